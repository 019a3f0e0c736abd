// The two MDPD passes over the cell list:
//   pass 1, CalcDensity::operator() (nbdf_calculator.hpp:11-60);
//   pass 2, CalcForceEpEpDPD::operator() (nbdf_calculator.hpp:63-145).
//
// FP32 passes (the engine): each pair is taken once, by the particle that
// owns it (owns()), and its term goes to both particles. Pass 1 runs one warp
// per particle over its kept list or its cells (the neighbour-cell segments
// cached in shared memory, swept 32 candidates at a time with coalesced
// float4 loads) and writes the owned pairs within the cutoff as the list of
// pass 2, which runs two particles per warp, 16 lanes each. Pair vectors come
// from cell-local FP32 coordinates; cutoff decisions within kGuard of the
// cutoff are re-taken in FP64 from the FP64 positions as the reference takes
// them; pairs within 0.01 of the cutoff take 1 - r from the compensated
// (hi + lo) coordinates; every pair term is summed as a 64-bit fixed-point
// integer, so the result is independent of the visiting order, of the cell
// size and of the launch shape.
//
// FP64 passes (the plain single-system baseline): one thread per particle,
// FP64 throughout, FP64 sums in cell order.
#include "pair_lists.cuh"

namespace idpd {

// One warp per particle, over the pairs it owns (owns(); the other particle
// gets the same weight by atomic add). Without kept lists: phase A sweeps the
// neighbour segments 32 candidates at a time and appends the owned pairs
// within the cutoff 1 to a list in shared memory; phase B takes the density
// weights from that list with every lane busy and copies the list out for
// pass 2 (a particle whose list overflows takes its weights during a second
// sweep). With kept lists (VERLET, owned candidates only): one pass over the
// particle's kept list tests each candidate, adds its weight and appends it
// to the list of pass 2. Each particle's own total is added to its sums in
// dsum as well; k_dens_finalize turns them into the FP32 densities.
// With MARKS, the precursor conversion's marks (phit): a pair of prop_from
// and prop_near within the cutoff marks the prop_from particle.
//
// Three forms (MODE): kDensSweep sweeps the cells of every row (no kept
// lists); kDensKept takes the rows whose kept list fit and uses no shared
// memory, which leaves the SM's L1 the room to cache the candidates' rows;
// kDensKeptOver takes the rows whose kept list did not fit and sweeps their
// cells (the ownership of the kept lists). The two kept-list forms run one
// after the other (with the sweep's 13.8 KB of shared memory per CTA in the
// kept-list kernel, pass 1 took 0.70 ms instead of 0.65 on membrane_1m). The sweeping forms keep per warp the neighbour segments
// and a list buffer in dynamic shared memory (dens_sweep_smem_bytes).
enum { kDensSweep = 0, kDensKept = 1, kDensKeptOver = 2 };
constexpr size_t dens_sweep_smem_bytes() {
  return kWarps * (sizeof(SegTable) + kNbrCap * sizeof(uint32_t));
}

template <int REACH, int MODE, bool MARKS>
__global__ void __launch_bounds__(kRowBlock, (MODE != kDensSweep && (REACH == 2 || MARKS)) ? 8 : 10) k_density_f32(DevState d) {
  constexpr bool VERLET = MODE != kDensSweep;
  extern __shared__ __align__(16) unsigned char dens_smem[];
  const int r = d.blk_rep[blockIdx.x];
  const RepDev* R = d.reps + r;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  SegTable& S = reinterpret_cast<SegTable*>(dens_smem)[wid];
  uint32_t* L = reinterpret_cast<uint32_t*>(dens_smem + kWarps * sizeof(SegTable)) + wid * kNbrCap;
  const int s0 = d.blk_row[blockIdx.x] + 32 * wid;
  const int s_end = min(s0 + 32, R->row_off + R->n);
  const bool warren = R->form == IDPD_FORM_WARREN_K;
  const float cutd2 = R->wrd * R->wrd;  // density cutoff^2 (1 unless Warren)
  const double cutd2d = (double)R->wrd * (double)R->wrd;
  const float inv_rd = R->winv_rd, wnorm = R->wnorm, pre = R->dens_prescale;
  const float csx = R->cs_f[0], csy = R->cs_f[1], csz = R->cs_f[2];
  const bool prec = MARKS && R->prec_on;
  constexpr int nseg = 2 * (2 * REACH + 1) * (2 * REACH + 1);
  const uint32_t lt_mask = (1u << lane) - 1u;
  int cached = -1;
  auto row = [&](const int s) {
    const float4 pi = d.posf[s];
    const uint32_t si = d.perm[s], pri = fbits(pi.w);
    const float ki = VERLET ? d.okey[s] : pi.x;  // the ownership key of the step
    int nl = 0;  // owned pairs within the cutoff
    int nw = 0;  // bound on the weighted pairs
    bool hit = false;
    uint32_t q0 = 0, q1 = 0, q2 = 0;
    // weight of one owned candidate, to both particles; called by every lane
    // together (valid = false for lanes without one) so that the rare FP64
    // recheck is warp-uniform. Returns whether the pair lies within the cutoff 1.
    auto test = [&](bool valid, int t, int dx, int dy, int dz, float4 pj, bool list_known) {
      const float ex = (pi.x - (float)dx * csx) - pj.x;
      const float ey = (pi.y - (float)dy * csy) - pj.y;
      const float ez = (pi.z - (float)dz * csz) - pj.z;
      const float dr2 = ex * ex + ey * ey + ez * ez;
      bool in1 = valid && (list_known || dr2 < 1.0f);
      bool ind = in1 && dr2 < cutd2 && dr2 >= 1.0e-10f;
      const bool near1 = valid && !list_known && fabsf(dr2 - 1.0f) <= kGuard;
      const bool near2 = valid && ((warren && fabsf(dr2 - cutd2) <= kGuard) || dr2 < 1.0e-10f);
      // rare: the FP64 decisions of the reference near the cutoffs and at
      // coincident positions (a warp-uniform branch keeps them out of the
      // common path)
      if (__any_sync(0xffffffffu, near1 || near2)) {
        if (near1 || near2) {
          const double e2 = exact_dr2(d, R, si, d.perm[t]);
          if (near1) in1 = e2 < 1.0;
          ind = in1 && (near2 ? (e2 < cutd2d && e2 != 0.0) : (dr2 < cutd2 && dr2 >= 1.0e-10f));
        }
      }
      const uint32_t prj = fbits(pj.w);
      if (ind) {
        const uint32_t w = dens_weight(dr2, warren, inv_rd, wnorm, pre);
        add_weight(q0, q1, q2, prj, w);
        atomicAdd(d.dsum + 4 * (size_t)t + (pri & 3u), (unsigned long long)w);
      }
      if (MARKS && prec && in1) {
        hit |= pri == R->prec_from && prj == R->prec_near;
        if (prj == R->prec_from && pri == R->prec_near) d.phit[t] = 1;
      }
      return in1;
    };
    const uint32_t nv = VERLET ? (uint32_t)d.vn[s] : kNbrFallback;
    bool fits = true;
    bool swept = true;  // the pairs came from a sweep of the cells (list out below)
    if constexpr (MODE == kDensKept) {
      // ---- the particle's kept list: test, weight and list out in one pass
      swept = false;
      const uint32_t* vl = d.vl + (size_t)s * kVerletCap;
      uint32_t* out = d.nbl + (size_t)s * kNbrCap;
      uint32_t e_next = lane < (int)nv ? vl[lane] : 0u;  // one round ahead
      for (int k0 = 0; k0 < (int)nv; k0 += 32) {
        const int k = k0 + lane;
        const bool valid = k < (int)nv;
        const uint32_t e = e_next;
        if (k + 32 < (int)nv) e_next = vl[k + 32];
        int t, dx, dy, dz;
        read_entry(e, t, dx, dy, dz);
        if (!valid) t = s;
        const bool in1 = test(valid, t, dx, dy, dz, __ldg(d.posf + t), false);
        const uint32_t mask = __ballot_sync(0xffffffffu, in1);
        if (in1) {
          const int pos = nl + __popc(mask & lt_mask);
          if (pos < kNbrCap) out[pos] = e;
        }
        nl += __popc(mask);
      }
      nw = (int)nv;
      fits = nl <= kNbrCap;
    } else {
      const int cell = (int)d.scell[s];
      if (cell != cached) {
        int cx, cy, cz;
        cell_xyz(cell - R->cell_off, R->nc, cx, cy, cz);
        __syncwarp();
        build_segments(S, d, R, cx, cy, cz, lane);
        __syncwarp();
        cached = cell;
      }
      // ---- phase A: the owned pairs within the cutoff 1
#pragma unroll 1
      for (int g = 0; g < nseg; g++) {
        const int tb = S.tb[g], te = S.te[g];
        if (tb >= te) continue;
        const int code = S.code[g];
        int b[2 * REACH];
#pragma unroll
        for (int q = 0; q < 2 * REACH; q++) b[q] = S.bnd[g][q];
        const int fx0 = (code & 7) - 4, dy = ((code >> 3) & 7) - 4, dz = ((code >> 6) & 7) - 4;
        const float by = pi.y - (float)dy * csy, bz = pi.z - (float)dz * csz;
        for (int t0 = tb; t0 < te; t0 += 32) {
          const int t = t0 + lane;
          bool in1 = false, near = false;
          int ddx = 0;
          if (t < te && t != s) {
            const float4 pj = __ldg(d.posf + t);
            ddx = frame_step<REACH>(t, b);
            if (owns(fx0 + ddx, VERLET ? d.okey[t] : pj.x, ki, t, s)) {
              const float ex = (pi.x - (float)(fx0 + ddx) * csx) - pj.x, ey = by - pj.y,
                          ez = bz - pj.z;
              const float dr2 = ex * ex + ey * ey + ez * ez;
              in1 = dr2 < 1.0f;
              near = fabsf(dr2 - 1.0f) <= kGuard;
            }
          }
          if (__any_sync(0xffffffffu, near)) {
            if (near) in1 = exact_dr2(d, R, si, d.perm[t]) < 1.0;
          }
          const uint32_t mask = __ballot_sync(0xffffffffu, in1);
          if (in1) {
            const int pos = nl + __popc(mask & lt_mask);
            if (pos < kNbrCap) L[pos] = make_entry(t, fx0 + ddx, dy, dz);
          }
          nl += __popc(mask);
        }
      }
      __syncwarp();
      fits = nl <= kNbrCap;
      nw = nl;
      // ---- phase B: density weights
      if (fits) {
        for (int k0 = 0; k0 < nl; k0 += 32) {
          const int k = k0 + lane;
          const bool valid = k < nl;
          int t = s, dx = 0, dy = 0, dz = 0;
          if (valid) read_entry(L[k], t, dx, dy, dz);
          test(valid, t, dx, dy, dz, valid ? __ldg(d.posf + t) : pi, true);
        }
      } else {
        // a lane takes at most nseg + nl / 32 weights below 2^23 each
        if (nl > kDensPairsMax && lane == 0) atomicCAS(d.err, 0, kErrDensPairs);
#pragma unroll 1
        for (int g = 0; g < nseg; g++) {
          const int tb = S.tb[g], te = S.te[g];
          if (tb >= te) continue;
          const int code = S.code[g];
          int b[2 * REACH];
#pragma unroll
          for (int q = 0; q < 2 * REACH; q++) b[q] = S.bnd[g][q];
          const int fx0 = (code & 7) - 4, dy = ((code >> 3) & 7) - 4, dz = ((code >> 6) & 7) - 4;
          for (int t0 = tb; t0 < te; t0 += 32) {
            const int t = t0 + lane;
            const int dx = fx0 + frame_step<REACH>(t, b);
            const float4 pj = t < te ? __ldg(d.posf + t) : pi;
            const bool valid =
                t < te && t != s && owns(dx, VERLET ? d.okey[t] : pj.x, ki, t, s);
            test(valid, valid ? t : s, dx, dy, dz, pj, false);
          }
        }
      }
    }
    __syncwarp();
    if (swept && fits) {  // list out for pass 2, coalesced
      uint32_t* out = d.nbl + (size_t)s * kNbrCap;
      for (int k = lane; k < nl; k += 32) out[k] = L[k];
    }
    // each weight is below 2^23, so up to 512 weighted pairs total below
    // 2^32 (nw bounds them: the kept list's length, or the pairs in range)
    unsigned long long a0, a1, a2;
    if (nw <= 512) {
      a0 = __reduce_add_sync(0xffffffffu, q0);
      a1 = __reduce_add_sync(0xffffffffu, q1);
      a2 = __reduce_add_sync(0xffffffffu, q2);
    } else {
      a0 = q0, a1 = q1, a2 = q2;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        a0 += __shfl_xor_sync(0xffffffffu, a0, o);
        a1 += __shfl_xor_sync(0xffffffffu, a1, o);
        a2 += __shfl_xor_sync(0xffffffffu, a2, o);
      }
    }
    if (MARKS) hit = __any_sync(0xffffffffu, hit);
    if (lane == 0) {
      unsigned long long* q = d.dsum + 4 * (size_t)s;
      if (a0) atomicAdd(q, a0);
      if (a1) atomicAdd(q + 1, a1);
      if (a2) atomicAdd(q + 2, a2);
      d.nbn[s] = fits ? (uint16_t)nl : (uint16_t)kNbrFallback;
      d.npair[s] = 2u * (uint32_t)nl;  // ordered pairs: each owned pair counts twice
      if (MARKS && hit) d.phit[s] = 1;
    }
    __syncwarp();
  };
  if constexpr (MODE == kDensKeptOver) {
    // the few rows whose kept list did not fit: lane k tests row s0 + k
    uint32_t rows = __ballot_sync(0xffffffffu, s0 + lane < s_end && d.vn[s0 + lane] == kNbrFallback);
    while (rows) {
      row(s0 + __ffs(rows) - 1);
      rows &= rows - 1;
    }
  } else {
    for (int s = s0; s < s_end; s++)
      if (MODE == kDensSweep || d.vn[s] != kNbrFallback) row(s);
  }
}

// Pass 1 over the kept lists with LP lanes per particle (LP 4, 8 or 16; 32 is
// k_density_f32's kDensKept form): for systems whose kept lists are short
// (a liquid at density 6 keeps ~20 owned candidates per particle), one warp
// per particle leaves most lanes idle and repeats the per-particle work (its
// row, the totals of its weights, its counts) for every particle. The warp
// sorts its 32 rows by kept-list length (as pass 2 does) and takes them
// 32 / LP at a time. Per candidate it does what k_density_f32 does over a
// kept list, and the pass-2 list comes out in the same order, so every LP
// gives the same densities and lists bit for bit. Rows whose kept list
// overflowed are left to kDensKeptOver.
template <int REACH, bool MARKS, int LP>
__global__ void __launch_bounds__(kRowBlock, 8) k_density_kept_lp(DevState d) {
  constexpr int G = 32 / LP;  // particles per warp at a time
  const int r = d.blk_rep[blockIdx.x];
  const RepDev* R = d.reps + r;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int h = lane / LP, sl = lane % LP;
  const int s0 = d.blk_row[blockIdx.x] + 32 * wid;
  const int s_end = min(s0 + 32, R->row_off + R->n);
  if (s0 >= s_end) return;
  const bool warren = R->form == IDPD_FORM_WARREN_K;
  const float cutd2 = R->wrd * R->wrd;  // density cutoff^2 (1 unless Warren)
  const double cutd2d = (double)R->wrd * (double)R->wrd;
  const float inv_rd = R->winv_rd, wnorm = R->wnorm, pre = R->dens_prescale;
  const float csx = R->cs_f[0], csy = R->cs_f[1], csz = R->cs_f[2];
  const bool prec = MARKS && R->prec_on;
  const uint32_t gmask = (LP == 32 ? 0xffffffffu : ((1u << LP) - 1u)) << (LP * h);
  const uint32_t group_lt = ((1u << lane) - 1u) & gmask;
  // the chunk's rows sorted by kept-list length (rows past the end and
  // overflowed lists count 0): key = length << 5 | row - s0
  uint32_t key;
  {
    const int sk = s0 + lane;
    const uint32_t c = sk < s_end ? (uint32_t)d.vn[sk] : 0u;
    key = ((c != kNbrFallback ? c : 0u) << 5) | (uint32_t)lane;
    key = warp_sort_asc(key, lane);
  }
  for (int i2 = 0; i2 < 32; i2 += G) {
    const int s2 = s0 + (int)(__shfl_sync(0xffffffffu, key, i2 + h) & 31u);
    const uint32_t nv0 = s2 < s_end ? (uint32_t)d.vn[s2] : kNbrFallback;
    const bool act = nv0 != kNbrFallback;
    if (!__any_sync(0xffffffffu, act)) continue;
    const int s = s2 < s_end ? s2 : s0;
    const int nv = act ? (int)nv0 : 0;
    int nmax = nv;  // rounds of the warp: the longest list of its groups
#pragma unroll
    for (int o = LP; o < 32; o <<= 1) nmax = max(nmax, __shfl_xor_sync(0xffffffffu, nmax, o));
    const float4 pi = d.posf[s];
    const uint32_t si = d.perm[s], pri = fbits(pi.w);
    int nl = 0;  // owned pairs within the cutoff
    bool hit = false;
    uint32_t q0 = 0, q1 = 0, q2 = 0;
    const uint32_t* vl = d.vl + (size_t)s * kVerletCap;
    uint32_t* out = d.nbl + (size_t)s * kNbrCap;
    uint32_t e_next = sl < nv ? vl[sl] : 0u;  // one round ahead
    for (int k0 = 0; k0 < nmax; k0 += LP) {
      const int k = k0 + sl;
      const bool valid = k < nv;
      const uint32_t e = e_next;
      if (k + LP < nv) e_next = vl[k + LP];
      int t, dx, dy, dz;
      read_entry(e, t, dx, dy, dz);
      if (!valid) t = s;
      const float4 pj = __ldg(d.posf + t);
      const float ex = (pi.x - (float)dx * csx) - pj.x;
      const float ey = (pi.y - (float)dy * csy) - pj.y;
      const float ez = (pi.z - (float)dz * csz) - pj.z;
      const float dr2 = ex * ex + ey * ey + ez * ez;
      bool in1 = valid && dr2 < 1.0f;
      bool ind = in1 && dr2 < cutd2 && dr2 >= 1.0e-10f;
      const bool near1 = valid && fabsf(dr2 - 1.0f) <= kGuard;
      const bool near2 = valid && ((warren && fabsf(dr2 - cutd2) <= kGuard) || dr2 < 1.0e-10f);
      // rare: the FP64 decisions of the reference near the cutoffs and at
      // coincident positions
      if (__any_sync(0xffffffffu, near1 || near2)) {
        if (near1 || near2) {
          const double e2 = exact_dr2(d, R, si, d.perm[t]);
          if (near1) in1 = e2 < 1.0;
          ind = in1 && (near2 ? (e2 < cutd2d && e2 != 0.0) : (dr2 < cutd2 && dr2 >= 1.0e-10f));
        }
      }
      const uint32_t prj = fbits(pj.w);
      if (ind) {
        const uint32_t w = dens_weight(dr2, warren, inv_rd, wnorm, pre);
        add_weight(q0, q1, q2, prj, w);
        atomicAdd(d.dsum + 4 * (size_t)t + (pri & 3u), (unsigned long long)w);
      }
      if (MARKS && prec && in1) {
        hit |= pri == R->prec_from && prj == R->prec_near;
        if (prj == R->prec_from && pri == R->prec_near) d.phit[t] = 1;
      }
      const uint32_t mask = __ballot_sync(0xffffffffu, in1);
      if (in1) {
        const int pos = nl + __popc(mask & group_lt);
        if (pos < kNbrCap) out[pos] = e;
      }
      nl += __popc(mask & gmask);
    }
    // the totals of each group's lanes: a kept list holds at most kVerletCap
    // (512) candidates, each weight is below 2^23, so a total is below 2^32
    uint32_t a0 = 0, a1 = 0, a2 = 0;
#pragma unroll
    for (int g = 0; g < G; g++) {
      const uint32_t t0 = __reduce_add_sync(0xffffffffu, h == g ? q0 : 0u);
      const uint32_t t1 = __reduce_add_sync(0xffffffffu, h == g ? q1 : 0u);
      const uint32_t t2 = __reduce_add_sync(0xffffffffu, h == g ? q2 : 0u);
      if (h == g) {
        a0 = t0;
        a1 = t1;
        a2 = t2;
      }
    }
    if (MARKS) hit = (__ballot_sync(0xffffffffu, hit) & gmask) != 0u;
    if (sl == 0 && act) {
      unsigned long long* q = d.dsum + 4 * (size_t)s;
      if (a0) atomicAdd(q, (unsigned long long)a0);
      if (a1) atomicAdd(q + 1, (unsigned long long)a1);
      if (a2) atomicAdd(q + 2, (unsigned long long)a2);
      d.nbn[s] = nl <= kNbrCap ? (uint16_t)nl : (uint16_t)kNbrFallback;
      d.npair[s] = 2u * (uint32_t)nl;  // ordered pairs: each owned pair counts twice
      if (MARKS && hit) d.phit[s] = 1;
    }
    __syncwarp();
  }
}
static_assert((long long)kVerletCap * (1ll << 23) <= (1ll << 32), "32-bit totals of pass 1");

// The FP32 densities of pass 1 from its fixed-point sums (and the fixed-point
// densities of the fine-grained API); the sums are zeroed for the next pass.
__global__ void __launch_bounds__(kRowBlock) k_dens_finalize(DevState d) {
  const int r = d.blk_rep[blockIdx.x];
  const int s = d.blk_row[blockIdx.x] + threadIdx.x;
  const RepDev* R = d.reps + r;
  if (s >= R->row_off + R->n) return;
  unsigned long long* q = d.dsum + 4 * (size_t)s;
  const long long a0 = (long long)q[0], a1 = (long long)q[1], a2 = (long long)q[2];
  const float u = R->dens_unscale_f;
  d.densf[s] = make_float4(fix_to_float(a0, u), fix_to_float(a1, u), fix_to_float(a2, u), 0.0f);
  if (d.dqx) {
    d.dqx[s] = a0;
    d.dqy[s] = a1;
    d.dqz[s] = a2;
  }
  q[0] = q[1] = q[2] = 0ull;
}

// The kept lists (rebuild steps only). The particles of one cell share its
// stencil of neighbour segments and, per candidate, the frame offset, so a
// warp takes one cell at a time and up to 32 of its particles at once: each
// lane loads one candidate, every particle of the batch is tested against
// the 32 candidates (one ballot per particle), and the lanes whose candidate
// is in range append it to that particle's list in one coalesced store. A
// candidate is kept when closer than 1 + skin in FP32 (with a margin: the
// list only has to hold every pair that can come within the cutoff before
// the next rebuild). Only the candidates the particle owns are kept (owns()
// on the cell-local x of the build, kept in okey): the stencil's -x third is
// never queued. Each warp builds the lists of exactly its 32-row chunk, one
// cell's share of the chunk at a time (a cell split between chunks has its
// stencil set up by each), so the warps of a CTA carry equal numbers of
// particles. Also records each row's delta_sumr for the displacement test.
template <int REACH>
__global__ void __launch_bounds__(kRowBlock) k_verlet_build(DevState d) {
  __shared__ SegTable seg[kWarps];
  __shared__ float4 bpos[kWarps][32];
  __shared__ float4 qpos[kWarps][64];
  __shared__ uint32_t qent[kWarps][64];
  if (!d.vdev->rebuild) return;
  const int r = d.blk_rep[blockIdx.x];
  const RepDev* R = d.reps + r;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  SegTable& S = seg[wid];
  float4* P = bpos[wid];
  float4* QX = qpos[wid];
  uint32_t* QE = qent[wid];
  const uint32_t lt_mask = (1u << lane) - 1u;
  const int s0 = d.blk_row[blockIdx.x] + 32 * wid;
  const int s_end = min(s0 + 32, R->row_off + R->n);
  const float rv2 = d.vdev->rv2;
  const float csx = R->cs_f[0], csy = R->cs_f[1], csz = R->cs_f[2];
  constexpr int nseg = 2 * (2 * REACH + 1) * (2 * REACH + 1);
  // the chunk's rows cell by cell: [cs, ce) are the chunk's rows of one cell
  for (int cs = s0; cs < s_end;) {
    const int cell = (int)d.scell[cs];
    const int ce = min(d.cell_start[cell + 1], s_end);
    int cx, cy, cz;
    cell_xyz(cell - R->cell_off, R->nc, cx, cy, cz);
    __syncwarp();
    build_segments(S, d, R, cx, cy, cz, lane);
    for (int b0 = cs; b0 < ce; b0 += 32) {
      const int nb = min(32, ce - b0);
      const int me = b0 + lane;  // the lane's particle (lane < nb)
      __syncwarp();
      const float4 pm = lane < nb ? d.posf[me] : d.posf[b0];
      P[lane] = pm;
      // the batch's bounding box: a candidate farther than 1 + skin from it
      // is no candidate of any particle of the batch (about a quarter of the
      // 27-cell stencil)
      float lox = pm.x, hix = pm.x, loy = pm.y, hiy = pm.y, loz = pm.z, hiz = pm.z;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        lox = fminf(lox, __shfl_xor_sync(0xffffffffu, lox, o));
        hix = fmaxf(hix, __shfl_xor_sync(0xffffffffu, hix, o));
        loy = fminf(loy, __shfl_xor_sync(0xffffffffu, loy, o));
        hiy = fmaxf(hiy, __shfl_xor_sync(0xffffffffu, hiy, o));
        loz = fminf(loz, __shfl_xor_sync(0xffffffffu, loz, o));
        hiz = fmaxf(hiz, __shfl_xor_sync(0xffffffffu, hiz, o));
      }
      __syncwarp();
      int cnt = 0;  // the list length of the lane's particle
      int qn = 0;   // candidates queued for the next full round
      // tests the 32 queued candidates against every particle of the batch:
      // the lanes whose candidate is in range of particle k write it to k's
      // list, consecutive lanes to consecutive slots
      auto round = [&](float qx, float qy, float qz, uint32_t e, int t) {
        const bool fwd = ((e >> kRowBits) & 3u) == 2u;  // frame offset +1: owned by all
#pragma unroll 4
        for (int k = 0; k < nb; k++) {
          const float4 pk = P[k];
          const float ex = pk.x - qx, ey = pk.y - qy, ez = pk.z - qz;
          // owns(): qx is the candidate's cell-local x when its offset is 0
          // (a particle never owns itself); predicate logic, no branches
          const bool own = fwd | (qx > pk.x) | ((qx == pk.x) & (t > b0 + k));
          const bool in = (ex * ex + ey * ey + ez * ez < rv2) & own;
          const uint32_t m = __ballot_sync(0xffffffffu, in);
          const int base = __shfl_sync(0xffffffffu, cnt, k);
          const int pos = base + __popc(m & lt_mask);
          if (in && pos < kVerletCap) d.vl[(size_t)(b0 + k) * kVerletCap + pos] = e;
          if (lane == k) cnt += __popc(m);
        }
      };
#pragma unroll 1
      for (int g = 0; g < nseg; g++) {
        const int tb = S.tb[g], te = S.te[g];
        if (tb >= te) continue;
        const int code = S.code[g];
        int b[2 * REACH];
#pragma unroll
        for (int q = 0; q < 2 * REACH; q++) b[q] = S.bnd[g][q];
        const int fx0 = (code & 7) - 4, dy = ((code >> 3) & 7) - 4, dz = ((code >> 6) & 7) - 4;
        for (int t0 = tb; t0 < te; t0 += 32) {
          const int t = t0 + lane;
          bool keep = false;
          float qx = 0.0f, qy = 0.0f, qz = 0.0f;
          uint32_t e = 0;
          if (t < te) {
            // the candidate in the frame of the cell's particles
            const float4 pj = __ldg(d.posf + t);
            const int fx = fx0 + frame_step<REACH>(t, b);
            qx = fmaf((float)fx, csx, pj.x);
            qy = fmaf((float)dy, csy, pj.y);
            qz = fmaf((float)dz, csz, pj.z);
            e = make_entry(t, fx, dy, dz);
            const float ox = fmaxf(fmaxf(lox - qx, qx - hix), 0.0f);
            const float oy = fmaxf(fmaxf(loy - qy, qy - hiy), 0.0f);
            const float oz = fmaxf(fmaxf(loz - qz, qz - hiz), 0.0f);
            keep = fx >= 0 && ox * ox + oy * oy + oz * oz < rv2;
          }
          const uint32_t mask = __ballot_sync(0xffffffffu, keep);
          if (keep) {
            const int at = qn + __popc(mask & lt_mask);
            QX[at] = make_float4(qx, qy, qz, __int_as_float(t));
            QE[at] = e;
          }
          qn += __popc(mask);
          if (qn >= 32) {
            __syncwarp();
            const float4 q = QX[lane];
            const uint32_t qe = QE[lane];
            __syncwarp();
            if (lane < qn - 32) {
              QX[lane] = QX[32 + lane];
              QE[lane] = QE[32 + lane];
            }
            __syncwarp();
            qn -= 32;
            round(q.x, q.y, q.z, qe, __float_as_int(q.w));
          }
        }
      }
      __syncwarp();
      if (qn > 0) {  // the last, partial round (absent lanes far away)
        float4 q = make_float4(1.0e30f, 0.0f, 0.0f, __int_as_float(-1));
        uint32_t qe = 0;
        if (lane < qn) {
          q = QX[lane];
          qe = QE[lane];
        }
        round(q.x, q.y, q.z, qe, __float_as_int(q.w));
      }
      __syncwarp();
      if (lane < nb) {
        d.vn[me] = cnt <= kVerletCap ? (uint16_t)cnt : (uint16_t)kNbrFallback;
        d.okey[me] = pm.x;
        const uint32_t i = d.perm[me];
        d.drx[me] = d.dsx[i];
        d.dry[me] = d.dsy[i];
        d.drz[me] = d.dsz[i];
      }
    }
    cs = ce;
  }
}

void launch_verlet_build(const DevState& d, int nblk, int reach, cudaStream_t st) {
  if (nblk == 0) return;
  if (reach == 2)
    k_verlet_build<2><<<nblk, kRowBlock, 0, st>>>(d);
  else
    k_verlet_build<1><<<nblk, kRowBlock, 0, st>>>(d);
}


// Plain FP64 pass 1 of one sorted row: FP64 positions of the storage rows,
// FP64 sums. Returns the row's ordered pairs within the cutoff 1.
__device__ __forceinline__ unsigned int density_f64_row(const DevState& d, int r, int s,
                                                        const RepDev* R) {
  const RepTab64* T = d.tab64 + r;
  const uint32_t i = d.perm[s];
  const double xi = d.px[i], yi = d.py[i], zi = d.pz[i];
  int cx, cy, cz;
  cell_xyz((int)d.scell[s] - R->cell_off, R->nc, cx, cy, cz);
  const bool warren = R->form == IDPD_FORM_WARREN_K;
  const double rd = T->wrd;
  const double cut2 = warren ? rd * rd : 1.0;
  const double wn = 15.0 / (2.0 * 3.14159265358979323846 * rd * rd * rd);
  double a0 = 0.0, a1 = 0.0, a2 = 0.0;
  unsigned int np = 0;  // ordered pairs within the cutoff 1
  for_each_cell(R, R->reach, cx, cy, cz, [&](int cn, int, int, int, int sx, int sy, int sz) {
    const double shx = (double)sx * R->box[0], shy = (double)sy * R->box[1],
                 shz = (double)sz * R->box[2];
    for (int t = d.cell_start[cn]; t < d.cell_start[cn + 1]; t++) {
      const uint32_t j = d.perm[t];
      const double ex = xi - (d.px[j] + shx), ey = yi - (d.py[j] + shy), ez = zi - (d.pz[j] + shz);
      const double dr2 = ex * ex + ey * ey + ez * ez;
      np += (dr2 < 1.0 && t != s) ? 1u : 0u;
      if (dr2 < cut2 && dr2 != 0.0) {
        const double dr = sqrt(dr2);
        double w;
        if (warren) {
          const double u = 1.0 - dr / rd;
          w = wn * (u * u);
        } else {
          w = (1.0 - dr) * (1.0 - dr);
        }
        const uint32_t pr = d.prop[j];
        if (pr == 0) a0 += w;
        else if (pr == 1) a1 += w;
        else a2 += w;
      }
    }
  });
  d.dens64[3 * s] = a0;
  d.dens64[3 * s + 1] = a1;
  d.dens64[3 * s + 2] = a2;
  d.densf[s] = make_float4((float)a0, (float)a1, (float)a2, 0.0f);
  if (d.dqx) {
    d.dqx[s] = __double2ll_rn(a0 / R->dens_unscale);
    d.dqy[s] = __double2ll_rn(a1 / R->dens_unscale);
    d.dqz[s] = __double2ll_rn(a2 / R->dens_unscale);
  }
  return np;
}

__global__ void __launch_bounds__(kRowBlock) k_density_f64(DevState d) {
  const int r = d.blk_rep[blockIdx.x];
  const int s = d.blk_row[blockIdx.x] + threadIdx.x;
  const RepDev* R = d.reps + r;
  if (s < R->row_off + R->n) d.npair[s] = density_f64_row(d, r, s, R);
}

template <int REACH, bool MARKS>
void launch_density_reach(const DevState& d, int nblk, bool verlet, int lanes, cudaStream_t st) {
  constexpr size_t sm = dens_sweep_smem_bytes();
  if (verlet) {
    if (lanes == 4)
      k_density_kept_lp<REACH, MARKS, 4><<<nblk, kRowBlock, 0, st>>>(d);
    else if (lanes == 8)
      k_density_kept_lp<REACH, MARKS, 8><<<nblk, kRowBlock, 0, st>>>(d);
    else if (lanes == 16)
      k_density_kept_lp<REACH, MARKS, 16><<<nblk, kRowBlock, 0, st>>>(d);
    else
      k_density_f32<REACH, kDensKept, MARKS><<<nblk, kRowBlock, 0, st>>>(d);
    k_density_f32<REACH, kDensKeptOver, MARKS><<<nblk, kRowBlock, sm, st>>>(d);
  } else {
    k_density_f32<REACH, kDensSweep, MARKS><<<nblk, kRowBlock, sm, st>>>(d);
  }
}

template <bool MARKS>
void launch_density_f32(const DevState& d, int nblk, int reach, bool verlet, int lanes,
                        cudaStream_t st) {
  if (reach == 2)
    launch_density_reach<2, MARKS>(d, nblk, verlet, lanes, st);
  else
    launch_density_reach<1, MARKS>(d, nblk, verlet, lanes, st);
}

// The reference's pair expression in FP64 (nbdf_calculator.hpp:84-132): the
// pair force over dr, for one pair within the cutoff, with the FP64 tables
// and the reference's FP64 Box-Muller.
__device__ __forceinline__ double pair_cf64(const RepTab64* T, int form, uint32_t pri,
                                            uint32_t prj, double dr2, double ex, double ey,
                                            double ez, double dvx, double dvy, double dvz,
                                            double di0, double di1, double di2, double dj0,
                                            double dj1, double dj2, uint32_t idi, uint32_t idj,
                                            uint32_t seed) {
  Saru sr(idi < idj ? idi : idj, idi < idj ? idj : idi, seed);
  const double rnd = saru_nrml_f64(sr);
  const double dr = sqrt(dr2);
  const double inv_dr = 1.0 / dr;
  const double w = 1.0 - dr;
  const int k = pri * 3 + prj;
  double cons;
  if (form == IDPD_FORM_PAIRWISE_K) {
    cons = 25.0 * w;
  } else if (form == IDPD_FORM_WARREN_K) {
    const double rho = (di0 + dj0) + (di1 + dj1) + (di2 + dj2);
    const double wb = dr < T->wrd ? 1.0 - dr / T->wrd : 0.0;
    cons = T->wa * w + T->wb * rho * wb;
  } else {
    const double cf_pair = T->cf_c[k] * (dr - kArcD) * (double)(dr >= kArcD);
    double cf_mbd = 0.0;
    cf_mbd += T->cf_m[3 * k] * (di0 + dj0);
    cf_mbd += T->cf_m[3 * k + 1] * (di1 + dj1);
    cf_mbd += T->cf_m[3 * k + 2] * (di2 + dj2);
    cons = (cf_pair + cf_mbd) * w;
  }
  return (cons + T->cf_r[k] * sqrt(w) * rnd -
          T->cf_g[k] * w * (ex * dvx + ey * dvy + ez * dvz) * inv_dr) *
         inv_dr;
}

// Plain FP64 pass 2 (the FP64 baseline): the reference's arithmetic on the
// FP64 rows with the FP64 coefficient tables, FP64 sums in cell order,
// stored in the engine's fixed point.
template <bool PRESS>
__global__ void __launch_bounds__(kRowBlock) k_force_f64(DevState d) {
  const int r = d.blk_rep[blockIdx.x];
  const int s = d.blk_row[blockIdx.x] + threadIdx.x;
  const RepDev* R = d.reps + r;
  if (s >= R->row_off + R->n) return;
  const RepTab64* T = d.tab64 + r;
  const uint32_t i = d.perm[s];
  const double xi = d.px[i], yi = d.py[i], zi = d.pz[i];
  const double vxi = d.vx[i], vyi = d.vy[i], vzi = d.vz[i];
  const uint32_t idi = d.id[i], pri = d.prop[i];
  const double di0 = d.dens64[3 * s], di1 = d.dens64[3 * s + 1], di2 = d.dens64[3 * s + 2];
  const uint32_t seed = R->seed + d.rep_time[r];
  const int form = R->form;
  int cx, cy, cz;
  cell_xyz((int)d.scell[s] - R->cell_off, R->nc, cx, cy, cz);
  double f0 = 0.0, f1 = 0.0, f2 = 0.0, p0 = 0.0, p1 = 0.0, p2 = 0.0;
  for_each_cell(R, R->reach, cx, cy, cz, [&](int cn, int, int, int, int sx, int sy, int sz) {
    const double shx = (double)sx * R->box[0], shy = (double)sy * R->box[1],
                 shz = (double)sz * R->box[2];
    for (int t = d.cell_start[cn]; t < d.cell_start[cn + 1]; t++) {
      const uint32_t j = d.perm[t];
      if (d.id[j] == idi) continue;
      const double ex = xi - (d.px[j] + shx), ey = yi - (d.py[j] + shy), ez = zi - (d.pz[j] + shz);
      const double dr2 = ex * ex + ey * ey + ez * ez;
      if (dr2 < 1.0) {
        const double all = pair_cf64(T, form, pri, d.prop[j], dr2, ex, ey, ez, vxi - d.vx[j],
                                     vyi - d.vy[j], vzi - d.vz[j], di0, di1, di2,
                                     d.dens64[3 * t], d.dens64[3 * t + 1], d.dens64[3 * t + 2],
                                     idi, d.id[j], seed);
        f0 += all * ex;
        f1 += all * ey;
        f2 += all * ez;
        if (PRESS) {
          p0 += all * ex * ex;
          p1 += all * ey * ey;
          p2 += all * ez * ez;
        }
      }
    }
  });
  long long* q = d.fq + 4 * (size_t)s;
  q[0] = __double2ll_rn(f0 * kForceScale);
  q[1] = __double2ll_rn(f1 * kForceScale);
  q[2] = __double2ll_rn(f2 * kForceScale);
  if (PRESS) {
    long long* pq = d.pq + 4 * (size_t)s;
    pq[0] = __double2ll_rn(p0 * kForceScale);
    pq[1] = __double2ll_rn(p1 * kForceScale);
    pq[2] = __double2ll_rn(p2 * kForceScale);
  }
}

// ================================================ FP64 engine algorithm
// The engine's algorithm with every pair term in FP64 (IDPD_CFG_FP64_KEPT):
// the same kept lists and rebuild schedule, the same ownership rule (each
// pair once, its term to both particles) and 64-bit fixed-point sums
// (densities in 2^-40, forces in 2^-26), with FP64 pair vectors from the
// cell-local coordinates (hi + lo of the packed split, exact to 2^-47
// relative), FP64 velocities and densities, the FP64 tables and the
// reference's FP64 Box-Muller. Pair-set decisions within 1e-10 of a cutoff
// take the reference's own FP64 distance. One warp per particle, cell reach 1.

__device__ __forceinline__ void pos64(const DevState& d, int s, double& x, double& y, double& z) {
  const float4 h = __ldg(d.posf + s), l = __ldg(d.poslo + s);
  x = (double)h.x + (double)l.x;
  y = (double)h.y + (double)l.y;
  z = (double)h.z + (double)l.z;
}

constexpr double kBand64 = 1.0e-10;

// Pass 1: over the kept list (VERLET) or the 27 cells, the owned candidates;
// each pair's weight goes to both particles, the pairs within the cutoff to
// the list of pass 2.
template <bool VERLET>
__global__ void __launch_bounds__(kRowBlock) k_density_kept64(DevState d) {
  const int r = d.blk_rep[blockIdx.x];
  const RepDev* R = d.reps + r;
  const RepTab64* T = d.tab64 + r;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int s0 = d.blk_row[blockIdx.x] + 32 * wid;
  const int s_end = min(s0 + 32, R->row_off + R->n);
  const bool warren = R->form == IDPD_FORM_WARREN_K;
  const double rd = T->wrd, cut2 = warren ? rd * rd : 1.0;
  const double wn = 15.0 / (2.0 * 3.14159265358979323846 * rd * rd * rd);
  const double csx = R->cs[0], csy = R->cs[1], csz = R->cs[2];
  const uint32_t lt_mask = (1u << lane) - 1u;
  for (int s = s0; s < s_end; s++) {
    double xi, yi, zi;
    pos64(d, s, xi, yi, zi);
    const uint32_t si = d.perm[s], pri = fbits(d.posf[s].w);
    const float ki = VERLET ? d.okey[s] : d.posf[s].x;
    long long q0 = 0, q1 = 0, q2 = 0;
    int nl = 0;
    uint32_t* out = d.nbl + (size_t)s * kNbrCap;
    // one owned candidate per lane, every lane together
    auto take = [&](bool valid, int t, int dx, int dy, int dz) {
      double dr2 = 4.0;
      uint32_t prj = 0;
      if (valid) {
        double xj, yj, zj;
        pos64(d, t, xj, yj, zj);
        prj = fbits(__ldg(d.posf + t).w);
        const double ex = (xi - (double)dx * csx) - xj, ey = (yi - (double)dy * csy) - yj,
                     ez = (zi - (double)dz * csz) - zj;
        dr2 = ex * ex + ey * ey + ez * ez;
      }
      bool in1 = valid && dr2 < 1.0;
      bool ind = valid && dr2 < cut2 && dr2 != 0.0;
      const bool near = valid && (fabs(dr2 - 1.0) < kBand64 || fabs(dr2 - cut2) < kBand64 ||
                                  dr2 < kBand64);
      if (__any_sync(0xffffffffu, near)) {
        if (near) {
          const double e2 = exact_dr2(d, R, si, d.perm[t]);
          in1 = e2 < 1.0;
          ind = e2 < cut2 && e2 != 0.0;
        }
      }
      if (ind) {
        const double dr = sqrt(dr2);
        double w;
        if (warren) {
          const double u = 1.0 - dr / rd;
          w = wn * (u * u);
        } else {
          w = (1.0 - dr) * (1.0 - dr);
        }
        const long long qw = __double2ll_rn(w * kDensScale);
        q0 += prj == 0 ? qw : 0ll;
        q1 += prj == 1 ? qw : 0ll;
        q2 += prj == 2 ? qw : 0ll;
        atomicAdd(d.dsum + 4 * (size_t)t + (pri & 3u), (unsigned long long)qw);
      }
      const uint32_t m = __ballot_sync(0xffffffffu, in1);
      if (in1) {
        const int pos = nl + __popc(m & lt_mask);
        if (pos < kNbrCap) out[pos] = make_entry(t, dx, dy, dz);
      }
      nl += __popc(m);
    };
    const uint32_t nv = VERLET ? (uint32_t)d.vn[s] : kNbrFallback;
    if (VERLET && nv != kNbrFallback) {
      const uint32_t* vl = d.vl + (size_t)s * kVerletCap;
      for (int k0 = 0; k0 < (int)nv; k0 += 32) {
        const int k = k0 + lane;
        const bool valid = k < (int)nv;
        int t = s, dx = 0, dy = 0, dz = 0;
        if (valid) read_entry(vl[k], t, dx, dy, dz);
        take(valid, t, dx, dy, dz);
      }
    } else {  // the 27 cells of the particle's cell (the build's cells with kept lists)
      int cx, cy, cz;
      cell_xyz((int)d.scell[s] - R->cell_off, R->nc, cx, cy, cz);
      for_each_cell(R, 1, cx, cy, cz, [&](int cn, int dx, int dy, int dz, int, int, int) {
        const int tb = d.cell_start[cn], te = d.cell_start[cn + 1];
        for (int t0 = tb; t0 < te; t0 += 32) {
          const int t = t0 + lane;
          const bool valid =
              t < te && t != s && owns(dx, VERLET ? d.okey[t] : __ldg(d.posf + t).x, ki, t, s);
          take(valid, valid ? t : s, dx, dy, dz);
        }
      });
    }
    q0 = warp_sum_ll(q0);
    q1 = warp_sum_ll(q1);
    q2 = warp_sum_ll(q2);
    if (lane == 0) {
      unsigned long long* q = d.dsum + 4 * (size_t)s;
      if (q0) atomicAdd(q, (unsigned long long)q0);
      if (q1) atomicAdd(q + 1, (unsigned long long)q1);
      if (q2) atomicAdd(q + 2, (unsigned long long)q2);
      d.nbn[s] = nl <= kNbrCap ? (uint16_t)nl : (uint16_t)kNbrFallback;
      d.npair[s] = 2u * (uint32_t)nl;
    }
    __syncwarp();
  }
}

// The FP64 densities of k_density_kept64 from its 2^-40 fixed-point sums
// (zeroed for the next pass).
__global__ void __launch_bounds__(kRowBlock) k_dens_finalize64(DevState d) {
  const int r = d.blk_rep[blockIdx.x];
  const int s = d.blk_row[blockIdx.x] + threadIdx.x;
  const RepDev* R = d.reps + r;
  if (s >= R->row_off + R->n) return;
  unsigned long long* q = d.dsum + 4 * (size_t)s;
  const double a0 = (double)(long long)q[0] * kDensUnscale,
               a1 = (double)(long long)q[1] * kDensUnscale,
               a2 = (double)(long long)q[2] * kDensUnscale;
  d.dens64[3 * s] = a0;
  d.dens64[3 * s + 1] = a1;
  d.dens64[3 * s + 2] = a2;
  d.densf[s] = make_float4((float)a0, (float)a1, (float)a2, 0.0f);
  if (d.dqx) {
    d.dqx[s] = __double2ll_rn(a0 / R->dens_unscale);
    d.dqy[s] = __double2ll_rn(a1 / R->dens_unscale);
    d.dqz[s] = __double2ll_rn(a2 / R->dens_unscale);
  }
  q[0] = q[1] = q[2] = 0ull;
}

// Pass 2: over the pass-1 list (or, when it overflowed, the owned pairs
// within the cutoff of the 27 cells), each pair's FP64 term rounded once to
// the 2^-26 fixed point: +q to the owner, -q to the other particle (the
// virial a e e to both). The sums start at zero (launch_force).
template <bool PRESS, bool VERLET>
__global__ void __launch_bounds__(kRowBlock) k_force_kept64(DevState d) {
  const int r = d.blk_rep[blockIdx.x];
  const RepDev* R = d.reps + r;
  const RepTab64* T = d.tab64 + r;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int s0 = d.blk_row[blockIdx.x] + 32 * wid;
  const int s_end = min(s0 + 32, R->row_off + R->n);
  const uint32_t seed = R->seed + d.rep_time[r];
  const int form = R->form;
  const double csx = R->cs[0], csy = R->cs[1], csz = R->cs[2];
  for (int s = s0; s < s_end; s++) {
    double xi, yi, zi;
    pos64(d, s, xi, yi, zi);
    const double* vi = d.svel + 4 * (size_t)s;
    const double vxi = vi[0], vyi = vi[1], vzi = vi[2];
    const double di0 = d.dens64[3 * s], di1 = d.dens64[3 * s + 1], di2 = d.dens64[3 * s + 2];
    const uint32_t idi = fbits(d.velf[s].w), pri = fbits(d.posf[s].w), si = d.perm[s];
    long long f[6] = {0, 0, 0, 0, 0, 0};
    auto eval = [&](int t, int dx, int dy, int dz) {
      const uint32_t idj = fbits(__ldg(d.velf + t).w);
      if (idj == idi) return;
      double xj, yj, zj;
      pos64(d, t, xj, yj, zj);
      const double ex = (xi - (double)dx * csx) - xj, ey = (yi - (double)dy * csy) - yj,
                   ez = (zi - (double)dz * csz) - zj;
      const double* vj = d.svel + 4 * (size_t)t;
      const double all = pair_cf64(T, form, pri, fbits(__ldg(d.posf + t).w),
                                   ex * ex + ey * ey + ez * ez, ex, ey, ez, vxi - vj[0],
                                   vyi - vj[1], vzi - vj[2], di0, di1, di2, d.dens64[3 * t],
                                   d.dens64[3 * t + 1], d.dens64[3 * t + 2], idi, idj, seed);
      const double g[3] = {all * ex, all * ey, all * ez};
      const double e[3] = {ex, ey, ez};
      long long* q = d.fq + 4 * (size_t)t;
#pragma unroll
      for (int c = 0; c < 3; c++) {
        const long long x = __double2ll_rn(g[c] * kForceScale);
        f[c] += x;
        red_add(q + c, -x);
      }
      if (PRESS) {
        long long* pq = d.pq + 4 * (size_t)t;
#pragma unroll
        for (int c = 0; c < 3; c++) {
          const long long x = __double2ll_rn(g[c] * e[c] * kForceScale);
          f[3 + c] += x;
          red_add(pq + c, x);
        }
      }
    };
    const uint32_t nu = d.nbn[s];
    if (nu != kNbrFallback) {
      const uint32_t* list = d.nbl + (size_t)s * kNbrCap;
      for (int k = lane; k < (int)nu; k += 32) {
        int t, dx, dy, dz;
        read_entry(list[k], t, dx, dy, dz);
        eval(t, dx, dy, dz);
      }
    } else {  // the list did not fit: the owned pairs within the cutoff of the 27 cells
      const float ki = VERLET ? d.okey[s] : d.posf[s].x;
      int cx, cy, cz;
      cell_xyz((int)d.scell[s] - R->cell_off, R->nc, cx, cy, cz);
      for_each_cell(R, 1, cx, cy, cz, [&](int cn, int dx, int dy, int dz, int, int, int) {
        const int tb = d.cell_start[cn], te = d.cell_start[cn + 1];
        for (int t0 = tb; t0 < te; t0 += 32) {
          const int t = t0 + lane;
          bool in = false, near = false;
          if (t < te && t != s &&
              owns(dx, VERLET ? d.okey[t] : __ldg(d.posf + t).x, ki, t, s)) {
            double xj, yj, zj;
            pos64(d, t, xj, yj, zj);
            const double ex = (xi - (double)dx * csx) - xj, ey = (yi - (double)dy * csy) - yj,
                         ez = (zi - (double)dz * csz) - zj;
            const double dr2 = ex * ex + ey * ey + ez * ez;
            in = dr2 < 1.0;
            near = fabs(dr2 - 1.0) < kBand64;
          }
          if (__any_sync(0xffffffffu, near)) {
            if (near) in = exact_dr2(d, R, si, d.perm[t]) < 1.0;
          }
          if (in) eval(t, dx, dy, dz);
        }
      });
    }
#pragma unroll
    for (int c = 0; c < (PRESS ? 6 : 3); c++) f[c] = warp_sum_ll(f[c]);
    if (lane == 0) {
      long long* q = d.fq + 4 * (size_t)s;
      red_add(q, f[0]);
      red_add(q + 1, f[1]);
      red_add(q + 2, f[2]);
      if (PRESS) {
        long long* pq = d.pq + 4 * (size_t)s;
        red_add(pq, f[3]);
        red_add(pq + 1, f[4]);
        red_add(pq + 2, f[5]);
      }
    }
    __syncwarp();
  }
}


// Sum of the per-row pair counts of rows [row0, row0 + n) (idpd_pair_count).
__global__ void __launch_bounds__(256) k_sum_pairs(const uint32_t* npair, int row0, int n,
                                                   unsigned long long* out) {
  unsigned long long v = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    v += npair[row0 + i];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0 && v) atomicAdd(out, v);
}

void launch_sum_pairs(const uint32_t* npair, int row0, int n, unsigned long long* out,
                      cudaStream_t st) {
  cudaMemsetAsync(out, 0, sizeof(unsigned long long), st);
  if (n > 0) k_sum_pairs<<<std::min((n + 255) / 256, 1024), 256, 0, st>>>(npair, row0, n, out);
}

void launch_force_fp64(const DevState& d, int nblk, int mode, bool with_press, bool kept,
                       cudaStream_t st) {
  if (mode == kPairsF64Kept) {
    if (with_press && kept)
      k_force_kept64<true, true><<<nblk, kRowBlock, 0, st>>>(d);
    else if (with_press)
      k_force_kept64<true, false><<<nblk, kRowBlock, 0, st>>>(d);
    else if (kept)
      k_force_kept64<false, true><<<nblk, kRowBlock, 0, st>>>(d);
    else
      k_force_kept64<false, false><<<nblk, kRowBlock, 0, st>>>(d);
  } else if (with_press) {
    k_force_f64<true><<<nblk, kRowBlock, 0, st>>>(d);
  } else {
    k_force_f64<false><<<nblk, kRowBlock, 0, st>>>(d);
  }
}

void launch_density(const DevState& d, int nblk, int mode, int reach, bool verlet, bool marks,
                    size_t rows, cudaStream_t st, int lanes) {
  if (nblk == 0) return;
  if (mode == kPairsF64) {
    k_density_f64<<<nblk, kRowBlock, 0, st>>>(d);
    return;
  }
  if (mode == kPairsF64Kept) {
    if (verlet)
      k_density_kept64<true><<<nblk, kRowBlock, 0, st>>>(d);
    else
      k_density_kept64<false><<<nblk, kRowBlock, 0, st>>>(d);
    k_dens_finalize64<<<nblk, kRowBlock, 0, st>>>(d);
    return;
  }
  if (marks) {
    cudaMemsetAsync(d.phit, 0, rows, st);
    launch_density_f32<true>(d, nblk, reach, verlet, lanes, st);
  } else {
    launch_density_f32<false>(d, nblk, reach, verlet, lanes, st);
  }
  k_dens_finalize<<<nblk, kRowBlock, 0, st>>>(d);
}

// ------------------------------------------- precursor conversion
// idpd_precursor: one warp per 32-row chunk, a particle at a time. A
// particle of prop_from looks for a particle of prop_near within the cutoff:
// the mark pass 1 left when it took such a pair (phit), or (FP64 arm) a sweep
// of the cells around it with the reference's FP64 distance. The draw is Saru(id, time, seed).u32() (saruprng.hpp:239-255,
// 322-333); properties change in the FP64 rows, so the pair passes see them
// from the next step's packing on.
__global__ void __launch_bounds__(kRowBlock) k_precursor(DevState d, int marks) {
  const int r = d.blk_rep[blockIdx.x];
  const RepDev* R = d.reps + r;
  if (!R->prec_on) return;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int s0 = d.blk_row[blockIdx.x] + 32 * wid;
  const int s_end = min(s0 + 32, R->row_off + R->n);
  const uint32_t from = R->prec_from, near_prop = R->prec_near;
  for (int s = s0; s < s_end; s++) {
    if (fbits(d.posf[s].w) != from) continue;
    bool near = false;
    if (marks) {
      near = d.phit[s] != 0;
    } else {
      const uint32_t i = d.perm[s];
      int cx, cy, cz;
      cell_xyz((int)d.scell[s] - R->cell_off, R->nc, cx, cy, cz);
      for_each_cell(R, R->reach, cx, cy, cz, [&](int c, int, int, int, int, int, int) {
        for (int t = d.cell_start[c] + lane; t < d.cell_start[c + 1]; t += 32)
          if (t != s && fbits(d.posf[t].w) == near_prop && exact_dr2(d, R, i, d.perm[t]) < 1.0)
            near = true;
      });
    }
    if (__any_sync(0xffffffffu, near) && lane == 0) {
      Saru g(fbits(d.velf[s].w), d.rep_time[r], R->prec_seed);
      if (g.next() < R->prec_thr) {
        d.prop[d.perm[s]] = R->prec_to;
        atomicAdd(d.prec_count + r, 1ull);
      }
    }
  }
}

void launch_precursor(const DevState& d, int nblk, bool marks, cudaStream_t st) {
  if (nblk > 0) k_precursor<<<nblk, kRowBlock, 0, st>>>(d, marks ? 1 : 0);
}

// -------------------------------------------- neighbour centre of mass
// The hydrophilic / hydrophobic neighbour sums of pass 1
// (nbdf_calculator.hpp:23-51) and FPDPD::copyFromForce (ptcl_class.hpp:53-57),
// for the fine-grained API and the chemistry: reach one more than the pair
// stencil (radius rn_c = 1.2), positions summed relative to the row's cell
// origin in 2^-40 fixed point, written per storage row.
__global__ void __launch_bounds__(kRowBlock) k_com(DevState d, double* cm, uint32_t* cnt_out) {
  const int r = d.blk_rep[blockIdx.x];
  const int s = d.blk_row[blockIdx.x] + threadIdx.x;
  const RepDev* R = d.reps + r;
  if (s >= R->row_off + R->n) return;
  const int reach = R->reach + 1;
  if (R->nc[0] < 2 * reach + 1 || R->nc[1] < 2 * reach + 1 || R->nc[2] < 2 * reach + 1) {
    atomicCAS(d.err, 0, kErrComBox);
    return;
  }
  const float4 pi = d.posf[s];
  int cx, cy, cz;
  cell_xyz((int)d.scell[s] - R->cell_off, R->nc, cx, cy, cz);
  const float rn2 = 1.44f;
  const double rn2d = 1.2 * 1.2;
  // hydrophilic sum starts at the row itself with count 1 (nbdf_calculator.hpp:23-24)
  long long hl[3] = {fix_from_float(pi.x, kPosBits), fix_from_float(pi.y, kPosBits),
                     fix_from_float(pi.z, kPosBits)};
  long long hb[3] = {0, 0, 0};
  uint32_t cl = 1, cb = 0;
  const uint32_t i = d.perm[s];
  const int rs = R->rshift;
  for_each_cell(R, reach, cx, cy, cz, [&](int cn, int dx, int dy, int dz, int sx, int sy, int sz) {
    // frame-cell offsets of the neighbour search cell
    const int fx = ((cx + dx) >> rs) - (cx >> rs), fy = ((cy + dy) >> rs) - (cy >> rs),
              fz = ((cz + dz) >> rs) - (cz >> rs);
    const float ox = (float)fx * R->cs_f[0], oy = (float)fy * R->cs_f[1],
                oz = (float)fz * R->cs_f[2];
    for (int t = d.cell_start[cn]; t < d.cell_start[cn + 1]; t++) {
      if (t == s) continue;
      const float4 pj = d.posf[t];
      const float jx = pj.x + ox, jy = pj.y + oy, jz = pj.z + oz;
      const float ex = pi.x - jx, ey = pi.y - jy, ez = pi.z - jz;
      const float dr2 = ex * ex + ey * ey + ez * ez;
      if (dr2 >= rn2 + kGuard) continue;
      bool in_b = dr2 < rn2, in_l = dr2 < 1.0f;
      if (fabsf(dr2 - rn2) <= kGuard || fabsf(dr2 - 1.0f) <= kGuard || dr2 < 1.0e-10f) {
        const double e2 = exact_dr2(d, R, i, d.perm[t]);
        in_b = e2 < rn2d && e2 != 0.0;
        in_l = in_b && e2 < 1.0;
      }
      const uint32_t pr = fbits(pj.w);
      if (in_b && pr == 1) {
        hb[0] += fix_from_float(jx, kPosBits);
        hb[1] += fix_from_float(jy, kPosBits);
        hb[2] += fix_from_float(jz, kPosBits);
        cb++;
      }
      if (in_l && pr == 0) {
        hl[0] += fix_from_float(jx, kPosBits);
        hl[1] += fix_from_float(jy, kPosBits);
        hl[2] += fix_from_float(jz, kPosBits);
        cl++;
      }
    }
  });
  const double org[3] = {(double)(cx >> rs) * R->cs[0], (double)(cy >> rs) * R->cs[1],
                         (double)(cz >> rs) * R->cs[2]};
  for (int k = 0; k < 3; k++) {
    cm[6 * i + k] = org[k] + ((double)hl[k] / kPosScale) / (double)cl;
    cm[6 * i + 3 + k] = org[k] + ((double)hb[k] / kPosScale) / (double)cb;
  }
  cnt_out[2 * i] = cl;
  cnt_out[2 * i + 1] = cb;
}

void launch_com(const DevState& d, int nblk, double* cm_out, uint32_t* cnt_out, cudaStream_t st) {
  if (nblk == 0) return;
  k_com<<<nblk, kRowBlock, 0, st>>>(d, cm_out, cnt_out);
}

}  // namespace idpd
