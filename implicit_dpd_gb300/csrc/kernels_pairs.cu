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
#include "pair_math.cuh"

namespace idpd {

__device__ __forceinline__ long long warp_sum_ll(long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// FP64 squared distance of rows i and j in the reference's operation order
// (nbdf_calculator.hpp:27-29, 86-87), j shifted to its image nearest to i.
// The image follows from the positions themselves, so it stays right while
// the cells are reused between list rebuilds.
__device__ __forceinline__ double exact_dr2(const DevState& d, const RepDev* R, uint32_t i,
                                            uint32_t j) {
  const double xi = d.px[i], yi = d.py[i], zi = d.pz[i];
  const double xj = d.px[j], yj = d.py[j], zj = d.pz[j];
  const int sx = nearest_image(xi, xj, R->box[0]), sy = nearest_image(yi, yj, R->box[1]),
            sz = nearest_image(zi, zj, R->box[2]);
  const double jx = __dadd_rn(xj, __dmul_rn((double)sx, R->box[0]));
  const double jy = __dadd_rn(yj, __dmul_rn((double)sy, R->box[1]));
  const double jz = __dadd_rn(zj, __dmul_rn((double)sz, R->box[2]));
  const double ex = __dsub_rn(xi, jx), ey = __dsub_rn(yi, jy), ez = __dsub_rn(zi, jz);
  return __dadd_rn(__dadd_rn(__dmul_rn(ex, ex), __dmul_rn(ey, ey)), __dmul_rn(ez, ez));
}

// ------------------------------------------------ neighbour segments
// A segment is a run of x-consecutive search cells of one (dy, dz) row with
// one image shift; its rows are contiguous in sorted order. The boundaries
// where the run enters a new frame cell give each candidate its x offset in
// frame cells (the unit of the stored cell-local coordinates).
constexpr int kMaxReach = 2;
constexpr int kMaxSeg = 2 * (2 * kMaxReach + 1) * (2 * kMaxReach + 1);  // 50
constexpr int kWarps = kRowBlock / 32;

struct SegTable {
  int tb[kMaxSeg], te[kMaxSeg];
  int bnd[kMaxSeg][2 * kMaxReach];  // first rows of the next frame cells (INT_MAX when absent)
  int code[kMaxSeg];  // frame offsets fx0+4 | (fy+4)<<3 | (fz+4)<<6, shifts (sx+1)<<9 | (sy+1)<<11 | (sz+1)<<13
};

// Lane k < (2m+1)^2 builds the (up to two) segments of row k of cell
// (cx, cy, cz); slots of a row that do not exist are left empty.
__device__ __forceinline__ void build_segments(SegTable& S, const DevState& d, const RepDev* R,
                                               int cx, int cy, int cz, int lane) {
  const int m = R->reach, w = 2 * m + 1, rs = R->rshift;
  const int nx = R->nc[0], ny = R->nc[1], nz = R->nc[2];
  for (int k = lane; k < w * w; k += 32) {
    const int dz = k / w - m, dy = k % w - m;
    const int qz = cz + dz, sz = qz < 0 ? -1 : (qz >= nz ? 1 : 0), wz = qz - sz * nz;
    const int qy = cy + dy, sy = qy < 0 ? -1 : (qy >= ny ? 1 : 0), wy = qy - sy * ny;
    const int base = R->cell_off + (wz * ny + wy) * nx;
    const int fy = (qy >> rs) - (cy >> rs), fz = (qz >> rs) - (cz >> rs);  // frame offsets
    // parts: [cx-m, -1] wrapped left (sx=-1), [max(cx-m,0), min(cx+m,nx-1)] (sx=0),
    // [nx, cx+m] wrapped right (sx=+1); at most two are non-empty.
    int slot = 2 * k;
    for (int part = -1; part <= 1; part++) {
      int lo, hi;  // unwrapped offsets lo..hi; wrapped index = cx + off - part * nx
      if (part == -1) {
        lo = -m;
        hi = -cx - 1;
      } else if (part == 0) {
        lo = cx - m < 0 ? -cx : -m;
        hi = cx + m >= nx ? nx - 1 - cx : m;
      } else {
        lo = nx - cx;
        hi = m;
      }
      if (lo > hi) continue;
      const int xs = cx + lo - part * nx;
      const int ncells = hi - lo + 1;
      S.tb[slot] = d.cell_start[base + xs];
      S.te[slot] = d.cell_start[base + xs + ncells];
      int nb = 0;
      for (int q = 1; q < ncells; q++)  // unwrapped search cell cx+lo+q starts a frame cell
        if (((cx + lo + q) & (m - 1)) == 0) S.bnd[slot][nb++] = d.cell_start[base + xs + q];
      for (; nb < 2 * kMaxReach; nb++) S.bnd[slot][nb] = 0x7fffffff;
      const int fx0 = ((cx + lo) >> rs) - (cx >> rs);
      S.code[slot] = (fx0 + 4) | ((fy + 4) << 3) | ((fz + 4) << 6) | ((part + 1) << 9) |
                     ((sy + 1) << 11) | ((sz + 1) << 13);
      slot++;
    }
    for (; slot < 2 * k + 2; slot++) {
      S.tb[slot] = 0;
      S.te[slot] = 0;
    }
  }
}

__device__ __forceinline__ int seg_dx(const SegTable& S, int g, int t) {
  int dx = (S.code[g] & 7) - 4;
#pragma unroll
  for (int q = 0; q < 2 * kMaxReach; q++) dx += t >= S.bnd[g][q];
  return dx;
}

struct PairCode {
  int dx, dy, dz, sx, sy, sz;
};
__device__ __forceinline__ uint32_t pack_code(int dx, int seg_code) {
  return (uint32_t)((dx + 4) | (seg_code & ~7));
}
__device__ __forceinline__ PairCode unpack_code(uint32_t c) {
  PairCode p;
  p.dx = (int)(c & 7) - 4;
  p.dy = (int)((c >> 3) & 7) - 4;
  p.dz = (int)((c >> 6) & 7) - 4;
  p.sx = (int)((c >> 9) & 3) - 1;
  p.sy = (int)((c >> 11) & 3) - 1;
  p.sz = (int)((c >> 13) & 3) - 1;
  return p;
}

// ------------------------------------------------------------- pass 1
// Neighbour list entry (32 bits): the candidate's sorted row (25 bits) and
// its frame cell's offset from the particle's frame cell, dx, dy, dz + 1 in
// 2 bits each. kNbrFallback marks a particle whose list did not fit (the
// next pass walks its cells again). Kept lists hold the candidates and
// pass-1 lists the pairs within the cutoff that the particle owns (owns()).
constexpr uint32_t kNbrFallback = 0xffffu;
constexpr int kRowBits = 25;
constexpr uint32_t kRowMask = (1u << kRowBits) - 1u;

// Both pair passes take each pair once, from the side of the particle that
// owns it: the frame offset dx of the other particle decides when nonzero,
// else (the same frame cell column) the larger cell-local x, else the larger
// sorted row. The x is that of the step (no kept lists) or of the kept
// lists' build (okey): rows and frame cells do not change between builds, so
// the two particles of a pair always agree. Each particle owns about half of
// its pairs (those on the +x side of the plane through it), which keeps the
// two particles of a half-warp pair in pass 2 near equal work.
__device__ __forceinline__ bool owns(int dx, float xj, float xi, int t, int s) {
  if (dx != 0) return dx > 0;
  return xj != xi ? xj > xi : t > s;
}

__device__ __forceinline__ uint32_t make_entry(int t, int dx, int dy, int dz) {
  return (uint32_t)t | ((uint32_t)(dx + 1) << kRowBits) | ((uint32_t)(dy + 1) << (kRowBits + 2)) |
         ((uint32_t)(dz + 1) << (kRowBits + 4));
}

__device__ __forceinline__ void read_entry(uint32_t e, int& t, int& dx, int& dy, int& dz) {
  t = (int)(e & kRowMask);
  dx = (int)((e >> kRowBits) & 3u) - 1;
  dy = (int)((e >> (kRowBits + 2)) & 3u) - 1;
  dz = (int)((e >> (kRowBits + 4)) & 3u) - 1;
}

template <int REACH>
__device__ __forceinline__ int frame_step(int t, const int* b) {
  int k = 0;
#pragma unroll
  for (int q = 0; q < 2 * REACH; q++) k += t >= b[q];
  return k;
}

// Density weight of one in-range pair, accumulated by the candidate's property.
__device__ __forceinline__ void add_weight(uint32_t& q0, uint32_t& q1, uint32_t& q2, uint32_t pr,
                                           uint32_t v) {
  q0 += pr == 0 ? v : 0u;
  q1 += pr == 1 ? v : 0u;
  q2 += pr == 2 ? v : 0u;
}

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
template <int REACH, bool VERLET, bool MARKS>
__global__ void __launch_bounds__(kRowBlock, 10) k_density_f32(DevState d) {
  __shared__ SegTable seg[kWarps];
  __shared__ uint32_t lst[kWarps][kNbrCap];
  const int r = d.blk_rep[blockIdx.x];
  const RepDev* R = d.reps + r;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  SegTable& S = seg[wid];
  uint32_t* L = lst[wid];
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
  for (int s = s0; s < s_end; s++) {
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
    if (VERLET && nv != kNbrFallback) {
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
      if (MARKS && hit) d.phit[s] = 1;
    }
    __syncwarp();
  }
}

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
// never queued. The warp of a 32-row chunk takes the cells whose first row
// lies in the chunk. Also records each row's delta_sumr for the displacement
// test.
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
  bool first = false;
  if (s0 + lane < s_end) first = d.cell_start[d.scell[s0 + lane]] == s0 + lane;
  uint32_t starts = __ballot_sync(0xffffffffu, first);
  while (starts) {
    const int cs = s0 + __ffs(starts) - 1;
    starts &= starts - 1;
    const int cell = (int)d.scell[cs];
    const int ce = d.cell_start[cell + 1];
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
  }
}

void launch_verlet_build(const DevState& d, int nblk, int reach, cudaStream_t st) {
  if (nblk == 0) return;
  if (reach == 2)
    k_verlet_build<2><<<nblk, kRowBlock, 0, st>>>(d);
  else
    k_verlet_build<1><<<nblk, kRowBlock, 0, st>>>(d);
}

// Visits every neighbour cell within the stencil of the given reach
// (plain FP64 kernels and the centre-of-mass pass).
template <class F>
__device__ __forceinline__ void for_each_cell(const RepDev* R, int reach, int cx, int cy, int cz,
                                              F&& f) {
  const int nx = R->nc[0], ny = R->nc[1], nz = R->nc[2];
  for (int dz = -reach; dz <= reach; dz++) {
    const int qz = cz + dz, sz = qz < 0 ? -1 : (qz >= nz ? 1 : 0), wz = qz - sz * nz;
    for (int dy = -reach; dy <= reach; dy++) {
      const int qy = cy + dy, sy = qy < 0 ? -1 : (qy >= ny ? 1 : 0), wy = qy - sy * ny;
      const int row = R->cell_off + (wz * ny + wy) * nx;
      for (int dx = -reach; dx <= reach; dx++) {
        const int qx = cx + dx, sx = qx < 0 ? -1 : (qx >= nx ? 1 : 0), wx = qx - sx * nx;
        f(row + wx, dx, dy, dz, sx, sy, sz);
      }
    }
  }
}

// Plain FP64 pass 1: FP64 positions of the storage rows, FP64 sums.
__global__ void __launch_bounds__(kRowBlock) k_density_f64(DevState d) {
  const int r = d.blk_rep[blockIdx.x];
  const int s = d.blk_row[blockIdx.x] + threadIdx.x;
  const RepDev* R = d.reps + r;
  if (s >= R->row_off + R->n) return;
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
  for_each_cell(R, R->reach, cx, cy, cz, [&](int cn, int, int, int, int sx, int sy, int sz) {
    const double shx = (double)sx * R->box[0], shy = (double)sy * R->box[1],
                 shz = (double)sz * R->box[2];
    for (int t = d.cell_start[cn]; t < d.cell_start[cn + 1]; t++) {
      const uint32_t j = d.perm[t];
      const double ex = xi - (d.px[j] + shx), ey = yi - (d.py[j] + shy), ez = zi - (d.pz[j] + shz);
      const double dr2 = ex * ex + ey * ey + ez * ez;
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
}

template <bool MARKS>
void launch_density_f32(const DevState& d, int nblk, int reach, bool verlet, cudaStream_t st) {
  if (verlet && reach == 2)
    k_density_f32<2, true, MARKS><<<nblk, kRowBlock, 0, st>>>(d);
  else if (verlet)
    k_density_f32<1, true, MARKS><<<nblk, kRowBlock, 0, st>>>(d);
  else if (reach == 2)
    k_density_f32<2, false, MARKS><<<nblk, kRowBlock, 0, st>>>(d);
  else
    k_density_f32<1, false, MARKS><<<nblk, kRowBlock, 0, st>>>(d);
}

void launch_density(const DevState& d, int nblk, bool fp64, int reach, bool verlet, bool marks,
                    size_t rows, cudaStream_t st) {
  if (nblk == 0) return;
  if (fp64) {
    k_density_f64<<<nblk, kRowBlock, 0, st>>>(d);
    return;
  }
  if (marks) {
    cudaMemsetAsync(d.phit, 0, rows, st);
    launch_density_f32<true>(d, nblk, reach, verlet, st);
  } else {
    launch_density_f32<false>(d, nblk, reach, verlet, st);
  }
  k_dens_finalize<<<nblk, kRowBlock, 0, st>>>(d);
}

// ------------------------------------------------------------- pass 2

// 1 - dr for a pair close to the cutoff, from the double-float cell-local
// coordinates (hi + lo) and the double-float cell side: every step below is
// an error-free transform or acts on terms below 1e-7, so 1 - dr^2 carries
// an absolute error near 1e-13 instead of the 1e-7 of the FP32 pair vector.
// The random term's sqrt(1 - r) amplifies the latter when r is near 1.
__device__ __forceinline__ float near_cut_w(float4 pi, float4 li, float4 pj, float4 lj, int dx,
                                            int dy, int dz, const RepDev* R, float dr) {
  const float hi_i[3] = {pi.x, pi.y, pi.z}, lo_i[3] = {li.x, li.y, li.z};
  const float hi_j[3] = {pj.x, pj.y, pj.z}, lo_j[3] = {lj.x, lj.y, lj.z};
  const int dk[3] = {dx, dy, dz};
  float p[3], err = 0.0f;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    float e1, e2, pe;
    const float s = two_sum(hi_i[k], -hi_j[k], e1);
    const float t = two_sum(s, -(float)dk[k] * R->cs_f[k], e2);
    const float lo = e1 + e2 + (lo_i[k] - lo_j[k]) - (float)dk[k] * R->cs_lo[k];
    p[k] = two_prod(t, t, pe);
    err += pe + 2.0f * t * lo;
  }
  float ea, eb;
  const float s1 = two_sum(p[0], p[1], ea);
  const float s2 = two_sum(s1, p[2], eb);
  const float w2 = (1.0f - s2) - (err + ea + eb);  // 1 - s2 is exact for s2 in [0.5, 2]
  return w2 / (1.0f + dr);
}

// The pair vector of a close pair from the double-float cell-local
// coordinates: the FP32 difference of the hi parts carries an absolute error
// near 1e-7, which is a large part of a vector a few hundredths long.
__device__ __forceinline__ void close_pair_vector(float4 pi, float4 li, float4 pj, float4 lj, int dx,
                                                  int dy, int dz, const RepDev* R, float& ex,
                                                  float& ey, float& ez) {
  const float hi_i[3] = {pi.x, pi.y, pi.z}, lo_i[3] = {li.x, li.y, li.z};
  const float hi_j[3] = {pj.x, pj.y, pj.z}, lo_j[3] = {lj.x, lj.y, lj.z};
  const int dk[3] = {dx, dy, dz};
  float e[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    float e1, e2;
    const float s = two_sum(hi_i[k], -hi_j[k], e1);
    const float t = two_sum(s, -(float)dk[k] * R->cs_f[k], e2);
    e[k] = t + (e1 + e2 + (lo_i[k] - lo_j[k]) - (float)dk[k] * R->cs_lo[k]);
  }
  ex = e[0];
  ey = e[1];
  ez = e[2];
}

// Pairs closer than 0.1 take their pair vector from close_pair_vector.
constexpr float kCloseCut2 = 0.01f;

// The particle of one (half) warp in pass 2 and its fixed-point sums.
struct PairI {
  float4 pi, vi, di;
  uint32_t idi, pri, seed;
  int row;  // the particle's row (its low position parts are read near the cutoff)
  float csx, csy, csz;
  long long fx, fy, fz, px, py, pz;
};

__device__ __forceinline__ void load_row(PairI& I, const DevState& d, int s) {
  I.pi = d.posf[s];
  I.vi = d.velf[s];
  I.di = d.densf[s];
  I.row = s;
  I.idi = fbits(I.vi.w);
  I.pri = fbits(I.pi.w);
}

// A lane's share of one fixed-point sum of pass 2 as the sums of the
// fix_force_parts of its terms. A list holds at most kNbrCap terms, so the
// parts' totals over a half warp stay below 2^30 and reduce in 32 bits.
struct FixSum {
  int hi, lo;
  __device__ __forceinline__ void add(float v, bool& range) {
    range &= fabsf(v) < 65536.0f;  // else the particle is summed again in 64 bits
    int h, l;
    fix_force_parts(v, h, l);
    hi += h;
    lo += l;
  }
  // the total over the lanes of half warp h (lanes 16 h .. 16 h + 15)
  __device__ __forceinline__ long long half_total(int h) const {
    const int hi0 = __reduce_add_sync(0xffffffffu, h ? 0 : hi);
    const int hi1 = __reduce_add_sync(0xffffffffu, h ? hi : 0);
    const int lo0 = __reduce_add_sync(0xffffffffu, h ? 0 : lo);
    const int lo1 = __reduce_add_sync(0xffffffffu, h ? lo : 0);
    return ((long long)(h ? hi1 : hi0) << 21) + (long long)(h ? lo1 : lo0);
  }
};
static_assert((long long)kNbrCap * (1 << 21) <= (1ll << 30), "32-bit totals of the fixed-point parts");

// The force and virial terms of one pair (the pair arithmetic of pass 2),
// from the side of the particle that owns the pair (a pair of equal ids is
// skipped, nbdf_calculator.hpp:84).
template <bool PRESS, bool CHECK, int FORM>
__device__ __forceinline__ bool pair_terms(const DevState& d, const RepDev* R, const PairTables& T,
                                           const PairI& I, int t, int dx, int dy, int dz,
                                           float g[6]) {
  const float4 vj = __ldg(d.velf + t);
  const uint32_t idj = fbits(vj.w);
  if (idj == I.idi) return false;
  const float4 pj = __ldg(d.posf + t);
  const float4 dj = __ldg(d.densf + t);
  float ex = (I.pi.x - (float)dx * I.csx) - pj.x;
  float ey = (I.pi.y - (float)dy * I.csy) - pj.y;
  float ez = (I.pi.z - (float)dz * I.csz) - pj.z;
  float dr2 = ex * ex + ey * ey + ez * ez;
  if (dr2 < kCloseCut2) {
    close_pair_vector(I.pi, __ldg(d.poslo + I.row), pj, __ldg(d.poslo + t), dx, dy, dz, R, ex, ey,
                      ez);
    dr2 = ex * ex + ey * ey + ez * ez;
  }
  const float inv_dr = rsqrtf(dr2);
  const float dr = dr2 * inv_dr;
  float w = 1.0f - dr;
  if (dr2 > kNearCut2)  // admitted pairs have 1 - r >= 0 up to ~1e-13
    w = fmaxf(near_cut_w(I.pi, __ldg(d.poslo + I.row), pj, __ldg(d.poslo + t), dx, dy, dz, R, dr),
              0.0f);
  const float a = pair_cf<FORM>(T, R, I.pri, fbits(pj.w), dr, inv_dr, w, ex, ey, ez, I.vi, vj,
                                I.di, dj, I.idi, idj, I.seed);
  // a non-finite term fails the range test of the 32-bit parts, and the 64-bit
  // pass (CHECK) reports it
  if (CHECK && !isfinite(a)) atomicCAS(d.err, 0, kErrNonFinite);
  g[0] = a * ex;
  g[1] = a * ey;
  g[2] = a * ez;
  if (PRESS) {
    g[3] = g[0] * ex;
    g[4] = g[1] * ey;
    g[5] = g[2] * ez;
  }
  return true;
}

__device__ __forceinline__ void red_add(long long* p, long long v) {
  atomicAdd(reinterpret_cast<unsigned long long*>(p), (unsigned long long)v);
}

// The other particle's share of one pair term: the force -g (the exact
// negation of the owner's fixed-point term) and the virial +g e.
template <bool PRESS>
__device__ __forceinline__ void add_to_other(const DevState& d, int t, const float g[6]) {
  red_add(d.fqx + t, -fix_force(g[0]));
  red_add(d.fqy + t, -fix_force(g[1]));
  red_add(d.fqz + t, -fix_force(g[2]));
  if (PRESS) {
    red_add(d.pqx + t, fix_force(g[3]));
    red_add(d.pqy + t, fix_force(g[4]));
    red_add(d.pqz + t, fix_force(g[5]));
  }
}

// One owned pair: the owner's term added to its sums in 32-bit parts, the
// other particle's term to its fixed-point sums in memory.
template <bool PRESS, int FORM>
__device__ __forceinline__ void eval_owned_parts(const DevState& d, const RepDev* R,
                                                 const PairTables& T, const PairI& I, int t,
                                                 int dx, int dy, int dz, FixSum f[6],
                                                 bool& range) {
  float g[6];
  if (!pair_terms<PRESS, false, FORM>(d, R, T, I, t, dx, dy, dz, g)) return;
#pragma unroll
  for (int c = 0; c < (PRESS ? 6 : 3); c++) f[c].add(g[c], range);
  add_to_other<PRESS>(d, t, g);
}

// One owned pair added to the owner's 64-bit sums (the lane's share) and,
// with OTHER, to the other particle's sums in memory.
template <bool PRESS, int FORM, bool OTHER>
__device__ __forceinline__ void eval_pair(const DevState& d, const RepDev* R, const PairTables& T,
                                          PairI& I, int t, int dx, int dy, int dz) {
  float g[6];
  if (!pair_terms<PRESS, true, FORM>(d, R, T, I, t, dx, dy, dz, g)) return;
  I.fx += fix_force(g[0]);
  I.fy += fix_force(g[1]);
  I.fz += fix_force(g[2]);
  if (PRESS) {
    I.px += fix_force(g[3]);
    I.py += fix_force(g[4]);
    I.pz += fix_force(g[5]);
  }
  if (OTHER) add_to_other<PRESS>(d, t, g);
}

// Each pair is evaluated once, by the particle that owns it (owns()), and
// its term goes to both particles (Newton's third law in exact fixed point: the
// sums equal those of the reference's two evaluations up to the FP32
// rounding of one of them). A warp takes two particles at a time, 16 lanes
// each, over their pass-1 lists (owned pairs only); the sums
// start at zero (launch_force) and every term arrives by atomic add. A
// particle whose list overflowed walks its cells again with the whole warp
// and queues the in-range pairs in shared memory; a particle with a term
// outside the 32-bit parts' range is summed again in 64 bits (its own side
// only). One launch per pair form present: a block whose replica has another
// form returns at once.
template <int REACH, bool PRESS, int FORM>
__global__ void __launch_bounds__(kRowBlock, 8) k_force_f32(DevState d, int kept) {
  __shared__ SegTable seg[kWarps];
  __shared__ uint32_t qt[kWarps][64], qc[kWarps][64];
  __shared__ PairTables T;
  const int r = d.blk_rep[blockIdx.x];
  const RepDev* R = d.reps + r;
  if (R->form != FORM) return;
  if (threadIdx.x < 9) fill_pair_table(T, *R, threadIdx.x);
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int h = lane >> 4, sl = lane & 15;
  SegTable& S = seg[wid];
  uint32_t* QT = qt[wid];
  uint32_t* QC = qc[wid];
  const int s0 = d.blk_row[blockIdx.x] + 32 * wid;
  const int s_end = min(s0 + 32, R->row_off + R->n);
  PairI I;
  I.seed = R->seed + d.rep_time[r];
  I.csx = R->cs_f[0];
  I.csy = R->cs_f[1];
  I.csz = R->cs_f[2];
  constexpr int nseg = 2 * (2 * REACH + 1) * (2 * REACH + 1);
  const uint32_t lt_mask = (1u << lane) - 1u;
  int cached = -1;
  for (int s2 = s0; s2 < s_end; s2 += 2) {
    // ---- two particles, 16 lanes each: the owned pairs of the lists
    const bool act = s2 + h < s_end;
    const int s = act ? s2 + h : s2;
    load_row(I, d, s);
    const uint32_t cnt = act ? (uint32_t)d.nbn[s] : 0u;
    const int nu = cnt != kNbrFallback ? (int)cnt : 0;
    const uint32_t* list = d.nbl + (size_t)s * kNbrCap;
    FixSum f[6];
#pragma unroll
    for (int c = 0; c < 6; c++) f[c].hi = f[c].lo = 0;
    bool range = true;
    for (int k = sl; k < nu; k += 16) {
      int t, dx, dy, dz;
      read_entry(list[k], t, dx, dy, dz);
      eval_owned_parts<PRESS, FORM>(d, R, T, I, t, dx, dy, dz, f, range);
    }
    __syncwarp();
    const uint32_t bad = __ballot_sync(0xffffffffu, !range);
    const bool ok = ((bad >> (16 * h)) & 0xffffu) == 0u;
    {
      const long long fx = f[0].half_total(h), fy = f[1].half_total(h), fz = f[2].half_total(h);
      long long px = 0, py = 0, pz = 0;
      if (PRESS) {
        px = f[3].half_total(h);
        py = f[4].half_total(h);
        pz = f[5].half_total(h);
      }
      if (sl == 0 && act && cnt != kNbrFallback && ok) {
        red_add(d.fqx + s, fx);
        red_add(d.fqy + s, fy);
        red_add(d.fqz + s, fz);
        if (PRESS) {
          red_add(d.pqx + s, px);
          red_add(d.pqy + s, py);
          red_add(d.pqz + s, pz);
        }
      }
    }
    // ---- the particles that need 64-bit sums, one at a time, whole warp
    uint32_t slow = __ballot_sync(0xffffffffu, sl == 0 && act && (cnt == kNbrFallback || !ok));
    while (slow) {
      const int ss = s2 + ((__ffs(slow) - 1) >> 4);
      slow &= slow - 1;
      load_row(I, d, ss);
      I.fx = I.fy = I.fz = I.px = I.py = I.pz = 0;
      const uint32_t c2 = d.nbn[ss];
      if (c2 != kNbrFallback) {  // a term outside the parts' range: the own side again
        const uint32_t* l2 = d.nbl + (size_t)ss * kNbrCap;
        const int n2 = (int)c2;
        for (int k = lane; k < n2; k += 32) {
          int t, dx, dy, dz;
          read_entry(l2[k], t, dx, dy, dz);
          eval_pair<PRESS, FORM, false>(d, R, T, I, t, dx, dy, dz);
        }
      } else {  // the list did not fit: walk the cells
        const int cell = (int)d.scell[ss];
        if (cell != cached) {  // the segments of the particle's cell (only this path walks cells)
          int cx, cy, cz;
          cell_xyz(cell - R->cell_off, R->nc, cx, cy, cz);
          __syncwarp();
          build_segments(S, d, R, cx, cy, cz, lane);
          __syncwarp();
          cached = cell;
        }
        int qn = 0;
#pragma unroll 1
        for (int g = 0; g < nseg; g++) {
          const int tb = S.tb[g], te = S.te[g];
          if (tb >= te) continue;
          const int code = S.code[g];
          int b[2 * REACH];
#pragma unroll
          for (int q = 0; q < 2 * REACH; q++) b[q] = S.bnd[g][q];
          const int fx0 = (code & 7) - 4, dy = ((code >> 3) & 7) - 4, dz = ((code >> 6) & 7) - 4;
          const float by = I.pi.y - (float)dy * I.csy, bz = I.pi.z - (float)dz * I.csz;
          for (int t0 = tb; t0 < te; t0 += 32) {
            const int t = t0 + lane;
            bool in = false, own = false;
            int dx = 0;
            bool near = false;
            if (t < te && t != ss) {
              const float4 pj = __ldg(d.posf + t);
              dx = fx0 + frame_step<REACH>(t, b);
              const float ex = (I.pi.x - (float)dx * I.csx) - pj.x, ey = by - pj.y,
                          ez = bz - pj.z;
              const float dr2 = ex * ex + ey * ey + ez * ez;
              in = dr2 < 1.0f;
              near = fabsf(dr2 - 1.0f) <= kGuard;
              own = owns(dx, kept ? d.okey[t] : pj.x, kept ? d.okey[ss] : I.pi.x, t, ss);
            }
            if (__any_sync(0xffffffffu, near) && near) {
              in = exact_dr2(d, R, d.perm[ss], d.perm[t]) < 1.0;
            }
            in = in && own;  // the pairs this particle owns
            const uint32_t mask = __ballot_sync(0xffffffffu, in);
            if (in) {
              const int pos = qn + __popc(mask & lt_mask);
              QT[pos] = (uint32_t)t;
              QC[pos] = pack_code(dx, code);
            }
            qn += __popc(mask);
            if (qn >= 32) {
              __syncwarp();
              const PairCode pc = unpack_code(QC[lane]);
              eval_pair<PRESS, FORM, true>(d, R, T, I, (int)QT[lane], pc.dx, pc.dy, pc.dz);
              __syncwarp();
              if (lane < qn - 32) {
                QT[lane] = QT[32 + lane];
                QC[lane] = QC[32 + lane];
              }
              __syncwarp();
              qn -= 32;
            }
          }
        }
        __syncwarp();
        if (lane < qn) {
          const PairCode pc = unpack_code(QC[lane]);
          eval_pair<PRESS, FORM, true>(d, R, T, I, (int)QT[lane], pc.dx, pc.dy, pc.dz);
        }
        __syncwarp();
      }
      const long long fx = warp_sum_ll(I.fx), fy = warp_sum_ll(I.fy), fz = warp_sum_ll(I.fz);
      long long px = 0, py = 0, pz = 0;
      if (PRESS) {
        px = warp_sum_ll(I.px);
        py = warp_sum_ll(I.py);
        pz = warp_sum_ll(I.pz);
      }
      if (lane == 0) {
        red_add(d.fqx + ss, fx);
        red_add(d.fqy + ss, fy);
        red_add(d.fqz + ss, fz);
        if (PRESS) {
          red_add(d.pqx + ss, px);
          red_add(d.pqy + ss, py);
          red_add(d.pqz + ss, pz);
        }
      }
    }
  }
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
  const double rd = T->wrd;
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
        const double dvx = vxi - d.vx[j], dvy = vyi - d.vy[j], dvz = vzi - d.vz[j];
        const uint32_t idj = d.id[j], prj = d.prop[j];
        const double dj0 = d.dens64[3 * t], dj1 = d.dens64[3 * t + 1], dj2 = d.dens64[3 * t + 2];
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
          const double wb = dr < rd ? 1.0 - dr / rd : 0.0;
          cons = T->wa * w + T->wb * rho * wb;
        } else {
          const double cf_pair = T->cf_c[k] * (dr - kArcD) * (double)(dr >= kArcD);
          double cf_mbd = 0.0;
          cf_mbd += T->cf_m[3 * k] * (di0 + dj0);
          cf_mbd += T->cf_m[3 * k + 1] * (di1 + dj1);
          cf_mbd += T->cf_m[3 * k + 2] * (di2 + dj2);
          cons = (cf_pair + cf_mbd) * w;
        }
        const double all = (cons + T->cf_r[k] * sqrt(w) * rnd -
                            T->cf_g[k] * w * (ex * dvx + ey * dvy + ez * dvz) * inv_dr) *
                           inv_dr;
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
  d.fqx[s] = __double2ll_rn(f0 * kForceScale);
  d.fqy[s] = __double2ll_rn(f1 * kForceScale);
  d.fqz[s] = __double2ll_rn(f2 * kForceScale);
  if (PRESS) {
    d.pqx[s] = __double2ll_rn(p0 * kForceScale);
    d.pqy[s] = __double2ll_rn(p1 * kForceScale);
    d.pqz[s] = __double2ll_rn(p2 * kForceScale);
  }
}

template <int FORM>
void launch_force_form(const DevState& d, int nblk, bool with_press, int reach, int kept,
                       cudaStream_t st) {
  if (reach == 2) {
    if (with_press)
      k_force_f32<2, true, FORM><<<nblk, kRowBlock, 0, st>>>(d, kept);
    else
      k_force_f32<2, false, FORM><<<nblk, kRowBlock, 0, st>>>(d, kept);
  } else {
    if (with_press)
      k_force_f32<1, true, FORM><<<nblk, kRowBlock, 0, st>>>(d, kept);
    else
      k_force_f32<1, false, FORM><<<nblk, kRowBlock, 0, st>>>(d, kept);
  }
}

void launch_force(const DevState& d, int nblk, bool fp64, bool with_press, bool kept,
                  const PairTuning& tu, int form_mask, size_t rows, cudaStream_t st) {
  if (nblk == 0) return;
  if (!fp64) {
    cudaMemsetAsync(d.fqx, 0, 3 * rows * sizeof(long long), st);
    if (with_press) cudaMemsetAsync(d.pqx, 0, 3 * rows * sizeof(long long), st);
  }
  if (fp64) {
    if (with_press)
      k_force_f64<true><<<nblk, kRowBlock, 0, st>>>(d);
    else
      k_force_f64<false><<<nblk, kRowBlock, 0, st>>>(d);
    return;
  }
  if (form_mask & (1 << IDPD_FORM_MDPD_K))
    launch_force_form<IDPD_FORM_MDPD_K>(d, nblk, with_press, tu.reach, kept ? 1 : 0, st);
  if (form_mask & (1 << IDPD_FORM_PAIRWISE_K))
    launch_force_form<IDPD_FORM_PAIRWISE_K>(d, nblk, with_press, tu.reach, kept ? 1 : 0, st);
  if (form_mask & (1 << IDPD_FORM_WARREN_K))
    launch_force_form<IDPD_FORM_WARREN_K>(d, nblk, with_press, tu.reach, kept ? 1 : 0, st);
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
