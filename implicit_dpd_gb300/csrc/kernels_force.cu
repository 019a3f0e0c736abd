// Pass 2 of the FP32 engine, CalcForceEpEpDPD::operator()
// (nbdf_calculator.hpp:63-145) with each pair taken once, by the particle
// that owns it, over the pass-1 lists; and the dispatch of every pass-2 arm.
#include "pair_lists.cuh"

namespace idpd {

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

// Frame-cell offsets (dx cs_x, dy cs_y, dz cs_z) of the 64 codes of a list
// entry's top bits (dx + 1 | (dy + 1) << 2 | (dz + 1) << 4): one shared load
// gives the shift of the other particle's cell-local coordinates. Each
// product is exact (dx in {-1, 0, 1}), so (x_i - off) - x_j rounds as the
// fused x_i - dx cs - x_j does.
struct OffTable {
  float4 o[64];
};

__device__ __forceinline__ void fill_off_table(OffTable& T, const RepDev& R, int c) {
  const float dx = (float)((c & 3) - 1), dy = (float)(((c >> 2) & 3) - 1),
              dz = (float)(((c >> 4) & 3) - 1);
  T.o[c] = make_float4(dx * R.cs_f[0], dy * R.cs_f[1], dz * R.cs_f[2], 0.0f);
}

// A lane's share of the owner's fixed-point sums of pass 2, kept as the sums
// of the fix_force_parts of its terms. A list holds at most kNbrCap terms, so
// the parts' totals over a half warp stay below 2^30 and reduce in 32 bits.
struct PartSums {
  int hi[6], lo[6];
};
static_assert((long long)kNbrCap * (1 << 21) <= (1ll << 30), "32-bit totals of the fixed-point parts");

// The total of parts c over the lanes of half warp h (lanes 16 h .. 16 h + 15).
__device__ __forceinline__ long long half_total(const PartSums& P, int c, int h) {
  const int hi0 = __reduce_add_sync(0xffffffffu, h ? 0 : P.hi[c]);
  const int hi1 = __reduce_add_sync(0xffffffffu, h ? P.hi[c] : 0);
  const int lo0 = __reduce_add_sync(0xffffffffu, h ? 0 : P.lo[c]);
  const int lo1 = __reduce_add_sync(0xffffffffu, h ? P.lo[c] : 0);
  return ((long long)(h ? hi1 : hi0) << 21) + (long long)(h ? lo1 : lo0);
}

// One component v of a pair term, converted to fixed point once for both
// particles: the owner subtracts its parts (its term is -v), the other
// particle's sum receives round(v 2^26) (NEG: -round(v 2^26)) by atomic add.
// A term beyond +-65536 goes to the other particle exactly (bit-level
// conversion) and marks the owner for the 64-bit sums.
template <bool NEG>
__device__ __forceinline__ void part_both(float v, int& hi, int& lo, long long* q, bool& range) {
  int h, l;
  fix_force_parts(v, h, l);
  hi -= h;
  lo -= l;
  long long x = (long long)h * 2097152ll + (long long)l;
  if (!(fabsf(v) < 65536.0f)) {
    x = fix_from_float(v, kForceBits);
    range = false;
  }
  red_add(q, NEG ? -x : x);
}

// One owned pair of a pass-1 list (fast path of pass 2), given the other
// particle's three rows (posf, velf, densf): the pair arithmetic runs in FP32
// (the compensated forms near the cutoff and for close pairs), and the term
// is split between the owner's 32-bit parts and the other particle's sums.
// A pair of equal ids contributes nothing (nbdf_calculator.hpp:84).
template <bool PRESS, int FORM>
__device__ __forceinline__ void owned_pair(const DevState& d, const RepDev* R, const PairTables& T,
                                           const OffTable& OT, const PairI& I, uint32_t e,
                                           float4 pj, float4 vj, float4 dj, PartSums& P,
                                           bool& range) {
  const int t = (int)(e & kRowMask);
  const float4 o = OT.o[e >> kRowBits];
  float ex = (I.pi.x - o.x) - pj.x;
  float ey = (I.pi.y - o.y) - pj.y;
  float ez = (I.pi.z - o.z) - pj.z;
  float dr2 = ex * ex + ey * ey + ez * ez;
  float inv_dr, dr, w;
  if (dr2 < kCloseCut2 || dr2 > kNearCut2) {  // rare: the compensated forms
    int tt, dx, dy, dz;
    read_entry(e, tt, dx, dy, dz);
    const float4 li = __ldg(d.poslo + I.row), lj = __ldg(d.poslo + t);
    if (dr2 < kCloseCut2) {
      close_pair_vector(I.pi, li, pj, lj, dx, dy, dz, R, ex, ey, ez);
      dr2 = ex * ex + ey * ey + ez * ez;
    }
    inv_dr = rsqrtf(dr2);
    dr = dr2 * inv_dr;
    w = 1.0f - dr;
    if (dr2 > kNearCut2)  // admitted pairs have 1 - r >= 0 up to ~1e-13
      w = fmaxf(near_cut_w(I.pi, li, pj, lj, dx, dy, dz, R, dr), 0.0f);
  } else {
    inv_dr = rsqrtf(dr2);
    dr = dr2 * inv_dr;
    w = 1.0f - dr;
  }
  const uint32_t idj = fbits(vj.w);
  const float a = pair_cf<FORM>(T, R, I.pri, fbits(pj.w), dr, inv_dr, w, ex, ey, ez, I.vi, vj,
                                I.di, dj, I.idi, idj, I.seed);
  const float an = idj == I.idi ? 0.0f : -a;  // the other particle's force is -a e
  const float gx = an * ex, gy = an * ey, gz = an * ez;
  long long* q = d.fq + 4 * (size_t)t;
  part_both<false>(gx, P.hi[0], P.lo[0], q, range);
  part_both<false>(gy, P.hi[1], P.lo[1], q + 1, range);
  part_both<false>(gz, P.hi[2], P.lo[2], q + 2, range);
  if (PRESS) {  // the virial a e e, the same for both particles
    long long* pq = d.pq + 4 * (size_t)t;
    part_both<true>(gx * ex, P.hi[3], P.lo[3], pq, range);
    part_both<true>(gy * ey, P.hi[4], P.lo[4], pq + 1, range);
    part_both<true>(gz * ez, P.hi[5], P.lo[5], pq + 2, range);
  }
}

// The force and virial terms of one pair (the pair arithmetic of pass 2),
// from the side of the particle that owns the pair (a pair of equal ids is
// skipped, nbdf_calculator.hpp:84); 64-bit path.
template <bool PRESS, bool CHECK, int FORM>
__device__ __forceinline__ bool pair_terms(const DevState& d, const RepDev* R, const PairTables& T,
                                           const PairI& I, int t, int dx, int dy, int dz,
                                           float g[6]) {
  const float4 vj = __ldg(d.velf + t);
  const float4 pj = __ldg(d.posf + t);
  const float4 dj = __ldg(d.densf + t);
  const uint32_t idj = fbits(vj.w);
  if (idj == I.idi) return false;
  float ex = (I.pi.x - (float)dx * R->cs_f[0]) - pj.x;
  float ey = (I.pi.y - (float)dy * R->cs_f[1]) - pj.y;
  float ez = (I.pi.z - (float)dz * R->cs_f[2]) - pj.z;
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
  // a non-finite term reports itself here (the fast path sends its particle
  // to this path through the range test of its parts)
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

// The other particle's share of one pair term: the force -g (the exact
// negation of the owner's fixed-point term) and the virial +g e.
template <bool PRESS>
__device__ __forceinline__ void add_to_other(const DevState& d, int t, const float g[6]) {
  long long* q = d.fq + 4 * (size_t)t;
  red_add(q, -fix_force(g[0]));
  red_add(q + 1, -fix_force(g[1]));
  red_add(q + 2, -fix_force(g[2]));
  if (PRESS) {
    long long* pq = d.pq + 4 * (size_t)t;
    red_add(pq, fix_force(g[3]));
    red_add(pq + 1, fix_force(g[4]));
    red_add(pq + 2, fix_force(g[5]));
  }
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

// The total of parts c over the LP lanes of group g (lanes LP g .. LP g + LP - 1).
template <int LP>
__device__ __forceinline__ long long group_total(const PartSums& P, int c, int g) {
  constexpr int G = 32 / LP;
  long long out = 0;
#pragma unroll
  for (int q = 0; q < G; q++) {
    const int hi = __reduce_add_sync(0xffffffffu, g == q ? P.hi[c] : 0);
    const int lo = __reduce_add_sync(0xffffffffu, g == q ? P.lo[c] : 0);
    if (g == q) out = ((long long)hi << 21) + (long long)lo;
  }
  return out;
}

// Shared memory of pass 2 (dynamic, sized by the launch): per 128-row block
// its replica's tables, per warp the segments and the queue of the
// cell-walk path.
struct ForceBlockSmem {
  PairTables T;
  OffTable OT;
};
struct ForceWarpSmem {
  SegTable seg;
  uint32_t qt[64], qc[64];
};



size_t force_smem_bytes(int fb) { return (size_t)fb * sizeof(ForceBlockSmem); }

// Each pair is evaluated once, by the particle that owns it (owns()), and
// its term goes to both particles (Newton's third law in exact fixed point: the
// sums equal those of the reference's two evaluations up to the FP32
// rounding of one of them). A warp takes the 32 particles of its chunk 32 / LP
// at a time, LP lanes each, over their pass-1 lists (owned pairs only),
// grouped by list length (the chunk sorted by length, neighbours in that
// order share a warp) so that the groups run about as long; each lane reads
// its next list entry one round ahead. The sums start at zero (launch_force)
// and every term arrives by atomic add. A particle with a term outside the
// 32-bit parts' range is summed again in 64 bits (its own side only). A
// particle whose list overflowed is left to k_force_walk, so that this pass
// keeps no walk state: no spills at 64 registers, and only the replica
// tables in shared memory, which leaves the SM's L1 the room to cache the
// other particles' rows (with the walk's 7.6 KB of shared memory per CTA in
// the same kernel the pass took 1.15 ms instead of 1.08 on membrane_1m).
// One launch per pair form present: a warp whose replica has another form
// returns at once.
//
// Pass 2 over the rows s0 .. s0 + 31 of replica r (one warp's chunk), the
// particles whose pass-1 list fit: G particles at a time, LP lanes each.
template <int REACH, bool PRESS, int FORM, int LP>
__device__ __forceinline__ void force_rows(const DevState& d, int s0, int r, const RepDev* R,
                                           const PairTables& T, const OffTable& OT, int lane) {
  constexpr int G = 32 / LP;  // particles per warp at a time
  const int h = lane / LP, sl = lane % LP;
  const int s_end = min(s0 + 32, R->row_off + R->n);
  if (s0 >= s_end) return;
  PairI I;
  I.seed = R->seed + d.rep_time[r];
  constexpr uint32_t group_mask = LP == 32 ? 0xffffffffu : ((1u << LP) - 1u);
  // the chunk's rows sorted by the length of their lists (rows past the end
  // and overflowed lists count 0): key = length << 5 | row - s0
  uint32_t key;
  {
    const int sk = s0 + lane;
    const uint32_t c = sk < s_end ? (uint32_t)d.nbn[sk] : 0u;
    key = ((c != kNbrFallback ? c : 0u) << 5) | (uint32_t)lane;
    key = warp_sort_asc(key, lane);
  }
  for (int i2 = 0; i2 < 32; i2 += G) {
    // ---- G particles, LP lanes each: the owned pairs of the lists
    const int s2 = s0 + (int)(__shfl_sync(0xffffffffu, key, i2 + h) & 31u);
    const bool act = s2 < s_end;
    const int s = act ? s2 : s0;
    load_row(I, d, s);
    const uint32_t cnt = act ? (uint32_t)d.nbn[s] : 0u;
    const int nu = cnt != kNbrFallback ? (int)cnt : 0;
    const uint32_t* list = d.nbl + (size_t)s * kNbrCap;
    PartSums P;
#pragma unroll
    for (int c = 0; c < 6; c++) P.hi[c] = P.lo[c] = 0;
    bool range = true;
    uint32_t e_next = sl < nu ? __ldg(list + sl) : 0u;  // one round ahead
    for (int k = sl; k < nu; k += LP) {
      const uint32_t e = e_next;
      if (k + LP < nu) e_next = __ldg(list + k + LP);
      const int t = (int)(e & kRowMask);
      owned_pair<PRESS, FORM>(d, R, T, OT, I, e, __ldg(d.posf + t), __ldg(d.velf + t),
                              __ldg(d.densf + t), P, range);
    }
    __syncwarp();
    const uint32_t bad = __ballot_sync(0xffffffffu, !range);
    const bool ok = ((bad >> (LP * h)) & group_mask) == 0u;
    {
      const long long fx = group_total<LP>(P, 0, h), fy = group_total<LP>(P, 1, h),
                      fz = group_total<LP>(P, 2, h);
      long long px = 0, py = 0, pz = 0;
      if (PRESS) {
        px = group_total<LP>(P, 3, h);
        py = group_total<LP>(P, 4, h);
        pz = group_total<LP>(P, 5, h);
      }
      if (sl == 0 && act && cnt != kNbrFallback && ok) {
        long long* q = d.fq + 4 * (size_t)s;
        red_add(q, fx);
        red_add(q + 1, fy);
        red_add(q + 2, fz);
        if (PRESS) {
          long long* pq = d.pq + 4 * (size_t)s;
          red_add(pq, px);
          red_add(pq + 1, py);
          red_add(pq + 2, pz);
        }
      }
    }
    // ---- a term outside the parts' range: the particle's own side again in
    // 64 bits, one particle at a time, whole warp (the other particles'
    // shares are already in memory)
    uint32_t slow = __ballot_sync(0xffffffffu, sl == 0 && act && cnt != kNbrFallback && !ok);
    while (slow) {
      const int hs = (__ffs(slow) - 1) / LP;
      slow &= slow - 1;
      const int ss = __shfl_sync(0xffffffffu, s, LP * hs);
      load_row(I, d, ss);
      I.fx = I.fy = I.fz = I.px = I.py = I.pz = 0;
      const uint32_t* l2 = d.nbl + (size_t)ss * kNbrCap;
      const int n2 = (int)d.nbn[ss];
      for (int k = lane; k < n2; k += 32) {
        int t, dx, dy, dz;
        read_entry(l2[k], t, dx, dy, dz);
        eval_pair<PRESS, FORM, false>(d, R, T, I, t, dx, dy, dz);
      }
      const long long fx = warp_sum_ll(I.fx), fy = warp_sum_ll(I.fy), fz = warp_sum_ll(I.fz);
      long long px = 0, py = 0, pz = 0;
      if (PRESS) {
        px = warp_sum_ll(I.px);
        py = warp_sum_ll(I.py);
        pz = warp_sum_ll(I.pz);
      }
      if (lane == 0) {
        long long* q = d.fq + 4 * (size_t)ss;
        red_add(q, fx);
        red_add(q + 1, fy);
        red_add(q + 2, fz);
        if (PRESS) {
          long long* pq = d.pq + 4 * (size_t)ss;
          red_add(pq, px);
          red_add(pq + 1, py);
          red_add(pq + 2, pz);
        }
      }
    }
  }
}

// Pass 2 for the particles of the chunk s0 .. s0 + 31 whose pass-1 list did
// not fit (more than kNbrCap owned pairs, only at extreme densities): one at
// a time, the whole warp walks the particle's cells again and queues its
// owned in-range pairs in shared memory; each term goes to both particles.
template <int REACH, bool PRESS, int FORM>
__device__ __forceinline__ void force_walk_rows(const DevState& d, int kept, int s0, int r,
                                                const RepDev* R, const PairTables& T,
                                                ForceWarpSmem& W, int lane) {
  const int s_end = min(s0 + 32, R->row_off + R->n);
  if (s0 >= s_end) return;
  SegTable& S = W.seg;
  uint32_t* QT = W.qt;
  uint32_t* QC = W.qc;
  PairI I;
  I.seed = R->seed + d.rep_time[r];
  constexpr int nseg = 2 * (2 * REACH + 1) * (2 * REACH + 1);
  const uint32_t lt_mask = (1u << lane) - 1u;
  int cached = -1;
  uint32_t slow = __ballot_sync(0xffffffffu, s0 + lane < s_end && d.nbn[s0 + lane] == kNbrFallback);
  while (slow) {
    const int ss = s0 + __ffs(slow) - 1;
    slow &= slow - 1;
    load_row(I, d, ss);
    I.fx = I.fy = I.fz = I.px = I.py = I.pz = 0;
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
      const float by = I.pi.y - (float)dy * R->cs_f[1], bz = I.pi.z - (float)dz * R->cs_f[2];
      for (int t0 = tb; t0 < te; t0 += 32) {
        const int t = t0 + lane;
        bool in = false, own = false;
        int dx = 0;
        bool near = false;
        if (t < te && t != ss) {
          const float4 pj = __ldg(d.posf + t);
          dx = fx0 + frame_step<REACH>(t, b);
          const float ex = (I.pi.x - (float)dx * R->cs_f[0]) - pj.x, ey = by - pj.y,
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
    const long long fx = warp_sum_ll(I.fx), fy = warp_sum_ll(I.fy), fz = warp_sum_ll(I.fz);
    long long px = 0, py = 0, pz = 0;
    if (PRESS) {
      px = warp_sum_ll(I.px);
      py = warp_sum_ll(I.py);
      pz = warp_sum_ll(I.pz);
    }
    if (lane == 0) {
      long long* q = d.fq + 4 * (size_t)ss;
      red_add(q, fx);
      red_add(q + 1, fy);
      red_add(q + 2, fz);
      if (PRESS) {
        long long* pq = d.pq + 4 * (size_t)ss;
        red_add(pq, px);
        red_add(pq + 1, py);
        red_add(pq + 2, pz);
      }
    }
  }
}

// Pass 2, grid order: CTA b takes row blocks b fb .. b fb + fb - 1, one warp
// per 32-row chunk. Its shared memory is the replica tables only (1.2 KB per
// row block), which leaves most of the SM's 256 KB of L1 and shared memory
// to the L1 that caches the other particles' rows.
template <int REACH, bool PRESS, int FORM, int LP>
__global__ void __launch_bounds__(1024, 1) k_force_f32(DevState d, int nblk) {
  extern __shared__ __align__(16) unsigned char force_smem[];
  ForceBlockSmem* BS = reinterpret_cast<ForceBlockSmem*>(force_smem);
  const int fb = blockDim.x >> 7;  // 128-row blocks of this CTA
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int rbl = wid / kWarps;              // the warp's row block within the CTA
  const int rb = blockIdx.x * fb + rbl;      // in the row-block map
  const int r = rb < nblk ? d.blk_rep[rb] : 0;
  const RepDev* R = d.reps + r;
  if (rb < nblk) {
    const int tb = threadIdx.x & (kRowBlock - 1);
    if (tb < 9) fill_pair_table(BS[rbl].T, *R, tb);
    if (tb < 64) fill_off_table(BS[rbl].OT, *R, tb);
  }
  __syncthreads();
  if (rb >= nblk || R->form != FORM) return;
  force_rows<REACH, PRESS, FORM, LP>(d, d.blk_row[rb] + 32 * (wid % kWarps), r, R, BS[rbl].T,
                                     BS[rbl].OT, lane);
}

// Pass 2 of the particles whose list overflowed (force_walk_rows), one warp
// per 32-row chunk, 128-row blocks per CTA; a chunk without such a particle
// costs one read of its list lengths.
template <int REACH, bool PRESS, int FORM>
__global__ void __launch_bounds__(kRowBlock) k_force_walk(DevState d, int kept, int nblk) {
  __shared__ ForceBlockSmem B;
  __shared__ ForceWarpSmem W[kWarps];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int rb = blockIdx.x;
  const int r = d.blk_rep[rb];
  const RepDev* R = d.reps + r;
  if (threadIdx.x < 9) fill_pair_table(B.T, *R, threadIdx.x);
  __syncthreads();
  if (R->form != FORM) return;
  force_walk_rows<REACH, PRESS, FORM>(d, kept, d.blk_row[rb] + 32 * wid, r, R, B.T, W[wid], lane);
}

// Pass 2 of one pair form: the shape of the tuning (lanes per particle,
// row blocks per CTA); the observation steps (PRESS) run 16 lanes, one row
// block per CTA.
template <int REACH, int FORM, bool PRESS, int LP>
void launch_force_kernel(const DevState& d, int nblk, int kept, int fb, cudaStream_t st) {
  k_force_f32<REACH, PRESS, FORM, LP>
      <<<(nblk + fb - 1) / fb, kRowBlock * fb, force_smem_bytes(fb), st>>>(d, nblk);
  k_force_walk<REACH, PRESS, FORM><<<nblk, kRowBlock, 0, st>>>(d, kept, nblk);
}

template <int FORM, bool PRESS, int LP>
void launch_force_shape(const DevState& d, int nblk, int reach, int kept, int fb,
                        cudaStream_t st) {
  if (reach == 2)
    launch_force_kernel<2, FORM, PRESS, LP>(d, nblk, kept, fb, st);
  else
    launch_force_kernel<1, FORM, PRESS, LP>(d, nblk, kept, fb, st);
}

template <int FORM>
void launch_force_form(const DevState& d, int nblk, bool with_press, const PairTuning& tu,
                       int kept, cudaStream_t st) {
  if (with_press) {
    launch_force_shape<FORM, true, 16>(d, nblk, tu.reach, kept, 1, st);
    return;
  }
  const int fb = tu.fblk == 2 || tu.fblk == 4 ? tu.fblk : 1;
  if (tu.lanes == 4)
    launch_force_shape<FORM, false, 4>(d, nblk, tu.reach, kept, fb, st);
  else if (tu.lanes == 8)
    launch_force_shape<FORM, false, 8>(d, nblk, tu.reach, kept, fb, st);
  else if (tu.lanes == 32)
    launch_force_shape<FORM, false, 32>(d, nblk, tu.reach, kept, fb, st);
  else
    launch_force_shape<FORM, false, 16>(d, nblk, tu.reach, kept, fb, st);
}

void launch_force(const DevState& d, int nblk, int mode, bool with_press, bool kept,
                  const PairTuning& tu, int form_mask, size_t rows, cudaStream_t st) {
  if (nblk == 0) return;
  if (mode != kPairsF64) {
    cudaMemsetAsync(d.fq, 0, 4 * rows * sizeof(long long), st);
    if (with_press) cudaMemsetAsync(d.pq, 0, 4 * rows * sizeof(long long), st);
  }
  if (mode != kPairsF32) {
    launch_force_fp64(d, nblk, mode, with_press, kept, st);
    return;
  }
  if (form_mask & (1 << IDPD_FORM_MDPD_K))
    launch_force_form<IDPD_FORM_MDPD_K>(d, nblk, with_press, tu, kept ? 1 : 0, st);
  if (form_mask & (1 << IDPD_FORM_PAIRWISE_K))
    launch_force_form<IDPD_FORM_PAIRWISE_K>(d, nblk, with_press, tu, kept ? 1 : 0, st);
  if (form_mask & (1 << IDPD_FORM_WARREN_K))
    launch_force_form<IDPD_FORM_WARREN_K>(d, nblk, with_press, tu, kept ? 1 : 0, st);
}

}  // namespace idpd
