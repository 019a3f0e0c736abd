// Pair arithmetic shared by the cell-list passes and the multi-walk passes.
#pragma once

#include "state.cuh"

namespace idpd {

// Density weight of one in-range pair (pass 1 arithmetic, FP32) in the
// 2^-23 fixed point of the replica: round(w * pre * 2^23) read from the
// mantissa of 1 + w * pre (w * pre in [0, 1]).
__device__ __forceinline__ uint32_t dens_weight(float dr2, bool warren, float inv_rd, float wnorm,
                                                float pre) {
  const float dr = dr2 * rsqrtf(dr2);
  float w = warren ? 1.0f - dr * inv_rd : 1.0f - dr;
  w = warren ? wnorm * (w * w) : w * w;
  return (uint32_t)(__float_as_int(fmaf(w, pre, 1.0f)) - 0x3f800000);
}

// The replica's FP32 coefficients per property pair k = 3 prop_i + prop_j,
// packed so that one pair reads two shared-memory words: a = (cf_c, cf_r,
// cf_g, cf_m[k][0]), b = (cf_m[k][1], cf_m[k][2]).
struct PairTables {
  float4 a[9];
  float2 b[9];
};

__host__ __device__ __forceinline__ void fill_pair_table(PairTables& T, const RepDev& R, int k) {
  T.a[k] = make_float4(R.cf_c[k], R.cf_r[k], R.cf_g[k], R.cf_m[3 * k]);
  T.b[k] = make_float2(R.cf_m[3 * k + 1], R.cf_m[3 * k + 2]);
}

// Conservative + random + dissipative magnitude over dr for one pair
// (nbdf_calculator.hpp:108-132), FP32, for the pair-force form FORM. dr, 1/dr
// and w = 1 - dr are passed in.
template <int FORM>
__device__ __forceinline__ float pair_cf(const PairTables& T, const RepDev* R, uint32_t pri,
                                         uint32_t prj, float dr, float inv_dr, float w, float ex,
                                         float ey, float ez, float4 vi, float4 vj, float4 di,
                                         float4 dj, uint32_t idi, uint32_t idj, uint32_t seed) {
  const float sqw = w > 0.0f ? w * rsqrtf(w) : 0.0f;  // sqrt(1 - r), 2 ulp
  const int k = pri * 3 + prj;
  const float4 ta = T.a[k];
  float cons;
  if constexpr (FORM == IDPD_FORM_PAIRWISE_K) {
    cons = 25.0f * w;
  } else if constexpr (FORM == IDPD_FORM_WARREN_K) {
    const float rho = (di.x + dj.x) + (di.y + dj.y) + (di.z + dj.z);
    const float wb = dr < R->wrd ? 1.0f - dr * R->winv_rd : 0.0f;
    cons = R->wa * w + R->wb * rho * wb;
  } else {
    const float2 tb = T.b[k];
    const float cf_pair = dr >= kArc ? ta.x * (dr - kArc) : 0.0f;
    const float cf_mbd = ta.w * (di.x + dj.x) + tb.x * (di.y + dj.y) + tb.y * (di.z + dj.z);
    cons = (cf_pair + cf_mbd) * w;
  }
  Saru sr(idi < idj ? idi : idj, idi < idj ? idj : idi, seed);
  const float rnd = saru_nrml_f32(sr);
  const float ddv = ex * (vi.x - vj.x) + ey * (vi.y - vj.y) + ez * (vi.z - vj.z);
  return (cons + ta.y * sqw * rnd - ta.z * w * ddv * inv_dr) * inv_dr;
}

// pair_cf with the form chosen at run time.
__device__ __forceinline__ float pair_all_cf(const PairTables& T, const RepDev* R, int form,
                                             uint32_t pri, uint32_t prj, float dr, float inv_dr,
                                             float w, float ex, float ey, float ez, float4 vi,
                                             float4 vj, float4 di, float4 dj, uint32_t idi,
                                             uint32_t idj, uint32_t seed) {
  if (form == IDPD_FORM_PAIRWISE_K)
    return pair_cf<IDPD_FORM_PAIRWISE_K>(T, R, pri, prj, dr, inv_dr, w, ex, ey, ez, vi, vj, di,
                                         dj, idi, idj, seed);
  if (form == IDPD_FORM_WARREN_K)
    return pair_cf<IDPD_FORM_WARREN_K>(T, R, pri, prj, dr, inv_dr, w, ex, ey, ez, vi, vj, di, dj,
                                       idi, idj, seed);
  return pair_cf<IDPD_FORM_MDPD_K>(T, R, pri, prj, dr, inv_dr, w, ex, ey, ez, vi, vj, di, dj, idi,
                                   idj, seed);
}

// Pairs with dr^2 above this take w = 1 - dr from the compensated path.
// Below it w > 1e-3, and the ~2e-7 absolute FP32 error of w moves the
// random-force weight sqrt(w) by less than 4e-6.
constexpr float kNearCut2 = 0.998f;

}  // namespace idpd
