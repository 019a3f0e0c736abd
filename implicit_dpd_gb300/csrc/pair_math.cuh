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

struct PairTables {
  float cf_c[9], cf_g[9], cf_r[9], cf_m[27];
};

// Conservative + random + dissipative magnitude over dr for one pair
// (nbdf_calculator.hpp:108-132), FP32. dr, 1/dr and w = 1 - dr are passed in.
__device__ __forceinline__ float pair_all_cf(const PairTables& T, const RepDev* R, int form,
                                             uint32_t pri, uint32_t prj, float dr, float inv_dr,
                                             float w, float ex, float ey, float ez, float4 vi,
                                             float4 vj, float4 di, float4 dj, uint32_t idi,
                                             uint32_t idj, uint32_t seed) {
  const float sqw = w > 0.0f ? w * rsqrtf(w) : 0.0f;  // sqrt(1 - r), 2 ulp
  const int k = pri * 3 + prj;
  float cons;
  if (form == IDPD_FORM_PAIRWISE_K) {
    cons = 25.0f * w;
  } else if (form == IDPD_FORM_WARREN_K) {
    const float rho = (di.x + dj.x) + (di.y + dj.y) + (di.z + dj.z);
    const float wb = dr < R->wrd ? 1.0f - dr * R->winv_rd : 0.0f;
    cons = R->wa * w + R->wb * rho * wb;
  } else {
    const float cf_pair = dr >= kArc ? T.cf_c[k] * (dr - kArc) : 0.0f;
    const float cf_mbd = T.cf_m[3 * k] * (di.x + dj.x) + T.cf_m[3 * k + 1] * (di.y + dj.y) +
                         T.cf_m[3 * k + 2] * (di.z + dj.z);
    cons = (cf_pair + cf_mbd) * w;
  }
  Saru sr(idi < idj ? idi : idj, idi < idj ? idj : idi, seed);
  const float rnd = saru_nrml_f32(sr);
  const float ddv = ex * (vi.x - vj.x) + ey * (vi.y - vj.y) + ez * (vi.z - vj.z);
  return (cons + T.cf_r[k] * sqw * rnd - T.cf_g[k] * w * ddv * inv_dr) * inv_dr;
}

// Pairs with dr^2 above this take w = 1 - dr from the compensated path.
// Below it w > 1e-3, and the ~2e-7 absolute FP32 error of w moves the
// random-force weight sqrt(w) by less than 4e-6.
constexpr float kNearCut2 = 0.998f;

}  // namespace idpd
