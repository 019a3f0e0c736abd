// Shared device-side definitions of the GB300 engine.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace idpd {

// Compile-time constants of the reference model (parameter.hpp:189-205).
constexpr int kAllUnit = 4;       // head_unit + tail_unit
constexpr double kBondLeng = 0.5; // bond_leng (ibond = 2)
constexpr float kArc = 0.9f;      // arc
constexpr double kArcD = 0.9;
constexpr uint32_t kCmCorr = 100; // cm_corr
constexpr uint32_t kNone = 0xffffffffu;

// Conservative-force forms (IDPD_FORM_* of include/idpd_engine.h).
constexpr int IDPD_FORM_MDPD_K = 0;
constexpr int IDPD_FORM_PAIRWISE_K = 1;
constexpr int IDPD_FORM_WARREN_K = 2;

// Fixed-point scales of the order-independent accumulators.
constexpr double kForceScale = 67108864.0;           // 2^26 per unit force
constexpr double kForceUnscale = 1.0 / 67108864.0;
constexpr double kDensScale = 1099511627776.0;        // 2^40 per unit density
constexpr float kDensScaleF = 1099511627776.0f;
constexpr double kDensUnscale = 1.0 / 1099511627776.0;
constexpr double kPosScale = 1099511627776.0;         // 2^40: COM sums, delta_sumr
constexpr float kPosScaleF = 1099511627776.0f;
constexpr int kForceBits = 26;
constexpr int kDensBits = 40;
constexpr int kPosBits = 40;
constexpr float kDensUnscaleF = 1.0f / 1099511627776.0f;

// FP32 pair-set decisions within this band of a cutoff are re-taken in FP64
// from the FP64 positions, exactly as the reference's FP64 test. The bound on
// the FP32 error of dr^2 for |d| <= 1.5 cells is below 2e-6.
constexpr float kGuard = 8.0e-6f;

// Per-replica parameters on the device. Pair tables are FP32 copies of the
// reference's FP64 tables; geometry is kept in FP64 for the exact paths.
struct RepDev {
  double box[3];
  double ibox[3];    // 1 / box (Parameter::ibox_leng)
  double inv_cs[3];  // search cells per unit length (nc / box)
  double cs[3];      // frame cell side (box / nf): cell-local coordinates refer to it
  float cs_f[3];     // frame cell side rounded to float
  float cs_lo[3];    // cs - cs_f
  int nc[3];         // search cells per axis (reach * nf)
  int nf[3];         // frame cells per axis (floor(box), side >= the cutoff)
  int rshift;        // log2(reach): search cell c lies in frame cell c >> rshift
  int cell_off;      // first global cell of the replica
  int ncell;
  int row_off;       // first row (storage and sorted) of the replica
  int n;             // rows in use
  int blk_off;       // first block of the replica in row-block launches
  int nblk;
  double dt;
  float cf_c[9], cf_g[9], cf_r[9], cf_m[27];
  float wa, wb, wrd, winv_rd, wnorm;  // Warren form
  float cf_s;
  uint32_t seed;
  int form;
  int n_amp;         // molecules of the replica
  int amp_off;       // first molecule slot in the global topology
  int reach;         // cells per cutoff: cell side >= 1 / reach, stencil (2 reach + 1)^3
  float dens_prescale;    // 2^-k with every density weight * 2^-k <= 1
  float dens_unscale_f;   // 2^(k - 23): one unit of the density fixed point
  double dens_unscale;
  // precursor conversion (idpd_precursor)
  int prec_on;
  uint32_t prec_from, prec_near, prec_to, prec_thr, prec_seed;
};

// FP64 coefficient tables of a replica (plain FP64 kernels).
struct RepTab64 {
  double cf_c[9], cf_g[9], cf_r[9], cf_m[27];
  double wa, wb, wrd;
};

// Row-block launch: block b covers rows [blk_row[b], blk_row[b] + blockDim)
// of replica blk_rep[b] (rows beyond the replica's end are idle).
struct BlockMap {
  const int* rep;
  const int* row;
};

__device__ __forceinline__ int sar(int x, int s) { return x >> s; }

// ---------------------------------------------------------------- Saru
// Saru(seed1, seed2, seed3) and u32() (saruprng.hpp:239-255, 322-333); the
// constants are the generator's definition and must match bit for bit.
struct Saru {
  uint32_t lcg, weyl;
  __device__ __forceinline__ Saru(uint32_t a, uint32_t b, uint32_t c) {
    c ^= (a << 7) ^ (b >> 6);
    b += (a >> 4) ^ (c >> 15);
    a ^= (b << 9) + (c << 8);
    c ^= 0xA5366B4Du * ((b >> 11) ^ (a << 1));
    b += 0x72BE1579u * ((a << 4) ^ (c >> 16));
    a ^= 0x3F38A6EDu * ((c >> 5) ^ (uint32_t)((int)b >> 22));
    b += a * c;
    a += c ^ (b >> 2);
    b ^= (uint32_t)((int)b >> 17);
    lcg = 0x79dedea3u * (a ^ (uint32_t)((int)a >> 14));
    weyl = (lcg + b) ^ (uint32_t)((int)lcg >> 8);
    lcg = lcg + (weyl * (weyl ^ 0xdddf97f5u));
    weyl = 0xABCB96F7u + (weyl >> 1);
  }
  __device__ __forceinline__ uint32_t next() {
    lcg = 0x4beb5d59u * lcg + 0x2600e1f7u;
    weyl = weyl + 0x8009d14bu + ((uint32_t)((int)weyl >> 31) & 0xda879addu);
    const uint32_t v = (lcg ^ (lcg >> 26)) + weyl;
    return (v ^ (v >> 20)) * 0x6957f5a7u;
  }
};

// Normal deviate of Saru::nrml() (saruprng.hpp:442-445) in FP32:
// sqrt(-2 ln u1) cos(2 pi u2) with u = (2 (draw >> 1) + 1) / 2^32.
//
// One logarithm per draw, by the same branch-free arithmetic on every lane:
//  * u1 = m1 2^-32 = f' 2^-j with f' in [1/sqrt 2, sqrt 2): j = clz(m1),
//    M = m1 << j in [2^31, 2^32) gives f = M 2^-32 in [1/2, 1), and f is
//    doubled (j + 1) when below 1/sqrt 2;
//  * c = 1 - f' is exact in integers: (2^32 - M) 2^-32, or (2^32 - 2M) 2^-32
//    when doubled, so -ln u1 keeps its relative accuracy as u1 -> 1;
//  * -ln u1 = j ln 2 + 2 atanh(z), z = c / (2 - c), |z| <= 0.1716, with the
//    Taylor series z + z^3/3 + ... + z^9/9 (truncation below 3e-9 relative);
//  * cos(2 pi u2) = cos(2 pi (u2 - 1)): the draw read as a signed integer
//    gives the argument in [-pi, pi), where the hardware cosine's absolute
//    error is below 2^-21.4 (the deviate's error stays below 2.4e-6 for the
//    largest radius, sqrt(2 ln 2^32) = 6.66).
__device__ __forceinline__ float saru_nrml_f32(Saru& s) {
  const uint32_t m1 = s.next() | 1u;  // 2 (draw >> 1) + 1 = u1 * 2^32
  const uint32_t m2 = s.next() | 1u;  // u2 * 2^32
  const float two_m32 = 2.3283064365386963e-10f;  // 2^-32
  const int j = __clz(m1);
  const uint32_t M = m1 << j;
  const int dbl = M < 0xB504F334u ? 1 : 0;  // f < 1/sqrt 2 (0xB504F334 = 2^32 / sqrt 2)
  const uint32_t Md = M << dbl;             // f' 2^32, modulo 2^32 when doubled
  const float c = __int2float_rn((int)(0u - Md)) * two_m32;  // 1 - f'
  const float z = __fdividef(c, 2.0f - c);
  const float z2 = z * z;
  float p = 1.0f / 9.0f;
  p = fmaf(p, z2, 1.0f / 7.0f);
  p = fmaf(p, z2, 1.0f / 5.0f);
  p = fmaf(p, z2, 1.0f / 3.0f);
  p = fmaf(p, z2, 1.0f);
  const float nlog = fmaf(__int2float_rn(j + dbl), 0.69314718055994531f, 2.0f * (z * p));
  // cos(2 pi u2) = cos(2 pi (u2 - 1)): the signed draw gives the argument in [-pi, pi)
  const float cs = __cosf(__int2float_rn((int)m2) * (6.28318530717958647692f * two_m32));
  const float r2 = 2.0f * nlog;
  return r2 * rsqrtf(r2) * cs;  // nlog > 0 for every odd m1
}

// FP64 normal exactly as the reference computes it (plain FP64 arm).
__device__ __forceinline__ double saru_nrml_f64(Saru& s) {
  const double u1 = ((double)(int)(s.next() >> 1) + 0.5) * (1.0 / 2147483648.0);
  const double u2 = ((double)(int)(s.next() >> 1) + 0.5) * (1.0 / 2147483648.0);
  return sqrt(-2.0 * log(u1)) * cos(2.0 * 3.14159265358979323846 * u2);
}

// Splits a double X (|X| < 2^8) into floats hi + lo with |X - hi - lo| below
// 2^-47 |X|, with integer operations only: hi keeps the leading 24 mantissa
// bits (truncated), lo the remaining 29 bits rounded to float.
__device__ __forceinline__ void split_double(double X, float& hi, float& lo) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(X);
  const uint32_t sign = (uint32_t)(b >> 32) & 0x80000000u;
  const int e = (int)(b >> 52) & 0x7ff;
  if (e < 897) {  // |X| < 2^-126: both parts are negligible
    hi = 0.0f;
    lo = 0.0f;
    return;
  }
  const unsigned long long m = (b & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull;
  const uint32_t hm = (uint32_t)(m >> 29);
  hi = __uint_as_float(sign | ((uint32_t)(e - 896) << 23) | (hm & 0x7FFFFFu));
  if (e < 949) {
    lo = 0.0f;
  } else {
    const float scale = __uint_as_float((uint32_t)(e - 948) << 23);  // 2^(e - 1075)
    lo = __uint_as_float(__float_as_uint(__uint2float_rn((uint32_t)(m & 0x1FFFFFFFull)) * scale) |
                         sign);
  }
}

// Error-free transforms (Knuth's TwoSum, fma-based TwoProduct).
__device__ __forceinline__ float two_sum(float a, float b, float& err) {
  const float s = a + b;
  const float bb = s - a;
  err = (a - (s - bb)) + (b - bb);
  return s;
}
__device__ __forceinline__ float two_prod(float a, float b, float& err) {
  const float p = a * b;
  err = fmaf(a, b, -p);
  return p;
}

// Round(v * 2^S) as int64 from the float's bits, without conversion
// instructions (float-to-int64 conversion runs on the FP64 pipe).
// Ties round away from zero; |v| 2^S must stay below 2^62.
__device__ __forceinline__ long long fix_from_float(float v, int S) {
  const uint32_t b = __float_as_uint(v);
  const int e = (int)((b >> 23) & 0xffu);
  const long long m = (long long)((b & 0x7fffffu) | 0x800000u);
  const int sh = e - 150 + S;
  long long q;
  if (sh >= 0)
    q = m << (sh < 39 ? sh : 39);
  else
    q = sh > -25 ? (m + (1ll << (-sh - 1))) >> (-sh) : 0ll;
  q = e == 0 ? 0ll : q;
  return (b >> 31) ? -q : q;
}

// Fixed-point sum back to float: two exact 32-bit halves.
__device__ __forceinline__ float fix_to_float(long long q, float unscale) {
  const float hi = (float)(int)(q >> 32) * 4294967296.0f;
  const float lo = (float)(uint32_t)(q & 0xffffffffll);
  return (hi + lo) * unscale;
}

// round(v * 2^26) as int64 for |v| < 2^16 from two float roundings: the
// mantissa of 1.5 * 2^23 + v 2^5 holds round(v 2^5) (hi); the remainder
// v - hi 2^-5 is exact and |.| <= 2^-6, so a second rounding gives the low
// 21 bits. Larger |v| take the bit-level path. Ties round to even.
// round(v * 2^26) = hi * 2^21 + lo for |v| < 65536: hi = round(v * 32)
// (|hi| <= 2^21) and lo = round((v - hi / 32) * 2^26) (|lo| <= 2^20), both
// read from the mantissa of 1.5 * 2^23 + x.
__device__ __forceinline__ void fix_force_parts(float v, int& hi, int& lo) {
  const float magic = 12582912.0f;  // 1.5 * 2^23
  const float a = fmaf(v, 32.0f, magic);
  hi = __float_as_int(a) - __float_as_int(magic);
  const float r = fmaf(-(a - magic), 0.03125f, v);
  lo = __float_as_int(fmaf(r, 67108864.0f, magic)) - __float_as_int(magic);
}

__device__ __forceinline__ long long fix_force(float v) {
  if (!(fabsf(v) < 65536.0f)) return fix_from_float(v, kForceBits);
  int hi, lo;
  fix_force_parts(v, hi, lo);
  return ((long long)hi << 21) + (long long)lo;
}

// Fixed-point sum to double, exactly for |q| < 2^51: the integer is added
// into the mantissa of 1.5 * 2^52 and the bias removed with one FP64 add
// (an int64-to-double conversion is a slower FP64-pipe instruction).
__device__ __forceinline__ double fix_to_double(long long q, double unscale) {
  const double magic = 6755399441055744.0;  // 1.5 * 2^52
  const double v = __longlong_as_double(q + __double_as_longlong(magic)) - magic;
  return v * unscale;
}

// Float with bits reinterpreted as a uint32 payload (prop / id in .w lanes).
__device__ __forceinline__ uint32_t fbits(float f) { return __float_as_uint(f); }

// Cell coordinates of a replica-local cell index (x fastest).
// Periodic image of j nearest to i along one axis (the one FDPS gathers:
// within the search radius 1.2 < L / 2 it is unique): j is taken at xj + s L.
__device__ __forceinline__ int nearest_image(double xi, double xj, double L) {
  const double e = xi - xj;
  return e > 0.5 * L ? 1 : (e < -0.5 * L ? -1 : 0);
}

__device__ __forceinline__ void cell_xyz(int lc, const int* nc, int& cx, int& cy, int& cz) {
  cx = lc % nc[0];
  const int t = lc / nc[0];
  cy = t % nc[1];
  cz = t / nc[1];
}

}  // namespace idpd
