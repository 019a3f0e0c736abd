// The FDPS multi-walk passes (the reference's GPU hook, f_calculator_gpu.cuh:
// 9-21): many interaction groups ("walks") of i particles, each with the j
// particles FDPS gathered for it, positions image-shifted. One warp per i
// particle sweeps its walk's j particles 32 at a time. Each walk's
// coordinates are taken relative to the walk's first i particle and split into
// FP32 hi + lo parts; pair decisions within kGuard of a cutoff are re-taken on
// the FP64 positions in the reference's operation order. Pass 2 queues the
// in-range pairs of a warp in shared memory and evaluates them 32 at a time;
// sums are 64-bit fixed point as in the cell-list passes.
#include <cstring>
#include <string>
#include <vector>

#include "pair_math.cuh"

namespace idpd {
namespace {

constexpr int kWalkWarps = 4;
constexpr float kRnC2f = 1.44f;    // Parameter::rn_c2 (parameter.hpp:204-205)
constexpr double kRnC2 = 1.2 * 1.2;

// Device view of one dispatch.
struct WalkDev {
  int ni, nj, n_walk;
  const int* walk_of_i;        // [ni]
  const int* j_off;            // [n_walk + 1]
  const double* ref;           // [3 n_walk] coordinate origin of each walk
  const double *xi, *xj;       // [3 ni], [3 nj] FP64 positions (j image-shifted)
  float4 *pi, *li, *vi, *di;   // i: local hi (+prop bits), lo, vel (+id bits), dens
  float4 *pj, *lj, *vj, *dj;   // j: the same
  double* out;                 // results, AoS of the kind's RESULT type
  uint32_t* out_cnt;           // density: nei_cnt [2 ni]
  int* err;
};

__device__ __forceinline__ void split_local(const double* x, const double* ref, float4& hi,
                                            float4& lo) {
  const double a = x[0] - ref[0], b = x[1] - ref[1], c = x[2] - ref[2];
  hi.x = (float)a;
  hi.y = (float)b;
  hi.z = (float)c;
  lo.x = (float)(a - (double)hi.x);
  lo.y = (float)(b - (double)hi.y);
  lo.z = (float)(c - (double)hi.z);
  lo.w = 0.0f;
}

// Unpacks the reference's EPI / EPJ structs (byte offsets of their fields).
template <bool DPD, bool IS_I>
__global__ void k_walk_unpack(const unsigned char* raw, int n, int stride, WalkDev w) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const unsigned char* p = raw + (size_t)k * stride;
  uint32_t id = 0, prop;
  const double *pos, *vel = nullptr, *dens = nullptr;
  if (DPD) {
    id = *reinterpret_cast<const uint32_t*>(p);
    prop = *reinterpret_cast<const uint32_t*>(p + 4);
    const int o = IS_I ? 8 : 16;  // EPJ::DPD carries amp_id and unit before pos
    pos = reinterpret_cast<const double*>(p + o);
    vel = pos + 3;
    dens = pos + 6;
  } else {
    prop = *reinterpret_cast<const uint32_t*>(p);
    pos = reinterpret_cast<const double*>(p + 8);
  }
  int walk;
  if (IS_I) {
    walk = w.walk_of_i[k];
  } else {  // the walk whose j range holds k
    int lo = 0, hi = w.n_walk - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (w.j_off[mid] <= k) lo = mid;
      else hi = mid - 1;
    }
    walk = lo;
  }
  double* x = (IS_I ? const_cast<double*>(w.xi) : const_cast<double*>(w.xj)) + 3 * (size_t)k;
  x[0] = pos[0];
  x[1] = pos[1];
  x[2] = pos[2];
  float4 hi, lo;
  split_local(pos, w.ref + 3 * walk, hi, lo);
  hi.w = __uint_as_float(prop);
  (IS_I ? w.pi : w.pj)[k] = hi;
  (IS_I ? w.li : w.lj)[k] = lo;
  if (DPD) {
    (IS_I ? w.vi : w.vj)[k] = make_float4((float)vel[0], (float)vel[1], (float)vel[2], __uint_as_float(id));
    (IS_I ? w.di : w.dj)[k] = make_float4((float)dens[0], (float)dens[1], (float)dens[2], 0.0f);
  }
}

__device__ __forceinline__ double exact_walk_dr2(const WalkDev& w, int i, int j) {
  const double* a = w.xi + 3 * (size_t)i;
  const double* b = w.xj + 3 * (size_t)j;
  const double ex = __dsub_rn(a[0], b[0]), ey = __dsub_rn(a[1], b[1]), ez = __dsub_rn(a[2], b[2]);
  return __dadd_rn(__dadd_rn(__dmul_rn(ex, ex), __dmul_rn(ey, ey)), __dmul_rn(ez, ez));
}

__device__ __forceinline__ float walk_dist2(float4 a, float4 b) {
  const float ex = a.x - b.x, ey = a.y - b.y, ez = a.z - b.z;
  return __fmaf_rn(ez, ez, __fmaf_rn(ey, ey, __fmul_rn(ex, ex)));
}

// Pass 1 of CalcDensity (nbdf_calculator.hpp:18-57) per i particle.
__global__ void __launch_bounds__(32 * kWalkWarps) k_walk_density(WalkDev w, RepDev R) {
  const int lane = threadIdx.x & 31;
  const int i = blockIdx.x * kWalkWarps + (threadIdx.x >> 5);
  if (i >= w.ni) return;
  const int walk = w.walk_of_i[i];
  const int jb = w.j_off[walk], je = w.j_off[walk + 1];
  const float4 pi = w.pi[i];
  const bool warren = R.form == IDPD_FORM_WARREN_K;
  const float cutd2 = R.wrd * R.wrd;
  const double cutd2d = (double)R.wrd * (double)R.wrd;
  unsigned long long q[3] = {0, 0, 0};
  double hb[3] = {0.0, 0.0, 0.0}, hl[3] = {0.0, 0.0, 0.0};
  uint32_t cb = 0, cl = 0;
  for (int j0 = jb; j0 < je; j0 += 32) {
    const int j = j0 + lane;
    const bool valid = j < je;
    const float4 pj = valid ? w.pj[j] : make_float4(1.0e18f, 0.0f, 0.0f, 0.0f);
    const float dr2 = walk_dist2(pi, pj);
    bool in_b = valid && dr2 < kRnC2f && dr2 != 0.0f;
    bool in_1 = valid && dr2 < 1.0f && dr2 != 0.0f;
    bool in_d = in_1 && dr2 < cutd2;
    const bool near = valid && (fabsf(dr2 - kRnC2f) <= kGuard || fabsf(dr2 - 1.0f) <= kGuard ||
                                dr2 < 1.0e-10f || (warren && fabsf(dr2 - cutd2) <= kGuard));
    if (__any_sync(0xffffffffu, near)) {
      if (near) {
        const double e2 = exact_walk_dr2(w, i, j);
        in_b = e2 < kRnC2 && e2 != 0.0;
        in_1 = e2 < 1.0 && e2 != 0.0;
        in_d = in_1 && e2 < cutd2d;
      }
    }
    if (!valid) continue;
    const uint32_t prj = __float_as_uint(pj.w);
    const double* xj = w.xj + 3 * (size_t)j;
    if (in_b && prj == 1u) {  // Hyphob within rn_c
      hb[0] += xj[0];
      hb[1] += xj[1];
      hb[2] += xj[2];
      cb++;
    }
    if (in_1 && prj == 0u) {  // Hyphil within 1
      hl[0] += xj[0];
      hl[1] += xj[1];
      hl[2] += xj[2];
      cl++;
    }
    if (in_d) {
      const unsigned long long v = dens_weight(dr2, warren, R.winv_rd, R.wnorm, R.dens_prescale);
      q[0] += prj == 0u ? v : 0ull;
      q[1] += prj == 1u ? v : 0ull;
      q[2] += prj == 2u ? v : 0ull;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
    for (int k = 0; k < 3; k++) {
      q[k] += __shfl_xor_sync(0xffffffffu, q[k], o);
      hb[k] += __shfl_xor_sync(0xffffffffu, hb[k], o);
      hl[k] += __shfl_xor_sync(0xffffffffu, hl[k], o);
    }
    cb += __shfl_xor_sync(0xffffffffu, cb, o);
    cl += __shfl_xor_sync(0xffffffffu, cl, o);
  }
  if (lane != 0) return;
  double* out = w.out + 10 * (size_t)i;  // RESULT::Density: dens[3], nei_pos_sum[2][3]
  const double* xi = w.xi + 3 * (size_t)i;
  for (int k = 0; k < 3; k++) {
    out[k] = (double)q[k] * R.dens_unscale;
    out[3 + k] = xi[k] + hl[k];  // the Hyphil sum starts at the particle itself
    out[6 + k] = hb[k];
  }
  w.out_cnt[2 * (size_t)i] = cl + 1;
  w.out_cnt[2 * (size_t)i + 1] = cb;
}

// Pass 2 of CalcForceEpEpDPD (nbdf_calculator.hpp:73-144) per i particle.
__global__ void __launch_bounds__(32 * kWalkWarps) k_walk_force(WalkDev w, RepDev R, PairTables T,
                                                                uint32_t seed) {
  __shared__ int queue[kWalkWarps][64];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int i = blockIdx.x * kWalkWarps + wid;
  if (i >= w.ni) return;
  const int walk = w.walk_of_i[i];
  const int jb = w.j_off[walk], je = w.j_off[walk + 1];
  const float4 pi = w.pi[i], li = w.li[i], vi = w.vi[i], di = w.di[i];
  const uint32_t idi = __float_as_uint(vi.w), pri = __float_as_uint(pi.w);
  long long f[6] = {0, 0, 0, 0, 0, 0};
  int* Q = queue[wid];
  int qn = 0;
  auto eval = [&](int j) {
    const float4 pj = w.pj[j], lj = w.lj[j], vj = w.vj[j], dj = w.dj[j];
    const float ex = (pi.x - pj.x) + (li.x - lj.x), ey = (pi.y - pj.y) + (li.y - lj.y),
                ez = (pi.z - pj.z) + (li.z - lj.z);
    const float dr2 = __fmaf_rn(ez, ez, __fmaf_rn(ey, ey, __fmul_rn(ex, ex)));
    const float inv_dr = rsqrtf(dr2);
    const float dr = dr2 * inv_dr;
    float wv = 1.0f - dr;
    if (dr2 > kNearCut2) {  // 1 - r from the FP64 positions near the cutoff
      const double e2 = exact_walk_dr2(w, i, j);
      wv = fmaxf((float)(1.0 - sqrt(e2)), 0.0f);
    }
    const float a = pair_all_cf(T, &R, R.form, pri, __float_as_uint(pj.w), dr, inv_dr, wv, ex, ey, ez,
                                vi, vj, di, dj, idi, __float_as_uint(vj.w), seed);
    if (!isfinite(a)) atomicCAS(w.err, 0, kErrNonFinite);
    const float gx = a * ex, gy = a * ey, gz = a * ez;
    f[0] += fix_force(gx);
    f[1] += fix_force(gy);
    f[2] += fix_force(gz);
    f[3] += fix_force(gx * ex);
    f[4] += fix_force(gy * ey);
    f[5] += fix_force(gz * ez);
  };
  for (int j0 = jb; j0 < je; j0 += 32) {
    const int j = j0 + lane;
    bool in = false, near = false;
    if (j < je && __float_as_uint(w.vj[j].w) != idi) {  // nbdf_calculator.hpp:84
      const float dr2 = walk_dist2(pi, w.pj[j]);
      in = dr2 < 1.0f;
      near = fabsf(dr2 - 1.0f) <= kGuard;
    }
    if (__any_sync(0xffffffffu, near)) {
      if (near) in = exact_walk_dr2(w, i, j) < 1.0;
    }
    const uint32_t m = __ballot_sync(0xffffffffu, in);
    if (in) Q[qn + __popc(m & ((1u << lane) - 1u))] = j;
    qn += __popc(m);
    __syncwarp();
    if (qn >= 32) {
      eval(Q[lane]);
      __syncwarp();
      if (lane < qn - 32) Q[lane] = Q[32 + lane];
      qn -= 32;
      __syncwarp();
    }
  }
  if (lane < qn) eval(Q[lane]);
#pragma unroll
  for (int k = 0; k < 6; k++)
    for (int o = 16; o > 0; o >>= 1) f[k] += __shfl_xor_sync(0xffffffffu, f[k], o);
  if (lane == 0) {
    double* out = w.out + 6 * (size_t)i;  // RESULT::ForceDPD: acc, press
    for (int k = 0; k < 6; k++) out[k] = fix_to_double(f[k], kForceUnscale);
  }
}

template <class T>
int grow(T** p, size_t& cap, size_t want, bool pinned) {
  if (want <= cap && *p) return 0;
  if (*p) {
    if (pinned) cudaFreeHost(*p);
    else cudaFree(*p);
    *p = nullptr;
  }
  const size_t n = want + want / 2 + 64;
  const cudaError_t e = pinned ? cudaMallocHost((void**)p, n * sizeof(T)) : cudaMalloc((void**)p, n * sizeof(T));
  if (e != cudaSuccess) {
    *p = nullptr;
    cap = 0;
    return 1;
  }
  cap = n;
  return 0;
}

}  // namespace

// Buffers and the in-flight dispatch of each kind.
struct WalkState {
  struct Kind {
    unsigned char *h_raw = nullptr, *d_raw = nullptr;
    size_t h_raw_cap = 0, d_raw_cap = 0;
    int *h_int = nullptr, *d_int = nullptr;  // walk_of_i, j_off
    size_t h_int_cap = 0, d_int_cap = 0;
    double *h_ref = nullptr, *d_ref = nullptr;
    size_t h_ref_cap = 0, d_ref_cap = 0;
    double *d_x = nullptr;
    size_t d_x_cap = 0;
    float4* d_f4 = nullptr;
    size_t d_f4_cap = 0;
    double *d_out = nullptr, *h_out = nullptr;
    size_t d_out_cap = 0, h_out_cap = 0;
    uint32_t *d_cnt = nullptr, *h_cnt = nullptr;
    size_t d_cnt_cap = 0, h_cnt_cap = 0;
    cudaEvent_t done = nullptr;
    bool pending = false;
    int tag = 0, ni = 0, n_walk = 0;
  } kind[2];
  int* d_err = nullptr;
};

WalkState* walk_create() {
  WalkState* s = new WalkState();
  for (auto& k : s->kind) cudaEventCreateWithFlags(&k.done, cudaEventDisableTiming);
  cudaMalloc((void**)&s->d_err, sizeof(int));
  cudaMemset(s->d_err, 0, sizeof(int));
  return s;
}

void walk_destroy(WalkState* s) {
  if (!s) return;
  for (auto& k : s->kind) {
    if (k.done) cudaEventSynchronize(k.done);
    cudaFreeHost(k.h_raw); cudaFree(k.d_raw);
    cudaFreeHost(k.h_int); cudaFree(k.d_int);
    cudaFreeHost(k.h_ref); cudaFree(k.d_ref);
    cudaFree(k.d_x); cudaFree(k.d_f4);
    cudaFree(k.d_out); cudaFreeHost(k.h_out);
    cudaFree(k.d_cnt); cudaFreeHost(k.h_cnt);
    if (k.done) cudaEventDestroy(k.done);
  }
  cudaFree(s->d_err);
  delete s;
}

int walk_dispatch(WalkState* s, cudaStream_t st, const RepDev& R, const idpd_params& p, int kind,
                  int tag, int n_walk, const void* const* epi, const int32_t* n_epi,
                  const void* const* epj, const int32_t* n_epj, std::string& err) {
  WalkState::Kind& K = s->kind[kind];
  if (K.pending) cudaEventSynchronize(K.done);  // its buffers are reused
  const bool dpd = kind == IDPD_WALK_FORCE;
  const size_t si = dpd ? sizeof(idpd_epi_dpd) : sizeof(idpd_epi_density);
  const size_t sj = dpd ? sizeof(idpd_epj_dpd) : sizeof(idpd_epj_density);
  long long ni = 0, nj = 0;
  for (int w = 0; w < n_walk; w++) {
    if (n_epi[w] < 0 || n_epj[w] < 0 || (n_epi[w] > 0 && !epi[w]) || (n_epj[w] > 0 && !epj[w])) {
      err = "walk sizes or pointers invalid";
      return IDPD_ERR_INVALID_ARG;
    }
    ni += n_epi[w];
    nj += n_epj[w];
  }
  if (ni + nj >= (1ll << 30)) {
    err = "too many particles in one dispatch";
    return IDPD_ERR_CAPACITY;
  }
  const size_t raw = ni * si + nj * sj, nint = ni + n_walk + 1;
  if (grow(&K.h_raw, K.h_raw_cap, raw, true) || grow(&K.d_raw, K.d_raw_cap, raw, false) ||
      grow(&K.h_int, K.h_int_cap, nint, true) || grow(&K.d_int, K.d_int_cap, nint, false) ||
      grow(&K.h_ref, K.h_ref_cap, 3 * (size_t)n_walk, true) ||
      grow(&K.d_ref, K.d_ref_cap, 3 * (size_t)n_walk, false) ||
      grow(&K.d_x, K.d_x_cap, 3 * (size_t)(ni + nj), false) ||
      grow(&K.d_f4, K.d_f4_cap, 4 * (size_t)(ni + nj), false) ||
      grow(&K.d_out, K.d_out_cap, (dpd ? 6 : 10) * (size_t)ni, false) ||
      grow(&K.h_out, K.h_out_cap, (dpd ? 6 : 10) * (size_t)ni, true) ||
      grow(&K.d_cnt, K.d_cnt_cap, 2 * (size_t)ni, false) ||
      grow(&K.h_cnt, K.h_cnt_cap, 2 * (size_t)ni, true)) {
    err = "walk buffer allocation failed";
    return IDPD_ERR_CUDA;
  }
  // the walks side by side: i structs, then j structs; walk of each i; j offsets
  unsigned char* hi = K.h_raw;
  unsigned char* hj = K.h_raw + ni * si;
  int* walk_of_i = K.h_int;
  int* j_off = K.h_int + ni;
  long long oi = 0, oj = 0;
  for (int w = 0; w < n_walk; w++) {
    if (n_epi[w]) std::memcpy(hi + oi * si, epi[w], n_epi[w] * si);
    if (n_epj[w]) std::memcpy(hj + oj * sj, epj[w], n_epj[w] * sj);
    for (int k = 0; k < n_epi[w]; k++) walk_of_i[oi + k] = w;
    j_off[w] = (int)oj;
    // origin of the walk's local coordinates: its first i particle
    const double* ref = n_epi[w] ? reinterpret_cast<const double*>(
                                       static_cast<const unsigned char*>(epi[w]) + 8)
                                 : nullptr;
    for (int k = 0; k < 3; k++) K.h_ref[3 * w + k] = ref ? ref[k] : 0.0;
    oi += n_epi[w];
    oj += n_epj[w];
  }
  j_off[n_walk] = (int)oj;
  cudaMemcpyAsync(K.d_raw, K.h_raw, raw, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(K.d_int, K.h_int, sizeof(int) * nint, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(K.d_ref, K.h_ref, sizeof(double) * 3 * n_walk, cudaMemcpyHostToDevice, st);
  WalkDev W;
  W.ni = (int)ni;
  W.nj = (int)nj;
  W.n_walk = n_walk;
  W.walk_of_i = K.d_int;
  W.j_off = K.d_int + ni;
  W.ref = K.d_ref;
  W.xi = K.d_x;
  W.xj = K.d_x + 3 * ni;
  float4* f4 = K.d_f4;
  W.pi = f4; W.li = f4 + ni; W.vi = f4 + 2 * ni; W.di = f4 + 3 * ni;
  f4 += 4 * ni;
  W.pj = f4; W.lj = f4 + nj; W.vj = f4 + 2 * nj; W.dj = f4 + 3 * nj;
  W.out = K.d_out;
  W.out_cnt = K.d_cnt;
  W.err = s->d_err;
  const unsigned char* di = K.d_raw;
  const unsigned char* dj = K.d_raw + ni * si;
  if (ni > 0) {
    if (dpd) k_walk_unpack<true, true><<<(unsigned)((ni + 255) / 256), 256, 0, st>>>(di, (int)ni, (int)si, W);
    else k_walk_unpack<false, true><<<(unsigned)((ni + 255) / 256), 256, 0, st>>>(di, (int)ni, (int)si, W);
  }
  if (nj > 0 && n_walk > 0) {
    if (dpd) k_walk_unpack<true, false><<<(unsigned)((nj + 255) / 256), 256, 0, st>>>(dj, (int)nj, (int)sj, W);
    else k_walk_unpack<false, false><<<(unsigned)((nj + 255) / 256), 256, 0, st>>>(dj, (int)nj, (int)sj, W);
  }
  if (ni > 0) {
    const unsigned nb = (unsigned)((ni + kWalkWarps - 1) / kWalkWarps);
    if (dpd) {
      PairTables T;
      for (int k = 0; k < 9; k++) fill_pair_table(T, R, k);
      k_walk_force<<<nb, 32 * kWalkWarps, 0, st>>>(W, R, T, p.seed + p.time);
    } else {
      k_walk_density<<<nb, 32 * kWalkWarps, 0, st>>>(W, R);
    }
  }
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    err = std::string("walk launch: ") + cudaGetErrorString(e);
    return IDPD_ERR_CUDA;
  }
  if (ni > 0) {
    cudaMemcpyAsync(K.h_out, K.d_out, sizeof(double) * (dpd ? 6 : 10) * ni, cudaMemcpyDeviceToHost, st);
    if (!dpd) cudaMemcpyAsync(K.h_cnt, K.d_cnt, sizeof(uint32_t) * 2 * ni, cudaMemcpyDeviceToHost, st);
  }
  cudaEventRecord(K.done, st);
  K.pending = true;
  K.tag = tag;
  K.ni = (int)ni;
  K.n_walk = n_walk;
  return IDPD_OK;
}

int walk_retrieve(WalkState* s, int kind, int tag, int n_walk, const int32_t* ni,
                  void* const* result, std::string& err) {
  WalkState::Kind& K = s->kind[kind];
  if (!K.pending || K.tag != tag || K.n_walk != n_walk) {
    err = "no dispatch with this kind, tag and walk count";
    return IDPD_ERR_STATE;
  }
  if (cudaEventSynchronize(K.done) != cudaSuccess) {
    err = "walk pass failed";
    return IDPD_ERR_CUDA;
  }
  K.pending = false;
  int flag = 0;
  cudaMemcpy(&flag, s->d_err, sizeof(int), cudaMemcpyDeviceToHost);
  if (flag) {
    cudaMemset(s->d_err, 0, sizeof(int));
    err = "non-finite pair force in a walk";
    return IDPD_ERR_NONFINITE;
  }
  long long o = 0;
  for (int w = 0; w < n_walk; w++) {
    if (o + ni[w] > K.ni) {
      err = "retrieve sizes exceed the dispatch";
      return IDPD_ERR_INVALID_ARG;
    }
    if (kind == IDPD_WALK_FORCE) {
      idpd_result_dpd* r = static_cast<idpd_result_dpd*>(result[w]);
      for (int k = 0; k < ni[w]; k++) {
        const double* v = K.h_out + 6 * (size_t)(o + k);
        for (int c = 0; c < 3; c++) {
          r[k].acc[c] = v[c];
          r[k].press[c] = v[3 + c];
        }
      }
    } else {
      idpd_result_density* r = static_cast<idpd_result_density*>(result[w]);
      for (int k = 0; k < ni[w]; k++) {
        const double* v = K.h_out + 10 * (size_t)(o + k);
        for (int c = 0; c < 3; c++) {
          r[k].dens[c] = v[c];
          r[k].nei_pos_sum[0][c] = v[3 + c];
          r[k].nei_pos_sum[1][c] = v[6 + c];
        }
        r[k].nei_cnt[0] = K.h_cnt[2 * (size_t)(o + k)];
        r[k].nei_cnt[1] = K.h_cnt[2 * (size_t)(o + k) + 1];
      }
    }
    o += ni[w];
  }
  return IDPD_OK;
}

}  // namespace idpd
