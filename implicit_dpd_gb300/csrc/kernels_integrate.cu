// Bonded forces, the second half of the velocity-Verlet step, the
// centre-of-mass drift removal and small utility kernels.
//   ForceBonded::CalcListedForce  bdf_calculator.hpp:153-220 (bond :95-115,
//                                 bend :117-150, cf_spring parameter.hpp:713-716)
//   kick                          driftkick.hpp:33-40
//   remove_cmdrift_global         driftkick.hpp:43-54
#include "state.cuh"

namespace idpd {

// Position of sorted slot t relative to the origin of the frame cell that
// holds search cell (cx, cy, cz) of the same replica, in FP32: frame-local
// coordinate plus the minimum-image frame-cell difference.
__device__ __forceinline__ float3 rel_pos(const DevState& d, const RepDev* R, int t, int cx, int cy,
                                          int cz) {
  const float4 p = d.posf[t];
  int tx, ty, tz;
  cell_xyz((int)d.scell[t] - R->cell_off, R->nc, tx, ty, tz);
  const int rs = R->rshift;
  int q[3] = {(tx >> rs) - (cx >> rs), (ty >> rs) - (cy >> rs), (tz >> rs) - (cz >> rs)};
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const int n = R->nf[k];
    if (2 * q[k] > n) q[k] -= n;
    if (2 * q[k] < -n) q[k] += n;
  }
  return make_float3(p.x + (float)q[0] * R->cs_f[0], p.y + (float)q[1] * R->cs_f[1],
                     p.z + (float)q[2] * R->cs_f[2]);
}

__device__ __forceinline__ float3 sub3(float3 a, float3 b) {
  return make_float3(a.x - b.x, a.y - b.y, a.z - b.z);
}
__device__ __forceinline__ float dot3(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

// Bond and bend forces of one 4-bead chain (CalcBondBendGlobalCell<4>), FP32.
// F[u] is the force on unit u; vir the bonded virial (twice, as the reference).
__device__ __forceinline__ void chain_forces(const float3 p[4], float cf_s, float cf_b, float3 F[4],
                                             float3* vir) {
  float3 dr[3];
  float inv[3];
#pragma unroll
  for (int u = 0; u < 4; u++) F[u] = make_float3(0.f, 0.f, 0.f);
  float3 v = make_float3(0.f, 0.f, 0.f);
#pragma unroll
  for (int u = 1; u < 4; u++) {
    dr[u - 1] = sub3(p[u], p[u - 1]);
    inv[u - 1] = rsqrtf(dot3(dr[u - 1], dr[u - 1]));
    const float cb = cf_s * (inv[u - 1] - (float)(1.0 / kBondLeng));
    const float3 fb = make_float3(cb * dr[u - 1].x, cb * dr[u - 1].y, cb * dr[u - 1].z);
    v.x += 2.0f * dr[u - 1].x * fb.x;
    v.y += 2.0f * dr[u - 1].y * fb.y;
    v.z += 2.0f * dr[u - 1].z * fb.z;
    F[u - 1] = sub3(F[u - 1], fb);
    F[u] = make_float3(F[u].x + fb.x, F[u].y + fb.y, F[u].z + fb.z);
    if (u >= 2) {
      const float3 a = dr[u - 2], b = dr[u - 1];
      const float i0 = inv[u - 2], i1 = inv[u - 1];
      const float in_prod = dot3(a, b);
      const float cf_bd = cf_b * (i0 * i1);
      const float c0 = in_prod * (i0 * i0), c1 = in_prod * (i1 * i1);
      const float3 t0 = make_float3(cf_bd * (b.x - c0 * a.x), cf_bd * (b.y - c0 * a.y),
                                    cf_bd * (b.z - c0 * a.z));
      const float3 t1 = make_float3(cf_bd * (a.x - c1 * b.x), cf_bd * (a.y - c1 * b.y),
                                    cf_bd * (a.z - c1 * b.z));
      v.x += 2.0f * (a.x * t0.x + b.x * t1.x);
      v.y += 2.0f * (a.y * t0.y + b.y * t1.y);
      v.z += 2.0f * (a.z * t0.z + b.z * t1.z);
      F[u - 2] = sub3(F[u - 2], t0);
      F[u - 1] = make_float3(F[u - 1].x + (t0.x - t1.x), F[u - 1].y + (t0.y - t1.y),
                             F[u - 1].z + (t0.z - t1.z));
      F[u] = make_float3(F[u].x + t1.x, F[u].y + t1.y, F[u].z + t1.z);
    }
  }
  if (vir) *vir = v;
}

// One thread per storage row: pair force + bonded force on this bead (the
// chain is re-evaluated per bead, no scatter), acc written in FP64, then
// kick: vel = vel_buf + dt/2 acc (vel holds vel_buf after the drift).
template <bool KICK>
__global__ void __launch_bounds__(kRowBlock) k_bonded_kick(DevState d) {
  const int r = d.blk_rep[blockIdx.x];
  const int i = d.blk_row[blockIdx.x] + threadIdx.x;
  const RepDev* R = d.reps + r;
  if (i >= R->row_off + R->n) return;
  const int s = (int)d.rank[i];
  const long long* fs = d.fq + 4 * (size_t)s;
  long long f[3] = {fs[0], fs[1], fs[2]};
  const uint32_t a = d.amp_id[i];
  if (a != kNone && R->n_amp > 0) {
    const int u = (int)d.unit[i];
    const int m = R->amp_off + (int)a;
    int cx, cy, cz;
    cell_xyz((int)d.scell[s] - R->cell_off, R->nc, cx, cy, cz);
    float3 p[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const int tk = (k == u) ? s : (int)d.rank[d.topol[4 * m + k]];
      p[k] = rel_pos(d, R, tk, cx, cy, cz);
    }
    float3 F[4];
    chain_forces(p, R->cf_s, d.cf_bend[m], F, nullptr);
    float3 fu = F[0];
#pragma unroll
    for (int k = 1; k < 4; k++)
      if (k == u) fu = F[k];
    f[0] += fix_force(fu.x);
    f[1] += fix_force(fu.y);
    f[2] += fix_force(fu.z);
  }
  const double acx = fix_to_double(f[0], kForceUnscale), acy = fix_to_double(f[1], kForceUnscale),
               acz = fix_to_double(f[2], kForceUnscale);
  d.ax[i] = acx;
  d.ay[i] = acy;
  d.az[i] = acz;
  if (KICK) {
    const double h = __dmul_rn(R->dt, 0.5);
    d.vx[i] = __dadd_rn(d.vx[i], __dmul_rn(h, acx));
    d.vy[i] = __dadd_rn(d.vy[i], __dmul_rn(h, acy));
    d.vz[i] = __dadd_rn(d.vz[i], __dmul_rn(h, acz));
  }
}

void launch_bonded_kick(const DevState& d, int nblk, bool kick, cudaStream_t st) {
  if (nblk == 0) return;
  if (kick)
    k_bonded_kick<true><<<nblk, kRowBlock, 0, st>>>(d);
  else
    k_bonded_kick<false><<<nblk, kRowBlock, 0, st>>>(d);
}

// Fine-grained ForceBonded::CalcListedForce: one thread per molecule adds
// its chain forces to the FP64 acc of its beads (each bead belongs to one
// molecule) and writes its virial for a host-side sum in molecule order.
__global__ void k_bonded_fine(DevState d, int n_amp_tot, const int* amp_rep, double* vir_part) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= n_amp_tot) return;
  const RepDev* R = d.reps + amp_rep[m];
  if (m - R->amp_off >= R->n_amp) {  // slot reserved for molecules a reaction may add
    vir_part[3 * m] = vir_part[3 * m + 1] = vir_part[3 * m + 2] = 0.0;
    return;
  }
  uint32_t rows[4];
  int t[4];
#pragma unroll
  for (int k = 0; k < 4; k++) {
    rows[k] = d.topol[4 * m + k];
    t[k] = (int)d.rank[rows[k]];
  }
  int cx, cy, cz;
  cell_xyz((int)d.scell[t[0]] - R->cell_off, R->nc, cx, cy, cz);
  float3 p[4];
#pragma unroll
  for (int k = 0; k < 4; k++) p[k] = rel_pos(d, R, t[k], cx, cy, cz);
  float3 F[4], v;
  chain_forces(p, R->cf_s, d.cf_bend[m], F, &v);
#pragma unroll
  for (int k = 0; k < 4; k++) {
    d.ax[rows[k]] += (double)F[k].x;
    d.ay[rows[k]] += (double)F[k].y;
    d.az[rows[k]] += (double)F[k].z;
  }
  vir_part[3 * m] = v.x;
  vir_part[3 * m + 1] = v.y;
  vir_part[3 * m + 2] = v.z;
}

void launch_bonded_fine(const DevState& d, int n_amp_tot, const int* amp_rep, double* vir_part,
                        cudaStream_t st) {
  if (n_amp_tot == 0) return;
  k_bonded_fine<<<(n_amp_tot + 127) / 128, 128, 0, st>>>(d, n_amp_tot, amp_rep, vir_part);
}

// kick alone (driftkick.hpp:33-40) on the FP64 acc.
__global__ void __launch_bounds__(kRowBlock) k_kick(DevState d) {
  const int r = d.blk_rep[blockIdx.x];
  const int i = d.blk_row[blockIdx.x] + threadIdx.x;
  const RepDev* R = d.reps + r;
  if (i >= R->row_off + R->n) return;
  const double h = __dmul_rn(R->dt, 0.5);
  d.vx[i] = __dadd_rn(d.vx[i], __dmul_rn(h, d.ax[i]));
  d.vy[i] = __dadd_rn(d.vy[i], __dmul_rn(h, d.ay[i]));
  d.vz[i] = __dadd_rn(d.vz[i], __dmul_rn(h, d.az[i]));
}

void launch_kick_only(const DevState& d, int nblk, cudaStream_t st) {
  if (nblk == 0) return;
  k_kick<<<nblk, kRowBlock, 0, st>>>(d);
}

// Write-back of pass 2 (FPDPD::copyFromForce, ptcl_class.hpp:48-51):
// acc overwritten with the pair force, press from the per-particle virial.
__global__ void __launch_bounds__(kRowBlock) k_fq_to_acc(DevState d, double* press) {
  const int r = d.blk_rep[blockIdx.x];
  const int s = d.blk_row[blockIdx.x] + threadIdx.x;
  const RepDev* R = d.reps + r;
  if (s >= R->row_off + R->n) return;
  const uint32_t i = d.perm[s];
  const long long* fs = d.fq + 4 * (size_t)s;
  d.ax[i] = (double)fs[0] * kForceUnscale;
  d.ay[i] = (double)fs[1] * kForceUnscale;
  d.az[i] = (double)fs[2] * kForceUnscale;
  if (press) {
    const long long* ps = d.pq + 4 * (size_t)s;
    press[3 * i] = (double)ps[0] * kForceUnscale;
    press[3 * i + 1] = (double)ps[1] * kForceUnscale;
    press[3 * i + 2] = (double)ps[2] * kForceUnscale;
  }
}

void launch_fq_to_acc(const DevState& d, int nblk, double* press_out, cudaStream_t st) {
  if (nblk == 0) return;
  k_fq_to_acc<<<nblk, kRowBlock, 0, st>>>(d, press_out);
}

// ------------------------------------------------- centre-of-mass drift
// Runs every step; a replica takes part only when its time is a multiple
// of cm_corr (src/main.cpp:184) or when forced. Velocities are summed as
// 2^-28 fixed-point integers, so the mean does not depend on the storage
// order of the rows (which follows the cell grid).
constexpr double kVelScale = 268435456.0;  // 2^28

__device__ __forceinline__ bool cm_due(const DevState& d, int r, int force_now) {
  return force_now || (d.rep_time[r] % kCmCorr) == 0;
}

__global__ void __launch_bounds__(kRowBlock) k_cm_partial(DevState d, int force_now) {
  __shared__ long long sh[3][kRowBlock / 32];
  const int r = d.blk_rep[blockIdx.x];
  if (!cm_due(d, r, force_now)) return;
  const int i = d.blk_row[blockIdx.x] + threadIdx.x;
  const RepDev* R = d.reps + r;
  long long v[3] = {0, 0, 0};
  if (i < R->row_off + R->n) {
    v[0] = __double2ll_rn(d.vx[i] * kVelScale);
    v[1] = __double2ll_rn(d.vy[i] * kVelScale);
    v[2] = __double2ll_rn(d.vz[i] * kVelScale);
  }
#pragma unroll
  for (int k = 0; k < 3; k++)
    for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0)
    for (int k = 0; k < 3; k++) sh[k][w] = v[k];
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 0; k < 3; k++) {
      long long t = 0;
      for (int q = 0; q < kRowBlock / 32; q++) t += sh[k][q];
      reinterpret_cast<long long*>(d.blk_part)[3 * blockIdx.x + k] = t;
    }
  }
}

// One block per replica sums its blocks' partial momenta (integers: any
// order gives the same total).
constexpr int kCmThreads = 256;
__global__ void __launch_bounds__(kCmThreads) k_cm_finalize(DevState d, int force_now) {
  __shared__ long long sh[3][kCmThreads / 32];
  const int r = blockIdx.x;
  if (!cm_due(d, r, force_now)) return;
  const RepDev* R = d.reps + r;
  const long long* part = reinterpret_cast<const long long*>(d.blk_part);
  long long s[3] = {0, 0, 0};
  for (int b = R->blk_off + threadIdx.x; b < R->blk_off + R->nblk; b += kCmThreads)
    for (int k = 0; k < 3; k++) s[k] += part[3 * b + k];
#pragma unroll
  for (int k = 0; k < 3; k++)
    for (int o = 16; o > 0; o >>= 1) s[k] += __shfl_down_sync(0xffffffffu, s[k], o);
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0)
    for (int k = 0; k < 3; k++) sh[k][w] = s[k];
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 0; k < 3; k++) {
      long long t = 0;
      for (int q = 0; q < kCmThreads / 32; q++) t += sh[k][q];
      d.rep_mean[3 * r + k] = ((double)t / kVelScale) / (double)R->n;
    }
  }
}

__global__ void __launch_bounds__(kRowBlock) k_cm_apply(DevState d, int force_now) {
  const int r = d.blk_rep[blockIdx.x];
  if (!cm_due(d, r, force_now)) return;
  const int i = d.blk_row[blockIdx.x] + threadIdx.x;
  const RepDev* R = d.reps + r;
  if (i >= R->row_off + R->n) return;
  d.vx[i] = __dsub_rn(d.vx[i], d.rep_mean[3 * r]);
  d.vy[i] = __dsub_rn(d.vy[i], d.rep_mean[3 * r + 1]);
  d.vz[i] = __dsub_rn(d.vz[i], d.rep_mean[3 * r + 2]);
}

void launch_cmdrift(const DevState& d, int nblk, int R, bool force_now, cudaStream_t st) {
  if (nblk == 0) return;
  k_cm_partial<<<nblk, kRowBlock, 0, st>>>(d, force_now ? 1 : 0);
  k_cm_finalize<<<R, kCmThreads, 0, st>>>(d, force_now ? 1 : 0);
  k_cm_apply<<<nblk, kRowBlock, 0, st>>>(d, force_now ? 1 : 0);
}

__global__ void k_time_advance(uint32_t* t, int R, const int* skip) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (skip && *skip) return;
  if (r < R) t[r] += 1u;
}

void launch_time_advance(const DevState& d, int R, cudaStream_t st, const int* skip) {
  k_time_advance<<<(R + 127) / 128, 128, 0, st>>>(d.rep_time, R, skip);
}

// ------------------------------------------- K steps in one graph launch
// The step repeated on the device by a WHILE conditional node: the count of
// steps left is set before the launch; the last node of each step takes one
// off and keeps the loop going while steps are left and, with the reaction
// enabled, while the reaction has not stopped the run (stop: its flag).
__global__ void k_loop_set(int* left, int n) { *left = n; }

__global__ void k_loop_tail(cudaGraphConditionalHandle cond, int* left, const int* stop) {
  const int l = *left - 1;
  *left = l;
  cudaGraphSetConditional(cond, (l > 0 && !(stop && *stop)) ? 1u : 0u);
}

void launch_loop_set(int* left, int n, cudaStream_t st) { k_loop_set<<<1, 1, 0, st>>>(left, n); }

// IF nodes of a captured step: work that most steps skip (the cell and list
// rebuild, the centre-of-mass drift removal every kCmCorr steps) sits in a
// conditional body whose condition one thread sets from the device state,
// so that a step without it launches none of its kernels.
__global__ void k_cond_flag(cudaGraphConditionalHandle cond, const int* flag) {
  cudaGraphSetConditional(cond, *flag ? 1u : 0u);
}

__global__ void k_cond_cm(cudaGraphConditionalHandle cond, const uint32_t* rep_time, int R) {
  int any = 0;
  for (int r = threadIdx.x; r < R; r += blockDim.x) any |= (rep_time[r] % kCmCorr) == 0u;
  any = __syncthreads_or(any);
  if (threadIdx.x == 0) cudaGraphSetConditional(cond, any ? 1u : 0u);
}

void launch_cond_flag(cudaGraphConditionalHandle cond, const int* flag, cudaStream_t st) {
  k_cond_flag<<<1, 1, 0, st>>>(cond, flag);
}

void launch_cond_cm(cudaGraphConditionalHandle cond, const uint32_t* rep_time, int R,
                    cudaStream_t st) {
  k_cond_cm<<<1, 256, 0, st>>>(cond, rep_time, R);
}

void launch_loop_tail(cudaGraphConditionalHandle cond, int* left, const int* stop,
                      cudaStream_t st) {
  k_loop_tail<<<1, 1, 0, st>>>(cond, left, stop);
}

// ----------------------------------------------------------- utilities
__global__ void k_saru_test(int n, const uint32_t* s1, const uint32_t* s2, const uint32_t* s3,
                            int draws, uint32_t* out_u, float* out_n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (out_u) {
    Saru s(s1[i], s2[i], s3[i]);
    for (int k = 0; k < draws; k++) out_u[(size_t)i * draws + k] = s.next();
  }
  if (out_n) {
    Saru s(s1[i], s2[i], s3[i]);
    out_n[i] = saru_nrml_f32(s);
  }
}

void launch_saru_test(int n, const uint32_t* s1, const uint32_t* s2, const uint32_t* s3, int draws,
                      uint32_t* out_u, float* out_n, cudaStream_t st) {
  if (n == 0) return;
  k_saru_test<<<(n + 255) / 256, 256, 0, st>>>(n, s1, s2, s3, draws, out_u, out_n);
}

__global__ void k_aos_to_soa(const double* aos, double* x, double* y, double* z, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  x[i] = aos[3 * (size_t)i];
  y[i] = aos[3 * (size_t)i + 1];
  z[i] = aos[3 * (size_t)i + 2];
}

void launch_aos_to_soa(const double* aos, double* x, double* y, double* z, int n, cudaStream_t st) {
  if (n == 0) return;
  k_aos_to_soa<<<(n + 255) / 256, 256, 0, st>>>(aos, x, y, z, n);
}

// Per-step host exchange: rows of one replica in upload order (pos, vel and
// acc as three arrays of 3 doubles per row) into the storage rows; invalid
// rows raise an error. The position change of a row counts, at its nearest
// image, as displacement for the kept lists (the delta_sumr of their last
// rebuild moves back by it), so a host that hands back the positions it read
// keeps the lists, and one that moves particles far enough triggers a rebuild.
// One thread per storage row, which reads its upload row's three records
// (orig maps storage to upload rows): the storage arrays are written in
// order, and only the 24-byte records are read out of order.
__global__ void k_set_dynamics(DevState d, const double* pos, const double* vel,
                               const double* acc, int row0, int n, double b0, double b1,
                               double b2, int kept) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const uint32_t i = (uint32_t)(row0 + j);
  const int k = (int)d.orig[i] - row0;
  const double* p = pos + 3 * (size_t)k;
  const double* v = vel + 3 * (size_t)k;
  const double* a = acc + 3 * (size_t)k;
  const double box[3] = {b0, b1, b2};
  bool ok = true;
#pragma unroll
  for (int c = 0; c < 3; c++) ok = ok && p[c] >= 0.0 && p[c] <= box[c] && isfinite(v[c]) && isfinite(a[c]);
  if (!ok) atomicCAS(d.err, 0, kErrBadCell);
  if (kept) {
    const uint32_t s = d.rank[i];
    const double old[3] = {d.px[i], d.py[i], d.pz[i]};
    double* dr[3] = {d.drx, d.dry, d.drz};
#pragma unroll
    for (int c = 0; c < 3; c++) {
      double e = p[c] - old[c];
      e = e > 0.5 * box[c] ? e - box[c] : (e < -0.5 * box[c] ? e + box[c] : e);
      dr[c][s] -= e;
    }
  }
  d.px[i] = p[0]; d.py[i] = p[1]; d.pz[i] = p[2];
  d.vx[i] = v[0]; d.vy[i] = v[1]; d.vz[i] = v[2];
  d.ax[i] = a[0]; d.ay[i] = a[1]; d.az[i] = a[2];
}

void launch_set_dynamics(const DevState& d, const double* pos, const double* vel,
                         const double* acc, int row0, int n, double box0, double box1,
                         double box2, bool kept, cudaStream_t st) {
  if (n == 0) return;
  k_set_dynamics<<<(n + 255) / 256, 256, 0, st>>>(d, pos, vel, acc, row0, n, box0, box1, box2,
                                                  kept ? 1 : 0);
}

// Storage rows of one replica back to upload order, three doubles per row:
// output row k comes from storage row loc[row0 + k], so the writes (to device
// memory or straight to page-locked host memory) are in order.
__global__ void k_soa_to_aos(const double* x, const double* y, const double* z,
                             const uint32_t* loc, int row0, double* aos, int n) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const uint32_t i = loc[row0 + k];
  aos[3 * (size_t)k] = x[i];
  aos[3 * (size_t)k + 1] = y[i];
  aos[3 * (size_t)k + 2] = z[i];
}

void launch_soa_to_aos(const double* x, const double* y, const double* z, const uint32_t* loc,
                       int row0, double* aos, int n, cudaStream_t st) {
  if (n == 0) return;
  k_soa_to_aos<<<(n + 255) / 256, 256, 0, st>>>(x, y, z, loc, row0, aos, n);
}

// The four u32 fields of rows row0 .. row0 + n - 1 in upload order (loc maps
// upload rows to storage rows): out[f * n + k] = field f of upload row k.
__global__ void k_gather_u32x4(const uint32_t* a, const uint32_t* b, const uint32_t* c,
                               const uint32_t* e, const uint32_t* loc, int row0, uint32_t* out,
                               int n) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const uint32_t i = loc[row0 + k];
  out[k] = a[i];
  out[(size_t)n + k] = b[i];
  out[2 * (size_t)n + k] = c[i];
  out[3 * (size_t)n + k] = e[i];
}

void launch_gather_u32x4(const uint32_t* a, const uint32_t* b, const uint32_t* c,
                         const uint32_t* e, const uint32_t* loc, int row0, uint32_t* out, int n,
                         cudaStream_t st) {
  if (n == 0) return;
  k_gather_u32x4<<<(n + 255) / 256, 256, 0, st>>>(a, b, c, e, loc, row0, out, n);
}

// ------------------------------------------------------------ observables
// Observer::KineticTempera, Pressure and Diffusion (observer.hpp:82-178) of
// the replicas whose step counter is a multiple of the period. Row sums are
// taken per row block, molecule values per molecule; one block per replica
// then reduces them in a fixed order, so a record does not depend on timing.
__device__ __forceinline__ bool obs_due(const DevState& d, int r, int period) {
  return period > 0 && (d.rep_time[r] % (uint32_t)period) == 0u;
}

__device__ __forceinline__ double sq3(double x, double y, double z) {
  return __dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z));
}

__global__ void __launch_bounds__(kRowBlock) k_obs_rows(DevState d, ObsBuffers b) {
  __shared__ double sv[5][kRowBlock / 32];
  __shared__ long long sq[3][kRowBlock / 32];
  const int r = d.blk_rep[blockIdx.x];
  if (!obs_due(d, r, b.period)) return;
  const int i = d.blk_row[blockIdx.x] + threadIdx.x;
  const RepDev* R = d.reps + r;
  double v[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  long long q[3] = {0, 0, 0};
  if (i < R->row_off + R->n) {
    v[0] = __dmul_rn(d.vx[i], d.vx[i]);
    v[1] = __dmul_rn(d.vy[i], d.vy[i]);
    v[2] = __dmul_rn(d.vz[i], d.vz[i]);
    v[3] = sq3(d.dsx[i], d.dsy[i], d.dsz[i]);
    // Diffusion's D_sol runs over the rows from amp_num on (observer.hpp:169-170)
    const uint32_t u = d.orig[i] - (uint32_t)R->row_off;
    v[4] = u >= (uint32_t)R->n_amp ? v[3] : 0.0;
    // press of rows that took part in the pair pass (rows a reaction added
    // in this step start with press 0, chemmanager.hpp:59)
    const int s = (int)d.rank[i];
    if (s < d.cell_start[R->cell_off + R->ncell]) {
      const long long* ps = d.pq + 4 * (size_t)s;
      q[0] = ps[0];
      q[1] = ps[1];
      q[2] = ps[2];
    }
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
    for (int k = 0; k < 5; k++) v[k] = __dadd_rn(v[k], __shfl_down_sync(0xffffffffu, v[k], o));
#pragma unroll
    for (int k = 0; k < 3; k++) q[k] += __shfl_down_sync(0xffffffffu, q[k], o);
  }
  if (lane == 0) {
    for (int k = 0; k < 5; k++) sv[k][w] = v[k];
    for (int k = 0; k < 3; k++) sq[k][w] = q[k];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    ObsPart P;
    double t[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    long long tq[3] = {0, 0, 0};
    for (int ww = 0; ww < kRowBlock / 32; ww++) {
      for (int k = 0; k < 5; k++) t[k] = __dadd_rn(t[k], sv[k][ww]);
      for (int k = 0; k < 3; k++) tq[k] += sq[k][ww];
    }
    for (int k = 0; k < 3; k++) {
      P.v2[k] = t[k];
      P.pq[k] = tq[k];
    }
    P.ds2 = t[3];
    P.dsol2 = t[4];
    b.part[blockIdx.x] = P;
  }
}

// Bonded virial per molecule (CalcBondBendGlobalCell's d_vir,
// bdf_calculator.hpp:160-189) of the molecules that took part in the step's
// bonded pass.
__global__ void k_obs_bonds(DevState d, ObsBuffers b, int n_amp_tot, const int* amp_rep) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= n_amp_tot) return;
  const int r = amp_rep[m];
  if (!obs_due(d, r, b.period)) return;
  const RepDev* R = d.reps + r;
  double* out = b.mvir + 3 * (size_t)m;
  if (m - R->amp_off >= R->n_amp) {
    out[0] = out[1] = out[2] = 0.0;
    return;
  }
  int t[4];
#pragma unroll
  for (int k = 0; k < 4; k++) t[k] = (int)d.rank[d.topol[4 * (size_t)m + k]];
  int cx, cy, cz;
  cell_xyz((int)d.scell[t[0]] - R->cell_off, R->nc, cx, cy, cz);
  float3 p[4];
#pragma unroll
  for (int k = 0; k < 4; k++) p[k] = rel_pos(d, R, t[k], cx, cy, cz);
  float3 F[4], v;
  chain_forces(p, R->cf_s, d.cf_bend[m], F, &v);
  out[0] = (double)v.x;
  out[1] = (double)v.y;
  out[2] = (double)v.z;
}

// Diffusion's molecule term (observer.hpp:157-165): the mean delta_sumr of
// rows 4i .. 4i+3 (upload order), squared.
__global__ void k_obs_lipid(DevState d, ObsBuffers b, int n_amp_tot, const int* amp_rep) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= n_amp_tot) return;
  const int r = amp_rep[m];
  if (!obs_due(d, r, b.period)) return;
  const RepDev* R = d.reps + r;
  const int a = m - R->amp_off;
  if (a >= R->n_amp) {
    b.mdif[m] = 0.0;
    return;
  }
  double s[3] = {0.0, 0.0, 0.0};
  for (int k = 0; k < kAllUnit; k++) {
    const int u = kAllUnit * a + k;
    if (u >= R->n) break;
    const uint32_t i = d.loc[R->row_off + u];
    s[0] = __dadd_rn(s[0], d.dsx[i]);
    s[1] = __dadd_rn(s[1], d.dsy[i]);
    s[2] = __dadd_rn(s[2], d.dsz[i]);
  }
  const double inv = (double)kAllUnit;
  b.mdif[m] = sq3(__ddiv_rn(s[0], inv), __ddiv_rn(s[1], inv), __ddiv_rn(s[2], inv));
}

// One block per replica: fixed-order reductions and the record.
constexpr int kObsThreads = 256;
__global__ void __launch_bounds__(kObsThreads) k_obs_finalize(DevState d, ObsBuffers b) {
  __shared__ double sh[11][kObsThreads];
  __shared__ long long shq[3][kObsThreads];
  const int r = blockIdx.x;
  if (!obs_due(d, r, b.period)) return;
  const RepDev* R = d.reps + r;
  const int t = threadIdx.x;
  double v[11];
  long long q[3] = {0, 0, 0};
  for (int k = 0; k < 11; k++) v[k] = 0.0;
  for (int k = R->blk_off + t; k < R->blk_off + R->nblk; k += kObsThreads) {
    const ObsPart& P = b.part[k];
    for (int c = 0; c < 3; c++) {
      v[c] = __dadd_rn(v[c], P.v2[c]);
      q[c] += P.pq[c];
    }
    v[3] = __dadd_rn(v[3], P.ds2);
    v[4] = __dadd_rn(v[4], P.dsol2);
  }
  for (int m = R->amp_off + t; m < R->amp_off + R->n_amp; m += kObsThreads) {
    for (int c = 0; c < 3; c++) v[5 + c] = __dadd_rn(v[5 + c], b.mvir[3 * (size_t)m + c]);
    v[8] = __dadd_rn(v[8], b.mdif[m]);
  }
  for (int k = 0; k < 11; k++) sh[k][t] = v[k];
  for (int k = 0; k < 3; k++) shq[k][t] = q[k];
  __syncthreads();
  for (int w = kObsThreads / 2; w > 0; w >>= 1) {
    if (t < w) {
      for (int k = 0; k < 11; k++) sh[k][t] = __dadd_rn(sh[k][t], sh[k][t + w]);
      for (int k = 0; k < 3; k++) shq[k][t] += shq[k][t + w];
    }
    __syncthreads();
  }
  if (t != 0) return;
  idpd_observation o;
  const double n = (double)R->n;
  o.time = d.rep_time[r];
  o.replica = r;
  o.n = R->n;
  o.n_amp = R->n_amp;
  const double ivol = __dmul_rn(__dmul_rn(R->ibox[0], R->ibox[1]), R->ibox[2]);
  for (int c = 0; c < 3; c++) {
    o.kin_temp[c] = __ddiv_rn(sh[c][0], n);
    o.pair_virial[c] = (double)shq[c][0] * kForceUnscale;
    o.bonded_virial[c] = sh[5 + c][0];
    o.pressure[c] = __dmul_rn(__dadd_rn(__dadd_rn(__dmul_rn(o.pair_virial[c], 0.5), sh[c][0]),
                                        __dmul_rn(o.bonded_virial[c], 0.5)),
                              ivol);
  }
  o.kin_temp[3] = __ddiv_rn(__dadd_rn(__dadd_rn(o.kin_temp[0], o.kin_temp[1]), o.kin_temp[2]), 3.0);
  const int sol = R->n - kAllUnit * R->n_amp;
  o.diffusion[0] = __ddiv_rn(sh[3][0], n);
  o.diffusion[1] = R->n_amp > 0 ? __ddiv_rn(sh[8][0], (double)R->n_amp) : 0.0;
  o.diffusion[2] = sol > 0 ? __ddiv_rn(sh[4][0], (double)sol) : 0.0;
  const int slot = atomicAdd(b.count, 1);
  if (slot < b.cap) b.rec[slot] = o;
}

void launch_observe_bonds(const DevState& d, const ObsBuffers& b, int n_amp_tot,
                          const int* amp_rep, cudaStream_t st) {
  if (n_amp_tot > 0) k_obs_bonds<<<(n_amp_tot + 127) / 128, 128, 0, st>>>(d, b, n_amp_tot, amp_rep);
}

void launch_observe(const DevState& d, const ObsBuffers& b, int nblk, int n_amp_tot,
                    const int* amp_rep, int R, cudaStream_t st) {
  if (nblk > 0) k_obs_rows<<<nblk, kRowBlock, 0, st>>>(d, b);
  if (n_amp_tot > 0) k_obs_lipid<<<(n_amp_tot + 127) / 128, 128, 0, st>>>(d, b, n_amp_tot, amp_rep);
  k_obs_finalize<<<R, kObsThreads, 0, st>>>(d, b);
}

// Density profile: particles per slab along `axis` and per property.
__global__ void k_density_profile(DevState d, int r, int row_off, int n, int axis, int nbins,
                                  unsigned long long* hist) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int i = row_off + k;
  const RepDev* R = d.reps + r;
  const double x = axis == 0 ? d.px[i] : (axis == 1 ? d.py[i] : d.pz[i]);
  int bin = (int)(x * R->ibox[axis] * (double)nbins);
  bin = bin < 0 ? 0 : (bin >= nbins ? nbins - 1 : bin);
  const uint32_t pr = d.prop[i];
  if (pr < 3u) atomicAdd(hist + 3 * bin + pr, 1ull);
}

void launch_density_profile(const DevState& d, int r, int row_off, int n, int axis, int nbins,
                            unsigned long long* hist, cudaStream_t st) {
  if (n > 0) k_density_profile<<<(n + 255) / 256, 256, 0, st>>>(d, r, row_off, n, axis, nbins, hist);
}

// Radial distribution: ordered pairs within r_max over the (2m+1)^3 search
// cells around each particle (FP64 storage positions, minimum image by the
// cells' periodic shifts). Shared-memory histogram per block.
constexpr int kRdfMaxBins = 1024;
__global__ void __launch_bounds__(256) k_rdf(DevState d, int r, int row_off, int n, int nbins,
                                             double r_max, int m, unsigned long long* hist) {
  __shared__ unsigned int h[kRdfMaxBins];
  for (int k = threadIdx.x; k < nbins; k += blockDim.x) h[k] = 0u;
  __syncthreads();
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const RepDev* R = d.reps + r;
  if (k < n) {
    const int i = row_off + k;
    const double xi = d.px[i], yi = d.py[i], zi = d.pz[i];
    int cx, cy, cz;
    cell_xyz((int)d.key[i] - R->cell_off, R->nc, cx, cy, cz);
    const double r2max = r_max * r_max, scale = (double)nbins / r_max;
    for (int dz = -m; dz <= m; dz++) {
      const int qz = cz + dz, sz = qz < 0 ? -1 : (qz >= R->nc[2] ? 1 : 0);
      for (int dy = -m; dy <= m; dy++) {
        const int qy = cy + dy, sy = qy < 0 ? -1 : (qy >= R->nc[1] ? 1 : 0);
        for (int dx = -m; dx <= m; dx++) {
          const int qx = cx + dx, sx = qx < 0 ? -1 : (qx >= R->nc[0] ? 1 : 0);
          const int cell = R->cell_off + ((qz - sz * R->nc[2]) * R->nc[1] + (qy - sy * R->nc[1])) *
                                             R->nc[0] + (qx - sx * R->nc[0]);
          const double shx = sx * R->box[0], shy = sy * R->box[1], shz = sz * R->box[2];
          for (int t = d.cell_start[cell]; t < d.cell_start[cell + 1]; t++) {
            const uint32_t j = d.perm[t];
            if ((int)j == i) continue;
            const double ex = xi - (d.px[j] + shx), ey = yi - (d.py[j] + shy),
                         ez = zi - (d.pz[j] + shz);
            const double dr2 = ex * ex + ey * ey + ez * ez;
            if (dr2 < r2max) {
              int bin = (int)(sqrt(dr2) * scale);
              bin = bin >= nbins ? nbins - 1 : bin;
              atomicAdd(h + bin, 1u);
            }
          }
        }
      }
    }
  }
  __syncthreads();
  for (int q = threadIdx.x; q < nbins; q += blockDim.x)
    if (h[q]) atomicAdd(hist + q, (unsigned long long)h[q]);
}

void launch_rdf(const DevState& d, int r, int row_off, int n, int nbins, double r_max, int m,
                unsigned long long* hist, cudaStream_t st) {
  if (n > 0 && nbins > 0 && nbins <= kRdfMaxBins)
    k_rdf<<<(n + 255) / 256, 256, 0, st>>>(d, r, row_off, n, nbins, r_max, m, hist);
}

}  // namespace idpd
