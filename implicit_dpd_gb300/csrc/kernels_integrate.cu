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
  long long f[3] = {d.fqx[s], d.fqy[s], d.fqz[s]};
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
  d.ax[i] = (double)d.fqx[s] * kForceUnscale;
  d.ay[i] = (double)d.fqy[s] * kForceUnscale;
  d.az[i] = (double)d.fqz[s] * kForceUnscale;
  if (press) {
    press[3 * i] = (double)d.pqx[s] * kForceUnscale;
    press[3 * i + 1] = (double)d.pqy[s] * kForceUnscale;
    press[3 * i + 2] = (double)d.pqz[s] * kForceUnscale;
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

__global__ void k_cm_finalize(DevState d, int R_n, int force_now) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= R_n) return;
  if (!cm_due(d, r, force_now)) return;
  const RepDev* R = d.reps + r;
  const long long* part = reinterpret_cast<const long long*>(d.blk_part);
  long long s[3] = {0, 0, 0};
  for (int b = R->blk_off; b < R->blk_off + R->nblk; b++)
    for (int k = 0; k < 3; k++) s[k] += part[3 * b + k];
  for (int k = 0; k < 3; k++) d.rep_mean[3 * r + k] = ((double)s[k] / kVelScale) / (double)R->n;
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
  k_cm_finalize<<<(R + 127) / 128, 128, 0, st>>>(d, R, force_now ? 1 : 0);
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

// Per-step host exchange: rows of one replica in upload order, 9 doubles
// each (pos, vel, acc), into the storage rows; invalid rows raise an error.
__global__ void k_set_dynamics(DevState d, const double* aos, int row0, int n, double b0, double b1,
                               double b2) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const uint32_t i = d.loc[row0 + k];
  const double* a = aos + 9 * (size_t)k;
  const double box[3] = {b0, b1, b2};
  bool ok = true;
#pragma unroll
  for (int c = 0; c < 3; c++) ok = ok && a[c] >= 0.0 && a[c] <= box[c];
#pragma unroll
  for (int c = 3; c < 9; c++) ok = ok && isfinite(a[c]);
  if (!ok) atomicCAS(d.err, 0, kErrBadCell);
  d.px[i] = a[0]; d.py[i] = a[1]; d.pz[i] = a[2];
  d.vx[i] = a[3]; d.vy[i] = a[4]; d.vz[i] = a[5];
  d.ax[i] = a[6]; d.ay[i] = a[7]; d.az[i] = a[8];
}

void launch_set_dynamics(const DevState& d, const double* aos, int row0, int n, double box0,
                         double box1, double box2, cudaStream_t st) {
  if (n == 0) return;
  k_set_dynamics<<<(n + 255) / 256, 256, 0, st>>>(d, aos, row0, n, box0, box1, box2);
}

// Storage rows [row0, row0 + n) back to upload order: aos[orig - row0] = row.
__global__ void k_soa_to_aos(const double* x, const double* y, const double* z,
                             const uint32_t* orig, int row0, double* aos, int n) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int i = row0 + k;
  const size_t o = (size_t)(orig[i] - (uint32_t)row0);
  aos[3 * o] = x[i];
  aos[3 * o + 1] = y[i];
  aos[3 * o + 2] = z[i];
}

void launch_soa_to_aos(const double* x, const double* y, const double* z, const uint32_t* orig,
                       int row0, double* aos, int n, cudaStream_t st) {
  if (n == 0) return;
  k_soa_to_aos<<<(n + 255) / 256, 256, 0, st>>>(x, y, z, orig, row0, aos, n);
}

}  // namespace idpd
