// The two MDPD passes over the cell list:
//   pass 1, CalcDensity::operator() (nbdf_calculator.hpp:11-60);
//   pass 2, CalcForceEpEpDPD::operator() (nbdf_calculator.hpp:63-145).
// The FP32 kernels form each pair vector from cell-local FP32 coordinates
// (error below 5e-7 per component, independent of the box size), take every
// cutoff decision within kGuard of the cutoff again in FP64 from the FP64
// positions exactly as the reference does (so pair sets are the reference's),
// and sum every pair term as a 64-bit fixed-point integer, which makes the
// result independent of the visiting order and of the launch shape.
// The plain FP64 kernels are the single-system FP64 baseline: the same cell
// list, FP64 throughout, FP64 sums in cell order.
#include "state.cuh"

namespace idpd {

// Pair vector test of one neighbour cell: visits every (dx, dy, dz) in
// dz-major order with the wrapped cell, its FP32 offset and its image shift.
template <class F>
__device__ __forceinline__ void for_each_cell27(const RepDev* R, int cx, int cy, int cz, F&& f) {
  const int nx = R->nc[0], ny = R->nc[1], nz = R->nc[2];
#pragma unroll 1
  for (int dz = -1; dz <= 1; dz++) {
    const int qz = cz + dz;
    const int sz = qz < 0 ? -1 : (qz >= nz ? 1 : 0);
    const int wz = qz - sz * nz;
#pragma unroll 1
    for (int dy = -1; dy <= 1; dy++) {
      const int qy = cy + dy;
      const int sy = qy < 0 ? -1 : (qy >= ny ? 1 : 0);
      const int wy = qy - sy * ny;
      const int row = R->cell_off + (wz * ny + wy) * nx;
#pragma unroll
      for (int dx = -1; dx <= 1; dx++) {
        const int qx = cx + dx;
        const int sx = qx < 0 ? -1 : (qx >= nx ? 1 : 0);
        const int wx = qx - sx * nx;
        f(row + wx, dx, dy, dz, sx, sy, sz);
      }
    }
  }
}

// FP64 squared distance of rows i and j (image shift s * L applied to j),
// in the reference's operation order (nbdf_calculator.hpp:27-29, 86-87).
__device__ __forceinline__ double exact_dr2(const DevState& d, const RepDev* R, uint32_t i,
                                            uint32_t j, int sx, int sy, int sz) {
  const double jx = __dadd_rn(d.px[j], __dmul_rn((double)sx, R->box[0]));
  const double jy = __dadd_rn(d.py[j], __dmul_rn((double)sy, R->box[1]));
  const double jz = __dadd_rn(d.pz[j], __dmul_rn((double)sz, R->box[2]));
  const double ex = __dsub_rn(d.px[i], jx), ey = __dsub_rn(d.py[i], jy),
               ez = __dsub_rn(d.pz[i], jz);
  return __dadd_rn(__dadd_rn(__dmul_rn(ex, ex), __dmul_rn(ey, ey)), __dmul_rn(ez, ez));
}

__device__ __forceinline__ long long to_fix(float v, float scale) {
  return __float2ll_rn(v * scale);
}

// ------------------------------------------------------------- pass 1
__global__ void __launch_bounds__(kRowBlock) k_density_f32(DevState d) {
  const int r = d.blk_rep[blockIdx.x];
  const int s = d.blk_row[blockIdx.x] + threadIdx.x;
  const RepDev* R = d.reps + r;
  if (s >= R->row_off + R->n) return;
  const float4 pi = d.posf[s];
  int cx, cy, cz;
  cell_xyz((int)d.scell[s] - R->cell_off, R->nc, cx, cy, cz);
  const bool warren = R->form == IDPD_FORM_WARREN_K;
  const float cut2 = warren ? R->wrd * R->wrd : 1.0f;
  const double cut2d = warren ? (double)R->wrd * (double)R->wrd : 1.0;
  const float inv_rd = R->winv_rd, wnorm = R->wnorm;
  const float csx = R->cs_f[0], csy = R->cs_f[1], csz = R->cs_f[2];
  long long q0 = 0, q1 = 0, q2 = 0;
  for_each_cell27(R, cx, cy, cz, [&](int cn, int dx, int dy, int dz, int sx, int sy, int sz) {
    const int tb = d.cell_start[cn], te = d.cell_start[cn + 1];
    const float bx = pi.x - (float)dx * csx, by = pi.y - (float)dy * csy,
                bz = pi.z - (float)dz * csz;
    for (int t = tb; t < te; t++) {
      if (t == s) continue;
      const float4 pj = __ldg(d.posf + t);
      const float ex = bx - pj.x, ey = by - pj.y, ez = bz - pj.z;
      const float dr2 = ex * ex + ey * ey + ez * ez;
      if (dr2 < cut2 + kGuard) {
        bool in = dr2 < cut2;
        if (fabsf(dr2 - cut2) <= kGuard || dr2 < 1.0e-10f) {
          const double e2 = exact_dr2(d, R, d.perm[s], d.perm[t], sx, sy, sz);
          in = e2 < cut2d && e2 != 0.0;
        }
        if (in) {
          const float dr = sqrtf(dr2);
          float w = warren ? 1.0f - dr * inv_rd : 1.0f - dr;
          w = warren ? wnorm * (w * w) : w * w;
          const long long v = to_fix(w, kDensScaleF);
          const uint32_t pr = fbits(pj.w);
          if (pr == 0) q0 += v;
          else if (pr == 1) q1 += v;
          else q2 += v;
        }
      }
    }
  });
  d.densf[s] = make_float4((float)((double)q0 * kDensUnscale), (float)((double)q1 * kDensUnscale),
                           (float)((double)q2 * kDensUnscale), 0.0f);
  if (d.dqx) {
    d.dqx[s] = q0;
    d.dqy[s] = q1;
    d.dqz[s] = q2;
  }
}

// Plain FP64 pass 1: FP64 positions of the storage rows, FP64 sums.
__global__ void __launch_bounds__(kRowBlock) k_density_f64(DevState d) {
  const int r = d.blk_rep[blockIdx.x];
  const int s = d.blk_row[blockIdx.x] + threadIdx.x;
  const RepDev* R = d.reps + r;
  if (s >= R->row_off + R->n) return;
  const uint32_t i = d.perm[s];
  const double xi = d.px[i], yi = d.py[i], zi = d.pz[i];
  int cx, cy, cz;
  cell_xyz((int)d.scell[s] - R->cell_off, R->nc, cx, cy, cz);
  const bool warren = R->form == IDPD_FORM_WARREN_K;
  const double rd = (double)R->wrd;
  const double cut2 = warren ? rd * rd : 1.0;
  const double wn = 15.0 / (2.0 * 3.14159265358979323846 * rd * rd * rd);
  double a0 = 0.0, a1 = 0.0, a2 = 0.0;
  for_each_cell27(R, cx, cy, cz, [&](int cn, int dx, int dy, int dz, int sx, int sy, int sz) {
    const int tb = d.cell_start[cn], te = d.cell_start[cn + 1];
    const double shx = (double)sx * R->box[0], shy = (double)sy * R->box[1],
                 shz = (double)sz * R->box[2];
    for (int t = tb; t < te; t++) {
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
}

void launch_density(const DevState& d, int nblk, bool fp64, cudaStream_t st) {
  if (nblk == 0) return;
  if (fp64)
    k_density_f64<<<nblk, kRowBlock, 0, st>>>(d);
  else
    k_density_f32<<<nblk, kRowBlock, 0, st>>>(d);
}

// ------------------------------------------------------------- pass 2
struct PairTables {
  float cf_c[9], cf_g[9], cf_r[9], cf_m[27];
};

// Conservative + random + dissipative magnitude over dr
// (nbdf_calculator.hpp:108-132) for one pair, FP32.
__device__ __forceinline__ float pair_all_cf(const PairTables& T, const RepDev* R, int form,
                                             uint32_t pri, uint32_t prj, float dr2, float ex,
                                             float ey, float ez, float4 vi, float4 vj, float4 di,
                                             float4 dj, uint32_t idi, uint32_t idj, uint32_t seed) {
  const float inv_dr = rsqrtf(dr2);
  const float dr = dr2 * inv_dr;
  const float w = 1.0f - dr;
  const float sqw = sqrtf(w);
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

// One thread per sorted slot. Phase A walks the 27 cells and writes the
// in-range neighbours (sorted index | cell-offset code << 27) into a
// per-thread column of shared memory; phase B evaluates the pairs of the
// column with all lanes busy. A full column is evaluated before the walk
// continues, so there is no neighbour limit.
template <bool PRESS>
__global__ void __launch_bounds__(kRowBlock) k_force_f32(DevState d, int cap) {
  extern __shared__ uint32_t lst[];
  __shared__ PairTables T;
  const int r = d.blk_rep[blockIdx.x];
  const RepDev* R = d.reps + r;
  for (int k = threadIdx.x; k < 54; k += blockDim.x) {
    float v;
    if (k < 9) v = R->cf_c[k];
    else if (k < 18) v = R->cf_g[k - 9];
    else if (k < 27) v = R->cf_r[k - 18];
    else v = R->cf_m[k - 27];
    (&T.cf_c[0])[k] = v;
  }
  __syncthreads();
  const int s = d.blk_row[blockIdx.x] + threadIdx.x;
  if (s >= R->row_off + R->n) return;
  const int B = blockDim.x;
  uint32_t* col = lst + threadIdx.x;
  const float4 pi = d.posf[s];
  const float4 vi = d.velf[s];
  const float4 di = d.densf[s];
  const uint32_t idi = fbits(vi.w), pri = fbits(pi.w);
  const uint32_t seed = R->seed + d.rep_time[r];
  const int form = R->form;
  const float csx = R->cs_f[0], csy = R->cs_f[1], csz = R->cs_f[2];
  int cx, cy, cz;
  cell_xyz((int)d.scell[s] - R->cell_off, R->nc, cx, cy, cz);
  long long fx = 0, fy = 0, fz = 0, px = 0, py = 0, pz = 0;

  auto flush = [&](int cnt) {
    for (int k = 0; k < cnt; k++) {
      const uint32_t e = col[k * B];
      const int t = (int)(e & 0x7ffffffu);
      const int code = (int)(e >> 27);
      const int dz = code / 9 - 1, dy = (code / 3) % 3 - 1, dx = code % 3 - 1;
      const float4 vj = __ldg(d.velf + t);
      const uint32_t idj = fbits(vj.w);
      if (idj == idi) continue;
      const float4 pj = __ldg(d.posf + t);
      const float4 dj = __ldg(d.densf + t);
      const float ex = (pi.x - (float)dx * csx) - pj.x;
      const float ey = (pi.y - (float)dy * csy) - pj.y;
      const float ez = (pi.z - (float)dz * csz) - pj.z;
      const float dr2 = ex * ex + ey * ey + ez * ez;
      const float a = pair_all_cf(T, R, form, pri, fbits(pj.w), dr2, ex, ey, ez, vi, vj, di, dj,
                                  idi, idj, seed);
      if (!isfinite(a)) atomicCAS(d.err, 0, kErrNonFinite);
      const float gx = a * ex, gy = a * ey, gz = a * ez;
      fx += to_fix(gx, kForceScaleF);
      fy += to_fix(gy, kForceScaleF);
      fz += to_fix(gz, kForceScaleF);
      if (PRESS) {
        px += to_fix(gx * ex, kForceScaleF);
        py += to_fix(gy * ey, kForceScaleF);
        pz += to_fix(gz * ez, kForceScaleF);
      }
    }
  };

  int cnt = 0;
  for_each_cell27(R, cx, cy, cz, [&](int cn, int dx, int dy, int dz, int sx, int sy, int sz) {
    const int tb = d.cell_start[cn], te = d.cell_start[cn + 1];
    const float bx = pi.x - (float)dx * csx, by = pi.y - (float)dy * csy,
                bz = pi.z - (float)dz * csz;
    const uint32_t code = (uint32_t)((dz + 1) * 9 + (dy + 1) * 3 + (dx + 1)) << 27;
    for (int t = tb; t < te; t++) {
      if (t == s) continue;
      const float4 pj = __ldg(d.posf + t);
      const float ex = bx - pj.x, ey = by - pj.y, ez = bz - pj.z;
      const float dr2 = ex * ex + ey * ey + ez * ez;
      if (dr2 < 1.0f + kGuard) {
        bool in = dr2 < 1.0f;
        if (fabsf(dr2 - 1.0f) <= kGuard)
          in = exact_dr2(d, R, d.perm[s], d.perm[t], sx, sy, sz) < 1.0;
        if (in) {
          col[cnt * B] = (uint32_t)t | code;
          if (++cnt == cap) {
            flush(cnt);
            cnt = 0;
          }
        }
      }
    }
  });
  flush(cnt);
  d.fqx[s] = fx;
  d.fqy[s] = fy;
  d.fqz[s] = fz;
  if (PRESS) {
    d.pqx[s] = px;
    d.pqy[s] = py;
    d.pqz[s] = pz;
  }
}

// Plain FP64 pass 2 (the FP64 baseline): the reference's arithmetic on the
// FP64 rows, FP64 sums in cell order, stored as 2^-32 fixed point.
template <bool PRESS>
__global__ void __launch_bounds__(kRowBlock) k_force_f64(DevState d) {
  const int r = d.blk_rep[blockIdx.x];
  const int s = d.blk_row[blockIdx.x] + threadIdx.x;
  const RepDev* R = d.reps + r;
  if (s >= R->row_off + R->n) return;
  const uint32_t i = d.perm[s];
  const double xi = d.px[i], yi = d.py[i], zi = d.pz[i];
  const double vxi = d.vx[i], vyi = d.vy[i], vzi = d.vz[i];
  const uint32_t idi = d.id[i], pri = d.prop[i];
  const double di0 = d.dens64[3 * s], di1 = d.dens64[3 * s + 1], di2 = d.dens64[3 * s + 2];
  const uint32_t seed = R->seed + d.rep_time[r];
  const int form = R->form;
  const double rd = (double)R->wrd;
  int cx, cy, cz;
  cell_xyz((int)d.scell[s] - R->cell_off, R->nc, cx, cy, cz);
  double f0 = 0.0, f1 = 0.0, f2 = 0.0, p0 = 0.0, p1 = 0.0, p2 = 0.0;
  for_each_cell27(R, cx, cy, cz, [&](int cn, int dx, int dy, int dz, int sx, int sy, int sz) {
    const int tb = d.cell_start[cn], te = d.cell_start[cn + 1];
    const double shx = (double)sx * R->box[0], shy = (double)sy * R->box[1],
                 shz = (double)sz * R->box[2];
    for (int t = tb; t < te; t++) {
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
          cons = (double)R->wa * w + (double)R->wb * rho * wb;
        } else {
          const double cf_pair = dr >= kArcD ? (double)R->cf_c[k] * (dr - kArcD) : 0.0;
          const double cf_mbd = (double)R->cf_m[3 * k] * (di0 + dj0) +
                                (double)R->cf_m[3 * k + 1] * (di1 + dj1) +
                                (double)R->cf_m[3 * k + 2] * (di2 + dj2);
          cons = (cf_pair + cf_mbd) * w;
        }
        const double all = (cons + (double)R->cf_r[k] * sqrt(w) * rnd -
                            (double)R->cf_g[k] * w * (ex * dvx + ey * dvy + ez * dvz) * inv_dr) *
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

void launch_force(const DevState& d, int nblk, bool fp64, bool with_press, const PairTuning& tu,
                  cudaStream_t st) {
  if (nblk == 0) return;
  if (fp64) {
    if (with_press)
      k_force_f64<true><<<nblk, kRowBlock, 0, st>>>(d);
    else
      k_force_f64<false><<<nblk, kRowBlock, 0, st>>>(d);
    return;
  }
  const size_t smem = (size_t)tu.list_cap * kRowBlock * sizeof(uint32_t);
  if (with_press)
    k_force_f32<true><<<nblk, kRowBlock, smem, st>>>(d, tu.list_cap);
  else
    k_force_f32<false><<<nblk, kRowBlock, smem, st>>>(d, tu.list_cap);
}

// -------------------------------------------- neighbour centre of mass
// The hydrophilic / hydrophobic neighbour sums of pass 1
// (nbdf_calculator.hpp:23-51) and FPDPD::copyFromForce (ptcl_class.hpp:53-57),
// for the fine-grained API and the chemistry: reach of two cells (radius
// rn_c = 1.2), positions summed relative to the row's cell origin in 2^-40
// fixed point, written per storage row.
__global__ void __launch_bounds__(kRowBlock) k_com(DevState d, double* cm, uint32_t* cnt_out) {
  const int r = d.blk_rep[blockIdx.x];
  const int s = d.blk_row[blockIdx.x] + threadIdx.x;
  const RepDev* R = d.reps + r;
  if (s >= R->row_off + R->n) return;
  const int nx = R->nc[0], ny = R->nc[1], nz = R->nc[2];
  if (nx < 5 || ny < 5 || nz < 5) {
    atomicCAS(d.err, 0, kErrComBox);
    return;
  }
  const float4 pi = d.posf[s];
  int cx, cy, cz;
  cell_xyz((int)d.scell[s] - R->cell_off, R->nc, cx, cy, cz);
  const float rn2 = 1.44f;
  const double rn2d = 1.2 * 1.2;
  // hydrophilic sum starts at the row itself with count 1 (nbdf_calculator.hpp:23-24)
  long long hl[3] = {to_fix(pi.x, kPosScaleF), to_fix(pi.y, kPosScaleF), to_fix(pi.z, kPosScaleF)};
  long long hb[3] = {0, 0, 0};
  uint32_t cl = 1, cb = 0;
  const uint32_t i = d.perm[s];
  for (int dz = -2; dz <= 2; dz++) {
    const int qz = cz + dz, sz = qz < 0 ? -1 : (qz >= nz ? 1 : 0), wz = qz - sz * nz;
    for (int dy = -2; dy <= 2; dy++) {
      const int qy = cy + dy, sy = qy < 0 ? -1 : (qy >= ny ? 1 : 0), wy = qy - sy * ny;
      for (int dx = -2; dx <= 2; dx++) {
        const int qx = cx + dx, sx = qx < 0 ? -1 : (qx >= nx ? 1 : 0), wx = qx - sx * nx;
        const int cn = R->cell_off + (wz * ny + wy) * nx + wx;
        const float ox = (float)dx * R->cs_f[0], oy = (float)dy * R->cs_f[1],
                    oz = (float)dz * R->cs_f[2];
        for (int t = d.cell_start[cn]; t < d.cell_start[cn + 1]; t++) {
          if (t == s) continue;
          const float4 pj = d.posf[t];
          const float jx = pj.x + ox, jy = pj.y + oy, jz = pj.z + oz;
          const float ex = pi.x - jx, ey = pi.y - jy, ez = pi.z - jz;
          const float dr2 = ex * ex + ey * ey + ez * ez;
          if (dr2 >= rn2 + kGuard) continue;
          bool in_b = dr2 < rn2, in_l = dr2 < 1.0f;
          if (fabsf(dr2 - rn2) <= kGuard || fabsf(dr2 - 1.0f) <= kGuard || dr2 < 1.0e-10f) {
            const double e2 = exact_dr2(d, R, i, d.perm[t], sx, sy, sz);
            in_b = e2 < rn2d && e2 != 0.0;
            in_l = in_b && e2 < 1.0;
          }
          const uint32_t pr = fbits(pj.w);
          if (in_b && pr == 1) {
            hb[0] += to_fix(jx, kPosScaleF);
            hb[1] += to_fix(jy, kPosScaleF);
            hb[2] += to_fix(jz, kPosScaleF);
            cb++;
          }
          if (in_l && pr == 0) {
            hl[0] += to_fix(jx, kPosScaleF);
            hl[1] += to_fix(jy, kPosScaleF);
            hl[2] += to_fix(jz, kPosScaleF);
            cl++;
          }
        }
      }
    }
  }
  const double org[3] = {(double)cx * R->cs[0], (double)cy * R->cs[1], (double)cz * R->cs[2]};
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
