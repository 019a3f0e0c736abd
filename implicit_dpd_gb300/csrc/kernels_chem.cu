// ChemManager::RandomChemEvent on the device: the single-node form with
// LOCAL_CHEM_EVENT, which every CHEM_MODE build of the reference uses
// (include/user_defs.h:6-8). It restates chemmanager.hpp:244-281 with
// DetermineTargetIdWithCorePos (:115-162), GetCorePos (:84-113),
// GetMembraneTangRandomVec (:164-172) and CreateAmpPart (:35-67).
//
// The reaction decisions consume the MT19937 stream of PS::MT in the
// reference's order: cores outer, molecules inner, one genrand_real1 per
// molecule whose head lies inside the reaction cone. The cone test is
// parallel over molecules and keeps the reference's FP64 operation order
// (no contraction), so the flags are exact; a single block then walks the
// flags in order, producing the stream 624 words at a time with a
// block-parallel twist, and places the new molecules. New particles are
// appended after the last row (ids, rows and molecule slots continue the
// existing ones) and their molecules are appended to the bonded topology, as
// the multi-rank reference rebuilds it from amp_id / unit every step.
#include "state.cuh"

namespace idpd {
namespace {

constexpr int kChemThreads = 1024;
constexpr int kMtN = 624;
constexpr int kMtM = 397;
constexpr double kTempera = 1.0;
constexpr double kPi = 3.14159265358979323846;
constexpr double kRnC2 = 1.2 * 1.2;  // Parameter::rn_c2 (parameter.hpp:204-205)

// ---------------------------------------------------------------- MT19937
// Matsumoto & Nishimura (1998), mt19937ar: genrand_int32 regenerates the
// 624-word state when it is used up and tempers each word on output.
__device__ __forceinline__ uint32_t mt_mix(uint32_t a, uint32_t b) {
  const uint32_t y = (a & 0x80000000u) | (b & 0x7fffffffu);
  return (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
}

__device__ __forceinline__ uint32_t mt_temper(uint32_t y) {
  y ^= y >> 11;
  y ^= (y << 7) & 0x9d2c5680u;
  y ^= (y << 15) & 0xefc60000u;
  y ^= y >> 18;
  return y;
}

struct MtBlock {
  uint32_t mt[kMtN];   // raw state
  uint32_t out[kMtN];  // tempered words of the current state
  int mti;             // next word to hand out
};

// The in-place regeneration of the state. Word k reads words k + 1 and
// k + 397 (mod 624); words below k are already new when the sequential loop
// reaches k. Words [0, 227) read only old words, [227, 454) and [454, 623)
// read new words of the previous range, and word 623 reads new words 0 and
// 396: four phases of the whole block. Needs blockDim.x >= 624.
__device__ void mt_twist(MtBlock& S) {
  const int k = threadIdx.x;
  uint32_t v = 0;
  if (k < 227) v = S.mt[k + kMtM] ^ mt_mix(S.mt[k], S.mt[k + 1]);
  __syncthreads();
  if (k < 227) S.mt[k] = v;
  __syncthreads();
  if (k >= 227 && k < 454) v = S.mt[k - 227] ^ mt_mix(S.mt[k], S.mt[k + 1]);
  __syncthreads();
  if (k >= 227 && k < 454) S.mt[k] = v;
  __syncthreads();
  if (k >= 454 && k < 623) v = S.mt[k - 227] ^ mt_mix(S.mt[k], S.mt[k + 1]);
  __syncthreads();
  if (k >= 454 && k < 623) S.mt[k] = v;
  __syncthreads();
  if (k == 623) S.mt[623] = S.mt[kMtM - 1] ^ mt_mix(S.mt[623], S.mt[0]);
  __syncthreads();
  if (k < kMtN) S.out[k] = mt_temper(S.mt[k]);
  if (k == 0) S.mti = 0;
  __syncthreads();
}

// The next `count` words of the stream: the thread of rank r < count (with
// want set) receives word r. Every thread of the block calls it with the
// same count.
__device__ uint32_t mt_serve(MtBlock& S, bool want, int rank, int count) {
  uint32_t val = 0;
  int done = 0;
  while (done < count) {
    if (S.mti >= kMtN) mt_twist(S);
    const int base = S.mti;
    const int take = min(kMtN - base, count - done);
    if (want && rank >= done && rank < done + take) val = S.out[base + rank - done];
    done += take;
    __syncthreads();
    if (threadIdx.x == 0) S.mti = base + take;
    __syncthreads();
  }
  return val;
}

// genrand_real1 = u / (2^32 - 1), genrand_real3 = (u + 0.5) / 2^32.
__device__ __forceinline__ double mt_real1(uint32_t u) {
  return __dmul_rn((double)u, 1.0 / 4294967295.0);
}
__device__ __forceinline__ double mt_real3(uint32_t u) {
  return __dmul_rn(__dadd_rn((double)u, 0.5), 1.0 / 4294967296.0);
}

__device__ int block_scan_excl(int v, int* ws, int& total) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) ws[w] = incl;
  __syncthreads();
  if (w == 0) {
    const int s = lane < (int)(blockDim.x >> 5) ? ws[lane] : 0;
    int si = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, si, o);
      if (lane >= o) si += t;
    }
    ws[lane] = si - s;
    if (lane == 31) ws[32] = si;
  }
  __syncthreads();
  total = ws[32];
  const int res = incl - v + ws[w];
  __syncthreads();
  return res;
}

// ------------------------------------------------------ FP64 vector steps
// ForceBonded::MinImage (bdf_calculator.hpp:55-59).
__device__ __forceinline__ void min_image(double* v, const RepDev* R) {
#pragma unroll
  for (int k = 0; k < 3; k++) v[k] = __dsub_rn(v[k], __dmul_rn(R->box[k], round(__dmul_rn(v[k], R->ibox[k]))));
}

__device__ __forceinline__ double dot3(const double* a, const double* b) {
  return __dadd_rn(__dadd_rn(__dmul_rn(a[0], b[0]), __dmul_rn(a[1], b[1])), __dmul_rn(a[2], b[2]));
}

// ChemManager::Normalize (chemmanager.hpp:8-10).
__device__ __forceinline__ void normalize(double* v) {
  const double s = sqrt(dot3(v, v));
#pragma unroll
  for (int k = 0; k < 3; k++) v[k] = __ddiv_rn(v[k], s);
}

// ChemManager::ApplyPBC (chemmanager.hpp:22-26).
__device__ __forceinline__ void apply_pbc(double* x, const RepDev* R) {
#pragma unroll
  for (int k = 0; k < 3; k++) x[k] = __dsub_rn(x[k], __dmul_rn(floor(__dmul_rn(x[k], R->ibox[k])), R->box[k]));
}

// GenThermalVeloc (chemmanager.hpp:18-20): the first draw feeds the log.
__device__ __forceinline__ double thermal_veloc(uint32_t u1, uint32_t u2) {
  const double a = sqrt(__dmul_rn(-2.0 * kTempera, log(mt_real3(u1))));
  return __dmul_rn(a, cos(__dmul_rn(2.0 * kPi, mt_real3(u2))));
}

// ------------------------------------------------------------- kernels
__global__ void k_chem_begin(ChemDev* c, const uint32_t* rep_time, int force) {
  if (threadIdx.x == 0) {
    const int act = !c->stopped && (force || rep_time[0] >= c->beg_chem);
    c->active = act;
    c->stop_now = 0;
    if (act) c->n_targets = 0;
  }
  if (threadIdx.x < kChemMaxCore) c->core_row[threadIdx.x] = -1;
}

// GetCorePos, first half: the row of each core particle (ids are unique).
__global__ void __launch_bounds__(kRowBlock) k_chem_find(DevState d, ChemDev* c) {
  if (!c->active) return;
  const int i = d.blk_row[blockIdx.x] + threadIdx.x;
  const RepDev* R = d.reps;
  if (i >= R->row_off + R->n) return;
  const uint32_t id = d.id[i];
  for (int k = 0; k < c->n_core; k++)
    if (c->core_id[k] == id) c->core_row[k] = i;
}

// GetCorePos, second half, and the core geometry of
// DetermineTargetIdWithCorePos (:126-138): one warp per core. The neighbour
// centres of mass are CalcDensity's (nbdf_calculator.hpp:22-55 and
// ptcl_class.hpp:53-57): hydrophobic beads within rn_c, hydrophilic beads
// within 1 plus the particle itself, over image-shifted positions.
__global__ void k_chem_geom(DevState d, ChemDev* c) {
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (!c->active || w >= c->n_core) return;
  const RepDev* R = d.reps;
  const int i = c->core_row[w];
  double raw[9];
#pragma unroll
  for (int k = 0; k < 9; k++) raw[k] = -1.0;
  if (i >= 0) {
    const double xi = d.px[i], yi = d.py[i], zi = d.pz[i];
    const int m = R->reach + 1;  // search cells >= 1 / reach: m layers cover rn_c
    if (R->nc[0] < 2 * m + 1 || R->nc[1] < 2 * m + 1 || R->nc[2] < 2 * m + 1) {
      if (lane == 0) atomicCAS(d.err, 0, kErrComBox);
      return;
    }
    int cx, cy, cz;
    cell_xyz((int)d.key[i] - R->cell_off, R->nc, cx, cy, cz);
    double hb[3] = {0.0, 0.0, 0.0}, hl[3] = {0.0, 0.0, 0.0};
    int cb = 0, cl = 0;
    for (int dz = -m; dz <= m; dz++) {
      const int qz = cz + dz, sz = qz < 0 ? -1 : (qz >= R->nc[2] ? 1 : 0);
      for (int dy = -m; dy <= m; dy++) {
        const int qy = cy + dy, sy = qy < 0 ? -1 : (qy >= R->nc[1] ? 1 : 0);
        for (int dx = -m; dx <= m; dx++) {
          const int qx = cx + dx, sx = qx < 0 ? -1 : (qx >= R->nc[0] ? 1 : 0);
          const int cell = R->cell_off + ((qz - sz * R->nc[2]) * R->nc[1] + (qy - sy * R->nc[1])) *
                                             R->nc[0] + (qx - sx * R->nc[0]);
          const int tb = d.cell_start[cell], te = d.cell_start[cell + 1];
          for (int t = tb + lane; t < te; t += 32) {
            const uint32_t j = d.perm[t];
            // the image nearest to the core (the cells may be those of an
            // earlier step while neighbour lists are reused)
            const double jx = __dadd_rn(d.px[j], __dmul_rn((double)nearest_image(xi, d.px[j], R->box[0]), R->box[0]));
            const double jy = __dadd_rn(d.py[j], __dmul_rn((double)nearest_image(yi, d.py[j], R->box[1]), R->box[1]));
            const double jz = __dadd_rn(d.pz[j], __dmul_rn((double)nearest_image(zi, d.pz[j], R->box[2]), R->box[2]));
            const double ex = __dsub_rn(xi, jx), ey = __dsub_rn(yi, jy), ez = __dsub_rn(zi, jz);
            const double dr2 = __dadd_rn(__dadd_rn(__dmul_rn(ex, ex), __dmul_rn(ey, ey)), __dmul_rn(ez, ez));
            if (dr2 < kRnC2 && dr2 != 0.0) {
              const uint32_t pj = d.prop[j];
              if (pj == 1u) {  // Hyphob
                hb[0] = __dadd_rn(hb[0], jx); hb[1] = __dadd_rn(hb[1], jy); hb[2] = __dadd_rn(hb[2], jz);
                cb++;
              }
              if (dr2 < 1.0 && pj == 0u) {  // Hyphil
                hl[0] = __dadd_rn(hl[0], jx); hl[1] = __dadd_rn(hl[1], jy); hl[2] = __dadd_rn(hl[2], jz);
                cl++;
              }
            }
          }
        }
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
      for (int k = 0; k < 3; k++) {
        hb[k] = __dadd_rn(hb[k], __shfl_xor_sync(0xffffffffu, hb[k], o));
        hl[k] = __dadd_rn(hl[k], __shfl_xor_sync(0xffffffffu, hl[k], o));
      }
      cb += __shfl_xor_sync(0xffffffffu, cb, o);
      cl += __shfl_xor_sync(0xffffffffu, cl, o);
    }
    const double pi3[3] = {xi, yi, zi};
#pragma unroll
    for (int k = 0; k < 3; k++) {
      raw[k] = pi3[k];
      raw[3 + k] = __ddiv_rn(hb[k], (double)cb);
      raw[6 + k] = __ddiv_rn(__dadd_rn(pi3[k], hl[k]), (double)(cl + 1));
    }
  }
  if (lane != 0) return;
  double h[3] = {raw[0], raw[1], raw[2]}, h2t[3], c2cm[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    h2t[k] = __dsub_rn(raw[3 + k], h[k]);
    c2cm[k] = __dsub_rn(raw[6 + k], h[k]);
  }
  min_image(h2t, R);
  normalize(h2t);
  min_image(c2cm, R);
  const double prj = dot3(c2cm, h2t);
#pragma unroll
  for (int k = 0; k < 3; k++) h[k] = __dadd_rn(h[k], __dmul_rn(prj, h2t[k]));
  apply_pbc(h, R);
#pragma unroll
  for (int k = 0; k < 9; k++) c->core_raw[w][k] = raw[k];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    c->core_h[w][k] = h[k];
    c->core_n[w][k] = h2t[k];
  }
}

// DetermineTargetIdWithCorePos (:141-160) without the draw: is the head of
// molecule j inside core k's reaction cone? flag[k * amp_cap + j].
__global__ void __launch_bounds__(kChemThreads) k_chem_cone(DevState d, const ChemDev* c,
                                                            uint8_t* flags, int* chunk,
                                                            int amp_cap) {
  if (!c->active) return;
  const int q = blockIdx.x * kChemThreads + threadIdx.x;
  const int core = q / amp_cap, j = q - core * amp_cap;
  const RepDev* R = d.reps;
  int f = 0;
  if (core < c->n_core && j < (int)c->amp_num) {
    const uint32_t head = d.topol[4 * (size_t)(R->amp_off + j)];
    if (head < (uint32_t)(R->row_off + R->n)) {
      double c2p[3] = {__dsub_rn(d.px[head], c->core_h[core][0]),
                       __dsub_rn(d.py[head], c->core_h[core][1]),
                       __dsub_rn(d.pz[head], c->core_h[core][2])};
      min_image(c2p, R);
      const double* nv = c->core_n[core];
      const double depth = dot3(nv, c2p);
      double tang[3];
#pragma unroll
      for (int k = 0; k < 3; k++) tang[k] = __dsub_rn(c2p[k], __dmul_rn(depth, nv[k]));
      const double rad = sqrt(dot3(tang, tang));
      const double rad_th = __dadd_rn(__dmul_rn(c->influ_grd, depth), c->influ_rad);
      f = (rad <= rad_th) && (depth >= -c->influ_hei) && (depth <= c->influ_dep);
    }
  }
  if (core < c->n_core) flags[q] = (uint8_t)f;
  const int cnt = __syncthreads_count(f);
  if (threadIdx.x == 0) chunk[blockIdx.x] = cnt;
}

// The ordered draws and the new molecules (RandomChemEvent :254-280): one
// block of 1024 threads.
__global__ void __launch_bounds__(kChemThreads) k_chem_event(DevState d, ChemBuffers b, int n_core,
                                                             int amp_cap) {
  __shared__ MtBlock S;
  __shared__ int ws[33];
  ChemDev* c = b.chem;
  if (!c->active) return;
  const int tid = threadIdx.x;
  RepDev* R = d.reps;
  if (tid < kMtN) {
    S.mt[tid] = c->mt[tid];
    S.out[tid] = mt_temper(S.mt[tid]);
  }
  if (tid == 0) S.mti = c->mti;
  __syncthreads();
  const double p_th = c->p_thresld;
  const int total = n_core * amp_cap;
  const int nchunk = (total + kChemThreads - 1) / kChemThreads;
  int nt = 0;
  for (int ch = 0; ch < nchunk; ch++) {
    if (b.chunk[ch] == 0) continue;
    const int q = ch * kChemThreads + tid;
    const int f = q < total ? (int)b.flags[q] : 0;
    int cnt, tcnt;
    const int rank = block_scan_excl(f, ws, cnt);
    const uint32_t u = mt_serve(S, f != 0, rank, cnt);
    const int dec = f && mt_real1(u) <= p_th;
    const int trank = block_scan_excl(dec, ws, tcnt);
    if (dec) {
      const int t = nt + trank;
      const int j = q % amp_cap;
      if (t < c->target_cap) {
        b.targets[2 * t] = d.topol[4 * (size_t)(R->amp_off + j)];
        b.targets[2 * t + 1] = d.topol[4 * (size_t)(R->amp_off + j) + 2];
      }
    }
    nt += tcnt;
  }
  const int n0 = R->n;
  const bool fits = nt <= c->target_cap && n0 + 4 * nt <= c->row_cap &&
                    (int)c->amp_num + nt <= c->amp_cap;
  if (!fits) {
    if (tid == 0) atomicCAS(d.err, 0, kErrChemCapacity);
    nt = 0;
  }
  // placement draws: per target one genrand_real1, then three thermal
  // velocities (two genrand_real3 each) for each of its four beads
  const int nd = 25 * nt;
  for (int base = 0; base < nd; base += kChemThreads) {
    const int cnt = min(kChemThreads, nd - base);
    const uint32_t u = mt_serve(S, tid < cnt, tid, cnt);
    if (tid < cnt) b.draws[base + tid] = u;
  }
  __syncthreads();
  if (tid < kMtN) c->mt[tid] = S.mt[tid];
  if (tid == 0) c->mti = S.mti;
  const uint32_t amp0 = c->amp_num;
  for (int t = tid; t < nt; t += kChemThreads) {
    const uint32_t hd = b.targets[2 * t], tl = b.targets[2 * t + 1];
    const uint32_t* dr = b.draws + 25 * (size_t)t;
    double h2e[3] = {__dsub_rn(d.px[tl], d.px[hd]), __dsub_rn(d.py[tl], d.py[hd]),
                     __dsub_rn(d.pz[tl], d.pz[hd])};
    min_image(h2e, R);
    normalize(h2e);
    // GetMembraneTangRandomVec
    const double theta = __dmul_rn(2.0 * kPi, mt_real1(dr[0]));
    const double base[3] = {cos(theta), sin(theta), 0.0};
    const double bdot = dot3(base, h2e);
    double tang[3];
#pragma unroll
    for (int k = 0; k < 3; k++) tang[k] = __dsub_rn(base[k], __dmul_rn(h2e[k], bdot));
    normalize(tang);
    const double hp[3] = {d.px[hd], d.py[hd], d.pz[hd]};
    double copied[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
      tang[k] = __dmul_rn(tang[k], c->eps);
      h2e[k] = __dmul_rn(h2e[k], kBondLeng);
      copied[k] = __dadd_rn(tang[k], hp[k]);
    }
    const uint32_t amp = amp0 + (uint32_t)t;
    for (int u = 0; u < kAllUnit; u++) {
      double x[3];
#pragma unroll
      for (int k = 0; k < 3; k++) x[k] = __dadd_rn(copied[k], __dmul_rn(h2e[k], (double)u));
      apply_pbc(x, R);
      const int row = n0 + 4 * t + u;
      d.px[row] = x[0];
      d.py[row] = x[1];
      d.pz[row] = x[2];
      const uint32_t* du = dr + 1 + 6 * u;
      d.vx[row] = thermal_veloc(du[0], du[1]);
      d.vy[row] = thermal_veloc(du[2], du[3]);
      d.vz[row] = thermal_veloc(du[4], du[5]);
      d.ax[row] = d.ay[row] = d.az[row] = 0.0;
      d.dsx[row] = d.dsy[row] = d.dsz[row] = 0.0;
      d.id[row] = (uint32_t)row;  // new_ptcl_id continues from the global count
      d.prop[row] = u == 0 ? 0u : 1u;  // head_unit 1: Hyphil, then Hyphob
      d.amp_id[row] = amp;
      d.unit[row] = (uint32_t)u;
      d.orig[row] = (uint32_t)row;  // appended rows keep their creation order
      d.loc[row] = (uint32_t)row;
      d.perm[row] = (uint32_t)row;  // a reorder before the next sort keeps them in place
      d.rank[row] = (uint32_t)row;
      d.topol[4 * (size_t)(R->amp_off + amp) + u] = (uint32_t)row;
    }
    d.cf_bend[R->amp_off + amp] = c->cf_bend;
  }
  __syncthreads();
  // the targets as rows in upload order (storage rows change at reorders)
  for (int k = tid; k < 2 * nt; k += kChemThreads) b.targets[k] = d.orig[b.targets[k]];
  if (tid == 0) {
    if (nt > 0 && d.vdev) d.vdev->force = 1;  // new rows: cells and kept lists are rebuilt
    R->n = n0 + 4 * nt;
    R->n_amp += nt;
    c->amp_num = amp0 + (uint32_t)nt;
    c->n_targets = nt;
    c->events += 1;
    if (c->amp_num >= c->max_amp_num) {
      c->stopped = 1;
      c->stop_now = 1;
    }
  }
}

}  // namespace

void launch_chem(const DevState& d, const ChemBuffers& b, int nblk, int n_core, int amp_cap,
                 bool force, cudaStream_t st) {
  k_chem_begin<<<1, 32, 0, st>>>(b.chem, d.rep_time, force ? 1 : 0);
  if (nblk > 0) k_chem_find<<<nblk, kRowBlock, 0, st>>>(d, b.chem);
  k_chem_geom<<<1, 32 * kChemMaxCore, 0, st>>>(d, b.chem);
  const int total = n_core * amp_cap;
  if (total > 0)
    k_chem_cone<<<(total + kChemThreads - 1) / kChemThreads, kChemThreads, 0, st>>>(
        d, b.chem, b.flags, b.chunk, amp_cap);
  k_chem_event<<<1, kChemThreads, 0, st>>>(d, b, n_core, amp_cap);
}

}  // namespace idpd
