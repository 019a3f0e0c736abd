// Drift and cell binning, the counting sort by cell, and the packed FP32
// copies that the pair passes read. Replaces the FDPS tree build and the j
// gather of TreeForForceShort::Gather (src/main.cpp:124-132, 173-174) and
// performs drift_and_predict (driftkick.hpp:6-27) in the same pass.
#include <algorithm>

#include "state.cuh"

namespace idpd {

// Periodic wrap of driftkick.hpp:19-21, t - floor(t / L) L with the
// reference's rounding. Rows that stay inside [0, hi) keep t unchanged
// without touching the FP64 pipe (the sign bit and the bit pattern order of
// non-negative doubles decide it); all others take the reference expression.
__device__ __forceinline__ double wrap_pbc(double t, double L, double iL, long long hi_bits) {
  const long long b = __double_as_longlong(t);
  if (b >= 0 && b < hi_bits) return t;
  const double f = floor(__dmul_rn(t, iL));
  return __dsub_rn(t, __dmul_rn(f, L));
}

__device__ __forceinline__ int cell_coord(double x, double inv_cs, int nc) {
  int c = __double2int_rz(__dmul_rn(x, inv_cs));
  c = c < 0 ? 0 : c;
  return c >= nc ? nc - 1 : c;
}

// drift_and_predict of one storage row (driftkick.hpp:6-27); x, y, z hold
// the row's position on entry and the new one on return.
__device__ __forceinline__ void drift_row(const DevState& d, const RepDev* R, int i, double& x,
                                          double& y, double& z) {
  {
    const double dt = R->dt;
    const double h = __dmul_rn(0.5, dt);
    double p[3] = {x, y, z};
    double* vv[3] = {d.vx, d.vy, d.vz};
    double* aa[3] = {d.ax, d.ay, d.az};
    double* ds[3] = {d.dsx, d.dsy, d.dsz};
#pragma unroll
    for (int k = 0; k < 3; k++) {
      const double vp = __dadd_rn(vv[k][i], __dmul_rn(h, aa[k][i]));
      const double dr = __dmul_rn(dt, vp);
      const double t = __dadd_rn(p[k], dr);
      ds[k][i] = __dadd_rn(ds[k][i], dr);
      // hi = L (1 - 2^-50): below it t / L rounds below 1 and floor() is 0.
      const double L = R->box[k];
      const long long hi = __double_as_longlong(L) - 4;
      p[k] = wrap_pbc(t, L, R->ibox[k], hi);
      vv[k][i] = vp;
    }
    x = p[0];
    y = p[1];
    z = p[2];
    d.px[i] = x;
    d.py[i] = y;
    d.pz[i] = z;
  }
}

// One thread per storage row: optional drift, then cell index and arrival slot.
__global__ void __launch_bounds__(kRowBlock) k_drift_bin(DevState d, int do_drift) {
  const int r = d.blk_rep[blockIdx.x];
  const int i = d.blk_row[blockIdx.x] + threadIdx.x;
  const RepDev* R = d.reps + r;
  if (i >= R->row_off + R->n) return;
  double x = d.px[i], y = d.py[i], z = d.pz[i];
  if (do_drift) drift_row(d, R, i, x, y, z);
  const int cx = cell_coord(x, R->inv_cs[0], R->nc[0]);
  const int cy = cell_coord(y, R->inv_cs[1], R->nc[1]);
  const int cz = cell_coord(z, R->inv_cs[2], R->nc[2]);
  const uint32_t key = (uint32_t)(R->cell_off + (cz * R->nc[1] + cy) * R->nc[0] + cx);
  d.key[i] = key;
  d.slot[i] = (uint32_t)atomicAdd(&d.cell_cnt[key], 1);
}

// Steps that keep the neighbour lists: drift, and the largest squared
// displacement since the last rebuild (delta_sumr accumulates every drift,
// unwrapped) into the rebuild record.
__global__ void __launch_bounds__(kRowBlock) k_drift_disp(DevState d) {
  __shared__ float wmax[kRowBlock / 32];
  const int r = d.blk_rep[blockIdx.x];
  const int i = d.blk_row[blockIdx.x] + threadIdx.x;
  const RepDev* R = d.reps + r;
  float m = 0.0f;
  if (i < R->row_off + R->n) {
    double x = d.px[i], y = d.py[i], z = d.pz[i];
    drift_row(d, R, i, x, y, z);
    const uint32_t s = d.rank[i];
    const double ex = d.dsx[i] - d.drx[s], ey = d.dsy[i] - d.dry[s], ez = d.dsz[i] - d.drz[s];
    m = (float)(ex * ex + ey * ey + ez * ez);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) wmax[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    float b = 0.0f;
    for (int w = 0; w < kRowBlock / 32; w++) b = fmaxf(b, wmax[w]);
    // non-negative floats order like their bit patterns; the running maximum
    // is read first, so only blocks that raise it take the (single-address) atomic
    const unsigned int bb = __float_as_uint(b);
    if (b > 0.0f && bb > *(volatile unsigned int*)&d.vdev->maxd2) atomicMax(&d.vdev->maxd2, bb);
  }
}

__global__ void k_vl_decide(VerletDev* v) {
  if (threadIdx.x != 0) return;
  const int rb = v->force || __uint_as_float(v->maxd2) > v->thr2;
  v->rebuild = rb;
  v->force = 0;
  v->maxd2 = 0u;
  v->rebuilds += (unsigned)rb;
}

// The binning of k_drift_bin on a rebuild step (positions already drifted).
__global__ void __launch_bounds__(kRowBlock) k_bin_gated(DevState d) {
  if (!d.vdev->rebuild) return;
  const int r = d.blk_rep[blockIdx.x];
  const int i = d.blk_row[blockIdx.x] + threadIdx.x;
  const RepDev* R = d.reps + r;
  if (i >= R->row_off + R->n) return;
  const int cx = cell_coord(d.px[i], R->inv_cs[0], R->nc[0]);
  const int cy = cell_coord(d.py[i], R->inv_cs[1], R->nc[1]);
  const int cz = cell_coord(d.pz[i], R->inv_cs[2], R->nc[2]);
  const uint32_t key = (uint32_t)(R->cell_off + (cz * R->nc[1] + cy) * R->nc[0] + cx);
  d.key[i] = key;
  d.slot[i] = (uint32_t)atomicAdd(&d.cell_cnt[key], 1);
}

void launch_drift_disp(const DevState& d, int nblk, cudaStream_t st) {
  if (nblk > 0) k_drift_disp<<<nblk, kRowBlock, 0, st>>>(d);
}

void launch_vl_decide(const DevState& d, cudaStream_t st) { k_vl_decide<<<1, 32, 0, st>>>(d.vdev); }

void launch_bin_gated(const DevState& d, int nblk, cudaStream_t st) {
  if (nblk > 0) k_bin_gated<<<nblk, kRowBlock, 0, st>>>(d);
}

// ---------------------------------------------------------------- scan
constexpr int kScanThreads = 1024;
constexpr int kScanPerThread = 4;
constexpr int kScanTile = kScanThreads * kScanPerThread;

__device__ __forceinline__ int block_exclusive_scan(int v, int* warp_sums, int& total) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) warp_sums[w] = incl;
  __syncthreads();
  if (w == 0) {
    int s = lane < (int)(blockDim.x >> 5) ? warp_sums[lane] : 0;
    int si = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, si, o);
      if (lane >= o) si += t;
    }
    warp_sums[lane] = si - s;
    if (lane == 31) warp_sums[32] = si;
  }
  __syncthreads();
  total = warp_sums[32];
  const int res = incl - v + warp_sums[w];
  __syncthreads();
  return res;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_tiles(const int* cnt, int* start, int* part,
                                                             int ncell, const int* gate) {
  __shared__ int ws[33];
  if (gate && !*gate) return;
  const int base = blockIdx.x * kScanTile + threadIdx.x * kScanPerThread;
  int c[kScanPerThread];
  int sum = 0;
#pragma unroll
  for (int k = 0; k < kScanPerThread; k++) {
    c[k] = (base + k < ncell) ? cnt[base + k] : 0;
    sum += c[k];
  }
  int total;
  int run = block_exclusive_scan(sum, ws, total);
#pragma unroll
  for (int k = 0; k < kScanPerThread; k++) {
    if (base + k < ncell) start[base + k] = run;
    run += c[k];
  }
  if (threadIdx.x == 0) part[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_parts(int* part, int nparts,
                                                             const int* gate) {
  __shared__ int ws[33];
  if (gate && !*gate) return;
  int carry = 0;
  for (int b = 0; b < nparts; b += kScanThreads) {
    const int i = b + threadIdx.x;
    const int v = i < nparts ? part[i] : 0;
    int total;
    const int ex = block_exclusive_scan(v, ws, total);
    if (i < nparts) part[i] = ex + carry;
    carry += total;
  }
}

__global__ void __launch_bounds__(kScanThreads) k_scan_finish(int* cnt, int* start, const int* part,
                                                              int ncell, int n_tot,
                                                              const RepDev* last,
                                                              const int* gate) {
  if (gate && !*gate) return;
  const int base = blockIdx.x * kScanTile + threadIdx.x * kScanPerThread;
  const int off = part[blockIdx.x];
#pragma unroll
  for (int k = 0; k < kScanPerThread; k++) {
    if (base + k < ncell) {
      start[base + k] += off;
      cnt[base + k] = 0;  // ready for the next binning
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) start[ncell] = last ? last->row_off + last->n : n_tot;
}

void launch_scan(const DevState& d, int ncell_tot, int last_rep, cudaStream_t st,
                 const int* gate) {
  const int nb = (ncell_tot + kScanTile - 1) / kScanTile;
  k_scan_tiles<<<nb, kScanThreads, 0, st>>>(d.cell_cnt, d.cell_start, d.scan_part, ncell_tot, gate);
  k_scan_parts<<<1, kScanThreads, 0, st>>>(d.scan_part, nb, gate);
  k_scan_finish<<<nb, kScanThreads, 0, st>>>(d.cell_cnt, d.cell_start, d.scan_part, ncell_tot, 0,
                                             d.reps + last_rep, gate);
}

// ------------------------------------------------- scatter / sort / pack
__global__ void __launch_bounds__(kRowBlock) k_scatter(DevState d, const int* gate) {
  if (gate && !*gate) return;
  const int r = d.blk_rep[blockIdx.x];
  const int i = d.blk_row[blockIdx.x] + threadIdx.x;
  const RepDev* R = d.reps + r;
  if (i >= R->row_off + R->n) return;
  const uint32_t s = (uint32_t)d.cell_start[d.key[i]] + d.slot[i];
  d.perm[s] = (uint32_t)i;
}

// Rows of one cell in ascending storage row: the order a stable counting
// sort gives, independent of the arrival order of the atomics. A warp per
// cell: each of up to 128 rows finds its place by counting the smaller rows
// (rows are distinct); a larger cell is sorted by one lane in place.
__device__ __forceinline__ void sort_cell(uint32_t* perm, int b, int e, int lane) {
  const int n = e - b;
  if (n <= 1) return;
  if (n <= 128) {
    uint32_t v[4];
    int rank[4];
#pragma unroll
    for (int q = 0; q < 4; q++) {
      v[q] = 32 * q + lane < n ? perm[b + 32 * q + lane] : 0xFFFFFFFFu;
      rank[q] = 0;
    }
#pragma unroll
    for (int q = 0; q < 4; q++) {
      if (32 * q >= n) break;  // warp-uniform
      for (int j = 0; j < 32; j++) {
        const uint32_t x = __shfl_sync(0xffffffffu, v[q], j);
#pragma unroll
        for (int m = 0; m < 4; m++) rank[m] += x < v[m];
      }
    }
    __syncwarp();
#pragma unroll
    for (int q = 0; q < 4; q++)
      if (32 * q + lane < n) perm[b + rank[q]] = v[q];
    __syncwarp();
    return;
  }
  if (lane == 0) {
    for (int k = b + 1; k < e; k++) {
      const uint32_t v = perm[k];
      int m = k - 1;
      while (m >= b && perm[m] > v) {
        perm[m + 1] = perm[m];
        m--;
      }
      perm[m + 1] = v;
    }
  }
  __syncwarp();
}

constexpr int kSortWarps = 8;
constexpr int kSortBlocks = 1216;  // 8 per SM of a GB300; the cells are strided over them

__global__ void __launch_bounds__(32 * kSortWarps) k_cell_sort(uint32_t* perm, const int* start,
                                                               int ncell, const int* gate) {
  if (gate && !*gate) return;
  const int lane = threadIdx.x & 31;
  for (int c = blockIdx.x * kSortWarps + (threadIdx.x >> 5); c < ncell; c += gridDim.x * kSortWarps)
    sort_cell(perm, start[c], start[c + 1], lane);
}

// Offset of x from its frame cell's origin o, at the periodic image nearest
// to the cell (a particle that crossed the box edge since the cells were
// built keeps its old cell). For a particle inside its cell, x - o is exact
// in FP64 (Sterbenz: x lies in [o, 2o] or o = 0).
__device__ __forceinline__ double cell_offset(double x, double o, double L) {
  double v = __dsub_rn(x, o);
  if (v > 0.5 * L) v = __dsub_rn(v, L);
  else if (v < -0.5 * L) v = __dadd_rn(v, L);
  return v;
}

// One thread per sorted slot: FP32 cell-local position, velocity and ids.
// gate (may be null): when it reads 0 the slots keep their rows and cells
// of the last rebuild.
__global__ void __launch_bounds__(kRowBlock) k_pack(DevState d, const int* gate) {
  const int r = d.blk_rep[blockIdx.x];
  const int s = d.blk_row[blockIdx.x] + threadIdx.x;
  const RepDev* R = d.reps + r;
  if (s >= R->row_off + R->n) return;
  const uint32_t i = d.perm[s];
  uint32_t key;
  if (!gate || *gate) {
    d.rank[i] = (uint32_t)s;
    key = d.key[i];
    d.scell[s] = key;
  } else {
    key = d.scell[s];
  }
  int cx, cy, cz;
  cell_xyz((int)key - R->cell_off, R->nc, cx, cy, cz);
  cx >>= R->rshift;  // frame cell
  cy >>= R->rshift;
  cz >>= R->rshift;
  // the float split keeps 48 bits for the near-cutoff pair terms
  float lx, ly, lz, ex, ey, ez;
  split_double(cell_offset(d.px[i], __dmul_rn((double)cx, R->cs[0]), R->box[0]), lx, ex);
  split_double(cell_offset(d.py[i], __dmul_rn((double)cy, R->cs[1]), R->box[1]), ly, ey);
  split_double(cell_offset(d.pz[i], __dmul_rn((double)cz, R->cs[2]), R->box[2]), lz, ez);
  d.posf[s] = make_float4(lx, ly, lz, __uint_as_float(d.prop[i]));
  d.poslo[s] = make_float4(ex, ey, ez, 0.0f);
  d.velf[s] = make_float4(__double2float_rn(d.vx[i]), __double2float_rn(d.vy[i]),
                          __double2float_rn(d.vz[i]), __uint_as_float(d.id[i]));
  if (d.svel) {  // FP64 engine-algorithm arm
    double* v = d.svel + 4 * (size_t)s;
    v[0] = d.vx[i];
    v[1] = d.vy[i];
    v[2] = d.vz[i];
  }
}

void launch_scan_raw(int* cnt, int* start, int* part, int ncell, int n_tot, cudaStream_t st) {
  const int nb = (ncell + kScanTile - 1) / kScanTile;
  k_scan_tiles<<<nb, kScanThreads, 0, st>>>(cnt, start, part, ncell, nullptr);
  k_scan_parts<<<1, kScanThreads, 0, st>>>(part, nb, nullptr);
  k_scan_finish<<<nb, kScanThreads, 0, st>>>(cnt, start, part, ncell, n_tot, nullptr, nullptr);
}

void launch_cell_sort_raw(uint32_t* perm, const int* start, int ncell, cudaStream_t st) {
  if (ncell > 0)
    k_cell_sort<<<std::min((ncell + kSortWarps - 1) / kSortWarps, kSortBlocks), 32 * kSortWarps,
                  0, st>>>(perm, start, ncell, nullptr);
}

// Cell index and arrival slot of rows given as x y z triples (one grid, no
// replicas): the binning of k_drift_bin without the drift.
__global__ void __launch_bounds__(256) k_bin_rows(const double* pos, int n, double ix, double iy,
                                                  double iz, int nx, int ny, int nz,
                                                  uint32_t* cell, uint32_t* slot, int* cnt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double* p = pos + 3 * (size_t)i;
  const int cx = cell_coord(p[0], ix, nx);
  const int cy = cell_coord(p[1], iy, ny);
  const int cz = cell_coord(p[2], iz, nz);
  const uint32_t c = (uint32_t)((cz * ny + cy) * nx + cx);
  cell[i] = c;
  slot[i] = (uint32_t)atomicAdd(&cnt[c], 1);
}

__global__ void __launch_bounds__(256) k_scatter_rows(const uint32_t* cell, const uint32_t* slot,
                                                      const int* start, int n, uint32_t* perm) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  perm[(uint32_t)start[cell[i]] + slot[i]] = (uint32_t)i;
}

void launch_bin_rows(const double* pos, int n, const double inv_cs[3], const int nc[3],
                     uint32_t* cell, uint32_t* slot, int* cnt, cudaStream_t st) {
  if (n > 0)
    k_bin_rows<<<(n + 255) / 256, 256, 0, st>>>(pos, n, inv_cs[0], inv_cs[1], inv_cs[2], nc[0],
                                                nc[1], nc[2], cell, slot, cnt);
}

void launch_scatter_rows(const uint32_t* cell, const uint32_t* slot, const int* start, int n,
                         uint32_t* perm, cudaStream_t st) {
  if (n > 0) k_scatter_rows<<<(n + 255) / 256, 256, 0, st>>>(cell, slot, start, n, perm);
}

void launch_drift_bin(const DevState& d, int nblk, bool do_drift, cudaStream_t st) {
  if (nblk == 0) return;
  k_drift_bin<<<nblk, kRowBlock, 0, st>>>(d, do_drift ? 1 : 0);
}

void launch_scatter_sort(const DevState& d, int nblk, int ncell_tot, bool stable, cudaStream_t st,
                         const int* gate) {
  if (nblk == 0) return;
  k_scatter<<<nblk, kRowBlock, 0, st>>>(d, gate);
  if (stable)
    k_cell_sort<<<std::min((ncell_tot + kSortWarps - 1) / kSortWarps, kSortBlocks),
                  32 * kSortWarps, 0, st>>>(d.perm, d.cell_start, ncell_tot, gate);
}

void launch_pack(const DevState& d, int nblk, cudaStream_t st, const int* gate) {
  if (nblk > 0) k_pack<<<nblk, kRowBlock, 0, st>>>(d, gate);
}

void launch_scatter_sort_pack(const DevState& d, int nblk, int ncell_tot, bool stable,
                              cudaStream_t st, const int* gate) {
  launch_scatter_sort(d, nblk, ncell_tot, stable, st, gate);
  launch_pack(d, nblk, st, gate);
}

// ------------------------------------------------------------- reorder
// Moves every storage-order field into sorted order (o holds scratch
// buffers of the same shape) and rewrites the topology to the new rows.
__global__ void __launch_bounds__(kRowBlock) k_reorder_gather(DevState d, DevState o) {
  const int r = d.blk_rep[blockIdx.x];
  const int s = d.blk_row[blockIdx.x] + threadIdx.x;
  const RepDev* R = d.reps + r;
  if (s >= R->row_off + R->n) return;
  const uint32_t i = d.perm[s];
  o.px[s] = d.px[i]; o.py[s] = d.py[i]; o.pz[s] = d.pz[i];
  o.vx[s] = d.vx[i]; o.vy[s] = d.vy[i]; o.vz[s] = d.vz[i];
  o.ax[s] = d.ax[i]; o.ay[s] = d.ay[i]; o.az[s] = d.az[i];
  o.dsx[s] = d.dsx[i]; o.dsy[s] = d.dsy[i]; o.dsz[s] = d.dsz[i];
  o.id[s] = d.id[i]; o.prop[s] = d.prop[i]; o.amp_id[s] = d.amp_id[i]; o.unit[s] = d.unit[i];
  o.orig[s] = d.orig[i];
  o.key[s] = d.key[i];
}

__global__ void __launch_bounds__(kRowBlock) k_reorder_loc(DevState d) {
  const int r = d.blk_rep[blockIdx.x];
  const int s = d.blk_row[blockIdx.x] + threadIdx.x;
  const RepDev* R = d.reps + r;
  if (s >= R->row_off + R->n) return;
  d.loc[d.orig[s]] = (uint32_t)s;
}

__global__ void k_reorder_topol(uint32_t* topol, const uint32_t* rank, int n) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) topol[k] = rank[topol[k]];
}

__global__ void __launch_bounds__(kRowBlock) k_identity_perm(DevState d) {
  const int r = d.blk_rep[blockIdx.x];
  const int s = d.blk_row[blockIdx.x] + threadIdx.x;
  const RepDev* R = d.reps + r;
  if (s >= R->row_off + R->n) return;
  d.perm[s] = (uint32_t)s;
  d.rank[s] = (uint32_t)s;
}

void launch_update_loc(const DevState& d, int nblk, cudaStream_t st) {
  if (nblk == 0) return;
  k_reorder_loc<<<nblk, kRowBlock, 0, st>>>(d);
}

void launch_reorder(const DevState& d, const DevState& o, int nblk, int n_topol, cudaStream_t st) {
  if (nblk == 0) return;
  k_reorder_gather<<<nblk, kRowBlock, 0, st>>>(d, o);
  if (n_topol > 0) k_reorder_topol<<<(n_topol + 255) / 256, 256, 0, st>>>(d.topol, d.rank, n_topol);
  k_identity_perm<<<nblk, kRowBlock, 0, st>>>(d);
}

}  // namespace idpd
