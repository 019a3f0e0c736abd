// Device helpers shared by the pair passes (kernels_pairs.cu: pass 1, the
// kept-list build and the FP64 arms; kernels_force.cu: the FP32 pass 2):
// the reference's FP64 pair distance, the neighbour-cell segments, the
// 32-bit list entries, the ownership rule of the once-per-pair passes and
// the cell-stencil walk.
#pragma once

#include "pair_math.cuh"

namespace idpd {

__device__ __forceinline__ long long warp_sum_ll(long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Sorts the 32 keys of a warp ascending (bitonic network over the lanes).
__device__ __forceinline__ uint32_t warp_sort_asc(uint32_t key, int lane) {
#pragma unroll
  for (int k = 2; k <= 32; k <<= 1) {
#pragma unroll
    for (int j = k >> 1; j > 0; j >>= 1) {
      const uint32_t other = __shfl_xor_sync(0xffffffffu, key, j);
      const bool up = (lane & k) == 0 || k == 32;
      const bool low = (lane & j) == 0;
      key = (low == up) ? min(key, other) : max(key, other);
    }
  }
  return key;
}

// FP64 squared distance of rows i and j in the reference's operation order
// (nbdf_calculator.hpp:27-29, 86-87), j shifted to its image nearest to i.
// The image follows from the positions themselves, so it stays right while
// the cells are reused between list rebuilds.
__device__ __forceinline__ double exact_dr2(const DevState& d, const RepDev* R, uint32_t i,
                                            uint32_t j) {
  const double xi = d.px[i], yi = d.py[i], zi = d.pz[i];
  const double xj = d.px[j], yj = d.py[j], zj = d.pz[j];
  const int sx = nearest_image(xi, xj, R->box[0]), sy = nearest_image(yi, yj, R->box[1]),
            sz = nearest_image(zi, zj, R->box[2]);
  const double jx = __dadd_rn(xj, __dmul_rn((double)sx, R->box[0]));
  const double jy = __dadd_rn(yj, __dmul_rn((double)sy, R->box[1]));
  const double jz = __dadd_rn(zj, __dmul_rn((double)sz, R->box[2]));
  const double ex = __dsub_rn(xi, jx), ey = __dsub_rn(yi, jy), ez = __dsub_rn(zi, jz);
  return __dadd_rn(__dadd_rn(__dmul_rn(ex, ex), __dmul_rn(ey, ey)), __dmul_rn(ez, ez));
}

// ------------------------------------------------ neighbour segments
// A segment is a run of x-consecutive search cells of one (dy, dz) row with
// one image shift; its rows are contiguous in sorted order. The boundaries
// where the run enters a new frame cell give each candidate its x offset in
// frame cells (the unit of the stored cell-local coordinates).
constexpr int kMaxReach = 2;
constexpr int kMaxSeg = 2 * (2 * kMaxReach + 1) * (2 * kMaxReach + 1);  // 50
constexpr int kWarps = kRowBlock / 32;

struct SegTable {
  int tb[kMaxSeg], te[kMaxSeg];
  int bnd[kMaxSeg][2 * kMaxReach];  // first rows of the next frame cells (INT_MAX when absent)
  int code[kMaxSeg];  // frame offsets fx0+4 | (fy+4)<<3 | (fz+4)<<6, shifts (sx+1)<<9 | (sy+1)<<11 | (sz+1)<<13
};

// Lane k < (2m+1)^2 builds the (up to two) segments of row k of cell
// (cx, cy, cz); slots of a row that do not exist are left empty.
__device__ __forceinline__ void build_segments(SegTable& S, const DevState& d, const RepDev* R,
                                               int cx, int cy, int cz, int lane) {
  const int m = R->reach, w = 2 * m + 1, rs = R->rshift;
  const int nx = R->nc[0], ny = R->nc[1], nz = R->nc[2];
  for (int k = lane; k < w * w; k += 32) {
    const int dz = k / w - m, dy = k % w - m;
    const int qz = cz + dz, sz = qz < 0 ? -1 : (qz >= nz ? 1 : 0), wz = qz - sz * nz;
    const int qy = cy + dy, sy = qy < 0 ? -1 : (qy >= ny ? 1 : 0), wy = qy - sy * ny;
    const int base = R->cell_off + (wz * ny + wy) * nx;
    const int fy = (qy >> rs) - (cy >> rs), fz = (qz >> rs) - (cz >> rs);  // frame offsets
    // parts: [cx-m, -1] wrapped left (sx=-1), [max(cx-m,0), min(cx+m,nx-1)] (sx=0),
    // [nx, cx+m] wrapped right (sx=+1); at most two are non-empty.
    int slot = 2 * k;
    for (int part = -1; part <= 1; part++) {
      int lo, hi;  // unwrapped offsets lo..hi; wrapped index = cx + off - part * nx
      if (part == -1) {
        lo = -m;
        hi = -cx - 1;
      } else if (part == 0) {
        lo = cx - m < 0 ? -cx : -m;
        hi = cx + m >= nx ? nx - 1 - cx : m;
      } else {
        lo = nx - cx;
        hi = m;
      }
      if (lo > hi) continue;
      const int xs = cx + lo - part * nx;
      const int ncells = hi - lo + 1;
      S.tb[slot] = d.cell_start[base + xs];
      S.te[slot] = d.cell_start[base + xs + ncells];
      int nb = 0;
      for (int q = 1; q < ncells; q++)  // unwrapped search cell cx+lo+q starts a frame cell
        if (((cx + lo + q) & (m - 1)) == 0) S.bnd[slot][nb++] = d.cell_start[base + xs + q];
      for (; nb < 2 * kMaxReach; nb++) S.bnd[slot][nb] = 0x7fffffff;
      const int fx0 = ((cx + lo) >> rs) - (cx >> rs);
      S.code[slot] = (fx0 + 4) | ((fy + 4) << 3) | ((fz + 4) << 6) | ((part + 1) << 9) |
                     ((sy + 1) << 11) | ((sz + 1) << 13);
      slot++;
    }
    for (; slot < 2 * k + 2; slot++) {
      S.tb[slot] = 0;
      S.te[slot] = 0;
    }
  }
}

__device__ __forceinline__ int seg_dx(const SegTable& S, int g, int t) {
  int dx = (S.code[g] & 7) - 4;
#pragma unroll
  for (int q = 0; q < 2 * kMaxReach; q++) dx += t >= S.bnd[g][q];
  return dx;
}

struct PairCode {
  int dx, dy, dz, sx, sy, sz;
};
__device__ __forceinline__ uint32_t pack_code(int dx, int seg_code) {
  return (uint32_t)((dx + 4) | (seg_code & ~7));
}
__device__ __forceinline__ PairCode unpack_code(uint32_t c) {
  PairCode p;
  p.dx = (int)(c & 7) - 4;
  p.dy = (int)((c >> 3) & 7) - 4;
  p.dz = (int)((c >> 6) & 7) - 4;
  p.sx = (int)((c >> 9) & 3) - 1;
  p.sy = (int)((c >> 11) & 3) - 1;
  p.sz = (int)((c >> 13) & 3) - 1;
  return p;
}

// ------------------------------------------------------------- pass 1
// Neighbour list entry (32 bits): the candidate's sorted row (25 bits) and
// its frame cell's offset from the particle's frame cell, dx, dy, dz + 1 in
// 2 bits each. kNbrFallback marks a particle whose list did not fit (the
// next pass walks its cells again). Kept lists hold the candidates and
// pass-1 lists the pairs within the cutoff that the particle owns (owns()).
constexpr uint32_t kNbrFallback = 0xffffu;
constexpr int kRowBits = 25;
constexpr uint32_t kRowMask = (1u << kRowBits) - 1u;

// Both pair passes take each pair once, from the side of the particle that
// owns it: the frame offset dx of the other particle decides when nonzero,
// else (the same frame cell column) the larger cell-local x, else the larger
// sorted row. The x is that of the step (no kept lists) or of the kept
// lists' build (okey): rows and frame cells do not change between builds, so
// the two particles of a pair always agree. Each particle owns about half of
// its pairs (those on the +x side of the plane through it), which keeps the
// two particles of a half-warp pair in pass 2 near equal work.
__device__ __forceinline__ bool owns(int dx, float xj, float xi, int t, int s) {
  if (dx != 0) return dx > 0;
  return xj != xi ? xj > xi : t > s;
}

__device__ __forceinline__ uint32_t make_entry(int t, int dx, int dy, int dz) {
  return (uint32_t)t | ((uint32_t)(dx + 1) << kRowBits) | ((uint32_t)(dy + 1) << (kRowBits + 2)) |
         ((uint32_t)(dz + 1) << (kRowBits + 4));
}

__device__ __forceinline__ void read_entry(uint32_t e, int& t, int& dx, int& dy, int& dz) {
  t = (int)(e & kRowMask);
  dx = (int)((e >> kRowBits) & 3u) - 1;
  dy = (int)((e >> (kRowBits + 2)) & 3u) - 1;
  dz = (int)((e >> (kRowBits + 4)) & 3u) - 1;
}

template <int REACH>
__device__ __forceinline__ int frame_step(int t, const int* b) {
  int k = 0;
#pragma unroll
  for (int q = 0; q < 2 * REACH; q++) k += t >= b[q];
  return k;
}

// Density weight of one in-range pair, accumulated by the candidate's property.
__device__ __forceinline__ void add_weight(uint32_t& q0, uint32_t& q1, uint32_t& q2, uint32_t pr,
                                           uint32_t v) {
  q0 += pr == 0 ? v : 0u;
  q1 += pr == 1 ? v : 0u;
  q2 += pr == 2 ? v : 0u;
}

// Visits every neighbour cell within the stencil of the given reach
// (plain FP64 kernels and the centre-of-mass pass).
template <class F>
__device__ __forceinline__ void for_each_cell(const RepDev* R, int reach, int cx, int cy, int cz,
                                              F&& f) {
  const int nx = R->nc[0], ny = R->nc[1], nz = R->nc[2];
  for (int dz = -reach; dz <= reach; dz++) {
    const int qz = cz + dz, sz = qz < 0 ? -1 : (qz >= nz ? 1 : 0), wz = qz - sz * nz;
    for (int dy = -reach; dy <= reach; dy++) {
      const int qy = cy + dy, sy = qy < 0 ? -1 : (qy >= ny ? 1 : 0), wy = qy - sy * ny;
      const int row = R->cell_off + (wz * ny + wy) * nx;
      for (int dx = -reach; dx <= reach; dx++) {
        const int qx = cx + dx, sx = qx < 0 ? -1 : (qx >= nx ? 1 : 0), wx = qx - sx * nx;
        f(row + wx, dx, dy, dz, sx, sy, sz);
      }
    }
  }
}

__device__ __forceinline__ void red_add(long long* p, long long v) {
  atomicAdd(reinterpret_cast<unsigned long long*>(p), (unsigned long long)v);
}

// 16-byte asynchronous copy global -> shared (cp.async, kept in L1 and L2),
// and its group commit / wait: a lane's copies of one round form one group.
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}
__device__ __forceinline__ void cp_async_wait_prev() {  // all groups but the newest done
  asm volatile("cp.async.wait_group 1;\n" ::: "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_group 0;\n" ::: "memory");
}

}  // namespace idpd
