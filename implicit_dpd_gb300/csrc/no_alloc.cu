// Cell order of rows that the caller already holds on the device, with every
// piece of scratch memory in one static device array of this library. For
// callers that must not allocate device memory: a host code whose own pool
// owns the device budget, or a step loop in which the device-wide
// synchronisation of cudaMalloc / cudaFree would stall the other streams.
// The grid is floor(box) cells per axis (cells of the pair cutoff 1.0), rows
// of a cell in ascending row order: idpd_cell_order's result for the same
// rows at the engine's default tuning (cell reach 1, skin 0). Other tunings
// give idpd_cell_order other grids (floor(box / (1 + skin)) * reach cells).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>

#include "idpd_engine.h"
#include "state.cuh"

using namespace idpd;

namespace {

constexpr int kMaxRows = IDPD_NOALLOC_MAX_ROWS;
constexpr int kMaxCells = IDPD_NOALLOC_MAX_CELLS;
constexpr int kPartWords = 256;  // scan tile sums: kMaxCells / 4096 = 128 used
static_assert(kMaxCells / 4096 + 1 <= kPartWords, "scan tile sums do not fit");

// Word offsets of the pieces, each on a 256-byte boundary.
constexpr size_t kOffSlot = 0;                         // arrival slot per row
constexpr size_t kOffCnt = kOffSlot + kMaxRows;        // rows per cell
constexpr size_t kOffStart = kOffCnt + kMaxCells;      // first slot per cell (+ end)
constexpr size_t kOffPart = kOffStart + kMaxCells + 64;
constexpr size_t kScratchWords = kOffPart + kPartWords;
static_assert(kScratchWords * 4 == IDPD_NOALLOC_SCRATCH_BYTES, "scratch size out of date");
static_assert(kOffCnt % 64 == 0 && kOffStart % 64 == 0 && kOffPart % 64 == 0, "alignment");

// The scratch. Host code may not use this name as an address; the device
// address comes from cudaGetSymbolAddress in the caller's current context.
static __device__ __align__(256) uint32_t g_scratch[kScratchWords];

int noalloc_fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  set_library_error(buf);
  return code;
}

}  // namespace

extern "C" int idpd_cell_order_noalloc(const double* pos, int32_t n, const double* box,
                                       uint32_t* cell_of_row, uint32_t* perm, void* stream) {
  if (n < 0 || !box) return noalloc_fail(IDPD_ERR_INVALID_ARG, "cell_order_noalloc: bad argument");
  if (n > 0 && (!pos || !cell_of_row || !perm))
    return noalloc_fail(IDPD_ERR_INVALID_ARG, "cell_order_noalloc: null array");
  int nc[3];
  double inv_cs[3];
  long long ncell = 1;
  for (int k = 0; k < 3; k++) {
    if (!std::isfinite(box[k]) || box[k] < 1.0)
      return noalloc_fail(IDPD_ERR_INVALID_ARG,
                          "cell_order_noalloc: box[%d] = %g, each side must be finite and >= 1",
                          k, box[k]);
    if (box[k] >= (double)kMaxCells + 1.0)
      return noalloc_fail(IDPD_ERR_CAPACITY,
                          "cell_order_noalloc: box[%d] = %g gives more than %d cells", k, box[k],
                          kMaxCells);
    nc[k] = (int)(box[k] / 1.0);
    inv_cs[k] = (double)nc[k] / box[k];
    ncell *= nc[k];
  }
  if (n > kMaxRows)
    return noalloc_fail(IDPD_ERR_CAPACITY,
                        "cell_order_noalloc: %d rows exceed the static scratch limit of %d rows",
                        n, kMaxRows);
  if (ncell > kMaxCells)
    return noalloc_fail(IDPD_ERR_CAPACITY,
                        "cell_order_noalloc: %lld cells exceed the static scratch limit of %d "
                        "cells",
                        ncell, kMaxCells);
  if (n == 0) return IDPD_OK;

  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess)
    return noalloc_fail(IDPD_ERR_NO_DEVICE, "cell_order_noalloc: cudaGetDevice: %s",
                        cudaGetErrorString(e));
  // The scratch's device address in the context current on this thread,
  // looked up on every call: no address is kept across calls, so a caller
  // that switches contexts, or a device reset by any library of the process,
  // cannot leave a stale address behind. The lookup allocates nothing; the
  // first call on a device also loads this library's device code there (set-up).
  void* p = nullptr;
  e = cudaGetSymbolAddress(&p, g_scratch);
  if (e != cudaSuccess)
    return noalloc_fail(IDPD_ERR_CUDA, "cell_order_noalloc: cudaGetSymbolAddress on device %d: %s",
                        dev, cudaGetErrorString(e));
  uint32_t* base = (uint32_t*)p;
  cudaStream_t st = (cudaStream_t)stream;
  uint32_t* slot = base + kOffSlot;
  int* cnt = (int*)(base + kOffCnt);
  int* start = (int*)(base + kOffStart);
  int* part = (int*)(base + kOffPart);
  const int nce = (int)ncell;
  // The counts keep the previous call's contents: clear them first.
  e = cudaMemsetAsync(cnt, 0, sizeof(int) * (size_t)nce, st);
  if (e != cudaSuccess)
    return noalloc_fail(IDPD_ERR_CUDA, "cell_order_noalloc: cudaMemsetAsync: %s",
                        cudaGetErrorString(e));
  launch_bin_rows(pos, n, inv_cs, nc, cell_of_row, slot, cnt, st);
  launch_scan_raw(cnt, start, part, nce, n, st);
  launch_scatter_rows(cell_of_row, slot, start, n, perm, st);
  launch_cell_sort_raw(perm, start, nce, st);
  e = cudaGetLastError();
  if (e != cudaSuccess)
    return noalloc_fail(IDPD_ERR_CUDA, "cell_order_noalloc: launch: %s", cudaGetErrorString(e));
  return IDPD_OK;
}
