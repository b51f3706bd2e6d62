// Device-wide exclusive scan (int32 or int64 values into int64), for the
// graph build and the BC BFS phase: per-tile sums, a recursive scan of the
// sums, then each tile scanned again with its base.  Internal linkage: every
// translation unit that includes it gets its own copy of the kernels.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>

#include "engine.h"

namespace gbbfs {
namespace {

constexpr int kScanThreads = 1024;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

// ---------------------------------------------------------------------------
// Exclusive scan of int32 / int64 values into int64.

template <typename T>
__device__ __forceinline__ int64_t block_exclusive_scan(int64_t x, int64_t* total) {
  __shared__ int64_t warp_sums[kScanThreads / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int64_t inc = x;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const int64_t y = __shfl_up_sync(kFull, inc, d);
    if (lane >= d) inc += y;
  }
  if (lane == 31) warp_sums[w] = inc;
  __syncthreads();
  if (w == 0) {
    int64_t s = lane < kScanThreads / 32 ? warp_sums[lane] : 0;
    int64_t si = s;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const int64_t y = __shfl_up_sync(kFull, si, d);
      if (lane >= d) si += y;
    }
    if (lane < kScanThreads / 32) warp_sums[lane] = si - s;   // exclusive warp bases
    if (lane == 31) *total = si;
  }
  __syncthreads();
  const int64_t r = warp_sums[w] + inc - x;
  __syncthreads();
  return r;
}

// Per tile: the sum of its values.
template <typename T>
__global__ void __launch_bounds__(kScanThreads) k_scan_sums(const T* in, int64_t len,
                                                            int64_t* sums) {
  __shared__ int64_t total;
  const int64_t base = (int64_t)blockIdx.x * kScanTile;
  int64_t s = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; i++) {
    const int64_t j = base + (int64_t)i * kScanThreads + threadIdx.x;
    if (j < len) s += (int64_t)in[j];
  }
  block_exclusive_scan<T>(s, &total);
  if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

// out[j] = tile_base[tile] + exclusive prefix of in within the tile.  A
// thread scans kScanItems consecutive values.
template <typename T>
__global__ void __launch_bounds__(kScanThreads) k_scan_apply(const T* in, int64_t len,
                                                             const int64_t* tile_base,
                                                             int64_t* out) {
  __shared__ int64_t total;
  const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  int64_t v[kScanItems];
  int64_t s = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; i++) {
    v[i] = base + i < len ? (int64_t)in[base + i] : 0;
    s += v[i];
  }
  int64_t run = block_exclusive_scan<T>(s, &total) + tile_base[blockIdx.x];
#pragma unroll
  for (int i = 0; i < kScanItems; i++) {
    if (base + i < len) out[base + i] = run;
    run += v[i];
  }
}

__global__ void k_put_total(const int64_t* sums_scan, const int64_t* sums, int64_t tiles,
                            int64_t* at) {
  *at = tiles > 0 ? sums_scan[tiles - 1] + sums[tiles - 1] : 0;
}

// Exclusive scan of len values; out[len] receives the total when with_total.
// The per-tile sums are temporary allocations (graph build only).
template <typename T>
int device_scan(const T* in, int64_t len, int64_t* out, bool with_total, cudaStream_t s) {
  const int64_t tiles = std::max<int64_t>(1, (len + kScanTile - 1) / kScanTile);
  int64_t *sums = nullptr, *sums_scan = nullptr;
  GB_CUDA(cudaMalloc(&sums, sizeof(int64_t) * tiles));
  GB_CUDA(cudaMalloc(&sums_scan, sizeof(int64_t) * tiles));
  int rc = GBBFS_OK;
  k_scan_sums<T><<<(unsigned)tiles, kScanThreads, 0, s>>>(in, len, sums);
  if (cudaGetLastError() != cudaSuccess) rc = GBBFS_ERR_CUDA;
  if (rc == GBBFS_OK) {
    if (tiles == 1) {
      if (cudaMemsetAsync(sums_scan, 0, sizeof(int64_t), s) != cudaSuccess) rc = GBBFS_ERR_CUDA;
    } else {
      rc = device_scan<int64_t>(sums, tiles, sums_scan, false, s);
    }
  }
  if (rc == GBBFS_OK) {
    k_scan_apply<T><<<(unsigned)tiles, kScanThreads, 0, s>>>(in, len, sums_scan, out);
    if (with_total) k_put_total<<<1, 1, 0, s>>>(sums_scan, sums, tiles, out + len);
    if (cudaGetLastError() != cudaSuccess) rc = GBBFS_ERR_CUDA;
  }
  if (rc == GBBFS_OK && cudaStreamSynchronize(s) != cudaSuccess) rc = GBBFS_ERR_CUDA;
  cudaFree(sums);
  cudaFree(sums_scan);
  if (rc != GBBFS_OK) last_error() = "device scan failed";
  return rc;
}

}  // namespace
}  // namespace gbbfs
