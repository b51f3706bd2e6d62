// Shared definitions of the GB300 BFS engine (device side and host side).
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

#include "gbbfs.h"

namespace gbbfs {

constexpr int kThreads = 256;            // threads per CTA for every kernel
constexpr int kWarpsPerCta = kThreads / 32;
constexpr unsigned kFull = 0xffffffffu;

// Device-side counters of one search.  qpacked[i] describes frontier queue i:
// (vertex count << shift) | (sum of their out-degrees).  One 64-bit atomicAdd
// therefore hands a warp both its queue slots and the edge offsets of its
// entries, so the queue carries an exact prefix sum of frontier degrees that
// the next top-down step uses to split edges evenly over warps.
struct DevCounters {
  unsigned long long qpacked[2];
  unsigned long long awake;     // bottom-up claims of the current step
  unsigned long long scanned;   // bottom-up in-neighbours scanned (instrumented)
  int error;                    // GBBFS_ERR_* raised on the device
  int pad[3];
};

template <typename T>
__device__ __forceinline__ T shfl(T x, int src) {
  if constexpr (sizeof(T) == 8) {
    unsigned long long y = (unsigned long long)x;
    unsigned lo = __shfl_sync(kFull, (unsigned)y, src);
    unsigned hi = __shfl_sync(kFull, (unsigned)(y >> 32), src);
    return (T)(((unsigned long long)hi << 32) | lo);
  } else {
    return __shfl_sync(kFull, x, src);
  }
}

template <typename T>
__device__ __forceinline__ T shfl_up(T x, int d) {
  if constexpr (sizeof(T) == 8) {
    unsigned long long y = (unsigned long long)x;
    unsigned lo = __shfl_up_sync(kFull, (unsigned)y, d);
    unsigned hi = __shfl_up_sync(kFull, (unsigned)(y >> 32), d);
    return (T)(((unsigned long long)hi << 32) | lo);
  } else {
    return __shfl_up_sync(kFull, x, d);
  }
}

// Inclusive warp scan (sum).
template <typename T>
__device__ __forceinline__ T warp_inclusive_sum(T x, int lane) {
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    T y = shfl_up(x, d);
    if (lane >= d) x += y;
  }
  return x;
}

__device__ __forceinline__ uint32_t ld_cg(const uint32_t* p) { return __ldcg(p); }

__device__ __forceinline__ bool test_bit(const uint32_t* bm, int32_t v) {
  return (__ldcg(bm + (v >> 5)) >> (v & 31)) & 1u;
}

}  // namespace gbbfs
