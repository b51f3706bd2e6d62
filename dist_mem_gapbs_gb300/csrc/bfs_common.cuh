// Shared definitions of the GB300 BFS engine (device side and host side).
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

#include "gbbfs.h"

namespace gbbfs {

constexpr int kThreads = 256;            // threads per CTA for every kernel
constexpr int kWarpsPerCta = kThreads / 32;
constexpr unsigned kFull = 0xffffffffu;
constexpr int kMaxTrace = 1024;          // step records kept on the device per search
constexpr int kTraceInline = 128;        // records copied back with every search

// Step kinds as the device control loop schedules them.
enum : int32_t {
  kKindInit = 0,
  kKindTD = GBBFS_STEP_TD,
  kKindE = GBBFS_STEP_E,
  kKindBU = GBBFS_STEP_BU,
  kKindC = GBBFS_STEP_C,
  kKindStop = 5,
  kKindTDB = 6,   // a top-down step run as claims into a bitmap, then a sweep (k_tdb)
};

// Branches of the per-step switch node.
enum : unsigned {
  kSelTD = 0, kSelQ2B = 1, kSelBU0 = 2, kSelBU1 = 3, kSelB2Q = 4, kSelTDB = 5, kSelNone = 6
};

// Device-side counters of the current step.  qpacked[i] describes frontier
// queue i: (vertex count << shift) | (sum of their out-degrees).  One 64-bit
// atomicAdd therefore hands a warp both its queue slots and the edge offsets
// of its entries, so the queue carries an exact prefix sum of frontier
// degrees that the next top-down step uses to split edges evenly over warps.
struct DevCounters {
  unsigned long long qpacked[2];
  unsigned long long awake;     // bottom-up claims of the current step
  unsigned long long scanned;   // bottom-up in-neighbours scanned (instrumented)
};

struct DevStep {
  int32_t kind;
  int32_t level;
  int64_t count;
  int64_t edges;
  int64_t unvisited;
  int64_t ns;                   // device time of the step's kernel
};

// State of one search.  The first block is written by the host before the
// search; the rest is owned by the device control loop (k_decide).
struct DevState {
  int32_t source, alpha, beta, want_depth;
  int32_t instrument, in_graph, pad0, pad1;
  int32_t* parent;    // this search's parent array (32 W entries)
  // DOBFS control (src/bfs.cc:158-185): the reference's int64 counters.
  int64_t edges_to_check, scout, cur_edges, awake, old_awake, visited, F;
  int64_t iter, max_iter;
  int32_t cur;        // index of the current queue
  int32_t parity;     // bottom-up frontier lives in bm[parity]
  int32_t level;      // depth the next step discovers
  int32_t next_kind;  // step scheduled (or just run, when k_decide starts)
  int32_t nsteps;
  int32_t error;
  unsigned long long t0, t1;    // first-CTA start / last-CTA end of the running kernel
  unsigned long long init_ns;
  DevStep trace[kMaxTrace];
};

// Device pointers and sizes of one graph handle, passed by value.
template <typename OffT>
struct Bufs {
  const OffT* off;
  const int32_t* nbr;
  const int2* head;   // first two neighbours per vertex, or null
  const uint32_t* iso;
  uint32_t* visited;
  uint32_t* bm0;
  uint32_t* bm1;
  int32_t* depth;
  int32_t* qv0;
  int32_t* qv1;
  OffT* qs0;
  OffT* qs1;
  DevCounters* ctr;
  DevState* st;
  int64_t n, m, W;
  int shift;
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

__device__ __forceinline__ unsigned long long globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Kernel start/end stamps: first CTA to start, last CTA to finish.
__device__ __forceinline__ void stamp_begin(DevState* st) {
  if (threadIdx.x == 0) atomicMin(&st->t0, globaltimer());
}
__device__ __forceinline__ void stamp_end(DevState* st) {
  __syncthreads();
  if (threadIdx.x == 0) atomicMax(&st->t1, globaltimer());
}

}  // namespace gbbfs
