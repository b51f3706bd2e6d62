// gbbfs_bfs_noalloc: one direction-optimizing BFS that allocates nothing.
//
// Some callers cannot allocate device memory at the moment they need a
// search: plugins that live inside a framework whose own caching allocator
// owns the device (memory taken behind its back is memory it cannot account
// for or reuse), and loops that cannot afford the device-wide
// synchronisation cudaMalloc / cudaFree may cause.  For them this entry point
// takes the graph and the result buffers as device pointers the caller
// already owns, and keeps every intermediate it needs (frontier bitmaps,
// queues, counters, control state) in one fixed array of device memory that
// is part of the library itself.
//
// The array is a file-scope __device__ variable of kNoAllocScratchBytes
// (about 8.2 MB), sized for graphs of at most kNoAllocMaxVertices vertices.
// Every GPU that loads the library holds it until the process exits.  All
// calls share it: calls that overlap on the GPU (two streams, two threads)
// race on it and must be serialised by the caller.  Each call clears and
// re-initialises what it reads before reading it.
//
// Host code cannot pass the array's name to a kernel: on the host that name
// is only a stand-in, not a device address.  The first call on each device
// therefore looks the address up with cudaGetSymbolAddress while that device
// is current, and caches it with the launch grids of the step kernels.  The
// cache assumes the device's primary context lives as long as the process
// (no cudaDeviceReset between calls).
//
// The search is stepped from the host: after each step the host reads the
// device's choice of the next one and synchronises the stream.  So the call
// must not be made on a stream that is being captured into a CUDA graph; it
// checks, and returns GBBFS_ERR_STATE without touching the stream.

#include <cuda_runtime.h>

#include <cstddef>
#include <cstring>
#include <mutex>

#include "bfs_kernels.cuh"
#include "engine.h"
#include "gbbfs.h"

namespace gbbfs {
namespace {

constexpr int64_t kNoAllocMaxVertices = int64_t(1) << 18;
constexpr int64_t kNoAllocMaxWords = kNoAllocMaxVertices / 32;

constexpr size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// Layout of the scratch array (byte offsets).
constexpr size_t kOffState = 0;
constexpr size_t kOffCtr = kOffState + align256(sizeof(DevState));
constexpr size_t kOffIso = kOffCtr + align256(sizeof(DevCounters));
constexpr size_t kOffVisited = kOffIso + align256(4 * kNoAllocMaxWords);
constexpr size_t kOffBm0 = kOffVisited + align256(4 * kNoAllocMaxWords);
constexpr size_t kOffBm1 = kOffBm0 + align256(4 * kNoAllocMaxWords);
constexpr size_t kOffParent = kOffBm1 + align256(4 * kNoAllocMaxWords);
constexpr size_t kOffDepth = kOffParent + align256(4 * 32 * kNoAllocMaxWords);
constexpr size_t kOffQv0 = kOffDepth + align256(4 * 32 * kNoAllocMaxWords);
constexpr size_t kOffQv1 = kOffQv0 + align256(4 * kNoAllocMaxVertices);
constexpr size_t kOffQs0 = kOffQv1 + align256(4 * kNoAllocMaxVertices);
constexpr size_t kOffQs1 = kOffQs0 + align256(8 * kNoAllocMaxVertices);
constexpr size_t kNoAllocScratchBytes = kOffQs1 + align256(8 * kNoAllocMaxVertices);

__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;

// Per device: the scratch array's address and the grids of the step kernels.
struct DeviceSetup {
  unsigned char* scratch = nullptr;
  int sms = 0;
  int g_init = 0, g_td = 0, g_bu = 0, g_q2b = 0, g_b2q = 0, g_tdb = 0;
};
std::mutex g_setup_mu;
DeviceSetup g_setup[kMaxDevices];

int bits(uint64_t x) {
  int b = 0;
  while (x) {
    b++;
    x >>= 1;
  }
  return b;
}

int occupancy(const void* fn, int sms, int* grid) {
  int per_sm = 0;
  GB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kThreads, 0));
  *grid = (per_sm > 0 ? per_sm : 1) * sms;
  return GBBFS_OK;
}

// Set-up of the current device, done once: the device address of the
// scratch array (cudaGetSymbolAddress, with that device current) and the
// launch grids.
int device_setup(const DeviceSetup** out) {
  typedef unsigned long long OffT;
  int dev = 0;
  GB_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) {
    last_error() = "device index beyond the scratch table";
    return GBBFS_ERR_ARG;
  }
  std::lock_guard<std::mutex> lk(g_setup_mu);
  DeviceSetup& d = g_setup[dev];
  if (!d.scratch) {
    DeviceSetup t;
    void* p = nullptr;
    GB_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    t.scratch = static_cast<unsigned char*>(p);
    GB_CUDA(cudaDeviceGetAttribute(&t.sms, cudaDevAttrMultiProcessorCount, dev));
    GB_TRY(occupancy((const void*)k_init<OffT>, t.sms, &t.g_init));
    GB_TRY(occupancy((const void*)k_td<OffT>, t.sms, &t.g_td));
    GB_TRY(occupancy((const void*)k_bu<OffT, 0>, t.sms, &t.g_bu));
    GB_TRY(occupancy((const void*)k_q2b<OffT>, t.sms, &t.g_q2b));
    GB_TRY(occupancy((const void*)k_b2q<OffT, false>, t.sms, &t.g_b2q));
    GB_TRY(occupancy((const void*)k_tdb<OffT>, t.sms, &t.g_tdb));
    d = t;
  }
  *out = &d;
  return GBBFS_OK;
}

}  // namespace
}  // namespace gbbfs

using namespace gbbfs;

extern "C" {

int gbbfs_bfs_noalloc(const int64_t* d_offsets, const int32_t* d_neigh, int64_t n,
                      int64_t m_dir, int32_t source, int alpha, int beta,
                      int32_t* d_parent_out, int32_t* d_depth_out, void* stream) {
  typedef unsigned long long OffT;
  if (!d_offsets || (m_dir > 0 && !d_neigh) || !d_parent_out || n <= 0 || m_dir < 0) {
    last_error() = "bad arguments";
    return GBBFS_ERR_ARG;
  }
  if (n > kNoAllocMaxVertices) {
    last_error() = "gbbfs_bfs_noalloc serves graphs of at most 262144 vertices";
    return GBBFS_ERR_ARG;
  }
  if (source < 0 || source >= n) {
    last_error() = "source out of range";
    return GBBFS_ERR_ARG;
  }
  const int shift = 64 - bits((uint64_t)n);
  if ((uint64_t)m_dir >= (1ull << shift)) {
    last_error() = "graph too large for the packed frontier counter";
    return GBBFS_ERR_ARG;
  }
  if (alpha <= 0) alpha = 15;
  if (beta <= 0) beta = 18;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaStreamCaptureStatus capturing = cudaStreamCaptureStatusNone;
  GB_CUDA(cudaStreamIsCapturing(s, &capturing));
  if (capturing != cudaStreamCaptureStatusNone) {
    last_error() = "gbbfs_bfs_noalloc synchronises its stream after every step and cannot "
                   "run on a stream that is being captured";
    return GBBFS_ERR_STATE;
  }

  const DeviceSetup* d = nullptr;
  GB_TRY(device_setup(&d));
  unsigned char* base = d->scratch;
  const int sms = d->sms;
  const int g_init = d->g_init, g_td = d->g_td, g_bu = d->g_bu, g_q2b = d->g_q2b,
            g_b2q = d->g_b2q, g_tdb = d->g_tdb;

  Bufs<OffT> b;
  b.off = reinterpret_cast<const OffT*>(d_offsets);
  b.nbr = d_neigh;
  b.head = nullptr;   // no room for the neighbour heads: first probes read nbr
  b.iso = reinterpret_cast<uint32_t*>(base + kOffIso);
  b.visited = reinterpret_cast<uint32_t*>(base + kOffVisited);
  b.bm0 = reinterpret_cast<uint32_t*>(base + kOffBm0);
  b.bm1 = reinterpret_cast<uint32_t*>(base + kOffBm1);
  int32_t* parent = reinterpret_cast<int32_t*>(base + kOffParent);
  b.depth = reinterpret_cast<int32_t*>(base + kOffDepth);
  b.qv0 = reinterpret_cast<int32_t*>(base + kOffQv0);
  b.qv1 = reinterpret_cast<int32_t*>(base + kOffQv1);
  b.qs0 = reinterpret_cast<OffT*>(base + kOffQs0);
  b.qs1 = reinterpret_cast<OffT*>(base + kOffQs1);
  b.ctr = reinterpret_cast<DevCounters*>(base + kOffCtr);
  b.st = reinterpret_cast<DevState*>(base + kOffState);
  b.n = n;
  b.m = m_dir;
  b.W = (n + 31) / 32;
  b.shift = shift;

  // Start from a clean control block (the previous call left its own state),
  // with the timer stamps at their neutral values.
  DevState head;
  memset(&head, 0, offsetof(DevState, trace));
  head.source = source;
  head.alpha = alpha;
  head.beta = beta;
  head.want_depth = d_depth_out ? 1 : 0;
  head.parent = parent;
  head.instrument = 0;
  head.in_graph = 0;
  head.t0 = ~0ull;
  head.t1 = 0;
  GB_CUDA(cudaMemcpyAsync(b.st, &head, offsetof(DevState, trace), cudaMemcpyHostToDevice, s));
  GB_CUDA(cudaMemsetAsync(b.ctr, 0, sizeof(DevCounters), s));
  k_iso_mask<OffT><<<sms * 4, kThreads, 0, s>>>(n, b.W, b.off, const_cast<uint32_t*>(b.iso));
  GB_CUDA(cudaGetLastError());
  k_init<OffT><<<g_init, kThreads, 0, s>>>(b);
  GB_CUDA(cudaGetLastError());
  // The DOBFS control loop, stepped from the host: k_decide picks the step,
  // the host reads its choice and launches that kernel.
  const size_t ctl = offsetof(DevState, cur);
  int32_t c4[4];
  for (;;) {
    k_decide<OffT><<<1, 32, 0, s>>>(b, 0, 0);
    GB_CUDA(cudaGetLastError());
    GB_CUDA(cudaMemcpyAsync(c4, reinterpret_cast<unsigned char*>(b.st) + ctl, sizeof c4,
                            cudaMemcpyDeviceToHost, s));
    GB_CUDA(cudaStreamSynchronize(s));
    const int parity = c4[1], kind = c4[3];
    if (kind == kKindStop) break;
    switch (kind) {
      case kKindTD: k_td<OffT><<<g_td, kThreads, 0, s>>>(b); break;
      case kKindTDB:
        k_tdb<OffT><<<g_tdb, kThreads, 0, s>>>(b);
        k_b2q<OffT, true><<<g_b2q, kThreads, 0, s>>>(b);
        break;
      case kKindE: k_q2b<OffT><<<g_q2b, kThreads, 0, s>>>(b); break;
      case kKindBU:
        if (parity)
          k_bu<OffT, 1><<<g_bu, kThreads, 0, s>>>(b);
        else
          k_bu<OffT, 0><<<g_bu, kThreads, 0, s>>>(b);
        break;
      case kKindC: k_b2q<OffT, false><<<g_b2q, kThreads, 0, s>>>(b); break;
      default:
        last_error() = "unknown step kind from the device";
        return GBBFS_ERR_STATE;
    }
    GB_CUDA(cudaGetLastError());
  }
  int32_t err = 0;
  GB_CUDA(cudaMemcpyAsync(&err, &b.st->error, sizeof err, cudaMemcpyDeviceToHost, s));
  GB_CUDA(cudaMemcpyAsync(d_parent_out, parent, sizeof(int32_t) * n, cudaMemcpyDeviceToDevice,
                          s));
  if (d_depth_out)
    GB_CUDA(cudaMemcpyAsync(d_depth_out, b.depth, sizeof(int32_t) * n, cudaMemcpyDeviceToDevice,
                            s));
  GB_CUDA(cudaStreamSynchronize(s));
  if (err) {
    last_error() = "device control loop exceeded its iteration bound";
    return err;
  }
  return GBBFS_OK;
}

}  // extern "C"
