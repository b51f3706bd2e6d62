// CSR construction in HBM: the squish of Builder::MakeGraph on the GPU.
//
// The reference builds the CSR on the host (gapbs-verify/builder.h:73-206:
// count degrees, prefix-sum them, scatter both directions of every edge,
// then sort each neighbour list, drop duplicates and self-loops).  The
// result is a function of the edge multiset alone: vertex u's list is the
// sorted set of its distinct neighbours other than u.  Here every directed
// edge becomes one key (u << bits) | v, an LSD radix sort orders the keys by
// (u, v) with 8-bit digits, and one pass keeps the first of each run of
// equal keys that is not a self-loop, writing v and counting u's degree.  A
// prefix sum of the degrees gives the offsets.  The handle is then created
// from the device arrays; no host CSR is made.
//
// Radix pass (per 8192-key tile, one block): digit counts per tile in
// digit-major order, one exclusive scan over all (digit, tile) counts, then a
// stable scatter: the tile is taken in 32 rounds of 256 keys in index order;
// within a round a key's rank is its lane rank among equal digits in its
// warp (__match_any_sync) plus the counts of earlier warps, and rounds add
// up per digit, so keys keep their input order inside every digit.

#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "engine.h"
#include "scan.cuh"

namespace gbbfs {
namespace {

constexpr int kRadixThreads = 256;
constexpr int kRadixRounds = 32;
constexpr int kRadixTile = kRadixThreads * kRadixRounds;   // keys per block
constexpr int kRadixWarps = kRadixThreads / 32;
constexpr int kDigits = 256;

struct DevBuf {
  void* p = nullptr;
  ~DevBuf() { cudaFree(p); }
  template <typename T>
  T* as() { return static_cast<T*>(p); }
};


// ---------------------------------------------------------------------------
// Radix sort of 64-bit keys.

__global__ void __launch_bounds__(kRadixThreads) k_radix_count(const uint64_t* keys, int64_t len,
                                                               int shift, int64_t tiles,
                                                               int32_t* counts) {
  __shared__ int32_t hist[kDigits];
  hist[threadIdx.x] = 0;
  __syncthreads();
  const int64_t base = (int64_t)blockIdx.x * kRadixTile;
  for (int r = 0; r < kRadixRounds; r++) {
    const int64_t j = base + (int64_t)r * kRadixThreads + threadIdx.x;
    if (j < len) atomicAdd(&hist[(keys[j] >> shift) & (kDigits - 1)], 1);
  }
  __syncthreads();
  counts[(int64_t)threadIdx.x * tiles + blockIdx.x] = hist[threadIdx.x];
}

__global__ void __launch_bounds__(kRadixThreads) k_radix_scatter(const uint64_t* in,
                                                                 uint64_t* out, int64_t len,
                                                                 int shift, int64_t tiles,
                                                                 const int64_t* starts) {
  __shared__ int32_t wcnt[kRadixWarps][kDigits];
  __shared__ int32_t wbase[kRadixWarps][kDigits];
  __shared__ int32_t running[kDigits];
  __shared__ int64_t gbase[kDigits];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int t = threadIdx.x;   // also the digit this thread keeps the books for
  gbase[t] = starts[(int64_t)t * tiles + blockIdx.x];
  running[t] = 0;
#pragma unroll
  for (int i = 0; i < kRadixWarps; i++) wcnt[i][t] = 0;
  __syncthreads();
  const int64_t base = (int64_t)blockIdx.x * kRadixTile;
  for (int r = 0; r < kRadixRounds; r++) {
    const int64_t j = base + (int64_t)r * kRadixThreads + t;
    const bool valid = j < len;
    const uint64_t key = valid ? in[j] : 0ull;
    const int d = valid ? (int)((key >> shift) & (kDigits - 1)) : kDigits;
    const unsigned peers = __match_any_sync(kFull, d);
    const int lrank = __popc(peers & ((1u << lane) - 1));
    if (valid && lrank == 0) wcnt[w][d] = __popc(peers);
    __syncthreads();
    {
      int s = running[t];
#pragma unroll
      for (int i = 0; i < kRadixWarps; i++) {
        const int c = wcnt[i][t];
        wbase[i][t] = s;
        s += c;
        wcnt[i][t] = 0;
      }
      running[t] = s;
    }
    __syncthreads();
    if (valid) out[gbase[d] + wbase[w][d] + lrank] = key;
  }
}

}  // namespace

// Sort len 64-bit keys on their low key_bits bits, stably (LSD, 8-bit
// digits).  keys and tmp hold len entries each; *out is the one that ends up
// holding the sorted keys.
int radix_sort64(uint64_t* keys, uint64_t* tmp, int64_t len, int key_bits, cudaStream_t s,
                 uint64_t** out) {
  *out = keys;
  if (len <= 0) return GBBFS_OK;
  const int64_t tiles = (len + kRadixTile - 1) / kRadixTile;
  DevBuf counts, starts;
  GB_CUDA(cudaMalloc(&counts.p, sizeof(int32_t) * kDigits * (size_t)tiles));
  GB_CUDA(cudaMalloc(&starts.p, sizeof(int64_t) * kDigits * (size_t)tiles));
  uint64_t* src = keys;
  uint64_t* dst = tmp;
  for (int shift = 0; shift < key_bits; shift += 8) {
    k_radix_count<<<(unsigned)tiles, kRadixThreads, 0, s>>>(src, len, shift, tiles,
                                                             counts.as<int32_t>());
    GB_CUDA(cudaGetLastError());
    GB_TRY(device_scan<int32_t>(counts.as<int32_t>(), kDigits * tiles, starts.as<int64_t>(),
                                false, s));
    k_radix_scatter<<<(unsigned)tiles, kRadixThreads, 0, s>>>(src, dst, len, shift, tiles,
                                                               starts.as<int64_t>());
    GB_CUDA(cudaGetLastError());
    std::swap(src, dst);
  }
  GB_CUDA(cudaStreamSynchronize(s));
  *out = src;
  return GBBFS_OK;
}

namespace {

// ---------------------------------------------------------------------------
// Edge list -> keys, and the squish of the sorted keys.

__global__ void k_max_id(const int32_t* el, int64_t count, int* max_id, int* negative) {
  int mx = 0;
  bool neg = false;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int x = el[i];
    mx = max(mx, x);
    neg = neg || x < 0;
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) mx = max(mx, __shfl_xor_sync(kFull, mx, o));
  const unsigned anyneg = __ballot_sync(kFull, neg);
  if ((threadIdx.x & 31) == 0) {
    atomicMax(max_id, mx);
    if (anyneg) atomicOr(negative, 1);
  }
}

__global__ void k_check_ids(const int32_t* el, int64_t count, int64_t n, int* bad) {
  bool b = false;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count;
       i += (int64_t)gridDim.x * blockDim.x)
    b = b || el[i] < 0 || el[i] >= n;
  if (__ballot_sync(kFull, b) && (threadIdx.x & 31) == 0) atomicOr(bad, 1);
}

// Both directions of every edge: (u << bits) | v and (v << bits) | u.
__global__ void k_make_keys(const int32_t* el, int64_t edges, int bits, uint64_t* keys) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < edges;
       e += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t u = (uint32_t)el[2 * e], v = (uint32_t)el[2 * e + 1];
    keys[2 * e] = (u << bits) | v;
    keys[2 * e + 1] = (v << bits) | u;
  }
}

// A sorted key is kept when it differs from the one before it and is not a
// self-loop.  A thread owns kSquishItems consecutive keys.
constexpr int kSquishItems = 32;
constexpr int kSquishTile = kScanThreads * kSquishItems;

__device__ __forceinline__ bool kept(const uint64_t* keys, int64_t j, int bits, uint64_t mask) {
  const uint64_t k = keys[j];
  return (k >> bits) != (k & mask) && (j == 0 || keys[j - 1] != k);
}

__global__ void __launch_bounds__(kScanThreads) k_squish_count(const uint64_t* keys, int64_t len,
                                                               int bits, int32_t* tile_kept,
                                                               int32_t* deg) {
  __shared__ int64_t total;
  const uint64_t mask = (1ull << bits) - 1;
  const int64_t base = (int64_t)blockIdx.x * kSquishTile + (int64_t)threadIdx.x * kSquishItems;
  int64_t c = 0;
  int64_t run_u = -1, run = 0;
  for (int i = 0; i < kSquishItems && base + i < len; i++) {
    if (!kept(keys, base + i, bits, mask)) continue;
    c++;
    const int64_t u = (int64_t)(keys[base + i] >> bits);
    if (u != run_u) {
      if (run) atomicAdd(deg + run_u, (int32_t)run);
      run_u = u;
      run = 0;
    }
    run++;
  }
  if (run) atomicAdd(deg + run_u, (int32_t)run);
  block_exclusive_scan<int64_t>(c, &total);
  if (threadIdx.x == 0) tile_kept[blockIdx.x] = (int32_t)total;
}

__global__ void __launch_bounds__(kScanThreads) k_squish_write(const uint64_t* keys, int64_t len,
                                                               int bits, const int64_t* tile_base,
                                                               int32_t* nbr) {
  __shared__ int64_t total;
  const uint64_t mask = (1ull << bits) - 1;
  const int64_t base = (int64_t)blockIdx.x * kSquishTile + (int64_t)threadIdx.x * kSquishItems;
  int64_t c = 0;
  for (int i = 0; i < kSquishItems && base + i < len; i++) c += kept(keys, base + i, bits, mask);
  int64_t at = block_exclusive_scan<int64_t>(c, &total) + tile_base[blockIdx.x];
  for (int i = 0; i < kSquishItems && base + i < len; i++)
    if (kept(keys, base + i, bits, mask)) nbr[at++] = (int32_t)(keys[base + i] & mask);
}

int bit_length64(uint64_t x) {
  int b = 0;
  while (x) {
    b++;
    x >>= 1;
  }
  return b;
}

// The squished CSR of the edge list in device memory.
int build_on_device(const int32_t* el_pairs, int64_t edges, int64_t num_nodes, cudaStream_t s,
                    DevBuf* off_out, DevBuf* nbr_out, int64_t* n_out, int64_t* m_out) {
  int sms = 0, dev = 0;
  GB_CUDA(cudaGetDevice(&dev));
  GB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const unsigned grid = (unsigned)(sms * 8);
  DevBuf el, flags;
  if (edges > 0) {
    GB_CUDA(cudaMalloc(&el.p, sizeof(int32_t) * 2 * (size_t)edges));
    GB_CUDA(cudaMemcpyAsync(el.p, el_pairs, sizeof(int32_t) * 2 * (size_t)edges,
                            cudaMemcpyDefault, s));
  }
  GB_CUDA(cudaMalloc(&flags.p, 2 * sizeof(int)));
  int h[2] = {0, 0};
  GB_CUDA(cudaMemcpyAsync(flags.p, h, sizeof h, cudaMemcpyHostToDevice, s));
  int64_t n = num_nodes;
  if (n < 0) {
    // num_nodes = largest id + 1 (gapbs-verify/builder.h:62-71, :213-214)
    if (edges > 0)
      k_max_id<<<grid, kThreads, 0, s>>>(el.as<int32_t>(), 2 * edges, flags.as<int>(),
                                         flags.as<int>() + 1);
    GB_CUDA(cudaGetLastError());
    GB_CUDA(cudaMemcpyAsync(h, flags.p, sizeof h, cudaMemcpyDeviceToHost, s));
    GB_CUDA(cudaStreamSynchronize(s));
    if (h[1]) {
      last_error() = "negative vertex id in the edge list";
      return GBBFS_ERR_ARG;
    }
    n = (int64_t)h[0] + 1;
  } else if (edges > 0) {
    k_check_ids<<<grid, kThreads, 0, s>>>(el.as<int32_t>(), 2 * edges, n, flags.as<int>());
    GB_CUDA(cudaGetLastError());
    GB_CUDA(cudaMemcpyAsync(h, flags.p, sizeof h, cudaMemcpyDeviceToHost, s));
    GB_CUDA(cudaStreamSynchronize(s));
    if (h[0]) {
      last_error() = "vertex id outside [0, num_nodes)";
      return GBBFS_ERR_ARG;
    }
  }
  if (n <= 0 || n > INT32_MAX) {
    last_error() = "bad vertex count";
    return GBBFS_ERR_ARG;
  }
  const int bits = std::max(1, bit_length64((uint64_t)(n - 1)));
  const int64_t len = 2 * edges;
  DevBuf a, b, deg;
  GB_CUDA(cudaMalloc(&deg.p, sizeof(int32_t) * (size_t)n));
  GB_CUDA(cudaMemsetAsync(deg.p, 0, sizeof(int32_t) * (size_t)n, s));
  int64_t m = 0;
  if (len > 0) {
    GB_CUDA(cudaMalloc(&a.p, sizeof(uint64_t) * (size_t)len));
    GB_CUDA(cudaMalloc(&b.p, sizeof(uint64_t) * (size_t)len));
    k_make_keys<<<grid, kThreads, 0, s>>>(el.as<int32_t>(), edges, bits, a.as<uint64_t>());
    GB_CUDA(cudaGetLastError());
    GB_CUDA(cudaStreamSynchronize(s));
    cudaFree(el.p);
    el.p = nullptr;
    // LSD radix sort over the 2 * bits key bits.
    uint64_t* src = nullptr;
    GB_TRY(radix_sort64(a.as<uint64_t>(), b.as<uint64_t>(), len, 2 * bits, s, &src));
    // Squish: kept keys per tile, their positions, the neighbour ids.
    const int64_t stiles = (len + kSquishTile - 1) / kSquishTile;
    DevBuf tile_kept, tile_base;
    GB_CUDA(cudaMalloc(&tile_kept.p, sizeof(int32_t) * (size_t)stiles));
    GB_CUDA(cudaMalloc(&tile_base.p, sizeof(int64_t) * (size_t)(stiles + 1)));
    k_squish_count<<<(unsigned)stiles, kScanThreads, 0, s>>>(src, len, bits,
                                                             tile_kept.as<int32_t>(),
                                                             deg.as<int32_t>());
    GB_CUDA(cudaGetLastError());
    GB_TRY(device_scan<int32_t>(tile_kept.as<int32_t>(), stiles, tile_base.as<int64_t>(), true,
                                s));
    GB_CUDA(cudaMemcpy(&m, tile_base.as<int64_t>() + stiles, sizeof(int64_t),
                       cudaMemcpyDeviceToHost));
    GB_CUDA(cudaMalloc(&nbr_out->p, sizeof(int32_t) * (size_t)std::max<int64_t>(m, 1)));
    k_squish_write<<<(unsigned)stiles, kScanThreads, 0, s>>>(src, len, bits,
                                                             tile_base.as<int64_t>(),
                                                             nbr_out->as<int32_t>());
    GB_CUDA(cudaGetLastError());
  } else {
    GB_CUDA(cudaMalloc(&nbr_out->p, sizeof(int32_t)));
  }
  GB_CUDA(cudaMalloc(&off_out->p, sizeof(int64_t) * (size_t)(n + 1)));
  GB_TRY(device_scan<int32_t>(deg.as<int32_t>(), n, off_out->as<int64_t>(), true, s));
  GB_CUDA(cudaStreamSynchronize(s));
  *n_out = n;
  *m_out = m;
  return GBBFS_OK;
}

}  // namespace
}  // namespace gbbfs

extern "C" {

int gbbfs_graph_create_from_edges(const int32_t* el_pairs, int64_t edges, int64_t num_nodes,
                                  gbbfs_graph** out) {
  if (!out || edges < 0 || (edges > 0 && !el_pairs)) return GBBFS_ERR_ARG;
  *out = nullptr;
  cudaStream_t s = nullptr;
  GB_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  gbbfs::DevBuf off, nbr;
  int64_t n = 0, m = 0;
  int rc = gbbfs::build_on_device(el_pairs, edges, num_nodes, s, &off, &nbr, &n, &m);
  cudaStreamDestroy(s);
  if (rc != GBBFS_OK) return rc;
  return gbbfs::graph_create_device(off.as<int64_t>(), nbr.as<int32_t>(), n, m, out);
}

int gbbfs_graph_csr(const gbbfs_graph* g, int64_t* offsets_out, int32_t* neigh_out) {
  if (!g) return GBBFS_ERR_ARG;
  GB_CUDA(cudaSetDevice(g->device));
  if (offsets_out) {
    if (g->off32) {
      std::vector<uint32_t> o((size_t)g->n + 1);
      GB_CUDA(cudaMemcpy(o.data(), g->off, sizeof(uint32_t) * o.size(), cudaMemcpyDeviceToHost));
      for (size_t i = 0; i < o.size(); i++) offsets_out[i] = (int64_t)o[i];
    } else {
      GB_CUDA(cudaMemcpy(offsets_out, g->off, sizeof(int64_t) * (size_t)(g->n + 1),
                         cudaMemcpyDeviceToHost));
    }
  }
  if (neigh_out && g->m > 0)
    GB_CUDA(cudaMemcpy(neigh_out, g->nbr, sizeof(int32_t) * (size_t)g->m,
                       cudaMemcpyDeviceToHost));
  return GBBFS_OK;
}

}  // extern "C"
