// Batched multi-source BFS: up to 256 sources per batch as a bitmask per vertex.
//
// This form has no counterpart in the reference: it answers many BFS queries
// of the same graph at once.  Its results are defined by the reference's
// single-source search (src/bfs.cc:142-188): depth[s][v] equals the depth that
// a plain DOBFS from source s gives vertex v, bit for bit.
//
// The kernel and the layout of its buffers are described in
// msbfs_kernels.cuh.  The search runs on a copy of the graph in which the
// vertices are grouped by the bit length of their degree, longest first
// (isolated vertices last): the frontier words the bottom-up levels read at
// random then gather on a compact, cache-resident range, and tiles hold
// vertices of similar degree.  This file builds that copy when the state is
// first made, owns the buffers, captures one CUDA graph per batch buffer
// (sources copy, buffer resets, the persistent cooperative kernel, the pass
// that writes the depth rows in original vertex order from the per-vertex
// depth log, a copy of the control block back to the host), runs batches back to back with the
// copy of one batch's depths overlapping the next batch, and holds the
// autotuner.  Depth rows are uint8 (255 = unreached) or int32 (-1).

#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "engine.h"
#include "msbfs_kernels.cuh"

namespace gbbfs {

constexpr int kSrcSlot = kMsMaxLanes + 1;   // per batch buffer: count, then the sources
constexpr int kLaneClasses = 4;              // lane words of 32 << cls bits

struct MsConfig {
  int lanes = 256;       // 32, 64, 128 or 256 sources per batch (the widest used)
  int batch = 8;         // neighbours per bottom-up round of one thread
  int alpha = 15;        // top-down while frontier degrees <= m / alpha
};

struct MsState {
  int64_t n = 0;
  int depth_bytes = 0;
  int lanes = 0;
  void* visit = nullptr;
  void* fr[2] = {nullptr, nullptr};
  void* acc = nullptr;
  uint32_t* fbits[2] = {nullptr, nullptr};
  int32_t* q[2] = {nullptr, nullptr};
  uint64_t* qe[2] = {nullptr, nullptr};
  int32_t* tq = nullptr;
  int32_t* hubs = nullptr;
  uint32_t* hub_chunk = nullptr;
  int64_t nhubs = 0;
  int32_t* unit_tile = nullptr;      // bottom-up work units (tile ranges)
  int64_t nunits = 0;
  void* roff = nullptr;              // search-ordered CSR (OffT offsets)
  int32_t* rnbr = nullptr;
  int32_t* perm = nullptr;           // original id -> search order id
  void* dtmp = nullptr;              // depth rows in search order (row stride dstride)
  int64_t dstride = 0;
  uint32_t* lvl = nullptr;           // per-vertex depth log: levels, lane masks, flags
  void* lmask = nullptr;
  uint8_t* spill = nullptr;
  uint32_t* tflag = nullptr;
  void* depth[2] = {nullptr, nullptr};
  int32_t* d_src[2] = {nullptr, nullptr};
  int32_t* h_src = nullptr;          // pinned, 2 x kSrcSlot: count, then the sources
  MsCtl* ctl[2] = {nullptr, nullptr};
  MsCtl* h_ctl = nullptr;            // pinned, 2
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t computed[2] = {nullptr, nullptr};
  cudaEvent_t copied[2] = {nullptr, nullptr};
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  // One captured graph per batch buffer and lane width (32, 64, 128, 256);
  // the source count is read on the device, so a graph serves every batch
  // size.
  cudaGraphExec_t exec[2][kLaneClasses] = {};
  MsConfig exec_cfg[2][kLaneClasses];
  int exec_sms[2][kLaneClasses] = {};
  MsConfig cfg;
  // SMs the persistent kernel's grid spans (0: all).  A query server gives
  // each graph a share, so batches of several graphs run on the GPU at once.
  int grid_sms = 0;
  int64_t bytes = 0;
  int last_buf = -1;
  int last_k = 0;
};

void msbfs_release(MsState* ms) {
  if (!ms) return;
  for (int i = 0; i < 2; i++) {
    for (int c = 0; c < kLaneClasses; c++)
      if (ms->exec[i][c]) cudaGraphExecDestroy(ms->exec[i][c]);
    cudaFree(ms->q[i]);
    cudaFree(ms->qe[i]);
    cudaFree(ms->depth[i]);
    cudaFree(ms->d_src[i]);
    cudaFree(ms->ctl[i]);
    if (ms->computed[i]) cudaEventDestroy(ms->computed[i]);
    if (ms->copied[i]) cudaEventDestroy(ms->copied[i]);
  }
  cudaFree(ms->visit);
  cudaFree(ms->fr[0]);
  cudaFree(ms->fr[1]);
  cudaFree(ms->acc);
  cudaFree(ms->fbits[0]);
  cudaFree(ms->fbits[1]);
  cudaFree(ms->tq);
  cudaFree(ms->hubs);
  cudaFree(ms->hub_chunk);
  cudaFree(ms->unit_tile);
  cudaFree(ms->roff);
  cudaFree(ms->rnbr);
  cudaFree(ms->perm);
  cudaFree(ms->dtmp);
  cudaFree(ms->lvl);
  cudaFree(ms->lmask);
  cudaFree(ms->spill);
  cudaFree(ms->tflag);
  if (ms->h_src) cudaFreeHost(ms->h_src);
  if (ms->h_ctl) cudaFreeHost(ms->h_ctl);
  if (ms->ev0) cudaEventDestroy(ms->ev0);
  if (ms->ev1) cudaEventDestroy(ms->ev1);
  if (ms->copy_stream) cudaStreamDestroy(ms->copy_stream);
  delete ms;
}

// ---------------------------------------------------------------------------
// Host side.

// Lane words are allocated at 256 bits so every lane width fits: visit, the
// two frontier buffers, acc; queues q0/q1 with their edge positions qe0/qe1,
// and tq; two frontier unions and the work-unit table; the search-ordered CSR (offsets counted at 8
// bytes) and its permutation; the per-vertex depth log (kLogSlots lane masks,
// levels, flags); depth rows of 256 sources in search order for what the log
// cannot hold and two buffers of rows in original order; slack for the hub
// list and control blocks.
size_t ms_state_bytes(int64_t n, int64_t m, int64_t W, int depth_bytes) {
  return 4 * sizeof(Lane256) * (size_t)n + 2 * 8 * (size_t)n + 3 * 4 * (size_t)n +
         12 * (size_t)(W + 1) + 8 * (size_t)(n + 1) + 4 * (size_t)m + 4 * (size_t)n +
         (kLogSlots * sizeof(Lane256) + 9) * (size_t)n +
         3 * (size_t)kMsMaxLanes * (n + kDepthTile) * depth_bytes + (16 << 20);
}

namespace {

#define ms_error (::gbbfs::last_error())

template <typename OffT, typename LaneT, typename DepthT, int kB>
const void* kernel_ptr() {
  return (const void*)k_msbfs<OffT, LaneT, DepthT, kB>;
}

template <typename OffT, typename LaneT, typename DepthT>
const void* pick_batch(int batch) {
  switch (batch) {
    case 4: return kernel_ptr<OffT, LaneT, DepthT, 4>();
    case 16: return kernel_ptr<OffT, LaneT, DepthT, 16>();
    default: return kernel_ptr<OffT, LaneT, DepthT, 8>();
  }
}

template <typename OffT, typename LaneT>
const void* pick_depth(int depth_bytes, int batch) {
  return depth_bytes == 1 ? pick_batch<OffT, LaneT, uint8_t>(batch)
                          : pick_batch<OffT, LaneT, int32_t>(batch);
}

template <typename OffT>
const void* pick_kernel(const MsConfig& cfg, int depth_bytes) {
  if (cfg.lanes == 256) return pick_depth<OffT, Lane256>(depth_bytes, cfg.batch);
  if (cfg.lanes == 128) return pick_depth<OffT, Lane128>(depth_bytes, cfg.batch);
  return cfg.lanes == 32 ? pick_depth<OffT, uint32_t>(depth_bytes, cfg.batch)
                         : pick_depth<OffT, unsigned long long>(depth_bytes, cfg.batch);
}

const void* kernel_for(const gbbfs_graph* g, const MsConfig& cfg, int depth_bytes) {
  return g->off32 ? pick_kernel<uint32_t>(cfg, depth_bytes)
                  : pick_kernel<unsigned long long>(cfg, depth_bytes);
}

// Batching keys.  A batch costs about as many full bottom-up levels as its
// slowest source needs, so sources that reach the bulk of the graph at the
// same level should share a batch.  The proxy for that level is the source's
// BFS depth from the highest-degree vertex; among sources at the same depth,
// one whose neighbours have more edges reaches the bulk sooner (the sum of
// the neighbours' degrees: the number of two-step walks from the source).
template <typename OffT>
__global__ void k_argmax_degree(const OffT* off, int64_t n, unsigned long long* best) {
  unsigned long long mine = 0;
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += (int64_t)gridDim.x * blockDim.x) {
    const unsigned long long d = (unsigned long long)(off[v + 1] - off[v]);
    const unsigned long long key = ((d < 0xffffffffull ? d : 0xffffffffull) << 32) |
                                   (0xffffffffull - (unsigned long long)v);   // lowest id wins ties
    mine = mine > key ? mine : key;
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    const unsigned long long x = __shfl_xor_sync(kFull, mine, o);
    mine = mine > x ? mine : x;
  }
  if ((threadIdx.x & 31) == 0 && mine) atomicMax(best, mine);
}

// Key of v: hub depth (255 = unreached, else at most 254) << 8, then
// 255 - q with q = the quarter-octave of s, the sum of v's neighbours'
// degrees (over the first kKeySample neighbours, scaled by deg / kKeySample,
// for larger degrees): with t = 4 s and b = its bit length, q = 4 b + the two
// bits of t below its leading one (0 when s = 0).
constexpr int kKeySample = 256;

template <typename OffT>
__global__ void k_batch_keys(const OffT* off, const int32_t* nbr, const int32_t* depth,
                             int64_t n, uint16_t* keys) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += (int64_t)gridDim.x * blockDim.x) {
    const int32_t d = depth[v];
    const uint32_t hd = d < 0 ? 255u : d > 254 ? 254u : (uint32_t)d;
    const uint64_t b = (uint64_t)off[v], deg = (uint64_t)off[v + 1] - b;
    const uint64_t take = deg < (uint64_t)kKeySample ? deg : (uint64_t)kKeySample;
    uint64_t s = 0;
    for (uint64_t j = 0; j < take; j++) {
      const int32_t u = nbr[b + j];
      s += (uint64_t)(off[u + 1] - off[u]);
    }
    if (deg > take) s = s * deg / take;
    uint32_t q = 0;
    if (s) {
      const uint64_t t = s << 2;
      const int bl = 64 - __clzll((long long)t);
      q = 4u * (uint32_t)bl + (uint32_t)((t >> (bl - 3)) & 3u);
      if (q > 255u) q = 255u;
    }
    keys[v] = (uint16_t)((hd << 8) | (255u - q));
  }
}

template <typename OffT>
int make_batch_keys(gbbfs_graph* g) {
  const int64_t n = g->n;
  const OffT* off = reinterpret_cast<const OffT*>(g->off);
  unsigned long long* d_best = nullptr;
  uint16_t* d_keys = nullptr;
  GB_CUDA(cudaMalloc(&d_best, sizeof(unsigned long long)));
  cudaError_t e = cudaMalloc(&d_keys, 2 * (size_t)n);
  if (e == cudaSuccess) e = cudaMemsetAsync(d_best, 0, sizeof(unsigned long long), g->stream);
  if (e == cudaSuccess) {
    k_argmax_degree<OffT><<<4 * g->sms, kThreads, 0, g->stream>>>(off, n, d_best);
    e = cudaGetLastError();
  }
  unsigned long long best = 0;
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(&best, d_best, sizeof best, cudaMemcpyDeviceToHost, g->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
  int rc = GBBFS_OK;
  if (e == cudaSuccess) {
    const int32_t hub = (int32_t)(0xffffffffull - (best & 0xffffffffull));
    rc = gbbfs_bfs_device(g, hub, 0, 0, 1, nullptr);
    const int32_t* depth = nullptr;
    if (rc == GBBFS_OK) rc = gbbfs_result_device_ptrs(g, nullptr, &depth);
    if (rc == GBBFS_OK) {
      k_batch_keys<OffT><<<4 * g->sms, kThreads, 0, g->stream>>>(off, g->nbr, depth, n, d_keys);
      e = cudaGetLastError();
      std::vector<uint16_t> keys((size_t)n);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(keys.data(), d_keys, 2 * (size_t)n, cudaMemcpyDeviceToHost, g->stream);
      if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
      if (e == cudaSuccess) g->batch_key.swap(keys);
    }
  }
  cudaFree(d_best);
  cudaFree(d_keys);
  if (rc != GBBFS_OK) return rc;
  if (e != cudaSuccess) {
    ms_error = std::string("batching keys: ") + cudaGetErrorString(e);
    return GBBFS_ERR_CUDA;
  }
  return GBBFS_OK;
}

// The search-ordered copy of the graph.  New ids: the vertices of degree
// kMsOrderDeg or more in buckets by the bit length of their degree, longest
// first, in id order inside each bucket; then the others in id order (a
// counting sort on the host over the offsets).  Inside a bucket vertices keep
// their order, so the rows put back into original order read from a few
// sequential runs.  The neighbour lists are then renamed and sorted by new
// id on the device (a radix sort of the directed edges' (new u, new v) keys),
// so every list starts with its highest-degree neighbours: they are in many
// sources' frontiers at once, and bottom-up scans that stop once every lane
// is found stop sooner.  Hubs (degree above kMsHubDeg) are listed in new-id
// order with their work chunks' prefix.
template <typename OffT, typename Alloc>
int build_order(gbbfs_graph* g, MsState* ms, Alloc&& alloc) {
  const int64_t n = g->n;
  std::vector<OffT> hoff((size_t)n + 1);
  GB_CUDA(cudaMemcpy(hoff.data(), g->off, sizeof(OffT) * (size_t)(n + 1),
                     cudaMemcpyDeviceToHost));
  auto deg = [&](int64_t v) { return (uint64_t)(hoff[v + 1] - hoff[v]); };
  auto key = [&](int64_t v) {
    const uint64_t d = deg(v);
    if (d < (uint64_t)kMsOrderDeg) return 64;
    int bits = 0;
    for (uint64_t x = d; x; x >>= 1) bits++;
    return 64 - bits;
  };
  std::vector<int64_t> pos(65, 0);
  for (int64_t v = 0; v < n; v++) pos[key(v)]++;
  int64_t run = 0;
  for (auto& p : pos) {
    const int64_t c = p;
    p = run;
    run += c;
  }
  std::vector<int32_t> perm((size_t)n), inv((size_t)n);
  for (int64_t v = 0; v < n; v++) {
    const int64_t r = pos[key(v)]++;
    perm[v] = (int32_t)r;
    inv[r] = (int32_t)v;
  }
  std::vector<OffT> noff((size_t)n + 1);
  noff[0] = 0;
  for (int64_t r = 0; r < n; r++) noff[r + 1] = noff[r] + (OffT)deg(inv[r]);
  std::vector<int32_t> hubs;
  std::vector<uint32_t> hub_chunk;
  uint64_t chunks = 0;
  for (int64_t r = 0; r < n; r++) {
    if (deg(inv[r]) <= (uint64_t)kMsHubDeg) continue;
    hubs.push_back((int32_t)r);
    hub_chunk.push_back((uint32_t)chunks);
    chunks += (deg(inv[r]) + kMsHubChunk - 1) / kMsHubChunk;
  }
  hub_chunk.push_back((uint32_t)chunks);
  // Bottom-up work units: runs of up to kMsGrab tiles, cut early once the
  // tiles' non-hub vertices hold kMsUnitEdges edges, so the high-degree
  // tiles at the front of the order do not pile up on one warp.
  std::vector<int32_t> unit_tile;
  const int64_t tiles = (n + 31) / 32;
  {
    int64_t in_unit = 0;
    uint64_t edges = 0;
    for (int64_t t = 0; t < tiles; t++) {
      if (in_unit == 0) unit_tile.push_back((int32_t)t);
      for (int64_t r = 32 * t; r < std::min<int64_t>(n, 32 * t + 32); r++) {
        const uint64_t d = deg(inv[r]);
        if (d <= (uint64_t)kMsHubDeg) edges += d;
      }
      if (++in_unit == kMsGrab || edges >= (uint64_t)kMsUnitEdges) {
        in_unit = 0;
        edges = 0;
      }
    }
    unit_tile.push_back((int32_t)tiles);
  }
  ms->nunits = (int64_t)unit_tile.size() - 1;
  GB_TRY(alloc(reinterpret_cast<void**>(&ms->unit_tile), 4 * unit_tile.size()));
  GB_CUDA(cudaMemcpy(ms->unit_tile, unit_tile.data(), 4 * unit_tile.size(),
                     cudaMemcpyHostToDevice));

  GB_TRY(alloc(&ms->roff, sizeof(OffT) * (size_t)(n + 1)));
  GB_TRY(alloc(reinterpret_cast<void**>(&ms->rnbr), 4 * (size_t)g->m));
  GB_TRY(alloc(reinterpret_cast<void**>(&ms->perm), 4 * (size_t)n));
  cudaError_t e = cudaMemcpy(ms->roff, noff.data(), sizeof(OffT) * (size_t)(n + 1),
                             cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(ms->perm, perm.data(), 4 * (size_t)n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && g->m > 0) {
    // Neighbour lists renamed and sorted by new id (hubs first): the keys
    // (new u, new v) of all directed edges, radix-sorted.
    int bits = 1;
    while (bits < 31 && (int64_t(1) << bits) < n) bits++;
    uint64_t *ka = nullptr, *kb = nullptr, *sorted = nullptr;
    e = cudaMalloc(&ka, 8 * (size_t)g->m);
    if (e == cudaSuccess) e = cudaMalloc(&kb, 8 * (size_t)g->m);
    if (e == cudaSuccess) {
      k_relabel_keys<OffT><<<8 * g->sms, kThreads, 0, g->stream>>>(
          reinterpret_cast<const OffT*>(g->off), g->nbr, ms->perm, n, bits, ka);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess &&
        radix_sort64(ka, kb, g->m, 2 * bits, g->stream, &sorted) != GBBFS_OK)
      e = cudaErrorUnknown;
    if (e == cudaSuccess) {
      k_low_bits<<<8 * g->sms, kThreads, 0, g->stream>>>(sorted, g->m, (1ull << bits) - 1,
                                                          ms->rnbr);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    cudaFree(ka);
    cudaFree(kb);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
  if (e != cudaSuccess) {
    ms_error = std::string("search-ordered graph copy: ") + cudaGetErrorString(e);
    return GBBFS_ERR_CUDA;
  }
  ms->nhubs = (int64_t)hubs.size();
  if (ms->nhubs) {
    GB_TRY(alloc(reinterpret_cast<void**>(&ms->hubs), 4 * (size_t)ms->nhubs));
    GB_TRY(alloc(reinterpret_cast<void**>(&ms->hub_chunk), 4 * (size_t)(ms->nhubs + 1)));
    GB_CUDA(cudaMemcpy(ms->hubs, hubs.data(), 4 * (size_t)ms->nhubs, cudaMemcpyHostToDevice));
    GB_CUDA(cudaMemcpy(ms->hub_chunk, hub_chunk.data(), 4 * (size_t)(ms->nhubs + 1),
                       cudaMemcpyHostToDevice));
  }
  return GBBFS_OK;
}

int build_state(gbbfs_graph* g, int depth_bytes);

// The batched-search state of a graph handle for this depth width: kept when
// it matches, else built anew.  A build that fails part way is released and
// detached, so a later call never finds a half-built state.
int ensure_state(gbbfs_graph* g, int depth_bytes) {
  if (g->ms && g->ms->depth_bytes == depth_bytes) return GBBFS_OK;
  const int rc = build_state(g, depth_bytes);
  if (rc != GBBFS_OK && g->ms) {
    msbfs_release(g->ms);
    g->ms = nullptr;
  }
  return rc;
}

int build_state(gbbfs_graph* g, int depth_bytes) {
  MsState* ms = g->ms;
  MsConfig keep;
  if (ms) {
    keep = ms->cfg;
    msbfs_release(ms);
    g->ms = nullptr;
  }
  const int64_t n = g->n;
  const size_t need = ms_state_bytes(n, g->m, g->W, depth_bytes);
  size_t free_b = 0, total_b = 0;
  GB_CUDA(cudaMemGetInfo(&free_b, &total_b));
  if (need > free_b) {
    ms_error = "multi-source BFS needs " + std::to_string(need) + " bytes, " +
               std::to_string(free_b) + " free";
    return GBBFS_ERR_NOMEM;
  }
  ms = new MsState();
  g->ms = ms;
  ms->cfg = keep;
  ms->n = n;
  ms->depth_bytes = depth_bytes;
  auto alloc = [&](void** p, size_t bytes) -> int {
    cudaError_t e = cudaMalloc(p, std::max<size_t>(bytes, 256));
    if (e != cudaSuccess) {
      ms_error = std::string("cudaMalloc: ") + cudaGetErrorString(e);
      return e == cudaErrorMemoryAllocation ? GBBFS_ERR_NOMEM : GBBFS_ERR_CUDA;
    }
    ms->bytes += (int64_t)bytes;
    return GBBFS_OK;
  };
  GB_TRY(alloc(&ms->visit, sizeof(Lane256) * (size_t)n));
  GB_TRY(alloc(&ms->fr[0], sizeof(Lane256) * (size_t)n));
  GB_TRY(alloc(&ms->fr[1], sizeof(Lane256) * (size_t)n));
  GB_TRY(alloc(&ms->acc, sizeof(Lane256) * (size_t)n));
  GB_TRY(alloc(reinterpret_cast<void**>(&ms->fbits[0]), 4 * (size_t)g->W));
  GB_TRY(alloc(reinterpret_cast<void**>(&ms->fbits[1]), 4 * (size_t)g->W));
  GB_TRY(alloc(reinterpret_cast<void**>(&ms->tq), 4 * (size_t)n));
  ms->dstride = (n + kDepthTile - 1) / kDepthTile * kDepthTile;
  GB_TRY(alloc(&ms->dtmp, (size_t)kMsMaxLanes * ms->dstride * depth_bytes));
  GB_TRY(alloc(reinterpret_cast<void**>(&ms->lvl), 4 * (size_t)n));
  GB_TRY(alloc(&ms->lmask, (size_t)kLogSlots * sizeof(Lane256) * n));
  GB_TRY(alloc(reinterpret_cast<void**>(&ms->spill), (size_t)n));
  GB_TRY(alloc(reinterpret_cast<void**>(&ms->tflag), 4 * (size_t)n));
  GB_TRY(g->off32 ? build_order<uint32_t>(g, ms, alloc)
                  : build_order<unsigned long long>(g, ms, alloc));
  for (int i = 0; i < 2; i++) {
    GB_TRY(alloc(reinterpret_cast<void**>(&ms->q[i]), 4 * (size_t)n));
    GB_TRY(alloc(reinterpret_cast<void**>(&ms->qe[i]), 8 * (size_t)n));
    GB_TRY(alloc(&ms->depth[i], (size_t)kMsMaxLanes * n * depth_bytes));
    GB_TRY(alloc(reinterpret_cast<void**>(&ms->d_src[i]), kSrcSlot * sizeof(int32_t)));
    GB_TRY(alloc(reinterpret_cast<void**>(&ms->ctl[i]), sizeof(MsCtl)));
    GB_CUDA(cudaEventCreateWithFlags(&ms->computed[i], cudaEventDisableTiming));
    GB_CUDA(cudaEventCreateWithFlags(&ms->copied[i], cudaEventDisableTiming));
  }
  GB_CUDA(cudaHostAlloc(reinterpret_cast<void**>(&ms->h_src), 2 * kSrcSlot * sizeof(int32_t),
                        cudaHostAllocDefault));
  GB_CUDA(cudaHostAlloc(reinterpret_cast<void**>(&ms->h_ctl), 2 * sizeof(MsCtl),
                        cudaHostAllocDefault));
  GB_CUDA(cudaStreamCreateWithFlags(&ms->copy_stream, cudaStreamNonBlocking));
  GB_CUDA(cudaEventCreate(&ms->ev0));
  GB_CUDA(cudaEventCreate(&ms->ev1));
  // Every batch's graph clears visit, acc, the level-1 frontier buffers and
  // the control block before the kernel runs; the other frontier buffers are
  // cleared or written densely by the kernel itself.
  return GBBFS_OK;
}

// SMs a batch's grid spans on this handle.
int grid_sms(const gbbfs_graph* g) {
  const int share = g->ms ? g->ms->grid_sms : 0;
  return share > 0 && share < g->sms ? share : g->sms;
}

template <typename OffT, typename LaneT, typename DepthT>
int capture_batch(gbbfs_graph* g, int buf, int cls) {
  MsState* ms = g->ms;
  MsConfig cfg = ms->cfg;
  cfg.lanes = 32 << cls;
  const void* fn = kernel_for(g, cfg, (int)sizeof(DepthT));
  int per_sm = 0;
  GB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kThreads, 0));
  if (per_sm < 1) {
    ms_error = "multi-source kernel does not fit on an SM";
    return GBBFS_ERR_CUDA;
  }
  const int grid = per_sm * grid_sms(g);
  MsArgs<OffT, LaneT, DepthT> a;
  a.off = reinterpret_cast<const OffT*>(ms->roff);
  a.nbr = ms->rnbr;
  a.n = g->n;
  a.m = g->m;
  a.visit = reinterpret_cast<LaneT*>(ms->visit);
  a.fr0 = reinterpret_cast<LaneT*>(ms->fr[0]);
  a.fr1 = reinterpret_cast<LaneT*>(ms->fr[1]);
  a.acc = reinterpret_cast<LaneT*>(ms->acc);
  a.W = g->W;
  a.fbits0 = ms->fbits[0];
  a.fbits1 = ms->fbits[1];
  a.q0 = ms->q[0];
  a.q1 = ms->q[1];
  a.qe0 = ms->qe[0];
  a.qe1 = ms->qe[1];
  a.tq = ms->tq;
  a.hubs = ms->hubs;
  a.unit_tile = ms->unit_tile;
  a.nunits = ms->nunits;
  a.hub_chunk = ms->hub_chunk;
  a.nhubs = ms->nhubs;
  a.depth = reinterpret_cast<DepthT*>(ms->dtmp);
  a.dstride = ms->dstride;
  a.lvl = ms->lvl;
  a.lmask = reinterpret_cast<LaneT*>(ms->lmask);
  a.spill = ms->spill;
  a.tflag = ms->tflag;
  a.nsrc = ms->d_src[buf];
  a.sources = ms->d_src[buf] + 1;
  a.perm = ms->perm;
  a.ctl = ms->ctl[buf];
  a.shift = g->shift;
  a.alpha = std::max(1, cfg.alpha);
  a.limit_ns = 5ull * 1000 * 1000 * 1000;  // 5 s per barrier

  cudaStream_t s = g->stream;
  const size_t lane_bytes = sizeof(LaneT) * (size_t)g->n;
  GB_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  cudaError_t e = cudaMemcpyAsync(ms->d_src[buf], ms->h_src + kSrcSlot * buf,
                                  kSrcSlot * sizeof(int32_t), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(ms->visit, 0, lane_bytes, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(ms->fr[1], 0, lane_bytes, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(ms->acc, 0, lane_bytes, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(ms->lvl, 0xff, 4 * (size_t)g->n, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(ms->spill, 0, (size_t)g->n, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(ms->tflag, 0, 4 * (size_t)g->n, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(ms->fbits[1], 0, 4 * (size_t)g->W, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(ms->ctl[buf], 0, sizeof(MsCtl), s);
  if (e == cudaSuccess) {
    cudaLaunchConfig_t lc;
    memset(&lc, 0, sizeof lc);
    lc.gridDim = dim3(grid);
    lc.blockDim = dim3(kThreads);
    lc.dynamicSmemBytes = 0;
    lc.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    lc.attrs = attr;
    lc.numAttrs = 1;
    void* args[] = {&a};
    e = cudaLaunchKernelExC(&lc, fn, args);
  }
  if (e == cudaSuccess) {
    constexpr int64_t kTileV = kDecodeTile / (int64_t)sizeof(DepthT);
    const unsigned blocks = (unsigned)((g->n + kTileV - 1) / kTileV);
    k_depth_decode<LaneT, DepthT><<<blocks, kThreads, 0, s>>>(
        ms->lvl, reinterpret_cast<const LaneT*>(ms->lmask), ms->spill,
        reinterpret_cast<const LaneT*>(ms->visit), reinterpret_cast<const DepthT*>(ms->dtmp),
        ms->dstride, ms->perm, reinterpret_cast<DepthT*>(ms->depth[buf]), g->n, ms->d_src[buf]);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(ms->h_ctl + buf, ms->ctl[buf], sizeof(MsCtl), cudaMemcpyDeviceToHost, s);
  cudaGraph_t graph = nullptr;
  cudaError_t e2 = cudaStreamEndCapture(s, &graph);
  if (e == cudaSuccess) e = e2;
  if (e == cudaSuccess) {
    if (ms->exec[buf][cls]) cudaGraphExecDestroy(ms->exec[buf][cls]);
    ms->exec[buf][cls] = nullptr;
    e = cudaGraphInstantiate(&ms->exec[buf][cls], graph, 0);
  }
  if (graph) cudaGraphDestroy(graph);
  if (e != cudaSuccess) {
    ms_error = std::string("multi-source graph capture: ") + cudaGetErrorString(e);
    return GBBFS_ERR_CUDA;
  }
  ms->exec_cfg[buf][cls] = cfg;
  ms->exec_sms[buf][cls] = grid_sms(g);
  return GBBFS_OK;
}

template <typename OffT, typename LaneT>
int capture_depth(gbbfs_graph* g, int buf, int cls) {
  return g->ms->depth_bytes == 1 ? capture_batch<OffT, LaneT, uint8_t>(g, buf, cls)
                                 : capture_batch<OffT, LaneT, int32_t>(g, buf, cls);
}

template <typename OffT>
int capture_lanes(gbbfs_graph* g, int buf, int cls) {
  if (cls == 3) return capture_depth<OffT, Lane256>(g, buf, cls);
  if (cls == 2) return capture_depth<OffT, Lane128>(g, buf, cls);
  return cls == 0 ? capture_depth<OffT, uint32_t>(g, buf, cls)
                  : capture_depth<OffT, unsigned long long>(g, buf, cls);
}

bool same_cfg(const MsConfig& a, const MsConfig& b) {
  return a.lanes == b.lanes && a.batch == b.batch && a.alpha == b.alpha;
}

// Capture every (buffer, lane width) graph that is missing or was made for
// another configuration, all at once: a first batch of a new width then
// costs no capture (and its stream synchronize) in the middle of a run.
int capture_all(gbbfs_graph* g) {
  MsState* ms = g->ms;
  bool synced = false;
  for (int buf = 0; buf < 2; buf++)
    for (int cls = 0; (32 << cls) <= ms->cfg.lanes; cls++) {
      MsConfig want = ms->cfg;
      want.lanes = 32 << cls;
      if (ms->exec[buf][cls] && same_cfg(ms->exec_cfg[buf][cls], want) &&
          ms->exec_sms[buf][cls] == grid_sms(g))
        continue;
      if (!synced) {
        GB_CUDA(cudaStreamSynchronize(g->stream));
        synced = true;
      }
      GB_TRY(g->off32 ? capture_lanes<uint32_t>(g, buf, cls)
                      : capture_lanes<unsigned long long>(g, buf, cls));
    }
  return GBBFS_OK;
}

// Launch one batch (k <= lanes sources) into depth buffer `buf`.
int launch_batch(gbbfs_graph* g, int buf, const int32_t* sources, int k) {
  MsState* ms = g->ms;
  for (int i = 0; i < k; i++) {
    if (sources[i] < 0 || sources[i] >= g->n) {
      ms_error = "source out of range";
      return GBBFS_ERR_ARG;
    }
  }
  // The narrowest lane word that holds the batch (never wider than the
  // configured one): a small batch costs a 32-lane search.
  int cls = 0;
  while ((32 << cls) < k) cls++;
  MsConfig want = ms->cfg;
  want.lanes = 32 << cls;
  // The buffer's previous results must have left the device first.
  GB_CUDA(cudaStreamWaitEvent(g->stream, ms->copied[buf], 0));
  if (!ms->exec[buf][cls] || !same_cfg(ms->exec_cfg[buf][cls], want) ||
      ms->exec_sms[buf][cls] != grid_sms(g))
    GB_TRY(capture_all(g));
  // The host copy of the sources is read by the graph's first node; wait
  // until the previous launch that read this slot is done.
  GB_CUDA(cudaEventSynchronize(ms->computed[buf]));
  int32_t* slot = ms->h_src + kSrcSlot * buf;
  slot[0] = k;
  memcpy(slot + 1, sources, sizeof(int32_t) * k);
  GB_CUDA(cudaGraphLaunch(ms->exec[buf][cls], g->stream));
  GB_CUDA(cudaEventRecord(ms->computed[buf], g->stream));
  return GBBFS_OK;
}

// Levels and per-direction device time of finished batches.
struct MsTally {
  int levels = 0;
  int td_levels = 0, bu_levels = 0;
  double td_ms = 0, bu_ms = 0;
  double phase[kMsPhases] = {};
  double level_ms[32] = {}, level_f[32] = {}, level_e[32] = {};
  int level_bu[32] = {};
};

int check_batch(gbbfs_graph* g, int buf, MsTally* t) {
  MsState* ms = g->ms;
  GB_CUDA(cudaEventSynchronize(ms->computed[buf]));
  const MsCtl& c = ms->h_ctl[buf];
  if (c.error) {
    ms_error = c.error == GBBFS_ERR_TIMEOUT
                   ? "multi-source grid barrier timed out"
                   : "a depth exceeds the uint8 output range (use 4-byte depths)";
    return c.error;
  }
  if (t) {
    for (int p = 0; p < kMsPhases; p++) t->phase[p] += (double)c.phase_cycles[p];
    t->levels = std::max(t->levels, c.levels);
    for (int l = 1; l <= c.levels && l < kMsTimedLevels; l++) {
      const double ms_l = (double)(c.level_end[l] - c.level_end[l - 1]) * 1e-6;
      if (l < 32) {
        t->level_ms[l] += ms_l;
        t->level_f[l] += (double)c.level_f[l];
        t->level_e[l] += (double)c.level_e[l];
        t->level_bu[l] += c.level_bu[l];
      }
      if (c.level_bu[l]) {
        t->bu_ms += ms_l;
        t->bu_levels++;
      } else {
        t->td_ms += ms_l;
        t->td_levels++;
      }
    }
  }
  return GBBFS_OK;
}

// Batches of sources[0..k) back to back.  With host_out, the row of
// sources[j] goes to row row_of[j] of host_out (row j when row_of is null).
int run_batches(gbbfs_graph* g, const int32_t* sources, int64_t k, int depth_bytes,
                void* host_out, gbbfs_ms_stats* st, const int32_t* row_of = nullptr) {
  if (!g || !sources || k <= 0 || (depth_bytes != 1 && depth_bytes != 4)) {
    ms_error = "bad multi-source arguments";
    return GBBFS_ERR_ARG;
  }
  GB_CUDA(cudaSetDevice(g->device));
  GB_TRY(ensure_state(g, depth_bytes));
  MsState* ms = g->ms;
  const int lanes = ms->cfg.lanes;
  const int64_t nb = (k + lanes - 1) / lanes;
  if (!host_out && nb > 1) {
    ms_error = "results left on the device hold one batch only";
    return GBBFS_ERR_ARG;
  }
  const size_t per_src = (size_t)g->n * depth_bytes;
  MsTally tally;
  GB_CUDA(cudaEventRecord(ms->ev0, g->stream));
  for (int64_t b = 0; b < nb; b++) {
    const int buf = (int)(b & 1);
    const int kb = (int)std::min<int64_t>(lanes, k - b * lanes);
    GB_TRY(launch_batch(g, buf, sources + b * lanes, kb));
    if (host_out) {
      // Copy this batch out on the copy stream while the next one computes.
      GB_CUDA(cudaStreamWaitEvent(ms->copy_stream, ms->computed[buf], 0));
      char* out = static_cast<char*>(host_out);
      if (!row_of) {
        GB_CUDA(cudaMemcpyAsync(out + (size_t)b * lanes * per_src, ms->depth[buf],
                                (size_t)kb * per_src, cudaMemcpyDeviceToHost, ms->copy_stream));
      } else {
        for (int j = 0; j < kb; j++)
          GB_CUDA(cudaMemcpyAsync(out + (size_t)row_of[b * lanes + j] * per_src,
                                  static_cast<const char*>(ms->depth[buf]) + (size_t)j * per_src,
                                  per_src, cudaMemcpyDeviceToHost, ms->copy_stream));
      }
      GB_CUDA(cudaEventRecord(ms->copied[buf], ms->copy_stream));
    }
    if (b >= 1) GB_TRY(check_batch(g, buf ^ 1, &tally));
    ms->last_buf = buf;
    ms->last_k = kb;
  }
  GB_CUDA(cudaEventRecord(ms->ev1, g->stream));
  GB_TRY(check_batch(g, ms->last_buf, &tally));
  GB_CUDA(cudaStreamSynchronize(ms->copy_stream));
  GB_CUDA(cudaStreamSynchronize(g->stream));
  if (st) {
    float ms_elapsed = 0;
    GB_CUDA(cudaEventElapsedTime(&ms_elapsed, ms->ev0, ms->ev1));
    st->device_ms = ms_elapsed;
    st->batches = (int32_t)nb;
    st->levels = tally.levels;
    st->lanes = lanes;
    st->batch = ms->cfg.batch;
    st->alpha = ms->cfg.alpha;
    st->td_levels = tally.td_levels;
    st->bu_levels = tally.bu_levels;
    st->td_ms = tally.td_ms;
    st->bu_ms = tally.bu_ms;
    double total = 0;
    for (int p = 0; p < kMsPhases; p++) total += tally.phase[p];
    for (int p = 0; p < kMsPhases && p < 8; p++)
      st->phase_share[p] = total > 0 ? tally.phase[p] / total : 0.0;
    for (int l = 0; l < 32; l++) {
      st->level_ms[l] = tally.level_ms[l];
      st->level_frontier[l] = tally.level_f[l];
      st->level_edges[l] = tally.level_e[l];
      st->level_bu[l] = tally.level_bu[l];
    }
  }
  return GBBFS_OK;
}

}  // namespace

int ms_prepare(gbbfs_graph* g, int depth_bytes) {
  GB_CUDA(cudaSetDevice(g->device));
  GB_TRY(ensure_state(g, depth_bytes));
  return capture_all(g);
}

int ms_lanes(const gbbfs_graph* g) { return g->ms ? g->ms->cfg.lanes : MsConfig().lanes; }

int ms_set_grid_sms(gbbfs_graph* g, int sms) {
  if (!g->ms) return GBBFS_ERR_STATE;
  g->ms->grid_sms = sms < 0 ? 0 : sms;   // graphs are recaptured on the next launch
  return GBBFS_OK;
}

int ms_launch(gbbfs_graph* g, int buf, const int32_t* sources, int k) {
  if (!g->ms || k < 1 || k > g->ms->cfg.lanes) return GBBFS_ERR_STATE;
  return launch_batch(g, buf, sources, k);
}

bool ms_ready(gbbfs_graph* g, int buf) {
  return cudaEventQuery(g->ms->computed[buf]) != cudaErrorNotReady;
}

int ms_finish(gbbfs_graph* g, int buf) {
  return check_batch(g, buf, nullptr);
}

void* ms_depth(gbbfs_graph* g, int buf) { return g->ms->depth[buf]; }

double ms_kernel_ms(const gbbfs_graph* g, int buf) {
  const MsCtl& c = g->ms->h_ctl[buf];
  return c.t_end > c.t_begin ? (double)(c.t_end - c.t_begin) * 1e-6 : 0.0;
}

void ms_kernel_stamps(const gbbfs_graph* g, int buf, uint64_t* begin_ns, uint64_t* end_ns) {
  const MsCtl& c = g->ms->h_ctl[buf];
  *begin_ns = c.t_begin;
  *end_ns = c.t_end;
}

cudaEvent_t ms_done_event(gbbfs_graph* g, int buf) { return g->ms->computed[buf]; }

void ms_mark_copied(gbbfs_graph* g, int buf, cudaStream_t s) {
  cudaEventRecord(g->ms->copied[buf], s);
}

int ms_order(gbbfs_graph* g, const int32_t* sources, int64_t k, int32_t* order) {
  for (int64_t i = 0; i < k; i++) {
    if (sources[i] < 0 || sources[i] >= g->n) {
      ms_error = "source out of range";
      return GBBFS_ERR_ARG;
    }
  }
  if ((int64_t)g->batch_key.size() != g->n) {
    GB_CUDA(cudaSetDevice(g->device));
    GB_TRY(g->off32 ? make_batch_keys<uint32_t>(g) : make_batch_keys<unsigned long long>(g));
  }
  for (int64_t i = 0; i < k; i++) order[i] = (int32_t)i;
  const uint16_t* key = g->batch_key.data();
  std::stable_sort(order, order + k,
                   [&](int32_t a, int32_t b) { return key[sources[a]] < key[sources[b]]; });
  return GBBFS_OK;
}

}  // namespace gbbfs

using namespace gbbfs;

extern "C" {

int gbbfs_msbfs(gbbfs_graph* g, const int32_t* sources, int64_t k, int depth_bytes,
                void* depth_out, gbbfs_ms_stats* st) {
  if (!g || !sources || !depth_out || k <= 0) return GBBFS_ERR_ARG;
  if (k <= ms_lanes(g)) return run_batches(g, sources, k, depth_bytes, depth_out, st);
  // Several batches: batch the sources in gbbfs_msbfs_order's order; each row
  // is copied to its caller's position.
  std::vector<int32_t> order((size_t)k), batched((size_t)k);
  GB_TRY(ms_order(g, sources, k, order.data()));
  for (int64_t j = 0; j < k; j++) batched[j] = sources[order[j]];
  return run_batches(g, batched.data(), k, depth_bytes, depth_out, st, order.data());
}

int gbbfs_msbfs_order(gbbfs_graph* g, const int32_t* sources, int64_t k, int32_t* order_out) {
  if (!g || k < 0 || (k > 0 && (!sources || !order_out))) return GBBFS_ERR_ARG;
  return ms_order(g, sources, k, order_out);
}

int gbbfs_msbfs_device(gbbfs_graph* g, const int32_t* sources, int64_t k, int depth_bytes,
                       const void** depth_dev, gbbfs_ms_stats* st) {
  if (!g) return GBBFS_ERR_ARG;
  int rc = run_batches(g, sources, k, depth_bytes, nullptr, st);
  if (rc != GBBFS_OK) return rc;
  if (depth_dev) *depth_dev = g->ms->depth[g->ms->last_buf];
  return GBBFS_OK;
}

int gbbfs_msbfs_set_config(gbbfs_graph* g, const gbbfs_ms_config* cfg) {
  if (!g || !cfg) return GBBFS_ERR_ARG;
  if ((cfg->lanes != 32 && cfg->lanes != 64 && cfg->lanes != 128 && cfg->lanes != 256) ||
      (cfg->batch != 4 && cfg->batch != 8 && cfg->batch != 16) || cfg->alpha < 1) {
    last_error() = "lanes must be 32, 64, 128 or 256, batch 4, 8 or 16, alpha >= 1";
    return GBBFS_ERR_ARG;
  }
  GB_CUDA(cudaSetDevice(g->device));
  if (!g->ms) {
    // keep the choice until the first batch allocates the state
    GB_TRY(ensure_state(g, 1));
  }
  g->ms->cfg.lanes = cfg->lanes;
  g->ms->cfg.batch = cfg->batch;
  g->ms->cfg.alpha = cfg->alpha;
  return GBBFS_OK;
}

int gbbfs_msbfs_get_config(const gbbfs_graph* g, gbbfs_ms_config* cfg) {
  if (!g || !cfg) return GBBFS_ERR_ARG;
  MsConfig d;
  const MsConfig& c = g->ms ? g->ms->cfg : d;
  cfg->lanes = c.lanes;
  cfg->batch = c.batch;
  cfg->alpha = c.alpha;
  return GBBFS_OK;
}

int64_t gbbfs_msbfs_state_bytes(int64_t n, int64_t m_dir, int depth_bytes) {
  if (n < 0 || m_dir < 0 || (depth_bytes != 1 && depth_bytes != 4)) return -1;
  return (int64_t)gbbfs::ms_state_bytes(n, m_dir, (n + 31) / 32, depth_bytes);
}

int gbbfs_msbfs_autotune(gbbfs_graph* g, const int32_t* sample, int64_t k, int depth_bytes,
                         gbbfs_ms_config* best) {
  if (!g || !sample || k <= 0) return GBBFS_ERR_ARG;
  // Time batches formed the way gbbfs_msbfs forms them.
  std::vector<int32_t> order((size_t)k), ordered((size_t)k);
  GB_TRY(ms_order(g, sample, k, order.data()));
  for (int64_t j = 0; j < k; j++) ordered[j] = sample[order[j]];
  sample = ordered.data();
  static const int kLanes[] = {32, 64, 128, 256};
  static const int kBatches[] = {4, 8, 16};
  static const int kAlphas[] = {2, 6, 15, 40, 200};
  // The same queries for every width: up to two batches of the widest word
  // (whole batches of every width), so one slow batch does not decide.
  int64_t base = std::min<int64_t>(k, 2 * kMsMaxLanes);
  if (base >= kMsMaxLanes) base -= base % kMsMaxLanes;
  double best_t = 1e300;
  gbbfs_ms_config pick = {64, 8, 15};
  for (int lanes : kLanes)
    for (int batch : kBatches)
      for (int alpha : kAlphas) {
        gbbfs_ms_config c = {lanes, batch, alpha};
        GB_TRY(gbbfs_msbfs_set_config(g, &c));
        const int64_t total = base >= lanes ? base / lanes * lanes : base;
        gbbfs_ms_stats st;
        GB_TRY(run_batches(g, sample, std::min<int64_t>(total, lanes), depth_bytes, nullptr,
                           &st));   // warm
        double ms = 0;
        for (int64_t b = 0; b < total; b += lanes) {
          GB_TRY(run_batches(g, sample + b, std::min<int64_t>(lanes, total - b), depth_bytes,
                             nullptr, &st));
          ms += st.device_ms;
        }
        const double per_query = ms / (double)total;
        if (per_query < best_t) {
          best_t = per_query;
          pick = c;
        }
      }
  GB_TRY(gbbfs_msbfs_set_config(g, &pick));
  if (best) *best = pick;
  return GBBFS_OK;
}

}  // extern "C"
