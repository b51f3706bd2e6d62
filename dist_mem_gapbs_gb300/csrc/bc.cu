// Betweenness centrality on the GPU: BC's BFS phase (src/bc.cc:55-102;
// gapbs-verify/bc.cc:51-92) and, for gbbfs_bc, Brandes' back-propagation and
// normalization (src/bc.cc:106-171).
//
// Brandes' betweenness centrality first runs, from each source, a
// level-synchronous BFS that records for every vertex its depth and its
// number of shortest paths from the source (path_counts), and for every
// directed edge whether it leads one level down (the successor bitmap the
// back-propagation phase reads).  Unlike DOBFS it visits every edge of every
// level, so this is top-down only.
//
// One kernel per level.  The level's frontier is a slice of the queue; a scan
// of its vertices' degrees gives each one's first edge in the concatenated
// adjacency, and warps take spans of consecutive edges of it (a 32-entry
// window of frontier vertices per warp maps an edge to its tail, as the
// batched search's top-down step does).  Per edge (u, v) at CSR position e:
// a vertex still at depth -1 is claimed with atomicCAS and queued; when v's
// depth is then the level's, e's successor bit is set (one atomicOr per
// bitmap word a warp touches) and path_counts[u] is added to path_counts[v]
// (64-bit atomicAdd, wrapping like the reference's unsigned long long adds).
// u's count is final: all of its in-edges lie in the level before.  Results
// equal the serial restatement exactly; only the order of vertices inside a
// level depends on timing, as in the reference.
//
// Back-propagation walks the levels from the deepest up (a thread per vertex
// of small degree, a warp per larger one, a block per hub):
// a vertex's dependency sums path_counts[u] / path_counts[v] * (1 + delta[v])
// over its successor edges (terms in double, as the DMM code computes them,
// summed in a fixed order), and is added to its score.  Scores are divided by
// their maximum at the end.

#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <vector>

#include "engine.h"
#include "scan.cuh"

namespace gbbfs {

struct BcState {
  int64_t n = 0, m = 0;
  float* delta = nullptr;    // dependency of the current source (Brandes)
  float* score = nullptr;    // scores summed over the sources
  unsigned long long* sigma = nullptr;
  int32_t* depth = nullptr;
  uint32_t* succ = nullptr;
  int32_t* queue = nullptr;
  int32_t* degs = nullptr;
  int64_t* epre = nullptr;
  unsigned long long* tail = nullptr;
};

void bc_release(BcState* b) {
  if (!b) return;
  cudaFree(b->sigma);
  cudaFree(b->depth);
  cudaFree(b->succ);
  cudaFree(b->queue);
  cudaFree(b->degs);
  cudaFree(b->epre);
  cudaFree(b->tail);
  cudaFree(b->delta);
  cudaFree(b->score);
  delete b;
}

namespace {

constexpr int kBcSpan = 2048;   // edges per warp span at most

template <typename OffT>
__global__ void k_bc_degs(const OffT* off, const int32_t* frontier, int64_t count, int32_t* degs) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t u = frontier[i];
    degs[i] = (int32_t)(off[u + 1] - off[u]);
  }
}

template <typename OffT>
__global__ void __launch_bounds__(kThreads) k_bc_expand(
    const OffT* off, const int32_t* nbr, const int32_t* frontier, int64_t F,
    const int64_t* epre, uint64_t E, uint64_t span, int level, int32_t* depth,
    unsigned long long* sigma, uint32_t* succ, int32_t* next, unsigned long long* tail) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int64_t nspans = (int64_t)((E + span - 1) / span);
  for (int64_t sp = warp; sp < nspans; sp += nwarps) {
    const uint64_t e_lo = (uint64_t)sp * span;
    const uint64_t e_hi = e_lo + span < E ? e_lo + span : E;
    int64_t lo = 0, hi = F - 1;
    while (lo < hi) {
      const int64_t mid = (lo + hi + 1) >> 1;
      if ((uint64_t)epre[mid] <= e_lo) lo = mid; else hi = mid - 1;
    }
    int64_t base = lo;
    uint64_t pre = ~0ull, ob = 0;
    unsigned long long su = 0;
    auto load_entry = [&](int64_t j) {
      if (j < F) {
        pre = (uint64_t)epre[j];
        const int32_t u = frontier[j];
        ob = (uint64_t)off[u];
        su = sigma[u];
      } else {
        pre = ~0ull;
        ob = 0;
        su = 0;
      }
    };
    load_entry(base + lane);
    for (uint64_t e0 = e_lo; e0 < e_hi; e0 += 32) {
      // slide so that the window's first entry holds edge e0
      for (;;) {
        const unsigned le = __ballot_sync(kFull, pre <= e0);
        const int s = 31 - __clz(le);
        if (s <= 0) break;
        const int src = lane + s;
        const uint64_t pre2 = shfl(pre, src & 31), ob2 = shfl(ob, src & 31);
        const unsigned long long su2 = shfl(su, src & 31);
        if (src < 32) {
          pre = pre2;
          ob = ob2;
          su = su2;
        } else {
          load_entry(base + src);
        }
        base += s;
      }
      const uint64_t e = e0 + lane;
      int seg = 0;
#pragma unroll
      for (int step = 16; step; step >>= 1)
        if (shfl(pre, seg + step) <= e) seg += step;
      const uint64_t pre_s = shfl(pre, seg), ob_s = shfl(ob, seg);
      const unsigned long long su_s = shfl(su, seg);
      bool claimed = false, down = false;
      int32_t v = 0;
      uint64_t eidx = 0;
      if (e < e_hi) {
        eidx = ob_s + (e - pre_s);
        v = __ldcs(nbr + eidx);
        int32_t d = __ldcg(depth + v);
        if (d == -1) {
          d = atomicCAS(depth + v, -1, level);
          claimed = d == -1;
          if (claimed) d = level;
        }
        down = d == level;
        if (down) atomicAdd(sigma + v, su_s);
      }
      // queue the claimed vertices: one atomic per warp
      const unsigned cm = __ballot_sync(kFull, claimed);
      if (cm) {
        unsigned long long at = 0;
        if (lane == 0) at = atomicAdd(tail, (unsigned long long)__popc(cm));
        at = shfl(at, 0);
        if (claimed) next[at + __popc(cm & ((1u << lane) - 1))] = v;
      }
      // successor bits: lanes of one bitmap word OR together first
      const unsigned long long wkey = down ? (eidx >> 5) : ~0ull;
      const unsigned grp = __match_any_sync(kFull, wkey);
      const uint32_t bits = __reduce_or_sync(grp, down ? 1u << (eidx & 31) : 0u);
      if (down && lane == __ffs(grp) - 1) atomicOr(succ + (eidx >> 5), bits);
    }
  }
}

// Dependencies of one level (src/bc.cc:129-152, gapbs-verify/bc.cc:128-141):
// for u in the level, delta[u] = sum over u's successor edges (u, v) of
// path_counts[u] / path_counts[v] * (1 + delta[v]), added to u's score.
// Terms in double, summed in a fixed order.  Vertices of degree up to
// kBcBackSmall take a thread each (k_bc_back_small, edges in order); larger
// ones a warp each (k_bc_back, lane-strided, then a fixed shuffle tree), and
// those above kBcBackHub a block each (k_bc_back_hub).
constexpr int kBcBackSmall = 32;
constexpr int kBcBackHub = 2048;   // above this degree a block per vertex

template <typename OffT>
__global__ void __launch_bounds__(kThreads) k_bc_back_small(const OffT* off, const int32_t* nbr,
                                                            const uint32_t* succ,
                                                            const unsigned long long* sigma,
                                                            const int32_t* level, int64_t count,
                                                            float* delta, float* score) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t u = level[i];
    const uint64_t b = (uint64_t)off[u], e = (uint64_t)off[u + 1];
    if (e - b > (uint64_t)kBcBackSmall) continue;
    const double su = (double)sigma[u];
    double sum = 0.0;
    for (uint64_t j = b; j < e; j++) {
      if ((__ldg(succ + (j >> 5)) >> (j & 31)) & 1u) {
        const int32_t v = nbr[j];
        sum += su / (double)sigma[v] * (1.0 + (double)delta[v]);
      }
    }
    delta[u] = (float)sum;
    score[u] += (float)sum;
  }
}

template <typename OffT>
__global__ void __launch_bounds__(kThreads) k_bc_back(const OffT* off, const int32_t* nbr,
                                                      const uint32_t* succ,
                                                      const unsigned long long* sigma,
                                                      const int32_t* level, int64_t count,
                                                      float* delta, float* score) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t i = warp; i < count; i += nwarps) {
    const int32_t u = level[i];
    const uint64_t b = (uint64_t)off[u], e = (uint64_t)off[u + 1];
    if (e - b <= (uint64_t)kBcBackSmall || e - b > (uint64_t)kBcBackHub) continue;
    const double su = (double)sigma[u];
    double sum = 0.0;
    for (uint64_t j = b + lane; j < e; j += 32) {
      if ((__ldg(succ + (j >> 5)) >> (j & 31)) & 1u) {
        const int32_t v = nbr[j];
        sum += su / (double)sigma[v] * (1.0 + (double)delta[v]);
      }
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) sum += __shfl_xor_sync(kFull, sum, o);
    if (lane == 0) {
      delta[u] = (float)sum;
      score[u] += (float)sum;
    }
  }
}

// Vertices above kBcBackHub: a block each, thread-strided over the edges,
// then a fixed-order tree over the block.
template <typename OffT>
__global__ void __launch_bounds__(kThreads) k_bc_back_hub(const OffT* off, const int32_t* nbr,
                                                          const uint32_t* succ,
                                                          const unsigned long long* sigma,
                                                          const int32_t* level, int64_t count,
                                                          float* delta, float* score) {
  __shared__ double part[kThreads];
  for (int64_t i = blockIdx.x; i < count; i += gridDim.x) {
    const int32_t u = level[i];
    const uint64_t b = (uint64_t)off[u], e = (uint64_t)off[u + 1];
    if (e - b <= (uint64_t)kBcBackHub) continue;   // block-uniform
    const double su = (double)sigma[u];
    double sum = 0.0;
    for (uint64_t j = b + threadIdx.x; j < e; j += blockDim.x) {
      if ((__ldg(succ + (j >> 5)) >> (j & 31)) & 1u) {
        const int32_t v = nbr[j];
        sum += su / (double)sigma[v] * (1.0 + (double)delta[v]);
      }
    }
    part[threadIdx.x] = sum;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
      if ((int)threadIdx.x < w) part[threadIdx.x] += part[threadIdx.x + w];
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      delta[u] = (float)part[0];
      score[u] += (float)part[0];
    }
    __syncthreads();
  }
}

__global__ void k_max_f(const float* x, int64_t n, unsigned int* out_bits) {
  float mx = 0.0f;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    mx = fmaxf(mx, x[i]);
#pragma unroll
  for (int o = 16; o; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(kFull, mx, o));
  // scores are >= 0, so their bit patterns order like the values
  if ((threadIdx.x & 31) == 0) atomicMax(out_bits, __float_as_uint(mx));
}

__global__ void k_scale_f(float* x, int64_t n, const unsigned int* max_bits) {
  const float mx = __uint_as_float(*max_bits);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    x[i] = x[i] / mx;
}

int ensure_bc(gbbfs_graph* g) {
  if (g->bc) return GBBFS_OK;
  BcState* b = new BcState();
  b->n = g->n;
  b->m = g->m;
  const size_t n = (size_t)g->n;
  const size_t words = (size_t)((g->m + 31) / 32) + 1;
  cudaError_t e = cudaMalloc(&b->sigma, 8 * n);
  if (e == cudaSuccess) e = cudaMalloc(&b->depth, 4 * n);
  if (e == cudaSuccess) e = cudaMalloc(&b->succ, 4 * words);
  if (e == cudaSuccess) e = cudaMalloc(&b->queue, 4 * (n + 1));
  if (e == cudaSuccess) e = cudaMalloc(&b->degs, 4 * (n + 1));
  if (e == cudaSuccess) e = cudaMalloc(&b->epre, 8 * (n + 2));
  if (e == cudaSuccess) e = cudaMalloc(&b->tail, 8);
  if (e == cudaSuccess) e = cudaMalloc(&b->delta, 4 * n);
  if (e == cudaSuccess) e = cudaMalloc(&b->score, 4 * n);
  if (e != cudaSuccess) {
    bc_release(b);
    last_error() = std::string("BC state: ") + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? GBBFS_ERR_NOMEM : GBBFS_ERR_CUDA;
  }
  g->bc = b;
  g->device_bytes += (int64_t)(8 * n + 4 * n + 4 * words + 8 * (n + 1) + 8 * (n + 2) + 8 + 8 * n);
  return GBBFS_OK;
}

template <typename OffT>
int run_bc(gbbfs_graph* g, int32_t source, std::vector<int64_t>* starts) {
  BcState* b = g->bc;
  cudaStream_t s = g->stream;
  const OffT* off = reinterpret_cast<const OffT*>(g->off);
  const size_t n = (size_t)g->n;
  GB_CUDA(cudaMemsetAsync(b->depth, 0xff, 4 * n, s));
  GB_CUDA(cudaMemsetAsync(b->sigma, 0, 8 * n, s));
  GB_CUDA(cudaMemsetAsync(b->succ, 0, 4 * (size_t)((g->m + 31) / 32 + 1), s));
  const int32_t zero = 0;
  const unsigned long long one = 1;
  GB_CUDA(cudaMemcpyAsync(b->depth + source, &zero, 4, cudaMemcpyHostToDevice, s));
  GB_CUDA(cudaMemcpyAsync(b->sigma + source, &one, 8, cudaMemcpyHostToDevice, s));
  GB_CUDA(cudaMemcpyAsync(b->queue, &source, 4, cudaMemcpyHostToDevice, s));
  GB_CUDA(cudaMemcpyAsync(b->tail, &one, 8, cudaMemcpyHostToDevice, s));
  GB_CUDA(cudaStreamSynchronize(s));
  starts->assign(1, 0);
  int64_t qs = 0, qe = 1;
  const int64_t nwarps = (int64_t)g->sms * 8 * (kThreads / 32);
  for (int level = 1; qs < qe; level++) {
    const int64_t F = qe - qs;
    k_bc_degs<OffT><<<g->sms * 8, kThreads, 0, s>>>(off, b->queue + qs, F, b->degs);
    GB_CUDA(cudaGetLastError());
    GB_TRY(device_scan<int32_t>(b->degs, F, b->epre, true, s));
    int64_t E = 0;
    GB_CUDA(cudaMemcpy(&E, b->epre + F, 8, cudaMemcpyDeviceToHost));
    if (E > 0) {
      uint64_t span = ((uint64_t)E + nwarps - 1) / nwarps;
      span = span < 32 ? 32 : span > (uint64_t)kBcSpan ? kBcSpan : (span + 31) & ~31ull;
      k_bc_expand<OffT><<<g->sms * 8, kThreads, 0, s>>>(
          off, g->nbr, b->queue + qs, F, b->epre, (uint64_t)E, span, level, b->depth, b->sigma,
          b->succ, b->queue, b->tail);
      GB_CUDA(cudaGetLastError());
    }
    unsigned long long t = 0;
    GB_CUDA(cudaMemcpyAsync(&t, b->tail, 8, cudaMemcpyDeviceToHost, s));
    GB_CUDA(cudaStreamSynchronize(s));
    starts->push_back(qe);
    qs = qe;
    qe = (int64_t)t;
  }
  return GBBFS_OK;
}

template <typename OffT>
int run_brandes(gbbfs_graph* g, const int32_t* sources, int64_t k) {
  BcState* b = g->bc;
  cudaStream_t s = g->stream;
  const OffT* off = reinterpret_cast<const OffT*>(g->off);
  GB_CUDA(cudaMemsetAsync(b->score, 0, 4 * (size_t)g->n, s));
  std::vector<int64_t> starts;
  for (int64_t i = 0; i < k; i++) {
    GB_TRY(run_bc<OffT>(g, sources[i], &starts));
    GB_CUDA(cudaMemsetAsync(b->delta, 0, 4 * (size_t)g->n, s));
    for (int64_t d = (int64_t)starts.size() - 2; d >= 0; d--) {
      const int64_t count = starts[d + 1] - starts[d];
      k_bc_back_small<OffT><<<g->sms * 8, kThreads, 0, s>>>(off, g->nbr, b->succ, b->sigma,
                                                             b->queue + starts[d], count,
                                                             b->delta, b->score);
      k_bc_back<OffT><<<g->sms * 8, kThreads, 0, s>>>(off, g->nbr, b->succ, b->sigma,
                                                       b->queue + starts[d], count, b->delta,
                                                       b->score);
      k_bc_back_hub<OffT><<<g->sms * 8, kThreads, 0, s>>>(off, g->nbr, b->succ, b->sigma,
                                                           b->queue + starts[d], count, b->delta,
                                                           b->score);
      GB_CUDA(cudaGetLastError());
    }
  }
  // scores / their maximum (src/bc.cc:160-167)
  GB_CUDA(cudaMemsetAsync(b->tail, 0, 8, s));
  unsigned int* mx = reinterpret_cast<unsigned int*>(b->tail);
  k_max_f<<<g->sms * 8, kThreads, 0, s>>>(b->score, g->n, mx);
  k_scale_f<<<g->sms * 8, kThreads, 0, s>>>(b->score, g->n, mx);
  GB_CUDA(cudaGetLastError());
  GB_CUDA(cudaStreamSynchronize(s));
  return GBBFS_OK;
}

}  // namespace
}  // namespace gbbfs

extern "C" {

int gbbfs_bc(gbbfs_graph* g, const int32_t* sources, int64_t k, float* scores_out) {
  if (!g || k < 1 || !sources) return GBBFS_ERR_ARG;
  for (int64_t i = 0; i < k; i++)
    if (sources[i] < 0 || sources[i] >= g->n) {
      gbbfs::last_error() = "source out of range";
      return GBBFS_ERR_ARG;
    }
  GB_CUDA(cudaSetDevice(g->device));
  GB_TRY(gbbfs::ensure_bc(g));
  GB_TRY(g->off32 ? gbbfs::run_brandes<uint32_t>(g, sources, k)
                  : gbbfs::run_brandes<unsigned long long>(g, sources, k));
  if (scores_out)
    GB_CUDA(cudaMemcpy(scores_out, g->bc->score, 4 * (size_t)g->n, cudaMemcpyDeviceToHost));
  return GBBFS_OK;
}


int gbbfs_bc_bfs(gbbfs_graph* g, int32_t source, uint64_t* path_counts, int32_t* depth,
                 uint32_t* succ, int32_t* order, int64_t* level_start, int32_t* levels) {
  if (!g) return GBBFS_ERR_ARG;
  if (source < 0 || source >= g->n) {
    gbbfs::last_error() = "source out of range";
    return GBBFS_ERR_ARG;
  }
  GB_CUDA(cudaSetDevice(g->device));
  GB_TRY(gbbfs::ensure_bc(g));
  std::vector<int64_t> starts;
  GB_TRY(g->off32 ? gbbfs::run_bc<uint32_t>(g, source, &starts)
                  : gbbfs::run_bc<unsigned long long>(g, source, &starts));
  gbbfs::BcState* b = g->bc;
  const size_t n = (size_t)g->n;
  const int64_t reached = starts.back();
  if (path_counts)
    GB_CUDA(cudaMemcpy(path_counts, b->sigma, 8 * n, cudaMemcpyDeviceToHost));
  if (depth) GB_CUDA(cudaMemcpy(depth, b->depth, 4 * n, cudaMemcpyDeviceToHost));
  if (succ)
    GB_CUDA(cudaMemcpy(succ, b->succ, 4 * (size_t)((g->m + 31) / 32), cudaMemcpyDeviceToHost));
  if (order) GB_CUDA(cudaMemcpy(order, b->queue, 4 * (size_t)reached, cudaMemcpyDeviceToHost));
  if (level_start) std::copy(starts.begin(), starts.end(), level_start);
  if (levels) *levels = (int32_t)starts.size() - 1;
  return GBBFS_OK;
}

}  // extern "C"
