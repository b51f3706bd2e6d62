// Host side of the GB300 BFS engine and its C ABI (include/gbbfs.h).
//
// gbbfs_graph holds the device CSR and the per-search state.  A search runs
// the DOBFS control loop of the reference (src/bfs.cc:142-188,
// gapbs-verify/bfs.cc:122-173) on the device: k_decide applies the same
// alpha/beta tests on the same int64 counters after every step, so the step
// sequence and its counts equal the reference's.
//
// Two drivers share those kernels:
//  * graph mode (default): one CUDA graph per handle —
//      init -> while(loop) { decide -> switch(sel) { td | q2b | bu0 | bu1 | b2q } }
//           -> copy of the state header back to pinned host memory
//    so a whole search is one cudaGraphLaunch with no host round trip;
//  * stepped mode: the host launches decide, reads the decision, launches the
//    chosen kernel between two CUDA events.  It gives per-kernel event times.

#include <cuda_runtime.h>

#include <algorithm>
#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "bfs_kernels.cuh"
#include "engine.h"
#include "msbfs_kernels.cuh"
#include "gbbfs.h"

using namespace gbbfs;

namespace {

#define g_last_error (::gbbfs::last_error())

int bit_length(uint64_t x) {
  int b = 0;
  while (x) {
    b++;
    x >>= 1;
  }
  return b;
}

constexpr size_t kParamBytes = offsetof(DevState, edges_to_check);
constexpr size_t kHeaderBytes = offsetof(DevState, trace);
constexpr size_t kReadbackBytes = kHeaderBytes + kTraceInline * sizeof(DevStep);

}  // namespace

namespace {

void release(gbbfs_graph* g) {
  if (!g) return;
  if (g->device >= 0) cudaSetDevice(g->device);
  if (g->stream) cudaStreamSynchronize(g->stream);
  msbfs_release(g->ms);
  g->ms = nullptr;
  bc_release(g->bc);
  g->bc = nullptr;
  if (g->copy_stream) cudaStreamSynchronize(g->copy_stream);
  for (int i = 0; i < 2; i++) {
    cudaFree(g->stage[i]);
    if (g->staged[i]) cudaEventDestroy(g->staged[i]);
    if (g->copied[i]) cudaEventDestroy(g->copied[i]);
  }
  if (g->copy_stream) cudaStreamDestroy(g->copy_stream);
  if (g->h_slot) cudaFreeHost(g->h_slot);
  if (g->exec) cudaGraphExecDestroy(g->exec);
  if (g->graph) cudaGraphDestroy(g->graph);
  cudaFree(g->off);
  cudaFree(g->nbr);
  cudaFree(g->head);
  cudaFree(g->iso);
  cudaFree(g->visited);
  cudaFree(g->bm[0]);
  cudaFree(g->bm[1]);
  cudaFree(g->parent);
  cudaFree(g->depth);
  cudaFree(g->qv[0]);
  cudaFree(g->qv[1]);
  cudaFree(g->qs[0]);
  cudaFree(g->qs[1]);
  cudaFree(g->ctr);
  cudaFree(g->st);
  if (g->h_st) cudaFreeHost(g->h_st);
  for (cudaEvent_t e : g->step_ev) cudaEventDestroy(e);
  if (g->ev_begin) cudaEventDestroy(g->ev_begin);
  if (g->ev_end) cudaEventDestroy(g->ev_end);
  if (g->stream) cudaStreamDestroy(g->stream);
  delete g;
}

template <typename T>
int dev_alloc(gbbfs_graph* g, T** p, size_t count) {
  size_t bytes = std::max<size_t>(count * sizeof(T), 256);
  cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), bytes);
  if (e != cudaSuccess) {
    g_last_error = std::string("cudaMalloc: ") + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? GBBFS_ERR_NOMEM : GBBFS_ERR_CUDA;
  }
  g->device_bytes += (int64_t)bytes;
  return GBBFS_OK;
}

template <typename OffT>
Bufs<OffT> bufs(const gbbfs_graph* g) {
  Bufs<OffT> b;
  b.off = reinterpret_cast<const OffT*>(g->off);
  b.nbr = g->nbr;
  b.head = g->head;
  b.iso = g->iso;
  b.visited = g->visited;
  b.bm0 = g->bm[0];
  b.bm1 = g->bm[1];
  b.depth = g->depth;
  b.qv0 = g->qv[0];
  b.qv1 = g->qv[1];
  b.qs0 = reinterpret_cast<OffT*>(g->qs[0]);
  b.qs1 = reinterpret_cast<OffT*>(g->qs[1]);
  b.ctr = g->ctr;
  b.st = g->st;
  b.n = g->n;
  b.m = g->m;
  b.W = g->W;
  b.shift = g->shift;
  return b;
}

// The sweep after a bitmap top-down step: the shared-memory tile version for
// 32-bit offsets, the per-vertex-load version otherwise.
template <typename OffT>
const void* sweep_kernel() {
  if constexpr (sizeof(OffT) == 4) return (const void*)k_sweep<OffT>;
  else return (const void*)k_b2q<OffT, true>;
}

int occupancy_grid(const void* fn, int sms, int* grid) {
  int per_sm = 0;
  GB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kThreads, 0));
  *grid = std::max(1, per_sm) * sms;
  return GBBFS_OK;
}

template <typename OffT>
int setup_grids(gbbfs_graph* g) {
  GB_TRY(occupancy_grid((const void*)k_init<OffT>, g->sms, &g->grid_init));
  GB_TRY(occupancy_grid((const void*)k_td<OffT>, g->sms, &g->grid_td));
  GB_TRY(occupancy_grid((const void*)k_bu<OffT, 0>, g->sms, &g->grid_bu));
  GB_TRY(occupancy_grid((const void*)k_q2b<OffT>, g->sms, &g->grid_q2b));
  GB_TRY(occupancy_grid((const void*)k_b2q<OffT, false>, g->sms, &g->grid_b2q));
  GB_TRY(occupancy_grid((const void*)k_tdb<OffT>, g->sms, &g->grid_tdb));
  GB_TRY(occupancy_grid(sweep_kernel<OffT>(), g->sms, &g->grid_sweep));
  return GBBFS_OK;
}

template <typename OffT>
int upload(gbbfs_graph* g, const int64_t* offsets, const int32_t* neigh) {
  // Offsets go up as int64 and are narrowed on the device when they fit.
  int64_t* tmp = nullptr;
  GB_CUDA(cudaMalloc(&tmp, sizeof(int64_t) * (g->n + 1)));
  cudaError_t e = cudaMemcpyAsync(tmp, offsets, sizeof(int64_t) * (g->n + 1),
                                  cudaMemcpyDefault, g->stream);
  if (e == cudaSuccess) {
    k_narrow_offsets<OffT><<<g->sms * 8, kThreads, 0, g->stream>>>(
        tmp, reinterpret_cast<OffT*>(g->off), g->n + 1);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
  cudaFree(tmp);
  if (e != cudaSuccess) {
    g_last_error = std::string("offset upload: ") + cudaGetErrorString(e);
    return GBBFS_ERR_CUDA;
  }
  if (g->m > 0)
    GB_CUDA(cudaMemcpyAsync(g->nbr, neigh, sizeof(int32_t) * g->m, cudaMemcpyDefault,
                            g->stream));
  k_iso_mask<OffT><<<g->sms * 8, kThreads, 0, g->stream>>>(
      g->n, g->W, reinterpret_cast<const OffT*>(g->off), g->iso);
  GB_CUDA(cudaGetLastError());
  k_heads<OffT><<<g->sms * 8, kThreads, 0, g->stream>>>(
      g->n, reinterpret_cast<const OffT*>(g->off), g->nbr, g->head);
  GB_CUDA(cudaGetLastError());
  GB_CUDA(cudaStreamSynchronize(g->stream));
  return setup_grids<OffT>(g);
}

int create(const int64_t* offsets, const int32_t* neigh, int64_t n, int64_t m,
           gbbfs_graph* g) {
  GB_CUDA(cudaGetDevice(&g->device));
  GB_CUDA(cudaDeviceGetAttribute(&g->sms, cudaDevAttrMultiProcessorCount, g->device));
  g->n = n;
  g->m = m;
  g->W = (n + 31) / 32;
  // GBBFS_FORCE_OFF64=1 selects the 64-bit offset kernels for any graph, so
  // the path that graphs with 2^32 or more directed edges take is testable on
  // small inputs.
  const char* force64 = getenv("GBBFS_FORCE_OFF64");
  g->off32 = m < (int64_t(1) << 32) && !(force64 && force64[0] == '1');
  g->shift = 64 - bit_length((uint64_t)n);
  if (g->shift < 33 || (uint64_t)m >= (1ull << g->shift)) {
    g_last_error = "graph too large for the packed frontier counter";
    return GBBFS_ERR_ARG;
  }
  const size_t offsz = g->off32 ? 4 : 8;
  // Admission: everything this handle allocates, against free HBM.
  const size_t need = offsz * (n + 1) + 4 * (size_t)m + 8 * (size_t)n + 4 * 4 * (size_t)g->W +
                      2 * 4 * 32 * (size_t)g->W + 2 * (4 + offsz) * (size_t)(n + 1) +
                      8 * (n + 1) + sizeof(DevState) + (64 << 20);
  size_t free_b = 0, total_b = 0;
  GB_CUDA(cudaMemGetInfo(&free_b, &total_b));
  if (need > free_b) {
    g_last_error = "graph needs " + std::to_string(need) + " bytes, " +
                   std::to_string(free_b) + " free";
    return GBBFS_ERR_NOMEM;
  }
  GB_CUDA(cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking));
  GB_CUDA(cudaEventCreate(&g->ev_begin));
  GB_CUDA(cudaEventCreate(&g->ev_end));
  if (g->off32) {
    GB_TRY(dev_alloc(g, reinterpret_cast<uint32_t**>(&g->off), n + 1));
  } else {
    GB_TRY(dev_alloc(g, reinterpret_cast<unsigned long long**>(&g->off), n + 1));
  }
  GB_TRY(dev_alloc(g, &g->nbr, (size_t)m));
  GB_TRY(dev_alloc(g, &g->head, (size_t)n));
  GB_TRY(dev_alloc(g, &g->iso, g->W));
  GB_TRY(dev_alloc(g, &g->visited, g->W));
  GB_TRY(dev_alloc(g, &g->bm[0], g->W));
  GB_TRY(dev_alloc(g, &g->bm[1], g->W));
  GB_TRY(dev_alloc(g, &g->parent, 32 * g->W));
  GB_TRY(dev_alloc(g, &g->depth, 32 * g->W));
  for (int i = 0; i < 2; i++) {
    GB_TRY(dev_alloc(g, &g->qv[i], n));
    if (g->off32) {
      GB_TRY(dev_alloc(g, reinterpret_cast<uint32_t**>(&g->qs[i]), n));
    } else {
      GB_TRY(dev_alloc(g, reinterpret_cast<unsigned long long**>(&g->qs[i]), n));
    }
  }
  GB_TRY(dev_alloc(g, &g->ctr, 1));
  GB_TRY(dev_alloc(g, &g->st, 1));
  GB_CUDA(cudaHostAlloc(&g->h_st, sizeof(DevState), cudaHostAllocDefault));
  memset(g->h_st, 0, sizeof(DevState));
  g->h_st->t0 = ~0ull;  // kernel stamps take the min start / max end
  GB_CUDA(cudaMemsetAsync(g->ctr, 0, sizeof(DevCounters), g->stream));
  GB_CUDA(cudaMemcpyAsync(g->st, g->h_st, sizeof(DevState), cudaMemcpyHostToDevice, g->stream));
  if (g->off32) return upload<uint32_t>(g, offsets, neigh);
  return upload<unsigned long long>(g, offsets, neigh);
}

// ---------------------------------------------------------------------------
// Graph mode.

int add_kernel(cudaGraphNode_t* node, cudaGraph_t graph, const cudaGraphNode_t* deps,
               size_t ndeps, const void* fn, int grid, int block, void** args) {
  cudaKernelNodeParams kp;
  memset(&kp, 0, sizeof kp);
  kp.func = const_cast<void*>(fn);
  kp.gridDim = dim3(grid);
  kp.blockDim = dim3(block);
  kp.sharedMemBytes = 0;
  kp.kernelParams = args;
  kp.extra = nullptr;
  GB_CUDA(cudaGraphAddKernelNode(node, graph, deps, ndeps, &kp));
  return GBBFS_OK;
}

template <typename OffT>
int build_graph(gbbfs_graph* g) {
  Bufs<OffT> b = bufs<OffT>(g);
  cudaGraph_t graph;
  GB_CUDA(cudaGraphCreate(&graph, 0));
  g->graph = graph;
  cudaGraphConditionalHandle h_loop;
  GB_CUDA(cudaGraphConditionalHandleCreate(&h_loop, graph, 1, cudaGraphCondAssignDefault));
  void* args_b[] = {&b};
  cudaGraphNode_t init_node;
  GB_TRY(add_kernel(&init_node, graph, nullptr, 0, (const void*)k_init<OffT>, g->grid_init,
                    kThreads, args_b));
  cudaGraphNodeParams wp = {cudaGraphNodeTypeConditional};
  wp.conditional.handle = h_loop;
  wp.conditional.type = cudaGraphCondTypeWhile;
  wp.conditional.size = 1;
  cudaGraphNode_t loop_node;
  GB_CUDA(cudaGraphAddNode(&loop_node, graph, &init_node, nullptr, 1, &wp));
  cudaGraph_t body = wp.conditional.phGraph_out[0];

  cudaGraphConditionalHandle h_sel;
  GB_CUDA(cudaGraphConditionalHandleCreate(&h_sel, body, kSelNone, cudaGraphCondAssignDefault));
  void* args_d[] = {&b, &h_loop, &h_sel};
  cudaGraphNode_t decide_node;
  GB_TRY(add_kernel(&decide_node, body, nullptr, 0, (const void*)k_decide<OffT>, 1, 32,
                    args_d));
  cudaGraphNodeParams sp = {cudaGraphNodeTypeConditional};
  sp.conditional.handle = h_sel;
  sp.conditional.type = cudaGraphCondTypeSwitch;
  sp.conditional.size = 6;
  cudaGraphNode_t switch_node;
  GB_CUDA(cudaGraphAddNode(&switch_node, body, &decide_node, nullptr, 1, &sp));
  cudaGraphNode_t k;
  GB_TRY(add_kernel(&k, sp.conditional.phGraph_out[kSelTD], nullptr, 0,
                    (const void*)k_td<OffT>, g->grid_td, kThreads, args_b));
  GB_TRY(add_kernel(&k, sp.conditional.phGraph_out[kSelQ2B], nullptr, 0,
                    (const void*)k_q2b<OffT>, g->grid_q2b, kThreads, args_b));
  GB_TRY(add_kernel(&k, sp.conditional.phGraph_out[kSelBU0], nullptr, 0,
                    (const void*)k_bu<OffT, 0>, g->grid_bu, kThreads, args_b));
  GB_TRY(add_kernel(&k, sp.conditional.phGraph_out[kSelBU1], nullptr, 0,
                    (const void*)k_bu<OffT, 1>, g->grid_bu, kThreads, args_b));
  GB_TRY(add_kernel(&k, sp.conditional.phGraph_out[kSelB2Q], nullptr, 0,
                    (const void*)k_b2q<OffT, false>, g->grid_b2q, kThreads, args_b));
  cudaGraphNode_t tdb;
  GB_TRY(add_kernel(&tdb, sp.conditional.phGraph_out[kSelTDB], nullptr, 0,
                    (const void*)k_tdb<OffT>, g->grid_tdb, kThreads, args_b));
  GB_TRY(add_kernel(&k, sp.conditional.phGraph_out[kSelTDB], &tdb, 1, sweep_kernel<OffT>(),
                    g->grid_sweep, kThreads, args_b));

  cudaGraphNode_t copy_node;
  GB_CUDA(cudaGraphAddMemcpyNode1D(&copy_node, graph, &loop_node, 1, g->h_st, g->st,
                                   kReadbackBytes, cudaMemcpyDeviceToHost));
  GB_CUDA(cudaGraphInstantiate(&g->exec, graph, 0));
  return GBBFS_OK;
}

template <typename OffT>
int run_graph(gbbfs_graph* g) {
  if (!g->exec) GB_TRY(build_graph<OffT>(g));
  GB_CUDA(cudaMemcpyAsync(g->st, g->h_st, kParamBytes, cudaMemcpyHostToDevice, g->stream));
  GB_CUDA(cudaEventRecord(g->ev_begin, g->stream));
  GB_CUDA(cudaGraphLaunch(g->exec, g->stream));
  GB_CUDA(cudaEventRecord(g->ev_end, g->stream));
  GB_CUDA(cudaEventSynchronize(g->ev_end));
  return GBBFS_OK;
}

// The trial loop's searches without stats: search i reads its parameters
// from host slot i & 1 and reads its header back into the same slot, so the
// host queues search i while search i-1 still runs and only waits for search
// i-2 (the last user of the slot).  The graph's own read-back into h_st
// still happens and is not used here.
template <typename OffT>
int run_many_graph(gbbfs_graph* g, const int32_t* sources, int64_t k, int alpha, int beta,
                   int32_t* const* parent_out) {
  if (!g->exec) GB_TRY(build_graph<OffT>(g));
  const size_t bytes = sizeof(int32_t) * (size_t)g->n;
  const size_t header = offsetof(DevState, trace);
  auto finish = [&](int64_t i) -> int {
    const int b = (int)(i & 1);
    GB_CUDA(cudaEventSynchronize(g->staged[b]));
    if (g->h_slot[b].error) {
      g_last_error = "device control loop exceeded its iteration bound";
      return g->h_slot[b].error;
    }
    return GBBFS_OK;
  };
  for (int64_t i = 0; i < k; i++) {
    const int b = (int)(i & 1);
    if (i >= 2) GB_TRY(finish(i - 2));
    DevState* h = g->h_slot + b;
    memset(h, 0, header);
    h->source = sources[i];
    h->alpha = alpha;
    h->beta = beta;
    h->in_graph = 1;
    h->parent = g->stage[b];
    // Parent array b is free once the copy of search i-2 has left it.
    GB_CUDA(cudaStreamWaitEvent(g->stream, g->copied[b], 0));
    GB_CUDA(cudaMemcpyAsync(g->st, h, kParamBytes, cudaMemcpyHostToDevice, g->stream));
    GB_CUDA(cudaGraphLaunch(g->exec, g->stream));
    GB_CUDA(cudaMemcpyAsync(h, g->st, header, cudaMemcpyDeviceToHost, g->stream));
    GB_CUDA(cudaEventRecord(g->staged[b], g->stream));
    GB_CUDA(cudaStreamWaitEvent(g->copy_stream, g->staged[b], 0));
    GB_CUDA(cudaMemcpyAsync(parent_out[i], g->stage[b], bytes, cudaMemcpyDeviceToHost,
                            g->copy_stream));
    GB_CUDA(cudaEventRecord(g->copied[b], g->copy_stream));
  }
  for (int64_t i = std::max<int64_t>(0, k - 2); i < k; i++) GB_TRY(finish(i));
  if (k > 0) {
    g->have_result = true;
    g->result_depth = false;
    g->last_parent = g->stage[(k - 1) & 1];
  }
  return GBBFS_OK;
}

// ---------------------------------------------------------------------------
// Stepped mode: same kernels, decisions read back after every k_decide.

int step_event(gbbfs_graph* g, size_t idx) {
  while (g->step_ev.size() <= idx) {
    cudaEvent_t e;
    GB_CUDA(cudaEventCreate(&e));
    g->step_ev.push_back(e);
  }
  GB_CUDA(cudaEventRecord(g->step_ev[idx], g->stream));
  return GBBFS_OK;
}

template <typename OffT>
int run_stepped(gbbfs_graph* g, std::vector<double>* kernel_seconds) {
  Bufs<OffT> b = bufs<OffT>(g);
  cudaStream_t s = g->stream;
  GB_CUDA(cudaMemcpyAsync(g->st, g->h_st, kParamBytes, cudaMemcpyHostToDevice, s));
  GB_CUDA(cudaEventRecord(g->ev_begin, s));
  k_init<OffT><<<g->grid_init, kThreads, 0, s>>>(b);
  GB_CUDA(cudaGetLastError());
  const size_t ctl = offsetof(DevState, cur);
  size_t steps = 0;
  for (;;) {
    k_decide<OffT><<<1, 32, 0, s>>>(b, 0, 0);
    GB_CUDA(cudaGetLastError());
    GB_CUDA(cudaMemcpyAsync(reinterpret_cast<char*>(g->h_st) + ctl,
                            reinterpret_cast<char*>(g->st) + ctl, 4 * sizeof(int32_t),
                            cudaMemcpyDeviceToHost, s));
    GB_CUDA(cudaStreamSynchronize(s));
    const int kind = g->h_st->next_kind;
    if (kind == kKindStop) break;
    GB_TRY(step_event(g, 2 * steps));
    switch (kind) {
      case kKindTD: k_td<OffT><<<g->grid_td, kThreads, 0, s>>>(b); break;
      case kKindTDB: {
        k_tdb<OffT><<<g->grid_tdb, kThreads, 0, s>>>(b);
        void* args[] = {&b};
        GB_CUDA(cudaLaunchKernel(sweep_kernel<OffT>(), dim3(g->grid_sweep), dim3(kThreads), args,
                                 0, s));
        break;
      }
      case kKindE: k_q2b<OffT><<<g->grid_q2b, kThreads, 0, s>>>(b); break;
      case kKindBU:
        if (g->h_st->parity)
          k_bu<OffT, 1><<<g->grid_bu, kThreads, 0, s>>>(b);
        else
          k_bu<OffT, 0><<<g->grid_bu, kThreads, 0, s>>>(b);
        break;
      case kKindC: k_b2q<OffT, false><<<g->grid_b2q, kThreads, 0, s>>>(b); break;
      default:
        g_last_error = "unknown step kind from the device";
        return GBBFS_ERR_STATE;
    }
    GB_CUDA(cudaGetLastError());
    GB_TRY(step_event(g, 2 * steps + 1));
    steps++;
  }
  GB_CUDA(cudaMemcpyAsync(g->h_st, g->st, kReadbackBytes, cudaMemcpyDeviceToHost, s));
  GB_CUDA(cudaEventRecord(g->ev_end, s));
  GB_CUDA(cudaEventSynchronize(g->ev_end));
  kernel_seconds->resize(steps);
  for (size_t i = 0; i < steps; i++) {
    float ms = 0;
    GB_CUDA(cudaEventElapsedTime(&ms, g->step_ev[2 * i], g->step_ev[2 * i + 1]));
    (*kernel_seconds)[i] = ms * 1e-3;
  }
  return GBBFS_OK;
}

int64_t alg_bytes(int64_t n, const gbbfs_step* steps, int count) {
  // InitParent 12n; TD 20|F| + 8 E_td + 8|N|; BU 4n + n/4 + 8|U| + 4 E_bu + 4|N|;
  // TD->BU 4|F| + n/8; BU->TD n/8 + 4|F'|.  |F| of a td step is the count of
  // the step before it.
  int64_t b = 12 * n;
  int64_t prev = 1;
  for (int i = 0; i < count; i++) {
    const gbbfs_step& s = steps[i];
    switch (s.kind) {
      case GBBFS_STEP_TD: b += 20 * prev + 8 * s.edges + 8 * s.count; break;
      case GBBFS_STEP_BU: b += 4 * n + n / 4 + 8 * s.unvisited + 4 * s.edges + 4 * s.count; break;
      case GBBFS_STEP_E: b += 4 * s.count + n / 8; break;
      case GBBFS_STEP_C: b += n / 8 + 4 * s.count; break;
    }
    prev = s.count;
  }
  return b;
}

// One search into parent_buf (32 W entries; the handle's own array when
// null).
int search(gbbfs_graph* g, int32_t source, int alpha, int beta, bool want_depth,
           gbbfs_stats* st, int32_t* parent_buf = nullptr) {
  if (!g) return GBBFS_ERR_ARG;
  if (source < 0 || source >= g->n) {
    g_last_error = "source out of range";
    return GBBFS_ERR_ARG;
  }
  if (alpha <= 0) alpha = 15;
  if (beta <= 0) beta = 18;
  GB_CUDA(cudaSetDevice(g->device));
  g->have_result = false;
  const bool instrument = st && st->instrument;
  const bool stepped = st && st->stepped;
  DevState* h = g->h_st;
  h->source = source;
  h->alpha = alpha;
  h->beta = beta;
  h->want_depth = want_depth ? 1 : 0;
  h->parent = parent_buf ? parent_buf : g->parent;
  h->instrument = instrument ? 1 : 0;
  h->in_graph = stepped ? 0 : 1;
  std::vector<double> kernel_seconds;
  int rc;
  if (stepped)
    rc = g->off32 ? run_stepped<uint32_t>(g, &kernel_seconds)
                  : run_stepped<unsigned long long>(g, &kernel_seconds);
  else
    rc = g->off32 ? run_graph<uint32_t>(g) : run_graph<unsigned long long>(g);
  if (rc != GBBFS_OK) return rc;
  if (h->error) {
    g_last_error = "device control loop exceeded its iteration bound";
    return h->error;
  }
  g->have_result = true;
  g->result_depth = want_depth;
  g->last_parent = parent_buf ? parent_buf : g->parent;
  if (st) {
    float ms = 0;
    GB_CUDA(cudaEventElapsedTime(&ms, g->ev_begin, g->ev_end));
    st->device_ms = ms;
    st->init_seconds = h->init_ns * 1e-9;
    st->num_steps = h->nsteps;
    st->levels = h->level - 1;
    st->reached = h->visited;
    const int have = std::min(h->nsteps, kMaxTrace);
    std::vector<DevStep> tr(have);
    if (have > 0) memcpy(tr.data(), h->trace, sizeof(DevStep) * std::min(have, kTraceInline));
    if (have > kTraceInline) {
      GB_CUDA(cudaMemcpy(tr.data() + kTraceInline, g->st->trace + kTraceInline,
                         sizeof(DevStep) * (have - kTraceInline), cudaMemcpyDeviceToHost));
    }
    std::vector<gbbfs_step> steps(have);
    for (int i = 0; i < have; i++) {
      steps[i].kind = tr[i].kind;
      steps[i].level = tr[i].level;
      steps[i].count = tr[i].count;
      steps[i].edges = tr[i].edges;
      steps[i].unvisited = tr[i].unvisited;
      steps[i].seconds = stepped && i < (int)kernel_seconds.size() ? kernel_seconds[i]
                                                                   : tr[i].ns * 1e-9;
    }
    st->alg_bytes = instrument ? alg_bytes(g->n, steps.data(), have) : 0;
    if (st->steps)
      for (int i = 0; i < st->max_steps && i < have; i++) st->steps[i] = steps[i];
  }
  return GBBFS_OK;
}

}  // namespace

namespace gbbfs {

int bfs_enqueue(gbbfs_graph* g, int32_t source, void* h_params) {
  if (source < 0 || source >= g->n) {
    g_last_error = "source out of range";
    return GBBFS_ERR_ARG;
  }
  if (!g->exec) GB_TRY(g->off32 ? build_graph<uint32_t>(g) : build_graph<unsigned long long>(g));
  DevState* h = static_cast<DevState*>(h_params);   // only the parameter head is written
  memset(h, 0, kParamBytes);
  h->source = source;
  h->alpha = 15;
  h->beta = 18;
  h->want_depth = 1;
  h->in_graph = 1;
  h->parent = g->parent;
  GB_CUDA(cudaMemcpyAsync(g->st, h, kParamBytes, cudaMemcpyHostToDevice, g->stream));
  GB_CUDA(cudaGraphLaunch(g->exec, g->stream));
  g->have_result = false;   // queued searches leave no result on the handle
  return GBBFS_OK;
}

const int32_t* bfs_depth(const gbbfs_graph* g) { return g->depth; }

int graph_set_stream_priority(gbbfs_graph* g, int priority) {
  GB_CUDA(cudaSetDevice(g->device));
  GB_CUDA(cudaStreamSynchronize(g->stream));
  cudaStream_t s = nullptr;
  GB_CUDA(cudaStreamCreateWithPriority(&s, cudaStreamNonBlocking, priority));
  cudaStreamDestroy(g->stream);
  g->stream = s;
  return GBBFS_OK;
}

const int32_t* bfs_error_word(const gbbfs_graph* g) { return &g->st->error; }

// A handle from a CSR already in device memory (offsets int64[n+1],
// neighbours int32[m]); the arrays are copied, the caller keeps them.
int graph_create_device(const int64_t* d_off, const int32_t* d_nbr, int64_t n, int64_t m,
                        gbbfs_graph** out) {
  gbbfs_graph* g = new (std::nothrow) gbbfs_graph();
  if (!g) return GBBFS_ERR_NOMEM;
  const int rc = create(d_off, d_nbr, n, m, g);
  if (rc != GBBFS_OK) {
    release(g);
    return rc;
  }
  *out = g;
  return GBBFS_OK;
}

}  // namespace gbbfs

extern "C" {

const char* gbbfs_strerror(int status) {
  switch (status) {
    case GBBFS_OK: return "ok";
    case GBBFS_ERR_ARG: return "invalid argument";
    case GBBFS_ERR_NOMEM: return "not enough device memory";
    case GBBFS_ERR_CUDA: return "CUDA error";
    case GBBFS_ERR_TIMEOUT: return "device wait timed out";
    case GBBFS_ERR_BOUNDS: return "device bounds check failed";
    case GBBFS_ERR_STATE: return "call out of order";
    case GBBFS_ERR_IO: return "file I/O error";
  }
  return "unknown status";
}

const char* gbbfs_last_error(void) { return g_last_error.c_str(); }

int gbbfs_graph_create(const int64_t* offsets, const int32_t* neigh, int64_t n, int64_t m_dir,
                       gbbfs_graph** out) {
  if (!out) return GBBFS_ERR_ARG;
  *out = nullptr;
  if (!offsets || n <= 0 || n > INT32_MAX || m_dir < 0 || (m_dir > 0 && !neigh)) {
    g_last_error = "bad graph arguments";
    return GBBFS_ERR_ARG;
  }
  if (offsets[0] != 0 || offsets[n] != m_dir) {
    g_last_error = "offsets[0] must be 0 and offsets[n] == m_dir";
    return GBBFS_ERR_ARG;
  }
  gbbfs_graph* g = new (std::nothrow) gbbfs_graph();
  if (!g) return GBBFS_ERR_NOMEM;
  int rc = create(offsets, neigh, n, m_dir, g);
  if (rc != GBBFS_OK) {
    release(g);
    return rc;
  }
  *out = g;
  return GBBFS_OK;
}

int gbbfs_graph_destroy(gbbfs_graph* g) {
  if (!g) return GBBFS_ERR_ARG;
  release(g);
  return GBBFS_OK;
}

int gbbfs_graph_info(const gbbfs_graph* g, int64_t* n, int64_t* m_dir, int64_t* device_bytes) {
  if (!g) return GBBFS_ERR_ARG;
  if (n) *n = g->n;
  if (m_dir) *m_dir = g->m;
  if (device_bytes) *device_bytes = g->device_bytes;
  return GBBFS_OK;
}

int gbbfs_bfs_device(gbbfs_graph* g, int32_t source, int alpha, int beta, int want_depth,
                     gbbfs_stats* st) {
  return search(g, source, alpha, beta, want_depth != 0, st);
}

int gbbfs_results(gbbfs_graph* g, int32_t* parent_out, int32_t* depth_out) {
  if (!g) return GBBFS_ERR_ARG;
  if (!g->have_result || (depth_out && !g->result_depth)) return GBBFS_ERR_STATE;
  GB_CUDA(cudaSetDevice(g->device));
  if (parent_out)
    GB_CUDA(cudaMemcpyAsync(parent_out, g->last_parent, sizeof(int32_t) * g->n,
                            cudaMemcpyDeviceToHost, g->stream));
  if (depth_out)
    GB_CUDA(cudaMemcpyAsync(depth_out, g->depth, sizeof(int32_t) * g->n,
                            cudaMemcpyDeviceToHost, g->stream));
  GB_CUDA(cudaStreamSynchronize(g->stream));
  return GBBFS_OK;
}

int gbbfs_result_device_ptrs(gbbfs_graph* g, const int32_t** parent, const int32_t** depth) {
  if (!g) return GBBFS_ERR_ARG;
  if (!g->have_result) return GBBFS_ERR_STATE;
  if (parent) *parent = g->last_parent;
  if (depth) *depth = g->result_depth ? g->depth : nullptr;
  return GBBFS_OK;
}

int gbbfs_bfs(gbbfs_graph* g, int32_t source, int alpha, int beta, int32_t* parent_out,
              int32_t* depth_out, gbbfs_stats* st) {
  int rc = search(g, source, alpha, beta, depth_out != nullptr, st);
  if (rc != GBBFS_OK) return rc;
  return gbbfs_results(g, parent_out, depth_out);
}

int gbbfs_bfs_many(gbbfs_graph* g, const int32_t* sources, int64_t k, int alpha, int beta,
                   int32_t* const* parent_out, gbbfs_stats* st) {
  if (!g || k < 0 || (k > 0 && (!sources || !parent_out))) return GBBFS_ERR_ARG;
  for (int64_t i = 0; i < k; i++)
    if (!parent_out[i]) return GBBFS_ERR_ARG;
  GB_CUDA(cudaSetDevice(g->device));
  // Made on first use; each resource is checked on its own, so a call after
  // a failed one completes the set-up instead of making any part twice.
  for (int i = 0; i < 2; i++) {
    if (!g->stage[i]) {
      cudaError_t e = cudaMalloc(&g->stage[i], sizeof(int32_t) * 32 * (size_t)g->W);
      if (e != cudaSuccess) {
        g->stage[i] = nullptr;
        g_last_error = std::string("parent arrays: ") + cudaGetErrorString(e);
        return e == cudaErrorMemoryAllocation ? GBBFS_ERR_NOMEM : GBBFS_ERR_CUDA;
      }
      g->device_bytes += (int64_t)sizeof(int32_t) * 32 * g->W;
    }
    if (!g->staged[i]) GB_CUDA(cudaEventCreateWithFlags(&g->staged[i], cudaEventDisableTiming));
    if (!g->copied[i]) GB_CUDA(cudaEventCreateWithFlags(&g->copied[i], cudaEventDisableTiming));
  }
  if (!g->copy_stream)
    GB_CUDA(cudaStreamCreateWithFlags(&g->copy_stream, cudaStreamNonBlocking));
  if (!g->h_slot)
    GB_CUDA(cudaHostAlloc(reinterpret_cast<void**>(&g->h_slot), 2 * sizeof(DevState),
                          cudaHostAllocDefault));
  if (!st) {
    if (alpha <= 0) alpha = 15;
    if (beta <= 0) beta = 18;
    for (int64_t i = 0; i < k; i++) {
      if (sources[i] < 0 || sources[i] >= g->n) {
        g_last_error = "source out of range";
        return GBBFS_ERR_ARG;
      }
    }
    g->have_result = false;
    int rc = g->off32 ? run_many_graph<uint32_t>(g, sources, k, alpha, beta, parent_out)
                      : run_many_graph<unsigned long long>(g, sources, k, alpha, beta, parent_out);
    GB_CUDA(cudaStreamSynchronize(g->copy_stream));
    GB_CUDA(cudaStreamSynchronize(g->stream));
    return rc;
  }
  const size_t bytes = sizeof(int32_t) * (size_t)g->n;
  int rc = GBBFS_OK;
  for (int64_t i = 0; i < k && rc == GBBFS_OK; i++) {
    const int b = (int)(i & 1);
    // Search i writes parent array b, which is free once the copy of search
    // i-2 has left it; its copy to the host then runs beside search i+1.
    GB_CUDA(cudaStreamWaitEvent(g->stream, g->copied[b], 0));
    rc = search(g, sources[i], alpha, beta, false, st ? st + i : nullptr, g->stage[b]);
    if (rc != GBBFS_OK) break;
    GB_CUDA(cudaEventRecord(g->staged[b], g->stream));
    GB_CUDA(cudaStreamWaitEvent(g->copy_stream, g->staged[b], 0));
    GB_CUDA(cudaMemcpyAsync(parent_out[i], g->stage[b], bytes, cudaMemcpyDeviceToHost,
                            g->copy_stream));
    GB_CUDA(cudaEventRecord(g->copied[b], g->copy_stream));
  }
  GB_CUDA(cudaStreamSynchronize(g->copy_stream));
  GB_CUDA(cudaStreamSynchronize(g->stream));
  return rc;
}

}  // extern "C"
