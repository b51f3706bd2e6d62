// Host side of the GB300 BFS engine and its C ABI (include/gbbfs.h).
//
// gbbfs_graph holds the device CSR and the per-search state.  gbbfs_bfs runs
// the DOBFS control loop of the reference (src/bfs.cc:142-188,
// gapbs-verify/bfs.cc:122-173): the same alpha/beta tests on the same int64
// counters, so the step sequence and its counts equal the reference's.

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "bfs_kernels.cuh"
#include "gbbfs.h"

using namespace gbbfs;

namespace {

thread_local std::string g_last_error;

#define GB_CUDA(call)                                                         \
  do {                                                                        \
    cudaError_t err_ = (call);                                                \
    if (err_ != cudaSuccess) {                                                \
      g_last_error = std::string(#call) + ": " + cudaGetErrorString(err_);    \
      return GBBFS_ERR_CUDA;                                                  \
    }                                                                         \
  } while (0)

int bit_length(uint64_t x) {
  int b = 0;
  while (x) {
    b++;
    x >>= 1;
  }
  return b;
}

}  // namespace

struct gbbfs_graph {
  int64_t n = 0, m = 0, W = 0;
  bool off32 = true;
  int shift = 32;           // packed queue counter: (count << shift) | edges
  int device = 0;
  int sms = 0;
  void* off = nullptr;      // uint32_t* or unsigned long long*
  int32_t* nbr = nullptr;
  uint32_t* iso = nullptr;
  uint32_t* visited = nullptr;
  uint32_t* bm[2] = {nullptr, nullptr};
  int32_t* parent = nullptr;
  int32_t* depth = nullptr;
  int32_t* qv[2] = {nullptr, nullptr};
  void* qs[2] = {nullptr, nullptr};
  DevCounters* ctr = nullptr;
  DevCounters* h_ctr = nullptr;   // pinned mirror
  cudaStream_t stream = nullptr;
  cudaEvent_t ev_begin = nullptr, ev_end = nullptr;
  std::vector<cudaEvent_t> step_ev;
  int grid_init = 0, grid_td = 0, grid_bu = 0, grid_q2b = 0, grid_b2q = 0;
  int64_t device_bytes = 0;
  bool have_result = false;
  bool result_depth = false;
};

namespace {

void release(gbbfs_graph* g) {
  if (!g) return;
  if (g->device >= 0) cudaSetDevice(g->device);
  cudaFree(g->off);
  cudaFree(g->nbr);
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
  if (g->h_ctr) cudaFreeHost(g->h_ctr);
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

#define GB_TRY(x)            \
  do {                       \
    int st_ = (x);           \
    if (st_ != GBBFS_OK) {   \
      return st_;            \
    }                        \
  } while (0)

template <typename OffT>
int occupancy_grid(const void* fn, int sms, int* grid) {
  int per_sm = 0;
  GB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kThreads, 0));
  *grid = std::max(1, per_sm) * sms;
  return GBBFS_OK;
}

template <typename OffT>
int setup_grids(gbbfs_graph* g) {
  GB_TRY(occupancy_grid<OffT>((const void*)k_init<OffT>, g->sms, &g->grid_init));
  GB_TRY(occupancy_grid<OffT>((const void*)k_td<OffT>, g->sms, &g->grid_td));
  GB_TRY(occupancy_grid<OffT>((const void*)k_bu<OffT, false>, g->sms, &g->grid_bu));
  GB_TRY(occupancy_grid<OffT>((const void*)k_q2b, g->sms, &g->grid_q2b));
  GB_TRY(occupancy_grid<OffT>((const void*)k_b2q<OffT>, g->sms, &g->grid_b2q));
  return GBBFS_OK;
}

template <typename OffT>
int upload(gbbfs_graph* g, const int64_t* offsets, const int32_t* neigh) {
  // Offsets go up as int64 and are narrowed on the device when they fit.
  int64_t* tmp = nullptr;
  GB_CUDA(cudaMalloc(&tmp, sizeof(int64_t) * (g->n + 1)));
  cudaError_t e = cudaMemcpyAsync(tmp, offsets, sizeof(int64_t) * (g->n + 1),
                                  cudaMemcpyHostToDevice, g->stream);
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
    GB_CUDA(cudaMemcpyAsync(g->nbr, neigh, sizeof(int32_t) * g->m, cudaMemcpyHostToDevice,
                            g->stream));
  k_iso_mask<OffT><<<g->sms * 8, kThreads, 0, g->stream>>>(
      g->n, g->W, reinterpret_cast<const OffT*>(g->off), g->iso);
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
  const size_t need = offsz * (n + 1) + 4 * (size_t)m + 4 * 4 * (size_t)g->W +
                      2 * 4 * 32 * (size_t)g->W + 2 * (4 + offsz) * (size_t)(n + 1) +
                      8 * (n + 1) + (64 << 20);
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
  GB_CUDA(cudaHostAlloc(&g->h_ctr, sizeof(DevCounters), cudaHostAllocDefault));
  GB_CUDA(cudaMemsetAsync(g->ctr, 0, sizeof(DevCounters), g->stream));
  if (g->off32) return upload<uint32_t>(g, offsets, neigh);
  return upload<unsigned long long>(g, offsets, neigh);
}

// Copy the counters to the pinned mirror and wait for them.
int read_counters(gbbfs_graph* g) {
  GB_CUDA(cudaMemcpyAsync(g->h_ctr, g->ctr, sizeof(DevCounters), cudaMemcpyDeviceToHost,
                          g->stream));
  GB_CUDA(cudaStreamSynchronize(g->stream));
  return GBBFS_OK;
}

struct StepLog {
  std::vector<gbbfs_step> steps;
  bool timed = false;
  double init_seconds = 0;
};

// The DOBFS control loop with one host round trip per step.
template <typename OffT>
int run_search(gbbfs_graph* g, int32_t source, int alpha, int beta, bool want_depth,
               bool instrument, StepLog* log, int* levels_out, int64_t* reached_out) {
  const OffT* off = reinterpret_cast<const OffT*>(g->off);
  OffT* qs[2] = {reinterpret_cast<OffT*>(g->qs[0]), reinterpret_cast<OffT*>(g->qs[1])};
  int32_t* depth = want_depth ? g->depth : nullptr;
  cudaStream_t s = g->stream;
  const int shift = g->shift;
  const unsigned long long emask = (1ull << shift) - 1;
  uint32_t* front = g->bm[0];
  uint32_t* next = g->bm[1];
  int cur = 0;

  auto mark = [&](size_t idx) -> int {
    if (!log->timed) return GBBFS_OK;
    while (g->step_ev.size() <= idx) {
      cudaEvent_t e;
      GB_CUDA(cudaEventCreate(&e));
      g->step_ev.push_back(e);
    }
    GB_CUDA(cudaEventRecord(g->step_ev[idx], s));
    return GBBFS_OK;
  };
  auto push = [&](int kind, int level, int64_t count, int64_t edges, int64_t unvisited) {
    gbbfs_step st;
    st.kind = kind;
    st.level = level;
    st.count = count;
    st.edges = edges;
    st.unvisited = unvisited;
    st.seconds = 0;
    log->steps.push_back(st);
  };

  GB_CUDA(cudaEventRecord(g->ev_begin, s));
  k_init<OffT><<<g->grid_init, kThreads, 0, s>>>(g->n, g->W, off, g->iso, g->visited, front,
                                                g->parent, depth, source, g->qv[0], qs[0],
                                                g->ctr, shift);
  GB_CUDA(cudaGetLastError());
  GB_TRY(mark(0));  // end of "i"
  GB_TRY(read_counters(g));
  int64_t F = (int64_t)(g->h_ctr->qpacked[0] >> shift);
  int64_t scout = (int64_t)(g->h_ctr->qpacked[0] & emask);
  int64_t cur_edges = scout;  // summed degrees of the current queue
  int64_t edges_to_check = g->m;
  int64_t visited = 1;
  int level = 1;
  while (F > 0) {
    if (scout > edges_to_check / alpha) {
      // QueueToBitmap ("e")
      GB_TRY(mark(1 + 2 * log->steps.size()));
      k_q2b<<<g->grid_q2b, kThreads, 0, s>>>(g->qv[cur], g->ctr, cur, shift, front);
      GB_CUDA(cudaGetLastError());
      GB_TRY(mark(2 + 2 * log->steps.size()));
      push(GBBFS_STEP_E, 0, F, 0, 0);
      int64_t awake = F, old_awake;
      do {
        old_awake = awake;
        GB_TRY(mark(1 + 2 * log->steps.size()));
        GB_CUDA(cudaMemsetAsync(&g->ctr->awake, 0, 2 * sizeof(unsigned long long), s));
        if (instrument)
          k_bu<OffT, true><<<g->grid_bu, kThreads, 0, s>>>(g->W, off, g->nbr, g->visited,
                                                          g->parent, depth, front, next,
                                                          g->ctr, level);
        else
          k_bu<OffT, false><<<g->grid_bu, kThreads, 0, s>>>(g->W, off, g->nbr, g->visited,
                                                           g->parent, depth, front, next,
                                                           g->ctr, level);
        GB_CUDA(cudaGetLastError());
        GB_TRY(mark(2 + 2 * log->steps.size()));
        GB_TRY(read_counters(g));
        awake = (int64_t)g->h_ctr->awake;
        push(GBBFS_STEP_BU, level, awake, instrument ? (int64_t)g->h_ctr->scanned : 0,
             g->n - visited);
        visited += awake;
        std::swap(front, next);
        level++;
      } while (awake >= old_awake || awake > g->n / beta);
      // BitmapToQueue ("c")
      GB_TRY(mark(1 + 2 * log->steps.size()));
      GB_CUDA(cudaMemsetAsync(&g->ctr->qpacked[cur], 0, sizeof(unsigned long long), s));
      k_b2q<OffT><<<g->grid_b2q, kThreads, 0, s>>>(g->W, off, front, g->qv[cur], qs[cur],
                                                    g->ctr, cur, shift);
      GB_CUDA(cudaGetLastError());
      GB_TRY(mark(2 + 2 * log->steps.size()));
      GB_TRY(read_counters(g));
      F = (int64_t)(g->h_ctr->qpacked[cur] >> shift);
      cur_edges = (int64_t)(g->h_ctr->qpacked[cur] & emask);
      push(GBBFS_STEP_C, 0, F, 0, 0);
      scout = 1;
    } else {
      edges_to_check -= scout;
      const int nxt = cur ^ 1;
      GB_TRY(mark(1 + 2 * log->steps.size()));
      GB_CUDA(cudaMemsetAsync(&g->ctr->qpacked[nxt], 0, sizeof(unsigned long long), s));
      k_td<OffT><<<g->grid_td, kThreads, 0, s>>>(off, g->nbr, g->visited, g->parent, depth,
                                                  g->qv[cur], qs[cur], g->qv[nxt], qs[nxt],
                                                  g->ctr, cur, shift, level);
      GB_CUDA(cudaGetLastError());
      GB_TRY(mark(2 + 2 * log->steps.size()));
      GB_TRY(read_counters(g));
      F = (int64_t)(g->h_ctr->qpacked[nxt] >> shift);
      scout = (int64_t)(g->h_ctr->qpacked[nxt] & emask);
      push(GBBFS_STEP_TD, level, F, cur_edges, 0);
      cur_edges = scout;
      visited += F;
      cur = nxt;
      level++;
    }
  }
  GB_CUDA(cudaEventRecord(g->ev_end, s));
  GB_CUDA(cudaEventSynchronize(g->ev_end));
  if (log->timed) {
    float init_ms = 0;
    GB_CUDA(cudaEventElapsedTime(&init_ms, g->ev_begin, g->step_ev[0]));
    log->init_seconds = init_ms * 1e-3;
    for (size_t i = 0; i < log->steps.size(); i++) {
      float ms = 0;
      GB_CUDA(cudaEventElapsedTime(&ms, g->step_ev[1 + 2 * i], g->step_ev[2 + 2 * i]));
      log->steps[i].seconds = ms * 1e-3;
    }
  }
  *levels_out = level;
  *reached_out = visited;
  return GBBFS_OK;
}

int64_t alg_bytes(int64_t n, const std::vector<gbbfs_step>& steps) {
  // InitParent 12n; TD 20|F| + 8 E_td + 8|N|; BU 4n + n/4 + 8|U| + 4 E_bu + 4|N|;
  // TD->BU 4|F| + n/8; BU->TD n/8 + 4|F'|.  |F| of a td step is the count of
  // the step before it.
  int64_t b = 12 * n;
  int64_t prev = 1;
  for (const gbbfs_step& s : steps) {
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

int search(gbbfs_graph* g, int32_t source, int alpha, int beta, bool want_depth,
           gbbfs_stats* st) {
  if (!g) return GBBFS_ERR_ARG;
  if (source < 0 || source >= g->n) {
    g_last_error = "source out of range";
    return GBBFS_ERR_ARG;
  }
  if (alpha <= 0) alpha = 15;
  if (beta <= 0) beta = 18;
  GB_CUDA(cudaSetDevice(g->device));
  g->have_result = false;
  StepLog log;
  log.timed = st && st->steps && st->max_steps > 0;
  const bool instrument = st && st->instrument;
  int levels = 0;
  int64_t reached = 0;
  int rc = g->off32
               ? run_search<uint32_t>(g, source, alpha, beta, want_depth, instrument, &log,
                                      &levels, &reached)
               : run_search<unsigned long long>(g, source, alpha, beta, want_depth,
                                                instrument, &log, &levels, &reached);
  if (rc != GBBFS_OK) return rc;
  g->have_result = true;
  g->result_depth = want_depth;
  if (st) {
    float ms = 0;
    GB_CUDA(cudaEventElapsedTime(&ms, g->ev_begin, g->ev_end));
    st->device_ms = ms;
    st->init_seconds = log.init_seconds;
    st->num_steps = (int32_t)log.steps.size();
    st->levels = levels;
    st->reached = reached;
    st->alg_bytes = instrument ? alg_bytes(g->n, log.steps) : 0;
    if (st->steps)
      for (int i = 0; i < st->max_steps && i < (int)log.steps.size(); i++)
        st->steps[i] = log.steps[i];
  }
  return GBBFS_OK;
}

}  // namespace

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
    GB_CUDA(cudaMemcpyAsync(parent_out, g->parent, sizeof(int32_t) * g->n,
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
  if (parent) *parent = g->parent;
  if (depth) *depth = g->result_depth ? g->depth : nullptr;
  return GBBFS_OK;
}

int gbbfs_bfs(gbbfs_graph* g, int32_t source, int alpha, int beta, int32_t* parent_out,
              int32_t* depth_out, gbbfs_stats* st) {
  int rc = search(g, source, alpha, beta, depth_out != nullptr, st);
  if (rc != GBBFS_OK) return rc;
  return gbbfs_results(g, parent_out, depth_out);
}

}  // extern "C"
