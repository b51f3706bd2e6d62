// Query server: (graph, source) BFS queries answered as they arrive.
//
// No counterpart in the reference.  A server holds a pool of resident graphs
// (gbbfs_graph handles the caller created).  A host thread batches the
// pending queries of each graph into the lanes of the multi-source search:
// whenever one of a graph's two batch buffers is free, up to `lanes` queued
// queries of that graph are launched together, so queries that arrive while
// a batch is on the GPU join the next one.  When more are queued than one
// batch holds, the batch is formed from queries whose sources have close
// batching keys (gbbfs_msbfs_order), around the oldest query.  A launch of
// few queries runs them as plain single-source searches instead when that
// is cheaper: per graph the server measures a plain search's device time
// when it admits the graph, keeps a running estimate of a batch's at each
// lane width (the search kernel's own start and end stamps, which exclude
// waits for other graphs' work; one 1-source batch is measured at
// admission too), and picks plain when k plain searches are estimated to
// take less than one batch and few batches are in flight: the small kernels
// of a plain search queue behind other graphs' batches, which hold the whole
// GPU, so under load a batch answers sooner.  Batches of different graphs run
// on their graphs' own streams.  By default each batch's persistent kernel
// spans the whole GPU and the graphs' batches take turns; grid_policy 1 gives
// each graph its own share of the SMs (a reserve for the small kernels
// around batches, at least 8 SMs per graph, the rest by the square root of
// the graph's measured batch cost), so a small graph's batch runs beside a
// large graph's instead of waiting for the whole GPU.  The per-graph
// search state (visit / frontier words, depth rows) is admitted against free
// HBM and an optional byte budget; an idle graph gives its state back when
// another graph needs the room.  mode 1 answers every query with its own
// single-source search instead (the plain per-query baseline).
//
// Every result carries the query's timestamps on the server clock (submit,
// launch, done) and a digest of its depth row: uint8 depths d[v] (255 =
// unreached), checksum = sum over v of (d[v] + 1) * ((v + 1) * 0x9E3779B97F4A7C15)
// mod 2^64, plus the number of reached vertices and the largest depth.

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <numeric>
#include <thread>
#include <vector>

#include "engine.h"
#include "msbfs_kernels.cuh"
#include "serve_policy.h"

namespace gbbfs {

struct RowStats {
  unsigned long long sum;
  unsigned long long reached;
  unsigned int max_depth;
  unsigned int pad;
};

// Digest of `rows` depth rows of n entries.  Depth type T: uint8 (255 =
// unreached) or int32 (-1 = unreached, mapped to 255).  Optionally writes
// the uint8 form to out8.
// With err (device, may be null), its value goes to stats[row].pad.
template <typename T>
__global__ void k_row_stats(const T* __restrict__ depth, int64_t n, int rows,
                            RowStats* __restrict__ stats, uint8_t* __restrict__ out8,
                            const int32_t* err) {
  const int row = blockIdx.y;
  if (row >= rows) return;
  if (err && blockIdx.x == 0 && threadIdx.x == 0) stats[row].pad = (unsigned int)*err;
  const T* d = depth + (int64_t)row * n;
  unsigned long long sum = 0, reached = 0;
  unsigned int mx = 0;
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += (int64_t)gridDim.x * blockDim.x) {
    int x = (int)d[v];
    unsigned int b = (x < 0 || x >= 255) ? 255u : (unsigned int)x;
    if (out8) out8[(int64_t)row * n + v] = (uint8_t)b;
    sum += (unsigned long long)(b + 1) * ((unsigned long long)(v + 1) * 0x9E3779B97F4A7C15ull);
    if (b != 255u) {
      reached++;
      mx = b > mx ? b : mx;
    }
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    sum += __shfl_xor_sync(kFull, sum, o);
    reached += __shfl_xor_sync(kFull, reached, o);
    mx = max(mx, __shfl_xor_sync(kFull, mx, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&stats[row].sum, sum);
    atomicAdd(&stats[row].reached, reached);
    atomicMax(&stats[row].max_depth, mx);
  }
}

namespace {

using Clock = std::chrono::steady_clock;

struct Query {
  uint64_t ticket;
  int32_t graph;
  int32_t source;
  uint8_t* out;
  double t_submit, t_start, t_done;
  int batch;
  bool plain;
  uint64_t dev_begin, dev_end;   // the answering batch kernel's device clock stamps
};

struct Inflight {
  bool busy = false;
  bool plain = false;            // plain single-source searches, not a batch
  int cls = 0;                   // lane width class of a batch (32 << cls lanes)
  std::vector<Query> q;
  cudaEvent_t done = nullptr;
};

struct Slot {
  gbbfs_graph* g = nullptr;
  std::deque<Query> pending;
  Inflight fl[2];
  RowStats* d_stats = nullptr;   // 2 x kMsMaxLanes (one block per batch buffer)
  RowStats* h_stats = nullptr;   // pinned 2 x kMsMaxLanes
  uint8_t* d_plain = nullptr;    // plain mode: uint8 depth row
  void* h_par = nullptr;         // pinned search parameters: 2 x kMsMaxLanes blocks
  bool admitted = false;
  double last_used = 0;
  // Device time estimates (ms): one plain search (at admission), and one
  // batch per lane width class (running); negative while unmeasured.
  double plain_ms = -1;
  double batch_ms[4] = {-1, -1, -1, -1};
  double full_batch_ms = -1;     // a 1-source batch on the whole GPU (at admission)
  int priority = 1 << 30;        // stream priority given (none yet)
};

constexpr size_t kParBlock = 64;   // bytes per parameter block in h_par
static_assert(kSearchParamBytes <= kParBlock, "parameter block too small");
constexpr double kEwma = 0.25;     // weight of a new measurement in the estimates

}  // namespace
}  // namespace gbbfs

using namespace gbbfs;

struct gbbfs_server {
  gbbfs_server_config cfg;
  Clock::time_point t0;
  std::vector<Slot> slots;
  std::mutex mu;
  std::condition_variable cv;
  std::deque<Query> inbox;
  std::deque<gbbfs_result> done;
  std::condition_variable done_cv;
  uint64_t next_ticket = 1;
  int64_t outstanding = 0;
  bool stop = false;
  bool started = false;
  int device = 0;
  int error = GBBFS_OK;
  std::string error_msg;
  std::thread worker;

  double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
};

namespace {

int64_t state_bytes_in_use(gbbfs_server* s) {
  int64_t b = 0;
  for (const Slot& sl : s->slots)
    if (sl.admitted) b += (int64_t)ms_state_bytes(sl.g->n, sl.g->m, sl.g->W, 1);
  return b;
}

// SMs a graph's batches span (0 = the whole GPU).  grid_policy 1 splits the
// SMs among the admitted graphs so that their batches run side by side: a
// reserve of kReserveSms is left for the small kernels around the batches
// (buffer clears, depth decode, digests), which would otherwise wait for a
// batch to finish; every graph gets kMinShareSms, and the rest goes in
// proportion to the square root of the graph's measured batch cost on the
// whole GPU.  (With equal query rates that split minimises the mean batch
// time when a batch's time scales with 1 / SMs; small graphs, whose batches
// do not, stay near the minimum.)  On the 8-graph pool of Kronecker 16-25 and
// uniform 20/23 graphs, whole-GPU batches taking turns measured better in
// both latency and saturation throughput, so grid_policy 0 is the default.
constexpr int kMinShareSms = 8;
constexpr int kReserveSms = 16;
void set_grid_shares(gbbfs_server* s) {
  if (s->cfg.grid_policy != 1) return;
  int count = 0;
  double wsum = 0;
  for (const Slot& o : s->slots)
    if (o.admitted) {
      count++;
      wsum += std::sqrt(std::max(1e-3, o.full_batch_ms));
    }
  if (count == 0) return;
  const int sms = s->slots[0].g->sms;
  const int avail = sms - kReserveSms - kMinShareSms * count;
  for (Slot& o : s->slots) {
    if (!o.admitted) continue;
    int share = 0;   // the whole GPU when there is nothing to split
    if (count > 1 && avail > 0)
      share = kMinShareSms +
              (int)(avail * std::sqrt(std::max(1e-3, o.full_batch_ms)) / wsum);
    ms_set_grid_sms(o.g, share);
  }
}

// Stream priorities by measured batch cost (priorities = 1): the admitted
// graphs are ranked by their whole-GPU batch time and spread over the
// device's priority range, the cheapest getting the highest priority, so
// that when SMs free up the GPU takes a small graph's waiting batch before a
// large graph's.  Under load this starves the costliest graphs (on the
// 8-graph pool at 10k queries/s some waited ~1 s), so it is off by default.
int set_priorities(gbbfs_server* s) {
  if (s->cfg.priorities != 1) return GBBFS_OK;
  int least = 0, greatest = 0;
  GB_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
  std::vector<size_t> idx;
  for (size_t i = 0; i < s->slots.size(); i++)
    if (s->slots[i].admitted) idx.push_back(i);
  std::stable_sort(idx.begin(), idx.end(), [&](size_t a, size_t b) {
    return s->slots[a].full_batch_ms < s->slots[b].full_batch_ms;
  });
  const int levels = least - greatest + 1;   // greatest is the numerically smaller
  for (size_t r = 0; r < idx.size(); r++) {
    Slot& o = s->slots[idx[r]];
    const int level = idx.size() > 1 ? (int)(r * (size_t)levels / idx.size()) : 0;
    const int prio = greatest + std::min(level, levels - 1);
    if (prio == o.priority) continue;
    GB_TRY(graph_set_stream_priority(o.g, prio));
    o.priority = prio;
  }
  return GBBFS_OK;
}

// Admission against free HBM and the configured budget; may evict idle slots.
bool admit(gbbfs_server* s, size_t idx) {
  Slot& sl = s->slots[idx];
  if (sl.admitted) return true;
  const int64_t need = (int64_t)ms_state_bytes(sl.g->n, sl.g->m, sl.g->W, 1);
  for (int pass = 0; pass < 2; pass++) {
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return false;
    const bool hbm_ok = (int64_t)free_b > need + s->cfg.hbm_reserve_bytes;
    const bool budget_ok = s->cfg.hbm_budget_bytes <= 0 ||
                           state_bytes_in_use(s) + need <= s->cfg.hbm_budget_bytes;
    if (hbm_ok && budget_ok) {
      if (ms_prepare(sl.g, 1) != GBBFS_OK) return false;
      if (ms_set_grid_sms(sl.g, 0) != GBBFS_OK) return false;   // measured on the whole GPU
      // Batching keys, once per graph (k = 0: keys only).
      if (s->cfg.order == 0 && ms_order(sl.g, nullptr, 0, nullptr) != GBBFS_OK) return false;
      // The plain search's cost, once per graph, from the oldest query's
      // source: the better of two runs (other graphs' work may overlap).
      if (s->cfg.batches_only == 0 && sl.plain_ms < 0) {
        for (int rep = 0; rep < 2; rep++) {
          gbbfs_stats st;
          memset(&st, 0, sizeof st);
          if (gbbfs_bfs_device(sl.g, sl.pending.front().source, 15, 18, 1, &st) != GBBFS_OK)
            return false;
          if (sl.plain_ms < 0 || st.device_ms < sl.plain_ms) sl.plain_ms = st.device_ms;
        }
      }
      // A 1-source batch's cost (32 lanes) on the whole GPU, from its kernel
      // stamps: the batch estimate's start and the weight of the SM split.
      const int32_t src = sl.pending.front().source;
      if (ms_launch(sl.g, 0, &src, 1) != GBBFS_OK || ms_finish(sl.g, 0) != GBBFS_OK) return false;
      sl.full_batch_ms = ms_kernel_ms(sl.g, 0);
      if (sl.batch_ms[0] < 0) sl.batch_ms[0] = sl.full_batch_ms;
      sl.admitted = true;
      set_grid_shares(s);
      if (set_priorities(s) != GBBFS_OK) return false;
      return true;
    }
    if (pass == 1) break;
    // Evict the least recently used idle slot that holds state.
    int victim = -1;
    for (size_t j = 0; j < s->slots.size(); j++) {
      Slot& o = s->slots[j];
      if (j == idx || !o.admitted || !o.pending.empty() || o.fl[0].busy || o.fl[1].busy) continue;
      if (victim < 0 || o.last_used < s->slots[victim].last_used) victim = (int)j;
    }
    if (victim < 0) return false;
    Slot& o = s->slots[victim];
    cudaStreamSynchronize(o.g->stream);
    msbfs_release(o.g->ms);
    o.g->ms = nullptr;
    o.admitted = false;
    set_grid_shares(s);
  }
  return false;
}

void complete(gbbfs_server* s, Slot& sl, Query& q, const RowStats& rs, int status) {
  gbbfs_result r;
  memset(&r, 0, sizeof r);
  r.ticket = q.ticket;
  r.graph_id = q.graph;
  r.source = q.source;
  r.status = status;
  r.batch_size = q.batch;
  r.submit_s = q.t_submit;
  r.start_s = q.t_start;
  r.done_s = q.t_done;
  r.checksum = rs.sum;
  r.reached = (int64_t)rs.reached;
  r.max_depth = (int32_t)rs.max_depth;
  r.plain = q.plain ? 1 : 0;
  r.device_begin_ns = q.dev_begin;
  r.device_end_ns = q.dev_end;
  std::lock_guard<std::mutex> lk(s->mu);
  s->done.push_back(r);
  s->outstanding--;
  s->done_cv.notify_all();
}

// Harvest finished batches of a slot.
void harvest(gbbfs_server* s, Slot& sl) {
  for (int b = 0; b < 2; b++) {
    Inflight& f = sl.fl[b];
    if (!f.busy || cudaEventQuery(f.done) == cudaErrorNotReady) continue;
    int st = f.plain ? GBBFS_OK : ms_finish(sl.g, b);
    if (!f.plain && st == GBBFS_OK) {
      const double x = ms_kernel_ms(sl.g, b);
      double& est = sl.batch_ms[f.cls];
      if (x > 0) est = est < 0 ? x : (1 - kEwma) * est + kEwma * x;
    }
    uint64_t dev_begin = 0, dev_end = 0;
    if (!f.plain && st == GBBFS_OK) ms_kernel_stamps(sl.g, b, &dev_begin, &dev_end);
    const double t = s->now();
    const size_t n = (size_t)sl.g->n;
    for (size_t i = 0; i < f.q.size(); i++) {
      Query& q = f.q[i];
      q.t_done = t;
      q.dev_begin = dev_begin;
      q.dev_end = dev_end;
      const RowStats& rs = sl.h_stats[kMsMaxLanes * b + i];
      int qst = st;
      if (qst == GBBFS_OK && f.plain && rs.pad) qst = (int)rs.pad;
      if (qst == GBBFS_OK && q.out)
        if (cudaMemcpy(q.out, static_cast<uint8_t*>(ms_depth(sl.g, b)) + i * n, n,
                       cudaMemcpyDeviceToHost) != cudaSuccess)
          qst = GBBFS_ERR_CUDA;
      complete(s, sl, q, rs, qst);
    }
    f.q.clear();
    f.busy = false;
    sl.last_used = t;
  }
}

// The queries of a slot's next batch (at most `lanes`): all of them when they
// fit, in arrival order when grouping is off, else pick_group's choice from
// the oldest kGroupWindow * lanes.
void take_batch(gbbfs_server* s, Slot& sl, size_t lanes, std::vector<Query>& out) {
  const size_t P = sl.pending.size();
  const std::vector<uint16_t>& keys = sl.g->batch_key;
  if (P <= lanes || s->cfg.order != 0 || keys.size() != (size_t)sl.g->n) {
    const size_t k = std::min(P, lanes);
    for (size_t i = 0; i < k; i++) {
      out.push_back(sl.pending.front());
      sl.pending.pop_front();
    }
    return;
  }
  const size_t W = std::min(P, kGroupWindow * lanes);
  std::vector<int> wkeys(W);
  for (size_t i = 0; i < W; i++) wkeys[i] = (int)keys[(size_t)sl.pending[i].source];
  std::vector<char> take(W, 0);
  for (uint32_t i : pick_group(wkeys, lanes)) take[i] = 1;
  std::vector<Query> rest;
  rest.reserve(W - lanes);
  for (size_t i = 0; i < W; i++) (take[i] ? out : rest).push_back(sl.pending[i]);
  sl.pending.erase(sl.pending.begin(), sl.pending.begin() + (std::ptrdiff_t)W);
  sl.pending.insert(sl.pending.begin(), rest.begin(), rest.end());
}

// Launch the next batch of a slot into a free buffer.
void launch(gbbfs_server* s, Slot& sl) {
  // Batches of one graph on the GPU at once (default 1).  A second batch in
  // flight only queues behind the first and behind other graphs' batches,
  // while the queries arriving meanwhile would have joined a later, fuller
  // batch: on the 8-graph pool at 10k queries/s one in flight gave p50 39 ms
  // against 65 ms for two, at the same saturation throughput.
  const int max_inflight = s->cfg.max_inflight > 0 ? s->cfg.max_inflight : 1;
  for (int b = 0; b < 2 && !sl.pending.empty(); b++) {
    Inflight& f = sl.fl[b];
    if (f.busy) continue;
    if (max_inflight == 1 && sl.fl[b ^ 1].busy) break;
    const int lanes = std::min<int>(ms_lanes(sl.g), std::max(1, s->cfg.max_batch));
    take_batch(s, sl, (size_t)lanes, f.q);
    const int k = (int)f.q.size();
    std::vector<int32_t> src(k);
    const double t = s->now();
    for (int i = 0; i < k; i++) {
      f.q[i].t_start = t;
      f.q[i].batch = k;
      src[i] = f.q[i].source;
    }
    int cls = 0;
    while ((32 << cls) < k) cls++;
    // Plain searches when k of them are estimated to take less than one
    // batch of this width (a width not yet measured runs as a batch) and the
    // GPU is lightly loaded.
    int in_flight = 0;
    for (const Slot& o : s->slots)
      for (const Inflight& x : o.fl) in_flight += (int)(x.busy && !x.plain);
    const bool plain = s->cfg.batches_only == 0 &&
                       plain_is_cheaper(k, sl.plain_ms, sl.batch_ms[cls], in_flight);
    cudaStream_t str = sl.g->stream;
    const int gx = std::max(1, std::min(1024, (int)((sl.g->n + 255) / 256)));
    int st = GBBFS_OK;
    // A failed CUDA call fails the whole launch (its queries end with the
    // status); work already queued still runs in stream order.
    auto cuda_ok = [&](cudaError_t e) {
      if (e != cudaSuccess && st == GBBFS_OK) {
        last_error() = std::string("query server launch: ") + cudaGetErrorString(e);
        st = GBBFS_ERR_CUDA;
      }
      return st == GBBFS_OK;
    };
    if (plain) {
      // Each search's depths become a uint8 row of buffer b and a digest,
      // before the next search reuses the handle's arrays.
      cuda_ok(cudaMemsetAsync(sl.d_stats + kMsMaxLanes * b, 0, sizeof(RowStats) * k, str));
      for (int i = 0; i < k && st == GBBFS_OK; i++) {
        st = bfs_enqueue(sl.g, src[i],
                         static_cast<char*>(sl.h_par) + ((size_t)b * kMsMaxLanes + i) * kParBlock);
        if (st != GBBFS_OK) break;
        k_row_stats<int32_t><<<dim3(gx, 1), 256, 0, str>>>(
            bfs_depth(sl.g), sl.g->n, 1, sl.d_stats + kMsMaxLanes * b + i,
            static_cast<uint8_t*>(ms_depth(sl.g, b)) + (size_t)i * sl.g->n,
            bfs_error_word(sl.g));
        cuda_ok(cudaGetLastError());
      }
    } else {
      st = ms_launch(sl.g, b, src.data(), k);
      if (st == GBBFS_OK &&
          cuda_ok(cudaMemsetAsync(sl.d_stats + kMsMaxLanes * b, 0, sizeof(RowStats) * k, str))) {
        k_row_stats<uint8_t><<<dim3(gx, k), 256, 0, str>>>(
            static_cast<const uint8_t*>(ms_depth(sl.g, b)), sl.g->n, k,
            sl.d_stats + kMsMaxLanes * b, nullptr, nullptr);
        cuda_ok(cudaGetLastError());
      }
    }
    for (Query& q : f.q) q.plain = plain;
    if (st == GBBFS_OK &&
        cuda_ok(cudaMemcpyAsync(sl.h_stats + kMsMaxLanes * b, sl.d_stats + kMsMaxLanes * b,
                                sizeof(RowStats) * k, cudaMemcpyDeviceToHost, str))) {
      ms_mark_copied(sl.g, b, str);
      cuda_ok(cudaEventRecord(f.done, str));
    }
    if (st == GBBFS_OK) {
      f.busy = true;
      f.plain = plain;
      f.cls = cls;
    } else {
      for (Query& q : f.q) {
        q.t_done = s->now();
        RowStats z = {0, 0, 0, 0};
        complete(s, sl, q, z, st);
      }
      f.q.clear();
    }
  }
}

// Plain mode: one single-source search per query.
void serve_plain(gbbfs_server* s, Slot& sl) {
  if (sl.pending.empty()) return;
  Query q = sl.pending.front();
  sl.pending.pop_front();
  q.t_start = s->now();
  q.batch = 1;
  q.plain = true;
  int st = gbbfs_bfs_device(sl.g, q.source, 15, 18, 1, nullptr);
  RowStats rs = {0, 0, 0, 0};
  if (st == GBBFS_OK) {
    const int32_t* dp = nullptr;
    gbbfs_result_device_ptrs(sl.g, nullptr, &dp);
    cudaStream_t str = sl.g->stream;
    cudaMemsetAsync(sl.d_stats, 0, sizeof(RowStats), str);
    const int gx = std::max(1, std::min(1024, (int)((sl.g->n + 255) / 256)));
    k_row_stats<int32_t><<<dim3(gx, 1), 256, 0, str>>>(dp, sl.g->n, 1, sl.d_stats,
                                                       q.out ? sl.d_plain : nullptr, nullptr);
    cudaMemcpyAsync(sl.h_stats, sl.d_stats, sizeof(RowStats), cudaMemcpyDeviceToHost, str);
    if (q.out) cudaMemcpyAsync(q.out, sl.d_plain, (size_t)sl.g->n, cudaMemcpyDeviceToHost, str);
    if (cudaStreamSynchronize(str) != cudaSuccess) st = GBBFS_ERR_CUDA;
    rs = sl.h_stats[0];
  }
  q.t_done = s->now();
  sl.last_used = q.t_done;
  complete(s, sl, q, rs, st);
}

void worker_loop(gbbfs_server* s) {
  cudaSetDevice(s->device);
  for (;;) {
    {
      std::unique_lock<std::mutex> lk(s->mu);
      bool busy = false;
      for (const Slot& sl : s->slots) busy = busy || sl.fl[0].busy || sl.fl[1].busy;
      if (s->inbox.empty() && !busy) {
        bool any_pending = false;
        for (const Slot& sl : s->slots) any_pending = any_pending || !sl.pending.empty();
        if (!any_pending) {
          if (s->stop) return;
          s->cv.wait_for(lk, std::chrono::microseconds(200));
        }
      }
      while (!s->inbox.empty()) {
        Query q = s->inbox.front();
        s->inbox.pop_front();
        s->slots[q.graph].pending.push_back(q);
      }
    }
    bool any_busy = false;
    for (size_t i = 0; i < s->slots.size(); i++) {
      Slot& sl = s->slots[i];
      if (s->cfg.mode == 1) {
        serve_plain(s, sl);
        continue;
      }
      harvest(s, sl);
      if (!sl.pending.empty()) {
        if (admit(s, i)) {
          launch(s, sl);
        } else {
          bool others = false;
          for (const Slot& o : s->slots) others = others || o.fl[0].busy || o.fl[1].busy;
          if (!others) {
            // Nothing in flight will free memory: the queries cannot be served.
            last_error() = "query state does not fit in free HBM / the server budget";
            while (!sl.pending.empty()) {
              Query q = sl.pending.front();
              sl.pending.pop_front();
              q.t_start = q.t_done = s->now();
              RowStats z = {0, 0, 0, 0};
              complete(s, sl, q, z, GBBFS_ERR_NOMEM);
            }
          }
        }
      }
      any_busy = any_busy || sl.fl[0].busy || sl.fl[1].busy;
    }
    if (any_busy) std::this_thread::sleep_for(std::chrono::microseconds(5));
  }
}

}  // namespace

extern "C" {

int gbbfs_server_open(const gbbfs_server_config* cfg, gbbfs_server** out) {
  if (!out) return GBBFS_ERR_ARG;
  *out = nullptr;
  gbbfs_server* s = new (std::nothrow) gbbfs_server();
  if (!s) return GBBFS_ERR_NOMEM;
  memset(&s->cfg, 0, sizeof s->cfg);
  s->cfg.max_batch = kMsMaxLanes;
  if (cfg) s->cfg = *cfg;
  if (s->cfg.max_batch <= 0) s->cfg.max_batch = kMsMaxLanes;
  if ((s->cfg.mode != 0 && s->cfg.mode != 1) || (s->cfg.order != 0 && s->cfg.order != 1) ||
      (s->cfg.batches_only != 0 && s->cfg.batches_only != 1) ||
      (s->cfg.priorities != 0 && s->cfg.priorities != 1) ||
      (s->cfg.grid_policy != 0 && s->cfg.grid_policy != 1) || s->cfg.max_inflight < 0 ||
      s->cfg.max_inflight > 2) {
    delete s;
    last_error() = "server mode must be 0 (batched) or 1 (plain), order 0 (grouped) or 1 "
                   "(arrival), batches_only 0 or 1, grid_policy 0 or 1, max_inflight 0..2, "
                   "priorities 0 or 1";
    return GBBFS_ERR_ARG;
  }
  s->t0 = Clock::now();
  cudaGetDevice(&s->device);
  *out = s;
  return GBBFS_OK;
}

int gbbfs_server_add_graph(gbbfs_server* s, gbbfs_graph* g, int32_t* graph_id) {
  if (!s || !g || !graph_id) return GBBFS_ERR_ARG;
  if (s->started) {
    last_error() = "graphs must be added before the first query";
    return GBBFS_ERR_STATE;
  }
  Slot sl;
  sl.g = g;
  cudaError_t e = cudaMalloc(&sl.d_stats, sizeof(RowStats) * 2 * kMsMaxLanes);
  if (e == cudaSuccess)
    e = cudaHostAlloc(&sl.h_stats, sizeof(RowStats) * 2 * kMsMaxLanes, cudaHostAllocDefault);
  if (e == cudaSuccess) e = cudaMalloc(&sl.d_plain, std::max<size_t>((size_t)g->n, 256));
  if (e == cudaSuccess)
    e = cudaHostAlloc(&sl.h_par, 2 * kMsMaxLanes * kParBlock, cudaHostAllocDefault);
  for (int b = 0; b < 2 && e == cudaSuccess; b++)
    e = cudaEventCreateWithFlags(&sl.fl[b].done, cudaEventDisableTiming);
  if (e != cudaSuccess) {
    // Give back what this call made; the server keeps its earlier graphs.
    cudaFree(sl.d_stats);
    if (sl.h_stats) cudaFreeHost(sl.h_stats);
    cudaFree(sl.d_plain);
    if (sl.h_par) cudaFreeHost(sl.h_par);
    for (int b = 0; b < 2; b++)
      if (sl.fl[b].done) cudaEventDestroy(sl.fl[b].done);
    last_error() = std::string("server graph slot: ") + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? GBBFS_ERR_NOMEM : GBBFS_ERR_CUDA;
  }
  s->slots.push_back(std::move(sl));
  *graph_id = (int32_t)s->slots.size() - 1;
  return GBBFS_OK;
}

int gbbfs_server_submit(gbbfs_server* s, int32_t graph_id, int32_t source, uint8_t* depth_out,
                        uint64_t* ticket) {
  if (!s || graph_id < 0 || graph_id >= (int32_t)s->slots.size()) return GBBFS_ERR_ARG;
  if (source < 0 || source >= s->slots[graph_id].g->n) {
    last_error() = "source out of range";
    return GBBFS_ERR_ARG;
  }
  std::lock_guard<std::mutex> lk(s->mu);
  if (s->stop) return GBBFS_ERR_STATE;
  if (!s->started) {
    s->started = true;
    s->worker = std::thread(worker_loop, s);
  }
  Query q;
  q.ticket = s->next_ticket++;
  q.graph = graph_id;
  q.source = source;
  q.out = depth_out;
  q.t_submit = s->now();
  q.t_start = q.t_done = 0;
  q.batch = 0;
  q.plain = false;
  q.dev_begin = q.dev_end = 0;
  s->inbox.push_back(q);
  s->outstanding++;
  if (ticket) *ticket = q.ticket;
  s->cv.notify_one();
  return GBBFS_OK;
}

int gbbfs_server_submit_many(gbbfs_server* s, int64_t count, const int32_t* graph_ids,
                             const int32_t* sources, uint8_t* const* depth_out,
                             uint64_t* tickets) {
  if (!s || count < 0 || (count > 0 && (!graph_ids || !sources))) return GBBFS_ERR_ARG;
  for (int64_t i = 0; i < count; i++) {
    if (graph_ids[i] < 0 || graph_ids[i] >= (int32_t)s->slots.size()) return GBBFS_ERR_ARG;
    if (sources[i] < 0 || sources[i] >= s->slots[graph_ids[i]].g->n) {
      last_error() = "source out of range";
      return GBBFS_ERR_ARG;
    }
  }
  std::lock_guard<std::mutex> lk(s->mu);
  if (s->stop) return GBBFS_ERR_STATE;
  if (!s->started) {
    s->started = true;
    s->worker = std::thread(worker_loop, s);
  }
  const double t = s->now();
  for (int64_t i = 0; i < count; i++) {
    Query q;
    q.ticket = s->next_ticket++;
    q.graph = graph_ids[i];
    q.source = sources[i];
    q.out = depth_out ? depth_out[i] : nullptr;
    q.t_submit = t;
    q.t_start = q.t_done = 0;
    q.batch = 0;
    q.plain = false;
    q.dev_begin = q.dev_end = 0;
    s->inbox.push_back(q);
    s->outstanding++;
    if (tickets) tickets[i] = q.ticket;
  }
  s->cv.notify_one();
  return GBBFS_OK;
}

int gbbfs_server_poll(gbbfs_server* s, gbbfs_result* out, int32_t max, int32_t* count,
                      int32_t wait_us) {
  if (!s || !count || (max > 0 && !out)) return GBBFS_ERR_ARG;
  std::unique_lock<std::mutex> lk(s->mu);
  if (s->done.empty() && wait_us > 0)
    s->done_cv.wait_for(lk, std::chrono::microseconds(wait_us), [&] { return !s->done.empty(); });
  int32_t c = 0;
  while (c < max && !s->done.empty()) {
    out[c++] = s->done.front();
    s->done.pop_front();
  }
  *count = c;
  return GBBFS_OK;
}

int gbbfs_server_drain(gbbfs_server* s, int32_t timeout_ms) {
  if (!s) return GBBFS_ERR_ARG;
  std::unique_lock<std::mutex> lk(s->mu);
  const bool ok = s->done_cv.wait_for(lk, std::chrono::milliseconds(timeout_ms),
                                      [&] { return s->outstanding == 0; });
  return ok ? GBBFS_OK : GBBFS_ERR_TIMEOUT;
}

double gbbfs_server_clock(const gbbfs_server* s) { return s ? s->now() : 0.0; }

int gbbfs_server_close(gbbfs_server* s) {
  if (!s) return GBBFS_ERR_ARG;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
    s->cv.notify_all();
  }
  if (s->worker.joinable()) s->worker.join();
  for (Slot& sl : s->slots) {
    if (sl.g && sl.g->stream) cudaStreamSynchronize(sl.g->stream);
    cudaFree(sl.d_stats);
    cudaFreeHost(sl.h_stats);
    cudaFree(sl.d_plain);
    if (sl.h_par) cudaFreeHost(sl.h_par);
    for (int b = 0; b < 2; b++)
      if (sl.fl[b].done) cudaEventDestroy(sl.fl[b].done);
  }
  delete s;
  return GBBFS_OK;
}

}  // extern "C"
