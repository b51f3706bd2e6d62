// CUDA kernels of the direction-optimizing BFS (sm_103a).
//
// Data layout in HBM (n vertices, W = ceil(n/32) bitmap words):
//   off      OffT[n+1]   CSR offsets; OffT = uint32 when m_dir < 2^32, else uint64
//   nbr      int32[m]    sorted neighbour lists (in == out: the graph is symmetric)
//   iso      u32[W]      bit set for degree-0 vertices and ids >= n
//   visited  u32[W]      bit set once a vertex has a parent
//   bm0/bm1  u32[W]      bottom-up frontier and the one being built (swap by parity)
//   parent   int32[32W]  the BFS tree, -1 while unvisited (the array the
//                        search's parameters name: the caller may alternate)
//   depth    int32[32W]  BFS depth, -1 while unvisited (kept on request)
//   qv/qs    frontier queues: vertex ids and the exclusive prefix sum of their
//            out-degrees, in queue order (two of each, current and next)
//
// A bitmap word w covers vertices [32w, 32w+32); in bottom-up steps one warp
// owns a word at a time, so next/visited/parent of that range have exactly
// one writer and need no atomics (the reference's per-PE vertex ranges of
// src/partition.h:69-161, one level finer).
//
// Every step kernel reads what changes from step to step (queue index,
// frontier parity, level) from DevState, which k_decide writes, so the same
// kernel nodes serve every level of a CUDA graph.
#pragma once

#include "bfs_common.cuh"

namespace gbbfs {

// ---------------------------------------------------------------------------
// InitParent (src/bfs.cc:131-140, gapbs-verify/bfs.cc:114-120) fused with the
// frontier set-up of DOBFS (src/bfs.cc:150-159): parent = -1 everywhere, the
// source its own parent, visited = iso | {source}, bm0 = 0, queue = {source}.
// The reference keeps -out_degree in parent for unvisited vertices so that
// scout_count can sum it; here the degree is read from the offsets at claim
// time instead, which keeps the init a pure store stream.
//
// The -1 fill is a TMA bulk store: each CTA fills a 16 KB tile of -1 in
// shared memory once, and one thread issues cp.async.bulk stores of that tile
// over the CTA's share of parent (and depth), 16 KB per instruction, then
// waits for them to complete.  The other threads meanwhile write the bitmaps.
// The source's own entries are written by k_decide's first call, after this
// kernel has completed, so no generic store races the bulk stores.
// (Every parent/depth array is 32 W entries from cudaMalloc or a 256-aligned
// slice: the addresses are 16-byte aligned and 128 W bytes is a multiple of 16.)
constexpr int kFillTile = 16384;
template <typename OffT>
__global__ void __launch_bounds__(kThreads) k_init(Bufs<OffT> b) {
  __shared__ __align__(128) int4 neg_tile[kFillTile / 16];
  DevState* st = b.st;
  stamp_begin(st);
  const int32_t source = st->source;
  unsigned char* parent = reinterpret_cast<unsigned char*>(st->parent);
  unsigned char* depth = st->want_depth ? reinterpret_cast<unsigned char*>(b.depth) : nullptr;
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int i = threadIdx.x; i < kFillTile / 16; i += blockDim.x)
    neg_tile[i] = make_int4(-1, -1, -1, -1);
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  __syncthreads();
  if (threadIdx.x == 0) {
    const uint32_t tile = (uint32_t)__cvta_generic_to_shared(neg_tile);
    const uint64_t total = (uint64_t)b.W * 128;   // bytes of 32 W int32 entries
    for (uint64_t o = (uint64_t)blockIdx.x * kFillTile; o < total;
         o += (uint64_t)gridDim.x * kFillTile) {
      const uint32_t sz = (uint32_t)(total - o < (uint64_t)kFillTile ? total - o : kFillTile);
      asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;"
                   :: "l"(parent + o), "r"(tile), "r"(sz) : "memory");
      if (depth)
        asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;"
                     :: "l"(depth + o), "r"(tile), "r"(sz) : "memory");
    }
    asm volatile("cp.async.bulk.commit_group;" ::: "memory");
    asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
  }
  const int64_t src_word = source >> 5;
  for (int64_t w = tid; w < b.W; w += stride) {
    uint32_t v = b.iso[w];
    if (w == src_word) v |= 1u << (source & 31);
    b.visited[w] = v;
    b.bm0[w] = 0;
  }
  if (tid == 0) {
    b.qv0[0] = source;
    b.qs0[0] = 0;
    const unsigned long long deg = (unsigned long long)(b.off[source + 1] - b.off[source]);
    b.ctr->qpacked[0] = (1ull << b.shift) | deg;
    b.ctr->qpacked[1] = 0;
    b.ctr->awake = 0;
    b.ctr->scanned = 0;
    st->cur = 0;
    st->parity = 0;
    st->level = 1;
    st->visited = 1;
    st->edges_to_check = b.m;
    st->iter = 0;
    st->max_iter = 4 * b.n + 64;
    st->nsteps = 0;
    st->error = 0;
    st->next_kind = kKindInit;
  }
  stamp_end(st);
}

// ---------------------------------------------------------------------------
// The DOBFS control loop (src/bfs.cc:158-185, gapbs-verify/bfs.cc:138-166),
// one decision per launch, on one thread.  It books the step that just ran
// (trace record, counters), then applies the reference's tests on the same
// int64 values:
//   scout_count > edges_to_check / alpha          -> switch to bottom-up
//   awake >= old_awake || awake > num_nodes / beta -> stay bottom-up
// and selects the next step.  Inside a CUDA graph it steers the per-step
// switch node and ends the while loop; stepped from the host it only writes
// st->next_kind.  A bound on the iteration count (4 * num_nodes + 64: a
// top-down or bottom-up step continues the loop only after claiming a vertex,
// and at most two conversions sit between two such steps) stops a run-away
// loop with GBBFS_ERR_TIMEOUT instead of spinning.
// Top-down steps whose frontier has more than n >> kTdBitmapShift edges run
// as k_tdb + sweep instead of k_td.
#ifndef GBBFS_TDB_SHIFT
#define GBBFS_TDB_SHIFT 3
#endif
constexpr int kTdBitmapShift = GBBFS_TDB_SHIFT;

template <typename OffT>
__global__ void k_decide(Bufs<OffT> b, cudaGraphConditionalHandle h_loop,
                         cudaGraphConditionalHandle h_sel) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  DevState* s = b.st;
  DevCounters* c = b.ctr;
  const unsigned long long emask = (1ull << b.shift) - 1;
  const int64_t ns = s->t1 > s->t0 ? (int64_t)(s->t1 - s->t0) : 0;
  auto rec = [&](int32_t kind, int32_t level, int64_t count, int64_t edges, int64_t unv) {
    if (s->nsteps < kMaxTrace) {
      DevStep& r = s->trace[s->nsteps];
      r.kind = kind;
      r.level = level;
      r.count = count;
      r.edges = edges;
      r.unvisited = unv;
      r.ns = ns;
    }
    s->nsteps++;
  };
  int32_t next = kKindStop;
  bool frontier_decision = false;
  switch (s->next_kind) {
    case kKindInit: {
      s->init_ns = ns;
      // The source's own entries, after k_init's bulk -1 stores completed.
      s->parent[s->source] = s->source;
      if (s->want_depth) b.depth[s->source] = 0;
      const unsigned long long p = c->qpacked[0];
      s->F = (int64_t)(p >> b.shift);
      s->scout = (int64_t)(p & emask);
      s->cur_edges = s->scout;
      frontier_decision = true;
      break;
    }
    case kKindTD:
    case kKindTDB: {
      const int nxt = s->cur ^ 1;
      const unsigned long long p = c->qpacked[nxt];
      s->F = (int64_t)(p >> b.shift);
      rec(kKindTD, s->level, s->F, s->cur_edges, 0);
      s->scout = (int64_t)(p & emask);
      s->cur_edges = s->scout;
      s->visited += s->F;
      s->cur = nxt;
      s->level++;
      frontier_decision = true;
      break;
    }
    case kKindE:
      rec(kKindE, 0, s->F, 0, 0);
      s->awake = s->F;
      next = kKindBU;
      break;
    case kKindBU: {
      const int64_t awake = (int64_t)c->awake;
      rec(kKindBU, s->level, awake, (int64_t)c->scanned, b.n - s->visited);
      s->awake = awake;
      s->visited += awake;
      s->parity ^= 1;
      s->level++;
      next = (awake >= s->old_awake || awake > b.n / s->beta) ? kKindBU : kKindC;
      break;
    }
    case kKindC: {
      const unsigned long long p = c->qpacked[s->cur];
      s->F = (int64_t)(p >> b.shift);
      s->cur_edges = (int64_t)(p & emask);
      rec(kKindC, 0, s->F, 0, 0);
      s->scout = 1;
      frontier_decision = true;
      break;
    }
    default:
      next = kKindStop;
  }
  if (frontier_decision) {
    if (s->F == 0) {
      next = kKindStop;
    } else if (s->scout > s->edges_to_check / s->alpha) {
      next = kKindE;
    } else {
      s->edges_to_check -= s->scout;
      // A frontier with many edges claims many vertices: its step runs as
      // claims into a bitmap and a sweep that builds the next queue (k_tdb).
      next = s->scout > (b.n >> kTdBitmapShift) ? kKindTDB : kKindTD;
    }
  }
  if (++s->iter > s->max_iter && next != kKindStop) {
    s->error = GBBFS_ERR_TIMEOUT;
    next = kKindStop;
  }
  if (next == kKindBU) {
    s->old_awake = s->awake;
    c->awake = 0;
    c->scanned = 0;
  } else if (next == kKindTD || next == kKindTDB) {
    c->qpacked[s->cur ^ 1] = 0;
  } else if (next == kKindC) {
    c->qpacked[s->cur] = 0;
  }
  s->next_kind = next;
  s->t0 = ~0ull;
  s->t1 = 0;
  if (s->in_graph) {
    unsigned sel = kSelNone;
    if (next == kKindTD) sel = kSelTD;
    else if (next == kKindTDB) sel = kSelTDB;
    else if (next == kKindE) sel = kSelQ2B;
    else if (next == kKindBU) sel = s->parity ? kSelBU1 : kSelBU0;
    else if (next == kKindC) sel = kSelB2Q;
    cudaGraphSetConditional(h_sel, sel);
    cudaGraphSetConditional(h_loop, next != kKindStop ? 1u : 0u);
  }
}

// ---------------------------------------------------------------------------
// Top-down step: TDStep (gapbs-verify/bfs.cc:67-89, src/bfs.cc:81-100).
//
// The frontier's edges are numbered 0..E-1 through the degree prefix sum qs.
// Each warp takes one contiguous span of edge numbers, finds the queue entry
// of its first edge by binary search, then walks the span 32 edges at a time
// (one edge per lane, consecutive lanes on consecutive neighbours: coalesced
// loads) while sliding a 32-entry window over the queue.  So a hub of degree
// 10^6 is spread over many warps and 32 degree-1 vertices fill one warp.
//
// A neighbour v is claimed by atomicOr on its visited bit (the reference's
// compare_and_swap on parent[v]); the winner writes parent[v] = u and appends
// v to the next queue.  scout_count (the summed degrees of claimed vertices)
// falls out of the packed queue counter.  Claims are staged per warp in
// shared memory and appended with one atomic per 256 claims.
constexpr int kTdStage = 256;
constexpr int kHub = 4;   // chunks per group on the hub fast path

template <typename OffT>
__global__ void __launch_bounds__(kThreads) k_td(Bufs<OffT> b) {
  __shared__ int32_t st_v[kWarpsPerCta][kTdStage];
  __shared__ OffT st_d[kWarpsPerCta][kTdStage];
  DevState* st = b.st;
  stamp_begin(st);
  const int cur = st->cur;
  const int level = st->level;
  int32_t* parent = st->parent;
  int32_t* depth = st->want_depth ? b.depth : nullptr;
  const int32_t* qv = cur ? b.qv1 : b.qv0;
  const OffT* qs = cur ? b.qs1 : b.qs0;
  int32_t* qv_out = cur ? b.qv0 : b.qv1;
  OffT* qs_out = cur ? b.qs0 : b.qs1;
  const OffT* __restrict__ off = b.off;
  const int32_t* __restrict__ nbr = b.nbr;
  uint32_t* visited = b.visited;
  const int shift = b.shift;
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const unsigned long long packed = b.ctr->qpacked[cur];
  const int64_t F = (int64_t)(packed >> shift);
  const unsigned long long emask = (1ull << shift) - 1;
  const uint64_t E = packed & emask;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const uint64_t nchunks = (E + 31) >> 5;
  const uint64_t per = (nchunks + nwarps - 1) / nwarps;
  const uint64_t c_begin = warp * per;
  const uint64_t c_end = c_begin + per < nchunks ? c_begin + per : nchunks;
  int staged = 0;

  auto flush = [&]() {
    // Degrees of the staged claims, loaded together (8 independent loads per
    // lane), then one atomic for the whole stage: (count << shift) + degrees.
    OffT red = 0;
#pragma unroll
    for (int q = 0; q < kTdStage / 32; q++) {
      const int i = lane + 32 * q;
      if (i < staged) {
        const int32_t v = st_v[wib][i];
        const OffT d = __ldg(off + v + 1) - __ldg(off + v);
        st_d[wib][i] = d;
        red += d;
      }
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) red += shfl(red, lane ^ o);
    unsigned long long base = 0;
    if (lane == 0)
      base = atomicAdd(&b.ctr->qpacked[cur ^ 1],
                       ((unsigned long long)staged << shift) + (unsigned long long)red);
    base = shfl(base, 0);
    const uint64_t qbase = base >> shift;
    OffT ebase = (OffT)(base & emask);
    for (int i0 = 0; i0 < staged; i0 += 32) {
      const int i = i0 + lane;
      const OffT d = i < staged ? st_d[wib][i] : 0;
      const OffT inc = warp_inclusive_sum(d, lane);
      if (i < staged) {
        qv_out[qbase + i] = st_v[wib][i];
        qs_out[qbase + i] = ebase + inc - d;
      }
      ebase += shfl(inc, 31);
    }
    __syncwarp();
    staged = 0;
  };
  // Append this lane's claim (if any) to the warp's stage.
  auto stage = [&](bool claimed, int32_t v) {
    const unsigned cm = __ballot_sync(kFull, claimed);
    if (cm) {
      const int cnt = __popc(cm);
      if (staged + cnt > kTdStage) flush();
      if (claimed) st_v[wib][staged + __popc(cm & ((1u << lane) - 1))] = v;
      staged += cnt;
      __syncwarp();
    }
  };

  if (c_begin < c_end) {
    uint64_t e0 = c_begin << 5;
    // Last queue entry whose first edge is <= e0.
    int64_t lo = 0, hi = F - 1;
    while (lo < hi) {
      const int64_t mid = (lo + hi + 1) >> 1;
      if ((uint64_t)qs[mid] <= e0) lo = mid; else hi = mid - 1;
    }
    int64_t i0 = lo;
    int64_t ij = -1;
    uint64_t sj = ~0ull;
    int32_t uj = 0;
    uint64_t rj = 0;
    for (uint64_t c = c_begin; c < c_end; c++, e0 += 32) {
      // The window of 32 queue entries from i0; unchanged while the walk
      // stays inside one entry (a hub), so it is reloaded only when i0 moved.
      if (ij != i0 + lane) {
        ij = i0 + lane;
        sj = ~0ull;
        uj = 0;
        rj = 0;
        if (ij < F) {
          sj = (uint64_t)qs[ij];
          uj = qv[ij];
          rj = (uint64_t)off[uj];
        }
      }
      // Hub fast path: when entry i0 covers the next kHub chunks, process them
      // together, every load of the group issued before any of them is used.
      const uint64_t s_next = shfl(sj, 1);   // first edge of entry i0 + 1
      if (c + kHub <= c_end && s_next >= e0 + 32 * kHub) {
        const int32_t u = __shfl_sync(kFull, uj, 0);
        const uint64_t base_nb = shfl(rj, 0) + (e0 - shfl(sj, 0)) + lane;
        int32_t v[kHub];
        uint32_t w[kHub];
#pragma unroll
        for (int q = 0; q < kHub; q++)
          v[q] = e0 + 32 * q + lane < E ? __ldg(nbr + base_nb + 32 * q) : -1;
#pragma unroll
        for (int q = 0; q < kHub; q++) w[q] = v[q] >= 0 ? __ldcg(visited + (v[q] >> 5)) : kFull;
        bool cl[kHub];
#pragma unroll
        for (int q = 0; q < kHub; q++) {
          cl[q] = false;
          if (v[q] >= 0 && !(w[q] & (1u << (v[q] & 31)))) {
            const uint32_t bit = 1u << (v[q] & 31);
            cl[q] = !(atomicOr(visited + (v[q] >> 5), bit) & bit);
          }
        }
#pragma unroll
        for (int q = 0; q < kHub; q++) {
          if (cl[q]) {
            parent[v[q]] = u;
            if (depth) depth[v[q]] = level;
          }
          stage(cl[q], v[q]);
        }
        if (s_next == e0 + 32 * kHub) i0 += 1;
        c += kHub - 1;
        e0 += 32 * (kHub - 1);
        continue;
      }
      // Bit p set <=> a window entry starts at edge e0 + p (entry i0 covers e0).
      unsigned mybit = 0;
      if (lane == 0) mybit = 1u;
      else if (ij < F && sj < e0 + 32) mybit = 1u << (unsigned)(sj - e0);
      const unsigned starts = __reduce_or_sync(kFull, mybit);
      const int k = __popc(starts & (kFull >> (31 - lane))) - 1;
      const int32_t u = __shfl_sync(kFull, uj, k);
      const uint64_t s = shfl(sj, k);
      const uint64_t r = shfl(rj, k);
      const uint64_t e = e0 + lane;
      bool claimed = false;
      int32_t v = 0;
      if (e < E) {
        v = __ldg(nbr + (r + (e - s)));
        const uint32_t bit = 1u << (v & 31);
        uint32_t* wp = visited + (v >> 5);
        if (!(__ldcg(wp) & bit)) {
          const uint32_t old = atomicOr(wp, bit);
          if (!(old & bit)) {
            claimed = true;
            parent[v] = u;
            if (depth) depth[v] = level;
          }
        }
      }
      stage(claimed, v);
      // Advance to the entry that covers edge e0 + 32.  The window holds 32
      // entries; when all of them start at or before e0 + 32, entry i0 + 32
      // may start exactly there.
      const unsigned le = __ballot_sync(kFull, lane == 0 || (ij < F && sj <= e0 + 32));
      int adv = __popc(le) - 1;
      if (le == kFull && i0 + 32 < F && (uint64_t)qs[i0 + 32] == e0 + 32) adv = 32;
      i0 += adv;
    }
  }
  if (staged) flush();
  stamp_end(st);
}

// ---------------------------------------------------------------------------
// Top-down step for frontiers with many edges (TDStep, gapbs-verify/bfs.cc:67-89,
// src/bfs.cc:81-100, as k_td splits it over warps).  Where a step claims
// millions of vertices, k_td's claim path is the cost: each claim waits on an
// atomicOr's returned value, then stages the vertex and later loads its
// degree.  Here a neighbour v not yet in visited (as of the step's start) or
// in the claim bitmap bm[parity] gets its bit set there by an atomicOr whose
// result is not used (a reduction: no round trip), and parent[v] = u.  Two
// frontier vertices may both reach v in the same step; each then stores
// itself as v's parent, and the last store stands: both are v's neighbours
// one level up, as the reference's own racing compare-and-swap allows.  The
// sweep that follows (k_b2q<OffT, true>) turns the bitmap into the next queue
// in vertex order, with degree prefix, packed counter and visited update, so
// the step's count and scout_count are the reference's exactly.
#ifndef GBBFS_TDB_GROUP
#define GBBFS_TDB_GROUP 8
#endif
constexpr int kTdbGroup = GBBFS_TDB_GROUP;   // ordinary chunks in flight per warp

template <typename OffT>
__global__ void __launch_bounds__(kThreads) k_tdb(Bufs<OffT> b) {
  DevState* st = b.st;
  stamp_begin(st);
  const int cur = st->cur;
  const int level = st->level;
  int32_t* parent = st->parent;
  int32_t* depth = st->want_depth ? b.depth : nullptr;
  const int32_t* qv = cur ? b.qv1 : b.qv0;
  const OffT* qs = cur ? b.qs1 : b.qs0;
  const OffT* __restrict__ off = b.off;
  const int32_t* __restrict__ nbr = b.nbr;
  const uint32_t* visited = b.visited;
  uint32_t* claim = st->parity ? b.bm1 : b.bm0;
  const int lane = threadIdx.x & 31;
  const unsigned long long packed = b.ctr->qpacked[cur];
  const int64_t F = (int64_t)(packed >> b.shift);
  const uint64_t E = packed & ((1ull << b.shift) - 1);
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const uint64_t nchunks = (E + 31) >> 5;
  const uint64_t per = (nchunks + nwarps - 1) / nwarps;
  const uint64_t c_begin = warp * per;
  const uint64_t c_end = c_begin + per < nchunks ? c_begin + per : nchunks;
  auto visit = [&](int32_t v, int32_t u) {
    const uint32_t bit = 1u << (v & 31);
    const uint32_t seen = __ldcg(visited + (v >> 5)) | __ldcg(claim + (v >> 5));
    if (!(seen & bit)) {
      atomicOr(claim + (v >> 5), bit);
      parent[v] = u;
      if (depth) depth[v] = level;
    }
  };
  if (c_begin < c_end) {
    uint64_t e0 = c_begin << 5;
    int64_t lo = 0, hi = F - 1;
    while (lo < hi) {
      const int64_t mid = (lo + hi + 1) >> 1;
      if ((uint64_t)qs[mid] <= e0) lo = mid; else hi = mid - 1;
    }
    int64_t i0 = lo;
    int64_t ij = -1;
    uint64_t sj = ~0ull;
    int32_t uj = 0;
    uint64_t rj = 0;
    auto reload = [&]() {
      ij = i0 + lane;
      sj = ~0ull;
      uj = 0;
      rj = 0;
      if (ij < F) {
        sj = (uint64_t)qs[ij];
        uj = qv[ij];
        rj = (uint64_t)off[uj];
      }
    };
    for (uint64_t c = c_begin; c < c_end;) {
      if (ij != i0 + lane) reload();
      const uint64_t s_next = shfl(sj, 1);
      if (c + kHub <= c_end && s_next >= e0 + 32 * kHub) {
        const int32_t u = __shfl_sync(kFull, uj, 0);
        const uint64_t base_nb = shfl(rj, 0) + (e0 - shfl(sj, 0)) + lane;
        int32_t v[kHub];
#pragma unroll
        for (int q = 0; q < kHub; q++)
          v[q] = e0 + 32 * q + lane < E ? __ldg(nbr + base_nb + 32 * q) : -1;
#pragma unroll
        for (int q = 0; q < kHub; q++)
          if (v[q] >= 0) visit(v[q], u);
        if (s_next == e0 + 32 * kHub) i0 += 1;
        c += kHub;
        e0 += 32 * kHub;
        continue;
      }
      // Up to kTdbGroup chunks of ordinary entries: each mapped to its queue
      // entries through the window first (the window is reloaded when the
      // walk moved past it), then all their neighbour loads issued together,
      // then all their bitmap tests, so a warp keeps several chunks' loads in
      // flight instead of one.
      int32_t gu[kTdbGroup];
      uint64_t gi[kTdbGroup];
      bool gv[kTdbGroup];
#pragma unroll
      for (int t = 0; t < kTdbGroup; t++) {
        gv[t] = false;
        gu[t] = 0;
        gi[t] = 0;
        if (c < c_end) {
          if (t > 0 && ij != i0 + lane) reload();
          unsigned mybit = 0;
          if (lane == 0) mybit = 1u;
          else if (ij < F && sj < e0 + 32) mybit = 1u << (unsigned)(sj - e0);
          const unsigned starts = __reduce_or_sync(kFull, mybit);
          const int k = __popc(starts & (kFull >> (31 - lane))) - 1;
          gu[t] = __shfl_sync(kFull, uj, k);
          const uint64_t sk = shfl(sj, k);
          const uint64_t rk = shfl(rj, k);
          const uint64_t e = e0 + lane;
          gv[t] = e < E;
          gi[t] = rk + (e - sk);
          const unsigned le = __ballot_sync(kFull, lane == 0 || (ij < F && sj <= e0 + 32));
          int adv = __popc(le) - 1;
          if (le == kFull && i0 + 32 < F && (uint64_t)qs[i0 + 32] == e0 + 32) adv = 32;
          i0 += adv;
          c++;
          e0 += 32;
        }
      }
      int32_t v[kTdbGroup];
#pragma unroll
      for (int t = 0; t < kTdbGroup; t++) v[t] = gv[t] ? __ldg(nbr + gi[t]) : -1;
      uint32_t w[kTdbGroup];
#pragma unroll
      for (int t = 0; t < kTdbGroup; t++)
        w[t] = v[t] >= 0 ? (__ldcg(visited + (v[t] >> 5)) | __ldcg(claim + (v[t] >> 5))) : kFull;
#pragma unroll
      for (int t = 0; t < kTdbGroup; t++) {
        if (v[t] >= 0 && !(w[t] & (1u << (v[t] & 31)))) {
          atomicOr(claim + (v[t] >> 5), 1u << (v[t] & 31));
          parent[v[t]] = gu[t];
          if (depth) depth[v[t]] = level;
        }
      }
    }
  }
  stamp_end(st);
}

// ---------------------------------------------------------------------------
// QueueToBitmap (gapbs-verify/bfs.cc:92-98, src/bfs.cc:104-112): set the bit
// of every queue entry in the bottom-up frontier bm[parity] (all zero on
// entry: BitmapToQueue clears what it reads, and the init clears bm0).
template <typename OffT>
__global__ void __launch_bounds__(kThreads) k_q2b(Bufs<OffT> b) {
  DevState* st = b.st;
  stamp_begin(st);
  const int cur = st->cur;
  const int32_t* qv = cur ? b.qv1 : b.qv0;
  uint32_t* front = st->parity ? b.bm1 : b.bm0;
  const int64_t F = (int64_t)(b.ctr->qpacked[cur] >> b.shift);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < F;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t v = qv[i];
    atomicOr(front + (v >> 5), 1u << (v & 31));
  }
  stamp_end(st);
}

// ---------------------------------------------------------------------------
// Bottom-up step: BUStep (gapbs-verify/bfs.cc:46-64, src/bfs.cc:57-78).
//
// Every unvisited vertex u looks for the FIRST neighbour (in sorted order)
// whose front bit is set, as the reference does, so bottom-up parents equal
// the reference's.  A warp takes 32 consecutive bitmap words per iteration,
// one word per lane (coalesced visited/next traffic, fully-visited words cost
// one bit test).  The unvisited vertices of those 32 words form a pool in
// shared memory; every lane scans one vertex at a time, in rounds of 2, 4,
// then kBatch neighbours with all loads of a round issued together, and takes
// the next vertex from the pool as soon as its own is resolved.  So a warp
// keeps 32 independent scans in flight whatever the degrees, and reads at
// most kBatch - 1 neighbours past the first hit.  Claims are gathered per word in
// shared memory; the lane that owns a word then writes next[w] and
// visited[w] whole, with no global atomics.  kParity fixes which bitmap is the
// frontier (two graph nodes).
constexpr int kBatch = 8;
// Neighbours probed in a vertex's first round; later rounds double up to
// kBatch.  In dense steps most vertices hit within their first neighbours,
// and every probe is an L2 request for a frontier word: on Kronecker-26,
// rounds of 2, 4, 8, 8, ... instead of 8 from the start took the search from
// 768 to 864 GTEPS (first 1: 839; first 2 without doubling: 854).
#ifndef GBBFS_BU_FIRST
#define GBBFS_BU_FIRST 2
#endif
#ifndef GBBFS_BU_GROW
#define GBBFS_BU_GROW 1
#endif
constexpr int kBatchFirst = GBBFS_BU_FIRST;
constexpr bool kBatchGrow = GBBFS_BU_GROW != 0;   // rounds double up to kBatch

template <typename OffT, int kParity>
__global__ void __launch_bounds__(kThreads) k_bu(Bufs<OffT> b) {
  __shared__ uint16_t pool[kWarpsPerCta][1024];
  __shared__ uint32_t got[kWarpsPerCta][32];
  DevState* st = b.st;
  stamp_begin(st);
  const int level = st->level;
  const bool instrument = st->instrument != 0;
  int32_t* depth = st->want_depth ? b.depth : nullptr;
  const uint32_t* __restrict__ front = kParity ? b.bm1 : b.bm0;
  uint32_t* __restrict__ next = kParity ? b.bm0 : b.bm1;
  const OffT* __restrict__ off = b.off;
  const int32_t* __restrict__ nbr = b.nbr;
  const int2* __restrict__ heads = kBatchFirst == 2 ? b.head : nullptr;
  uint32_t* __restrict__ visited = b.visited;
  int32_t* __restrict__ parent = st->parent;
  const int64_t W = b.W;
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  uint16_t* my_pool = pool[wib];
  unsigned long long awake = 0, scanned = 0;
  for (int64_t base = warp << 5; base < W; base += nwarps << 5) {
    const int64_t w = base + lane;
    const bool valid = w < W;
    const uint32_t vis = valid ? visited[w] : kFull;
    uint32_t todo = ~vis;
    // Pool of this chunk's unvisited vertices (chunk-local index 32*lane + bit),
    // word by word, so lanes that start together read neighbouring offsets.
    const int cnt = __popc(todo);
    const int incl = warp_inclusive_sum(cnt, lane);
    const int total = __shfl_sync(kFull, incl, 31);
    got[wib][lane] = 0;
    if (total == 0) {
      if (valid) next[w] = 0;
      continue;
    }
    for (int k = incl - cnt; todo; k++) {
      const int j = __ffs(todo) - 1;
      todo &= todo - 1;
      my_pool[k] = (uint16_t)((lane << 5) | j);
    }
    __syncwarp();
    int taken = 0;           // pool entries handed out (warp-uniform)
    int item = -1;           // chunk-local index of my vertex, -1 when idle
    uint64_t pos = 0, end = 0, start = 0;
    uint32_t lim = kBatchFirst;   // neighbours of this round
    int2 hd = make_int2(-1, -1);  // its neighbour heads (first round)
    for (;;) {
      const unsigned needy = __ballot_sync(kFull, item < 0);
      if (item < 0) {
        const int idx = taken + __popc(needy & ((1u << lane) - 1));
        if (idx < total) {
          item = my_pool[idx];
          const int64_t u = ((base + (item >> 5)) << 5) + (item & 31);
          start = pos = (uint64_t)off[u];
          end = (uint64_t)off[u + 1];
          if (heads) hd = __ldg(heads + u);
          lim = kBatchFirst;
        }
      }
      taken += __popc(needy);
      if (!__any_sync(kFull, item >= 0)) break;
      if (item >= 0) {
        int32_t v[kBatch];
        if (heads && pos == start) {   // first round: the two neighbour heads
          v[0] = hd.x;
          v[1] = hd.y;
#pragma unroll
          for (int k = 2; k < kBatch; k++) v[k] = -1;
        } else {
#pragma unroll
          for (int k = 0; k < kBatch; k++)
            v[k] = (k < (int)lim && pos + k < end) ? __ldg(nbr + pos + k) : -1;
        }
        uint32_t hits = 0;
#pragma unroll
        for (int k = 0; k < kBatch; k++)
          if (v[k] >= 0 && ((__ldg(front + (v[k] >> 5)) >> (v[k] & 31)) & 1u)) hits |= 1u << k;
        if (hits) {
          const int k = __ffs(hits) - 1;
          int32_t p = v[0];
#pragma unroll
          for (int q = 1; q < kBatch; q++) p = k == q ? v[q] : p;
          const int64_t u = ((base + (item >> 5)) << 5) + (item & 31);
          parent[u] = p;
          if (depth) depth[u] = level;
          atomicOr(&got[wib][item >> 5], 1u << (item & 31));
          if (instrument) scanned += pos + k + 1 - start;
          item = -1;
        } else {
          pos += lim;
          lim = kBatchGrow ? (lim * 2 < (uint32_t)kBatch ? lim * 2 : (uint32_t)kBatch)
                           : (uint32_t)kBatch;
          if (pos >= end) {
            if (instrument) scanned += end - start;
            item = -1;
          }
        }
      }
    }
    __syncwarp();
    const uint32_t claimed = got[wib][lane];
    if (valid) {
      next[w] = claimed;
      if (claimed) visited[w] = vis | claimed;
    }
    awake += __popc(claimed);
    __syncwarp();
  }
  // One atomic per CTA.
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    awake += __shfl_xor_sync(kFull, awake, o);
    scanned += __shfl_xor_sync(kFull, scanned, o);
  }
  __shared__ unsigned long long red[2][kWarpsPerCta];
  if (lane == 0) {
    red[0][threadIdx.x >> 5] = awake;
    red[1][threadIdx.x >> 5] = scanned;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long a = 0, s = 0;
    for (int i = 0; i < kWarpsPerCta; i++) {
      a += red[0][i];
      s += red[1][i];
    }
    if (a) atomicAdd(&b.ctr->awake, a);
    if (s) atomicAdd(&b.ctr->scanned, s);
  }
  stamp_end(st);
}

// ---------------------------------------------------------------------------
// BitmapToQueue (gapbs-verify/bfs.cc:100-112, src/bfs.cc:115-125): every set
// bit of the frontier bm[parity] becomes an entry of queue `cur` (with its
// degree prefix), and the bitmap is cleared on the way so it is all-zero for
// the next QueueToBitmap.  Thread per word; one atomic per CTA-iteration.
//
// kAfterTd: the sweep after k_tdb.  The bitmap holds that step's claims; they
// go to the next queue (cur ^ 1) and into visited.
template <typename OffT, bool kAfterTd>
__global__ void __launch_bounds__(kThreads) k_b2q(Bufs<OffT> b) {
  __shared__ unsigned long long warp_tot[kWarpsPerCta];
  __shared__ unsigned long long cta_base;
  DevState* st = b.st;
  if (!kAfterTd) stamp_begin(st);
  const int dst = kAfterTd ? st->cur ^ 1 : st->cur;
  uint32_t* front = st->parity ? b.bm1 : b.bm0;
  int32_t* qv_out = dst ? b.qv1 : b.qv0;
  OffT* qs_out = dst ? b.qs1 : b.qs0;
  const OffT* __restrict__ off = b.off;
  const int shift = b.shift;
  const int64_t W = b.W;
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const unsigned long long emask = (1ull << shift) - 1;
  const int64_t span = (int64_t)gridDim.x * blockDim.x;
  for (int64_t w0 = (int64_t)blockIdx.x * blockDim.x; w0 < W; w0 += span) {
    const int64_t w = w0 + threadIdx.x;
    uint32_t bits = 0;
    if (w < W) {
      bits = front[w];
      if (bits) {
        front[w] = 0;
        if (kAfterTd) b.visited[w] |= bits;
      }
    }
    unsigned long long degsum = 0;
    for (uint32_t x = bits; x; x &= x - 1) {
      const int64_t u = (w << 5) + (__ffs(x) - 1);
      degsum += (unsigned long long)(off[u + 1] - off[u]);
    }
    // packed (count, degree sum) per thread; inclusive scan over the CTA
    const unsigned long long mine = ((unsigned long long)__popc(bits) << shift) + degsum;
    const unsigned long long inc = warp_inclusive_sum(mine, lane);
    if (lane == 31) warp_tot[wib] = inc;
    __syncthreads();
    if (threadIdx.x == 0) {
      unsigned long long t = 0;
      for (int i = 0; i < kWarpsPerCta; i++) {
        const unsigned long long x = warp_tot[i];
        warp_tot[i] = t;
        t += x;
      }
      cta_base = t ? atomicAdd(&b.ctr->qpacked[dst], t) : 0;
    }
    __syncthreads();
    if (bits) {
      const unsigned long long at = cta_base + warp_tot[wib] + inc - mine;
      uint64_t qpos = at >> shift;
      uint64_t epos = at & emask;
      for (uint32_t x = bits; x; x &= x - 1) {
        const int64_t u = (w << 5) + (__ffs(x) - 1);
        qv_out[qpos] = (int32_t)u;
        qs_out[qpos] = (OffT)epos;
        qpos++;
        epos += (uint64_t)(off[u + 1] - off[u]);
      }
    }
    __syncthreads();
  }
  stamp_end(st);
}

// ---------------------------------------------------------------------------
// The sweep after k_tdb, for 32-bit offsets: the same result as
// k_b2q<OffT, true> (claims to the next queue in vertex order with their
// degree prefix, claim bitmap cleared, visited updated), for the dense claim
// bitmaps such steps leave.  A CTA takes 256 bitmap words (8192 vertices) at
// a time and first copies their 8193 offsets into shared memory with
// coalesced loads; each thread then reads the degrees of its word's claimed
// vertices from there, instead of a chain of two random offset loads per
// claimed vertex, twice.  (The copy is skipped for a tile without claims.)
constexpr int kSweepOffs = kThreads * 32 + 1;
__device__ __forceinline__ int sweep_slot(int i) { return (i >> 5) * 33 + (i & 31); }

template <typename OffT>
__global__ void __launch_bounds__(kThreads) k_sweep(Bufs<OffT> b) {
  static_assert(sizeof(OffT) == 4, "the shared tile holds 32-bit offsets");
  __shared__ OffT so[kThreads * 33 + 1];   // padded: thread t's 33 offsets at t*33
  __shared__ unsigned long long warp_tot[kWarpsPerCta];
  __shared__ unsigned long long cta_base;
  DevState* st = b.st;
  const int dst = st->cur ^ 1;
  uint32_t* claim = st->parity ? b.bm1 : b.bm0;
  int32_t* qv_out = dst ? b.qv1 : b.qv0;
  OffT* qs_out = dst ? b.qs1 : b.qs0;
  const OffT* __restrict__ off = b.off;
  const int shift = b.shift;
  const int64_t W = b.W, n = b.n;
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const unsigned long long emask = (1ull << shift) - 1;
  const int64_t span = (int64_t)gridDim.x * blockDim.x;
  for (int64_t w0 = (int64_t)blockIdx.x * blockDim.x; w0 < W; w0 += span) {
    const int64_t w = w0 + threadIdx.x;
    uint32_t bits = 0;
    if (w < W) {
      bits = claim[w];
      if (bits) {
        claim[w] = 0;
        b.visited[w] |= bits;
      }
    }
    if (!__syncthreads_or(bits != 0)) continue;
    const int64_t v0 = w0 << 5;
    for (int i = threadIdx.x; i < kSweepOffs; i += kThreads) {
      const int64_t v = v0 + i;
      so[sweep_slot(i)] = off[v < n ? v : n];   // ids past n: degree 0
    }
    __syncthreads();
    const int t0 = threadIdx.x << 5;
    unsigned long long degsum = 0;
    for (uint32_t x = bits; x; x &= x - 1) {
      const int j = __ffs(x) - 1;
      degsum += (unsigned long long)(so[sweep_slot(t0 + j + 1)] - so[sweep_slot(t0 + j)]);
    }
    const unsigned long long mine = ((unsigned long long)__popc(bits) << shift) + degsum;
    const unsigned long long inc = warp_inclusive_sum(mine, lane);
    if (lane == 31) warp_tot[wib] = inc;
    __syncthreads();
    if (threadIdx.x == 0) {
      unsigned long long t = 0;
      for (int i = 0; i < kWarpsPerCta; i++) {
        const unsigned long long x = warp_tot[i];
        warp_tot[i] = t;
        t += x;
      }
      cta_base = t ? atomicAdd(&b.ctr->qpacked[dst], t) : 0;
    }
    __syncthreads();
    if (bits) {
      const unsigned long long at = cta_base + warp_tot[wib] + inc - mine;
      uint64_t qpos = at >> shift;
      uint64_t epos = at & emask;
      for (uint32_t x = bits; x; x &= x - 1) {
        const int j = __ffs(x) - 1;
        qv_out[qpos] = (int32_t)((w << 5) + j);
        qs_out[qpos] = (OffT)epos;
        qpos++;
        epos += (uint64_t)(so[sweep_slot(t0 + j + 1)] - so[sweep_slot(t0 + j)]);
      }
    }
    __syncthreads();
  }
  stamp_end(st);
}

// ---------------------------------------------------------------------------
// Graph upload helpers.
template <typename OffT>
__global__ void k_narrow_offsets(const int64_t* __restrict__ in, OffT* __restrict__ out,
                                 int64_t count) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count;
       i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (OffT)in[i];
}

// head[u] = (first, second) neighbour of u in sorted order, -1 past its
// degree: the bottom-up step's first round of probes reads these 8 bytes,
// which lie next to those of the vertices the warp's other lanes take,
// instead of a 32-byte sector of nbr per vertex.
template <typename OffT>
__global__ void k_heads(int64_t n, const OffT* __restrict__ off, const int32_t* __restrict__ nbr,
                        int2* __restrict__ head) {
  for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < n;
       u += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t a = (uint64_t)off[u], e = (uint64_t)off[u + 1];
    head[u] = make_int2(a < e ? nbr[a] : -1, a + 1 < e ? nbr[a + 1] : -1);
  }
}

// iso bit = degree 0 or id >= n: never visited, never scanned.
template <typename OffT>
__global__ void k_iso_mask(int64_t n, int64_t W, const OffT* __restrict__ off,
                           uint32_t* __restrict__ iso) {
  for (int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; w < W;
       w += (int64_t)gridDim.x * blockDim.x) {
    uint32_t m = 0;
    for (int i = 0; i < 32; i++) {
      const int64_t u = (w << 5) + i;
      if (u >= n || off[u + 1] == off[u]) m |= 1u << i;
    }
    iso[w] = m;
  }
}

}  // namespace gbbfs
