// Device side of the batched multi-source BFS (sm_103a).
//
// Layout in HBM (n vertices, W = ceil(n/32), L = lane word of 32 or 64 bits):
//   visit      L[n]     bit i set once source i has reached v
//   fr0/fr1    L[n]     frontier of level l in fr[l & 1]: bit i set if v is in
//                       the frontier of source i
//   fbits0/1   u32[W]   union of all lanes of fr[l & 1] (v has fr != 0); tested
//                       before fr[v] is read, so neighbours outside every
//                       frontier cost one L2-resident bit instead of a word
//   acc        L[n]     bits merged by atomics (top-down levels and hubs)
//   q0/q1      int32    top-down queue of a frontier and qc0/qc1, the first
//                       work chunk of each entry
//   tq         int32    vertices whose acc received bits in this level
//   hubs       int32    vertices of degree > kMsHubDeg, with their chunk prefix
//   depth      D[k][n]  per-source depth, [source][vertex] order
//
// One persistent cooperative kernel runs all levels of a batch.  Level l
// reads the frontier in fr[l & 1] and writes the next one to fr[(l+1) & 1]:
//   top-down (frontier summed degree <= m / alpha): the next buffer is
//     cleared densely; a warp per kMsTdChunk-edge work item of a queued
//     frontier vertex ORs fr[u] & ~visit[v] into acc[v] (atomicOr) and queues
//     first touches; after a grid barrier every touched vertex is installed
//     (visit, depth, next frontier, next queue).  The queue of a frontier
//     that a bottom-up level produced is first compacted from its fbits.
//   bottom-up: a warp per 32 consecutive vertices.  The concatenated
//     adjacency of the tile's unfinished vertices of degree up to kMsSmall is
//     streamed 32 edges per lane-step into per-vertex words in shared
//     memory; vertices up to kMsHubDeg get the whole warp with early exit
//     once every lane is found.  The warp then writes visit, the depth rows
//     (coalesced per source), the next frontier words and their fbits word
//     densely, so no clear or install pass follows.  Hub adjacency is cut
//     into kMsHubChunk-edge items merged into acc and installed after the
//     barrier.
// Grid barriers spin on a generation word with a time bound; a barrier that
// runs out sets an error word and every block returns.
#pragma once

#include "bfs_common.cuh"

namespace gbbfs {

constexpr int kMsTimedLevels = 64;   // levels whose end time and direction are kept
// Phases whose warp time the kernel accounts (SM cycles summed over warps).
enum MsPhase {
  kPhTopDown = 0, kPhSmall, kPhMid, kPhWrite, kPhHub, kPhClear, kPhInstall, kPhBarrier,
  kMsPhases
};
constexpr int kMsSmall = 256;
constexpr int kMsHubDeg = 2048;
constexpr int kMsHubChunk = 2048;
constexpr int kMsTdChunk = 1024;

struct MsCtl {
  unsigned long long q_packed[2];   // top-down queue q[i]: (count << shift) | chunks
  unsigned long long f_count[3];    // frontier of level l: vertices (slot l % 3)
  unsigned long long f_edges[3];    //   and their summed degree
  unsigned long long touched[3];    // tq entries of level l (slot l % 3)
  unsigned int bar_count;
  unsigned int bar_gen;
  int error;
  int levels;
  unsigned long long t_begin, t_end;
  unsigned long long level_end[kMsTimedLevels];   // %globaltimer at the end of each level
  int level_bu[kMsTimedLevels];                    // 1 when the level ran bottom-up
  unsigned long long phase_cycles[kMsPhases];      // SM cycles per phase, summed over warps
};

template <typename OffT, typename LaneT, typename DepthT>
struct MsArgs {
  const OffT* off;
  const int32_t* nbr;
  int64_t n, m, W;
  LaneT* visit;
  LaneT* fr0;
  LaneT* fr1;
  LaneT* acc;
  uint32_t* fbits0;
  uint32_t* fbits1;
  int32_t* q0;
  int32_t* q1;
  uint32_t* qc0;
  uint32_t* qc1;
  int32_t* tq;
  const int32_t* hubs;
  const uint32_t* hub_chunk;   // nhubs + 1 entries
  int64_t nhubs;
  DepthT* depth;
  const int32_t* sources;
  MsCtl* ctl;
  int k;
  int shift;
  int alpha;
  unsigned long long limit_ns;
};

template <typename LaneT>
__device__ __forceinline__ LaneT atomic_or_lane(LaneT* p, LaneT v) {
  if constexpr (sizeof(LaneT) == 8)
    return (LaneT)atomicOr(reinterpret_cast<unsigned long long*>(p), (unsigned long long)v);
  else
    return (LaneT)atomicOr(reinterpret_cast<unsigned int*>(p), (unsigned int)v);
}

template <typename LaneT>
__device__ __forceinline__ LaneT ld_lane(const LaneT* p) {
  if constexpr (sizeof(LaneT) == 8)
    return (LaneT)__ldcg(reinterpret_cast<const unsigned long long*>(p));
  else
    return (LaneT)__ldcg(reinterpret_cast<const unsigned int*>(p));
}

template <typename LaneT>
__device__ __forceinline__ LaneT warp_or(LaneT x) {
#pragma unroll
  for (int o = 16; o; o >>= 1) x |= shfl(x, (int)(threadIdx.x & 31) ^ o);
  return x;
}

template <typename LaneT>
__device__ __forceinline__ int lowest_bit(LaneT x) {
  if constexpr (sizeof(LaneT) == 8)
    return __ffsll((long long)x) - 1;
  else
    return __ffs((int)x) - 1;
}

__device__ __forceinline__ bool in_frontier(const uint32_t* fbits, int32_t u) {
  return (__ldcg(fbits + (u >> 5)) >> (u & 31)) & 1u;
}

// Grid-wide barrier with a time bound.  Returns false (and every later call
// returns false at once) when any block has given up.
__device__ __forceinline__ bool grid_barrier(MsCtl* c, unsigned nblocks,
                                             unsigned long long limit_ns) {
  __syncthreads();
  __shared__ int ok;
  if (threadIdx.x == 0) {
    ok = 1;
    volatile unsigned* vgen = &c->bar_gen;
    const unsigned gen = *vgen;
    __threadfence();
    if (atomicAdd(&c->bar_count, 1u) == nblocks - 1) {
      c->bar_count = 0;
      __threadfence();
      atomicAdd(&c->bar_gen, 1u);
    } else {
      const unsigned long long t0 = globaltimer();
      while (*vgen == gen) {
        if (*(volatile int*)&c->error) {
          ok = 0;
          break;
        }
        if (globaltimer() - t0 > limit_ns) {
          atomicExch(&c->error, GBBFS_ERR_TIMEOUT);
          ok = 0;
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
    if (*(volatile int*)&c->error) ok = 0;
  }
  __syncthreads();
  return ok != 0;
}

// Depth `level` for every source bit of `nb` at vertex v.  Called by a whole
// warp; lanes with consecutive v write consecutive entries of each row.
template <typename LaneT, typename DepthT>
__device__ __forceinline__ void write_depths(DepthT* depth, int64_t n, int64_t v, LaneT nb,
                                             int level) {
  LaneT any = warp_or(nb);
  while (any) {
    const int i = lowest_bit(any);
    any &= any - 1;
    if ((nb >> i) & 1) depth[(int64_t)i * n + v] = (DepthT)level;
  }
}

// Append the lanes with `keep` to a vertex list (one atomic per warp).
__device__ __forceinline__ void warp_append(unsigned long long* counter, int32_t* list,
                                            bool keep, int32_t v) {
  const int lane = threadIdx.x & 31;
  const unsigned km = __ballot_sync(kFull, keep);
  if (km) {
    unsigned long long base = 0;
    if (lane == 0) base = atomicAdd(counter, (unsigned long long)__popc(km));
    base = shfl(base, 0);
    if (keep) list[base + __popc(km & ((1u << lane) - 1))] = v;
  }
}

// Append the lanes with `keep` to a top-down queue with its work-chunk
// prefix, and add them to the frontier totals.  Whole warp.
__device__ __forceinline__ void warp_enqueue(unsigned long long* packed, int32_t* q, uint32_t* qc,
                                             unsigned long long* f_count,
                                             unsigned long long* f_edges, int shift, bool keep,
                                             int32_t v, unsigned long long deg) {
  const int lane = threadIdx.x & 31;
  const unsigned km = __ballot_sync(kFull, keep);
  if (!km) return;
  const unsigned long long emask = (1ull << shift) - 1;
  const unsigned long long chunks = keep ? (deg + kMsTdChunk - 1) / kMsTdChunk : 0;
  const unsigned long long mine = keep ? (1ull << shift) + chunks : 0;
  const unsigned long long inc = warp_inclusive_sum(mine, lane);
  unsigned long long dsum = keep ? deg : 0;
#pragma unroll
  for (int o = 16; o; o >>= 1) dsum += __shfl_xor_sync(kFull, dsum, o);
  unsigned long long base = 0;
  if (lane == 31) {
    base = atomicAdd(packed, inc);
    atomicAdd(f_count, (unsigned long long)__popc(km));
    atomicAdd(f_edges, dsum);
  }
  base = shfl(base, 31);
  if (keep) {
    const unsigned long long at = base + inc - mine;
    q[at >> shift] = v;
    qc[at >> shift] = (uint32_t)(at & emask);
  }
}

// OR of fr[u] over the neighbours nbr[b..e) of one vertex, by the whole warp:
// 4 x 32 neighbours per round, every load of a round issued before any is
// used, early exit once (result | vis) covers every lane.
template <typename LaneT>
__device__ __forceinline__ LaneT warp_gather_or(const int32_t* nbr, const uint32_t* fbits,
                                                const LaneT* fr, uint64_t b, uint64_t e,
                                                LaneT vis, LaneT all) {
  const int lane = threadIdx.x & 31;
  LaneT got = 0;
  for (uint64_t e0 = b; e0 < e; e0 += 128) {
    int32_t u[4];
#pragma unroll
    for (int r = 0; r < 4; r++) {
      const uint64_t idx = e0 + 32 * r + lane;
      u[r] = idx < e ? __ldg(nbr + idx) : -1;
    }
    bool in[4];
#pragma unroll
    for (int r = 0; r < 4; r++) in[r] = u[r] >= 0 && in_frontier(fbits, u[r]);
    LaneT x = 0;
#pragma unroll
    for (int r = 0; r < 4; r++)
      if (in[r]) x |= ld_lane(fr + u[r]);
    got |= warp_or(x);
    if (((got | vis) & all) == all) break;
  }
  return got;
}

template <typename OffT, typename LaneT, typename DepthT, int kBatchN>
__global__ void __launch_bounds__(kThreads) k_msbfs(MsArgs<OffT, LaneT, DepthT> a) {
  __shared__ LaneT tile_acc[kWarpsPerCta][32];
  __shared__ unsigned long long blk_count, blk_edges;
  __shared__ unsigned long long ph_acc[kMsPhases];
  MsCtl* c = a.ctl;
  const unsigned nblocks = gridDim.x;
  const int lane = threadIdx.x & 31;
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t nthreads = (int64_t)gridDim.x * blockDim.x;
  const int64_t warp = tid >> 5;
  const int64_t nwarps = nthreads >> 5;
  const unsigned long long emask = (1ull << a.shift) - 1;
  const LaneT all = a.k >= (int)(8 * sizeof(LaneT)) ? (LaneT)~(LaneT)0
                                                     : (LaneT)(((LaneT)1 << a.k) - 1);
  const int max_level = sizeof(DepthT) == 1 ? 254 : 0x7ffffffe;
  const int64_t hub_chunks = a.nhubs ? (int64_t)a.hub_chunk[a.nhubs] : 0;
  if (tid == 0) c->t_begin = globaltimer();
  // Warp time per phase (for the stats): lane 0 of each warp adds its SM
  // cycles since the previous mark.
  if (threadIdx.x < kMsPhases) ph_acc[threadIdx.x] = 0;
  __syncthreads();
  long long ph_t = clock64();
  auto mark = [&](int phase) {
    const long long now = clock64();
    if (lane == 0) atomicAdd(&ph_acc[phase], (unsigned long long)(now - ph_t));
    ph_t = now;
  };
  // Grid barrier; the time spent waiting in it is its own phase.
  auto barrier = [&]() {
    const bool ok = grid_barrier(c, nblocks, a.limit_ns);
    mark(kPhBarrier);
    return ok;
  };

  // Level 1's frontier: lane i starts at sources[i] with depth 0.  A vertex
  // that is the source of several lanes is queued once.
  if (blockIdx.x == 0 && threadIdx.x < a.k) {
    const int i = threadIdx.x;
    const int32_t s = a.sources[i];
    const LaneT bit = (LaneT)1 << i;
    atomic_or_lane(a.visit + s, bit);
    a.depth[(int64_t)i * a.n + s] = 0;
    if (atomic_or_lane(a.fr1 + s, bit) == 0) {
      const unsigned long long deg = (unsigned long long)(a.off[s + 1] - a.off[s]);
      const unsigned long long chunks = (deg + kMsTdChunk - 1) / kMsTdChunk;
      const unsigned long long at = atomicAdd(&c->q_packed[1], (1ull << a.shift) + chunks);
      a.q1[at >> a.shift] = s;
      a.qc1[at >> a.shift] = (uint32_t)(at & emask);
      atomicAdd(&c->f_count[1], 1ull);
      atomicAdd(&c->f_edges[1], deg);
      atomicOr(a.fbits1 + (s >> 5), 1u << (s & 31));
    }
  }
  if (!barrier()) return;
  if (tid == 0) c->level_end[0] = globaltimer();

  bool have_queue = true;   // the top-down queue of the current frontier exists
  for (int level = 1;; level++) {
    const int cur = level & 1, nxt = cur ^ 1;
    const int64_t F = (int64_t)__ldcg(&c->f_count[level % 3]);
    const unsigned long long E = __ldcg(&c->f_edges[level % 3]);
    if (F == 0) break;
    if (level > max_level) {
      if (tid == 0) atomicExch(&c->error, GBBFS_ERR_ARG);
      break;
    }
    const LaneT* fr = cur ? a.fr1 : a.fr0;
    LaneT* frn = cur ? a.fr0 : a.fr1;
    const uint32_t* fb = cur ? a.fbits1 : a.fbits0;
    uint32_t* fbn = cur ? a.fbits0 : a.fbits1;
    int32_t* q = cur ? a.q1 : a.q0;
    uint32_t* qc = cur ? a.qc1 : a.qc0;
    int32_t* qn = cur ? a.q0 : a.q1;
    uint32_t* qcn = cur ? a.qc0 : a.qc1;
    unsigned long long* touched = &c->touched[level % 3];
    unsigned long long* nf_count = &c->f_count[(level + 1) % 3];
    unsigned long long* nf_edges = &c->f_edges[(level + 1) % 3];
    const bool bottom_up = E > (unsigned long long)(a.m / a.alpha);
    // Slots this level does not touch are reset for the levels ahead.
    if (tid == 0) {
      c->f_count[(level + 2) % 3] = 0;
      c->f_edges[(level + 2) % 3] = 0;
      c->touched[(level + 2) % 3] = 0;
      c->q_packed[nxt] = 0;
    }

    if (!bottom_up) {
      if (!have_queue) {
        // The frontier came from a bottom-up level: queue it from its fbits.
        // (q_packed[cur] was reset by the previous level.)
        for (int64_t w0 = warp << 5; w0 < a.W; w0 += nwarps << 5) {
          const int64_t w = w0 + lane;
          uint32_t bits = w < a.W ? __ldcg(fb + w) : 0u;
          while (__any_sync(kFull, bits != 0)) {
            const bool keep = bits != 0;
            int32_t v = 0;
            unsigned long long deg = 0;
            if (keep) {
              v = (int32_t)((w << 5) + (__ffs(bits) - 1));
              bits &= bits - 1;
              deg = (unsigned long long)(a.off[v + 1] - a.off[v]);
            }
            const unsigned long long chunks = keep ? (deg + kMsTdChunk - 1) / kMsTdChunk : 0;
            const unsigned long long mine = keep ? (1ull << a.shift) + chunks : 0;
            const unsigned long long inc = warp_inclusive_sum(mine, lane);
            unsigned long long base = 0;
            if (lane == 31) base = atomicAdd(&c->q_packed[cur], inc);
            base = shfl(base, 31);
            if (keep) {
              const unsigned long long at = base + inc - mine;
              q[at >> a.shift] = v;
              qc[at >> a.shift] = (uint32_t)(at & emask);
            }
          }
        }
        mark(kPhInstall);
        if (!barrier()) return;
      }
      const unsigned long long qp = __ldcg(&c->q_packed[cur]);
      const int64_t C = (int64_t)(qp & emask);
      const int64_t Q = (int64_t)(qp >> a.shift);
      // The next frontier buffers are written sparsely: clear them first.
      for (int64_t v = tid; v < a.n; v += nthreads) frn[v] = 0;
      for (int64_t w = tid; w < a.W; w += nthreads) fbn[w] = 0;
      mark(kPhClear);
      // Top-down: a warp per work chunk of one frontier vertex.
      for (int64_t ch = warp; ch < C; ch += nwarps) {
        int64_t lo = 0, hi = Q - 1;
        while (lo < hi) {
          const int64_t mid = (lo + hi + 1) >> 1;
          if ((int64_t)qc[mid] <= ch) lo = mid; else hi = mid - 1;
        }
        const int32_t u = q[lo];
        const LaneT f = ld_lane(fr + u);
        const uint64_t b = (uint64_t)a.off[u] + (uint64_t)(ch - qc[lo]) * kMsTdChunk;
        const uint64_t ue = (uint64_t)a.off[u + 1];
        const uint64_t e = b + kMsTdChunk < ue ? b + kMsTdChunk : ue;
        for (uint64_t e0 = b; e0 < e; e0 += 128) {
          int32_t v[4];
          LaneT vis[4];
#pragma unroll
          for (int r = 0; r < 4; r++) {
            const uint64_t idx = e0 + 32 * r + lane;
            v[r] = idx < e ? __ldg(a.nbr + idx) : -1;
          }
#pragma unroll
          for (int r = 0; r < 4; r++) vis[r] = v[r] >= 0 ? ld_lane(a.visit + v[r]) : all;
          bool first[4];
#pragma unroll
          for (int r = 0; r < 4; r++) {
            const LaneT nb = f & ~vis[r];
            first[r] = v[r] >= 0 && nb && atomic_or_lane(a.acc + v[r], nb) == 0;
          }
#pragma unroll
          for (int r = 0; r < 4; r++) warp_append(touched, a.tq, first[r], v[r]);
        }
      }
      mark(kPhTopDown);
      if (!barrier()) return;
      // Install every touched vertex.
      const int64_t T = (int64_t)__ldcg(touched);
      for (int64_t i0 = warp << 5; i0 < T; i0 += nwarps << 5) {
        const int64_t i = i0 + lane;
        int32_t v = 0;
        LaneT nb = 0;
        unsigned long long deg = 0;
        if (i < T) {
          v = a.tq[i];
          nb = a.acc[v];
          a.acc[v] = 0;
          const LaneT vis = a.visit[v];
          nb &= ~vis;
          if (nb) {
            a.visit[v] = vis | nb;
            for (LaneT x = nb; x; x &= x - 1)
              a.depth[(int64_t)lowest_bit(x) * a.n + v] = (DepthT)level;
            frn[v] = nb;
            atomicOr(fbn + (v >> 5), 1u << (v & 31));
            deg = (unsigned long long)(a.off[v + 1] - a.off[v]);
          }
        }
        warp_enqueue(&c->q_packed[nxt], qn, qcn, nf_count, nf_edges, a.shift, nb != 0, v, deg);
      }
      have_queue = true;
      mark(kPhInstall);
      if (!barrier()) return;
    } else {
      // Bottom-up over tiles of 32 consecutive vertices.
      if (threadIdx.x == 0) {
        blk_count = 0;
        blk_edges = 0;
      }
      __syncthreads();
      unsigned long long my_count = 0, my_edges = 0;
      for (int64_t v0 = warp << 5; v0 < a.n; v0 += nwarps << 5) {
        const int64_t v = v0 + lane;
        LaneT vis = all;
        uint64_t b = 0, e = 0;
        if (v < a.n) {
          vis = ld_lane(a.visit + v);
          b = (uint64_t)a.off[v];
          e = (uint64_t)a.off[v + 1];
        }
        const bool need = ((vis & all) != all) && e > b;
        const uint64_t deg = e - b;
        LaneT nb = 0;
        // Small vertices: the warp streams their concatenated adjacency,
        // kBatchN/2 x 32 edges per round, loads issued together; bits are
        // ORed into per-vertex words in shared memory.
        const bool small = need && deg <= (uint64_t)kMsSmall;
        const unsigned sd = small ? (unsigned)deg : 0u;
        const unsigned sincl = warp_inclusive_sum(sd, lane);
        const unsigned sstart = sincl - sd;
        const unsigned stotal = __shfl_sync(kFull, sincl, 31);
        LaneT* tacc = tile_acc[threadIdx.x >> 5];
        tacc[lane] = 0;
        __syncwarp();
        constexpr int kR = kBatchN / 2 > 0 ? kBatchN / 2 : 1;
        for (unsigned t0 = 0; t0 < stotal; t0 += 32 * kR) {
          int seg[kR];
          int32_t u[kR];
#pragma unroll
          for (int r = 0; r < kR; r++) {
            const unsigned t = t0 + 32 * r + lane;
            const unsigned tc = t < stotal ? t : stotal - 1;
            // last vertex of the tile whose stream starts at or before tc
            // (every lane takes part in the shuffles)
            int lo = 0;
#pragma unroll
            for (int step = 16; step; step >>= 1) {
              const unsigned st = __shfl_sync(kFull, sstart, lo + step);
              if (st <= tc) lo += step;
            }
            const uint64_t bs = shfl(b, lo);
            const unsigned ss = __shfl_sync(kFull, sstart, lo);
            seg[r] = t < stotal ? lo : -1;
            u[r] = t < stotal ? __ldg(a.nbr + bs + (t - ss)) : -1;
          }
          bool in[kR];
#pragma unroll
          for (int r = 0; r < kR; r++) in[r] = u[r] >= 0 && in_frontier(fb, u[r]);
#pragma unroll
          for (int r = 0; r < kR; r++) {
            if (in[r]) {
              const LaneT x = ld_lane(fr + u[r]);
              if (x) atomic_or_lane(tacc + seg[r], x);
            }
          }
        }
        __syncwarp();
        if (small) nb = tacc[lane] & ~vis & all;
        mark(kPhSmall);
        unsigned mids = __ballot_sync(kFull, need && deg > kMsSmall && deg <= kMsHubDeg);
        while (mids) {
          const int t = __ffs(mids) - 1;
          mids &= mids - 1;
          const LaneT vt = shfl(vis, t);
          const uint64_t bt = shfl(b, t), et = shfl(e, t);
          const LaneT got = warp_gather_or(a.nbr, fb, fr, bt, et, vt, all);
          if (lane == t) nb = got & ~vt & all;
        }
        mark(kPhMid);
        // Dense writes of this tile: visit, depths, next frontier and fbits.
        if (nb) a.visit[v] = vis | nb;
        if (v < a.n) frn[v] = nb;
        const unsigned nm = __ballot_sync(kFull, nb != 0);
        if (lane == 0 && (v0 >> 5) < a.W) fbn[v0 >> 5] = nm;
        write_depths(a.depth, a.n, v, nb, level);
        if (nb) {
          my_count++;
          my_edges += deg;
        }
        mark(kPhWrite);
      }
      // Hubs: their adjacency cut into work items, merged by atomicOr.
      for (int64_t hc = warp; hc < hub_chunks; hc += nwarps) {
        int64_t lo = 0, hi = a.nhubs - 1;
        while (lo < hi) {
          const int64_t mid = (lo + hi + 1) >> 1;
          if ((int64_t)a.hub_chunk[mid] <= hc) lo = mid; else hi = mid - 1;
        }
        const int32_t v = a.hubs[lo];
        const LaneT vis = ld_lane(a.visit + v);
        if ((vis & all) == all) continue;
        const uint64_t b = (uint64_t)a.off[v] + (uint64_t)(hc - a.hub_chunk[lo]) * kMsHubChunk;
        const uint64_t ve = (uint64_t)a.off[v + 1];
        const uint64_t e = b + kMsHubChunk < ve ? b + kMsHubChunk : ve;
        const LaneT got = warp_gather_or(a.nbr, fb, fr, b, e, vis, all);
        const LaneT part = got & ~vis & all;
        bool first = false;
        if (lane == 0 && part) first = atomic_or_lane(a.acc + v, part) == 0;
        warp_append(touched, a.tq, first, v);
      }
      mark(kPhHub);
      // One pair of counter atomics per block.
#pragma unroll
      for (int o = 16; o; o >>= 1) {
        my_count += __shfl_xor_sync(kFull, my_count, o);
        my_edges += __shfl_xor_sync(kFull, my_edges, o);
      }
      if (lane == 0) {
        atomicAdd(&blk_count, my_count);
        atomicAdd(&blk_edges, my_edges);
      }
      __syncthreads();
      if (threadIdx.x == 0 && blk_count) {
        atomicAdd(nf_count, blk_count);
        atomicAdd(nf_edges, blk_edges);
      }
      if (!barrier()) return;
      // Install the hubs that received bits (their words were written as 0
      // by the tile pass).
      const int64_t T = (int64_t)__ldcg(touched);
      if (T > 0) {
        for (int64_t i = tid; i < T; i += nthreads) {
          const int32_t v = a.tq[i];
          LaneT nb = a.acc[v];
          a.acc[v] = 0;
          const LaneT vis = a.visit[v];
          nb &= ~vis;
          if (nb) {
            a.visit[v] = vis | nb;
            for (LaneT x = nb; x; x &= x - 1)
              a.depth[(int64_t)lowest_bit(x) * a.n + v] = (DepthT)level;
            frn[v] = nb;
            atomicOr(fbn + (v >> 5), 1u << (v & 31));
            atomicAdd(nf_count, 1ull);
            atomicAdd(nf_edges, (unsigned long long)(a.off[v + 1] - a.off[v]));
          }
        }
        mark(kPhInstall);
        if (!barrier()) return;
      }
      have_queue = false;
    }
    if (tid == 0) {
      c->levels = level;
      if (level < kMsTimedLevels) {
        c->level_end[level] = globaltimer();
        c->level_bu[level] = bottom_up ? 1 : 0;
      }
    }
  }
  if (tid == 0) c->t_end = globaltimer();
  __syncthreads();
  if (threadIdx.x < kMsPhases) atomicAdd(&c->phase_cycles[threadIdx.x], ph_acc[threadIdx.x]);
}

}  // namespace gbbfs
