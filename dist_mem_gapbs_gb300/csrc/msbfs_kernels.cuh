// Device side of the batched multi-source BFS (sm_103a).
//
// Layout in HBM (n vertices, W = ceil(n/32), L = lane word of 32, 64, 128 or
// 256 bits; a 256-bit word is one 32-byte DRAM sector):
//   visit      L[n]     bit i set once source i has reached v
//   fr0/fr1    L[n]     frontier of level l in fr[l & 1]: bit i set if v is in
//                       the frontier of source i
//   fbits0/1   u32[W]   union of all lanes of fr[l & 1] (v has fr != 0); tested
//                       before fr[v] is read, so neighbours outside every
//                       frontier cost one L2-resident bit instead of a word
//   acc        L[n]     bits merged by atomics (top-down levels and hubs)
//   q0/q1      int32    top-down queue of a frontier (vertices with edges) and
//   qe0/qe1    u64      the position of each entry's first edge in the
//                       concatenated adjacency of the queue
//   tq         int32    vertices whose acc received bits in this level
//   hubs       int32    vertices of degree > kMsHubDeg, with their chunk prefix
//   lvl        u32[n]   depth log: the levels of up to kLogSlots entries per
//   lmask      L[4n]    vertex (0xff = empty) and the lanes each entry found
//   spill      u8[n]    1 if some of the vertex's depths are in the rows instead
//   tflag      u32[n]   touched in this level (128- and 256-lane words)
//   depth      D[k][s]  rows in search order (stride s) for what the log cannot
//                       hold: a source's own depth 0, a fifth level, levels
//                       above 254; k_depth_decode writes the rows callers see
//                       in original vertex order from the log and these
//
// One persistent cooperative kernel runs all levels of a batch.  Level l
// reads the frontier in fr[l & 1] and writes the next one to fr[(l+1) & 1]:
//   top-down (frontier summed degree <= m / alpha): warps take spans of
//     kMsTdSpan consecutive edges of the queue's concatenated adjacency and
//     OR fr[u] & ~visit[v] into acc[v] (atomicOr).  After a grid barrier the
//     next frontier is installed (visit, depth, next frontier words): for a
//     frontier with few edges from a list of first touches into a cleared
//     buffer, queueing the vertices as they are installed; for one with
//     more than n/16 edges by a pass over all vertices that writes every
//     word.  A frontier that was written densely is queued from its fbits
//     when a top-down level needs it.
//   bottom-up: a warp per tile of 32 consecutive vertices, tiles handed out
//     in work units from a counter (up to kMsGrab tiles, fewer where the
//     tiles hold many edges).  The concatenated adjacency of the
//     tile's unfinished vertices of degree below kMsSmall is streamed 32
//     edges per lane-step into per-vertex words in shared memory; vertices
//     up to kMsHubDeg get the whole warp with early exit once every lane is
//     found.  The warp then writes visit, the depth log entries, the next
//     frontier words and their fbits word densely, so no clear or install
//     pass follows.  Hub adjacency is cut
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
constexpr int kMsSmall = 32;        // bottom-up: lower degrees share a streamed pass
// Vertices of at least this degree are numbered first in the search, in
// buckets by the bit length of the degree, longest first; the others keep
// their relative order after them (with 1: isolated vertices last).
#ifndef GBBFS_MS_ORDER_DEG
#define GBBFS_MS_ORDER_DEG 1
#endif
constexpr int kMsOrderDeg = GBBFS_MS_ORDER_DEG;
constexpr int kDepthTile = 128;     // rows in search order: stride a multiple of this
constexpr int kDecodeTile = 64;     // bytes of each row per block of the depth decode
constexpr int kMsMaxLanes = 256;    // sources per batch at most (depth record length)
constexpr int kMsGrab = 8;          // tiles of 32 vertices in a bottom-up work unit at most
constexpr int kMsUnitEdges = 4096;  // a unit also ends once its tiles hold this many edges
constexpr int kMsHubDeg = 4096;
constexpr int kMsHubChunk = 2048;
constexpr int kMsTdSpan = 2048;     // edges per warp span of a top-down level

struct MsCtl {
  unsigned long long q_packed[2];   // top-down queue q[i]: (count << shift) | chunks
  unsigned long long f_count[3];    // frontier of level l: vertices (slot l % 3)
  unsigned long long f_edges[3];    //   and their summed degree
  unsigned long long touched[3];    // tq entries of level l (slot l % 3)
  unsigned long long tile_next[3];  // next bottom-up tile of level l (slot l % 3)
  unsigned int bar_count;
  unsigned int bar_gen;
  int error;
  int levels;
  unsigned long long t_begin, t_end;
  unsigned long long level_end[kMsTimedLevels];   // %globaltimer at the end of each level
  int level_bu[kMsTimedLevels];                    // 1 when the level ran bottom-up
  unsigned long long level_f[kMsTimedLevels];      // frontier vertices of each level
  unsigned long long level_e[kMsTimedLevels];      //   and their summed degree
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
  uint64_t* qe0;   // first edge of each queue entry in the queue's concatenated adjacency
  uint64_t* qe1;
  int32_t* tq;
  const int32_t* hubs;
  const int32_t* unit_tile;  // bottom-up work unit u = tiles [unit_tile[u], unit_tile[u+1])
  int64_t nunits;
  const uint32_t* hub_chunk;   // nhubs + 1 entries
  int64_t nhubs;
  DepthT* depth;             // [source][search-order vertex] rows: entries the log cannot hold
  int64_t dstride;           // row stride of depth (elements, a multiple of kDepthTile)
  uint32_t* lvl;             // per vertex: levels of its kLogSlots log entries (0xff = empty)
  LaneT* lmask;              // per vertex: the lanes each log entry found
  uint8_t* spill;            // per vertex: 1 if some depths are in the rows instead
  uint32_t* tflag;           // per vertex: touched in this level (128/256-lane words)
  const int32_t* nsrc;      // sources in this batch (device, set per launch)
  const int32_t* sources;   // original vertex ids
  const int32_t* perm;      // original id -> search order id
  MsCtl* ctl;
  int shift;
  int alpha;
  unsigned long long limit_ns;
};

// A lane word of 128 sources (two 64-bit halves, lo = sources 0..63).
struct __align__(16) Lane128 {
  unsigned long long lo, hi;
  Lane128() = default;
  __host__ __device__ constexpr Lane128(unsigned long long x) : lo(x), hi(0) {}
  __host__ __device__ constexpr Lane128(unsigned long long l, unsigned long long h) : lo(l), hi(h) {}
  __host__ __device__ explicit operator bool() const { return (lo | hi) != 0; }
};
__host__ __device__ inline Lane128 operator&(Lane128 a, Lane128 b) { return {a.lo & b.lo, a.hi & b.hi}; }
__host__ __device__ inline Lane128 operator|(Lane128 a, Lane128 b) { return {a.lo | b.lo, a.hi | b.hi}; }
__host__ __device__ inline Lane128 operator~(Lane128 a) { return {~a.lo, ~a.hi}; }
__host__ __device__ inline Lane128& operator&=(Lane128& a, Lane128 b) { return a = a & b; }
__host__ __device__ inline Lane128& operator|=(Lane128& a, Lane128 b) { return a = a | b; }
__host__ __device__ inline bool operator==(Lane128 a, Lane128 b) { return a.lo == b.lo && a.hi == b.hi; }
__host__ __device__ inline bool operator!=(Lane128 a, Lane128 b) { return !(a == b); }

__device__ __forceinline__ Lane128 shfl(Lane128 x, int src) {
  return {shfl(x.lo, src), shfl(x.hi, src)};
}

// A lane word of 256 sources (q[0] = sources 0..63): one 32-byte sector, so
// a random frontier read fetches no bytes it does not use.  Indexes into q
// are compile-time constants everywhere (a run-time index would put the word
// in local memory).
struct __align__(32) Lane256 {
  unsigned long long q[4];
  Lane256() = default;
  __host__ __device__ constexpr Lane256(unsigned long long x) : q{x, 0ull, 0ull, 0ull} {}
  __host__ __device__ constexpr Lane256(unsigned long long a, unsigned long long b,
                                        unsigned long long c, unsigned long long d)
      : q{a, b, c, d} {}
  __host__ __device__ explicit operator bool() const { return (q[0] | q[1] | q[2] | q[3]) != 0; }
};
__host__ __device__ inline Lane256 operator&(Lane256 a, Lane256 b) {
  return {a.q[0] & b.q[0], a.q[1] & b.q[1], a.q[2] & b.q[2], a.q[3] & b.q[3]};
}
__host__ __device__ inline Lane256 operator|(Lane256 a, Lane256 b) {
  return {a.q[0] | b.q[0], a.q[1] | b.q[1], a.q[2] | b.q[2], a.q[3] | b.q[3]};
}
__host__ __device__ inline Lane256 operator~(Lane256 a) { return {~a.q[0], ~a.q[1], ~a.q[2], ~a.q[3]}; }
__host__ __device__ inline Lane256& operator&=(Lane256& a, Lane256 b) { return a = a & b; }
__host__ __device__ inline Lane256& operator|=(Lane256& a, Lane256 b) { return a = a | b; }
__host__ __device__ inline bool operator==(Lane256 a, Lane256 b) {
  return ((a.q[0] ^ b.q[0]) | (a.q[1] ^ b.q[1]) | (a.q[2] ^ b.q[2]) | (a.q[3] ^ b.q[3])) == 0;
}
__host__ __device__ inline bool operator!=(Lane256 a, Lane256 b) { return !(a == b); }

__device__ __forceinline__ Lane256 shfl(Lane256 x, int src) {
  return {shfl(x.q[0], src), shfl(x.q[1], src), shfl(x.q[2], src), shfl(x.q[3], src)};
}

// 64-bit word j (0..3) of a 256-lane word, j known only at run time.
__device__ __forceinline__ unsigned long long word64(const Lane256& x, int j) {
  return j < 2 ? (j == 0 ? x.q[0] : x.q[1]) : (j == 2 ? x.q[2] : x.q[3]);
}

// Lane-word helpers for the four widths (uint32, uint64, Lane128, Lane256).
template <typename LaneT>
__device__ __forceinline__ uint32_t word32(LaneT x, int h) {   // 32-bit word h
  if constexpr (sizeof(LaneT) == 32)
    return (uint32_t)(word64(x, h >> 1) >> (32 * (h & 1)));
  else if constexpr (sizeof(LaneT) == 16)
    return (uint32_t)((h < 2 ? x.lo : x.hi) >> (32 * (h & 1)));
  else
    return (uint32_t)((unsigned long long)x >> (32 * h));
}

template <typename LaneT>
__device__ __forceinline__ LaneT from_words(const uint32_t* w) {
  if constexpr (sizeof(LaneT) == 32)
    return Lane256(((unsigned long long)w[1] << 32) | w[0], ((unsigned long long)w[3] << 32) | w[2],
                   ((unsigned long long)w[5] << 32) | w[4], ((unsigned long long)w[7] << 32) | w[6]);
  else if constexpr (sizeof(LaneT) == 16)
    return Lane128(((unsigned long long)w[1] << 32) | w[0], ((unsigned long long)w[3] << 32) | w[2]);
  else if constexpr (sizeof(LaneT) == 8)
    return (LaneT)(((unsigned long long)w[1] << 32) | w[0]);
  else
    return (LaneT)w[0];
}

template <typename LaneT>
__device__ __forceinline__ bool lane_test(LaneT x, int i) {
  return (word32(x, i >> 5) >> (i & 31)) & 1u;
}

template <typename LaneT>
__device__ __forceinline__ LaneT lane_bit(int i) {
  if constexpr (sizeof(LaneT) == 32) {
    const unsigned long long b = 1ull << (i & 63);
    const int j = i >> 6;
    return Lane256(j == 0 ? b : 0ull, j == 1 ? b : 0ull, j == 2 ? b : 0ull, j == 3 ? b : 0ull);
  } else if constexpr (sizeof(LaneT) == 16)
    return i < 64 ? Lane128(1ull << i, 0) : Lane128(0, 1ull << (i - 64));
  else
    return (LaneT)((LaneT)1 << i);
}

// The k lowest lanes.
template <typename LaneT>
__device__ __forceinline__ LaneT lane_ones(int k) {
  if constexpr (sizeof(LaneT) == 32) {
    auto part = [k](int j) {
      return k >= 64 * (j + 1) ? ~0ull : k > 64 * j ? (1ull << (k - 64 * j)) - 1 : 0ull;
    };
    return Lane256(part(0), part(1), part(2), part(3));
  } else if constexpr (sizeof(LaneT) == 16)
    return Lane128(k >= 64 ? ~0ull : (1ull << k) - 1,
                   k >= 128 ? ~0ull : k > 64 ? (1ull << (k - 64)) - 1 : 0ull);
  else
    return k >= (int)(8 * sizeof(LaneT)) ? (LaneT)~(LaneT)0 : (LaneT)(((LaneT)1 << k) - 1);
}

template <typename LaneT>
__device__ __forceinline__ int lowest_bit(LaneT x) {
  if constexpr (sizeof(LaneT) == 32)
    return x.q[0] ? __ffsll((long long)x.q[0]) - 1
         : x.q[1] ? 63 + __ffsll((long long)x.q[1])
         : x.q[2] ? 127 + __ffsll((long long)x.q[2])
                  : 191 + __ffsll((long long)x.q[3]);
  else if constexpr (sizeof(LaneT) == 16)
    return x.lo ? __ffsll((long long)x.lo) - 1 : 63 + __ffsll((long long)x.hi);
  else if constexpr (sizeof(LaneT) == 8)
    return __ffsll((long long)x) - 1;
  else
    return __ffs((int)x) - 1;
}

template <typename LaneT>
__device__ __forceinline__ LaneT clear_lowest(LaneT x) {
  if constexpr (sizeof(LaneT) == 32) {
    if (x.q[0]) x.q[0] &= x.q[0] - 1;
    else if (x.q[1]) x.q[1] &= x.q[1] - 1;
    else if (x.q[2]) x.q[2] &= x.q[2] - 1;
    else x.q[3] &= x.q[3] - 1;
    return x;
  } else if constexpr (sizeof(LaneT) == 16)
    return x.lo ? Lane128(x.lo & (x.lo - 1), x.hi) : Lane128(0, x.hi & (x.hi - 1));
  else
    return (LaneT)(x & (x - 1));
}

// OR into a lane word in global memory (result not needed).
template <typename LaneT>
__device__ __forceinline__ void atomic_or_lane(LaneT* p, LaneT v) {
  if constexpr (sizeof(LaneT) == 32) {
#pragma unroll
    for (int j = 0; j < 4; j++)
      if (v.q[j]) atomicOr(&p->q[j], v.q[j]);
  } else if constexpr (sizeof(LaneT) == 16) {
    if (v.lo) atomicOr(&p->lo, v.lo);
    if (v.hi) atomicOr(&p->hi, v.hi);
  } else if constexpr (sizeof(LaneT) == 8) {
    atomicOr(reinterpret_cast<unsigned long long*>(p), (unsigned long long)v);
  } else {
    atomicOr(reinterpret_cast<unsigned int*>(p), (unsigned int)v);
  }
}

// OR into a lane word; true for the call that first made it non-zero.  A
// 128- or 256-lane word is several 64-bit atomics, so there each part has its
// own first caller: a word can report several first touches, never none.
template <typename LaneT>
__device__ __forceinline__ bool first_or_lane(LaneT* p, LaneT v) {
  if constexpr (sizeof(LaneT) == 32) {
    bool first = false;
#pragma unroll
    for (int j = 0; j < 4; j++)
      if (v.q[j]) first |= atomicOr(&p->q[j], v.q[j]) == 0;
    return first;
  } else if constexpr (sizeof(LaneT) == 16) {
    bool first = false;
    if (v.lo) first |= atomicOr(&p->lo, v.lo) == 0;
    if (v.hi) first |= atomicOr(&p->hi, v.hi) == 0;
    return first;
  } else if constexpr (sizeof(LaneT) == 8) {
    return atomicOr(reinterpret_cast<unsigned long long*>(p), (unsigned long long)v) == 0;
  } else {
    return atomicOr(reinterpret_cast<unsigned int*>(p), (unsigned int)v) == 0;
  }
}

// OR nb into acc[v]; true for the one call per level that first touched v.
// 32/64-lane words take it from the atomic's old value; a wider word is
// several 64-bit atomics, so there a per-vertex flag (cleared by the install)
// decides instead.
template <typename LaneT>
__device__ __forceinline__ bool touch_or(LaneT* acc, uint32_t* tflag, int64_t v, LaneT nb) {
  if constexpr (sizeof(LaneT) >= 16) {
    atomic_or_lane(acc + v, nb);
    return atomicOr(tflag + v, 1u) == 0;
  } else {
    return first_or_lane(acc + v, nb);
  }
}

// Per-vertex depth log: up to kLogSlots entries (level, lanes found at that
// level).  A vertex is logged by one thread per level.  Returns true when
// the entry does not fit (slots full, or a level above 254): the caller then
// writes those depths into the rows and flags the vertex.
constexpr int kLogSlots = 4;

template <typename LaneT>
__device__ __forceinline__ bool log_found(uint32_t* lvl, LaneT* lmask, int64_t v, LaneT nb,
                                          int level) {
  if (level > 254) return true;
  const uint32_t w = __ldcg(lvl + v);
  const uint32_t x = ~w;                                   // empty slots read 0x00
  const uint32_t zero = (x - 0x01010101u) & ~x & 0x80808080u;
  if (!zero) return true;
  const int slot = (__ffs(zero) - 1) >> 3;                 // first empty slot
  lmask[v * kLogSlots + slot] = nb;
  lvl[v] = (w & ~(0xffu << (8 * slot))) | ((uint32_t)level << (8 * slot));
  return false;
}

template <typename LaneT>
__device__ __forceinline__ LaneT ld_lane(const LaneT* p) {
  if constexpr (sizeof(LaneT) == 32) {
    const ulonglong2 t = __ldcg(reinterpret_cast<const ulonglong2*>(p));
    const ulonglong2 u = __ldcg(reinterpret_cast<const ulonglong2*>(p) + 1);
    return Lane256(t.x, t.y, u.x, u.y);
  } else if constexpr (sizeof(LaneT) == 16) {
    const ulonglong2 t = __ldcg(reinterpret_cast<const ulonglong2*>(p));
    return Lane128(t.x, t.y);
  } else if constexpr (sizeof(LaneT) == 8) {
    return (LaneT)__ldcg(reinterpret_cast<const unsigned long long*>(p));
  } else {
    return (LaneT)__ldcg(reinterpret_cast<const unsigned int*>(p));
  }
}

// OR over the lanes of `grp` (the calling lane included), one warp reduction
// per 32-bit word.
template <typename LaneT>
__device__ __forceinline__ LaneT group_or(unsigned grp, LaneT x) {
  uint32_t w[sizeof(LaneT) / 4];
#pragma unroll
  for (int h = 0; h < (int)(sizeof(LaneT) / 4); h++) w[h] = __reduce_or_sync(grp, word32(x, h));
  return from_words<LaneT>(w);
}

template <typename LaneT>
__device__ __forceinline__ LaneT warp_or(LaneT x) {
  return group_or(kFull, x);
}

// Neighbour lists are read once per level: loads marked evict-first, so the
// stream does not push the frontier words out of L2.
__device__ __forceinline__ int32_t ld_stream(const int32_t* p) { return __ldcs(p); }

// Frontier words and bits are read with L1-cached loads: they are written
// only in the level before, and the acquire fence of the grid barrier in
// between makes those writes visible to the weak loads after it.
template <typename LaneT>
__device__ __forceinline__ LaneT ld_frontier(const LaneT* p) {
  return *p;
}

__device__ __forceinline__ bool in_frontier(const uint32_t* fbits, int32_t u) {
  return (fbits[u >> 5] >> (u & 31)) & 1u;
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
// Rows are visited one 32-bit half of the lane word at a time: a half with
// many rows set runs every row unrolled, a sparse one only its set rows.
template <typename LaneT, typename DepthT>
__device__ __forceinline__ void write_depths(DepthT* depth, int64_t n, int64_t v, LaneT nb,
                                             int level) {
  const LaneT any = warp_or(nb);
  const DepthT d = (DepthT)level;
#pragma unroll
  for (int h = 0; h < (int)(sizeof(LaneT) / 4); h++) {
    unsigned anyh = word32(any, h);
    if (!anyh) continue;
    unsigned bits = word32(nb, h);
    DepthT* p = depth + (int64_t)(32 * h) * n + v;
    if (__popc(anyh) > 12) {
#pragma unroll 8
      for (int i = 0; i < 32; i++) {
        if (bits & 1u) *p = d;
        bits >>= 1;
        p += n;
      }
    } else {
      while (anyh) {
        const int i = __ffs(anyh) - 1;
        anyh &= anyh - 1;
        if ((bits >> i) & 1u) p[(int64_t)i * n] = d;
      }
    }
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

// Append the lanes with `keep` and a non-empty adjacency to a top-down queue.
// The packed counter is (entries << shift) | summed degree, so one atomic
// gives each entry its slot and the position of its first edge in the
// concatenated adjacency of the queue (qe).  Whole warp.
__device__ __forceinline__ void warp_queue(unsigned long long* packed, int32_t* q, uint64_t* qe,
                                           int shift, bool keep, int32_t v,
                                           unsigned long long deg) {
  const int lane = threadIdx.x & 31;
  keep = keep && deg > 0;
  if (!__any_sync(kFull, keep)) return;
  const unsigned long long emask = (1ull << shift) - 1;
  const unsigned long long mine = keep ? (1ull << shift) + deg : 0;
  const unsigned long long inc = warp_inclusive_sum(mine, lane);
  unsigned long long base = 0;
  if (lane == 31) base = atomicAdd(packed, inc);
  base = shfl(base, 31);
  if (keep) {
    const unsigned long long at = base + inc - mine;
    q[at >> shift] = v;
    qe[at >> shift] = at & emask;
  }
}

// warp_queue, and the lanes with `keep` added to the frontier totals.
__device__ __forceinline__ void warp_enqueue(unsigned long long* packed, int32_t* q, uint64_t* qe,
                                             unsigned long long* f_count,
                                             unsigned long long* f_edges, int shift, bool keep,
                                             int32_t v, unsigned long long deg) {
  const int lane = threadIdx.x & 31;
  const unsigned km = __ballot_sync(kFull, keep);
  if (!km) return;
  warp_queue(packed, q, qe, shift, keep, v, deg);
  unsigned long long dsum = keep ? deg : 0;
#pragma unroll
  for (int o = 16; o; o >>= 1) dsum += __shfl_xor_sync(kFull, dsum, o);
  if (lane == 0) {
    atomicAdd(f_count, (unsigned long long)__popc(km));
    atomicAdd(f_edges, dsum);
  }
}

// OR of fr[u] over the neighbours nbr[b..e) of one vertex, by the whole warp:
// 4 x 32 neighbours per round, every load of a round issued before any is
// used, early exit once (result | vis) covers every lane.
template <typename LaneT>
__device__ __forceinline__ LaneT warp_gather_or(const int32_t* nbr, const uint32_t* fbits,
                                                const LaneT* fr, uint64_t b, uint64_t e,
                                                LaneT vis, LaneT all, bool filter) {
  const int lane = threadIdx.x & 31;
  LaneT got = 0;
  for (uint64_t e0 = b; e0 < e; e0 += 128) {
    int32_t u[4];
#pragma unroll
    for (int r = 0; r < 4; r++) {
      const uint64_t idx = e0 + 32 * r + lane;
      u[r] = idx < e ? ld_stream(nbr + idx) : -1;
    }
    bool in[4];
#pragma unroll
    for (int r = 0; r < 4; r++) in[r] = u[r] >= 0 && (!filter || in_frontier(fbits, u[r]));
    LaneT x = 0;
#pragma unroll
    for (int r = 0; r < 4; r++)
      if (in[r]) x |= ld_frontier(fr + u[r]);
    got |= warp_or(x);
    if (((got | vis) & all) == all) break;
  }
  return got;
}

// Resident blocks per SM the register allocation is held to.  The 256-lane
// word's values take twice the registers, so it spills a little at 4 blocks
// (176 bytes of spill stores); it still ran faster there than at 3 or 2,
// since the kernel is latency-bound and occupancy decides.
#ifndef GBBFS_MS_MIN_BLOCKS
#define GBBFS_MS_MIN_BLOCKS 4
#endif
#ifndef GBBFS_MS_MIN_BLOCKS_WIDE
#define GBBFS_MS_MIN_BLOCKS_WIDE 4
#endif
template <typename LaneT>
constexpr int ms_min_blocks() {
  return sizeof(LaneT) > 16 ? GBBFS_MS_MIN_BLOCKS_WIDE : GBBFS_MS_MIN_BLOCKS;
}

template <typename OffT, typename LaneT, typename DepthT, int kBatchN>
__global__ void __launch_bounds__(kThreads, ms_min_blocks<LaneT>()) k_msbfs(MsArgs<OffT, LaneT, DepthT> a) {
  __shared__ LaneT tile_acc[kWarpsPerCta][32];
  __shared__ int64_t tile_base[kWarpsPerCta][32];
  __shared__ uint8_t tile_owner[kWarpsPerCta][32 * kMsSmall];
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
  const int k = *a.nsrc;
  const LaneT all = lane_ones<LaneT>(k);
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
  if (blockIdx.x == 0 && threadIdx.x < k) {
    const int i = threadIdx.x;
    const int32_t s = a.perm[a.sources[i]];
    const LaneT bit = lane_bit<LaneT>(i);
    atomic_or_lane(a.visit + s, bit);
    a.depth[(int64_t)i * a.dstride + s] = 0;   // depth 0 lives in the rows
    a.spill[s] = 1;
    if (first_or_lane(a.fr1 + s, bit)) {
      const unsigned long long deg = (unsigned long long)(a.off[s + 1] - a.off[s]);
      if (deg) {
        const unsigned long long at = atomicAdd(&c->q_packed[1], (1ull << a.shift) + deg);
        a.q1[at >> a.shift] = s;
        a.qe1[at >> a.shift] = at & emask;
      }
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
    uint64_t* qe = cur ? a.qe1 : a.qe0;
    int32_t* qn = cur ? a.q0 : a.q1;
    uint64_t* qen = cur ? a.qe0 : a.qe1;
    unsigned long long* touched = &c->touched[level % 3];
    unsigned long long* nf_count = &c->f_count[(level + 1) % 3];
    unsigned long long* nf_edges = &c->f_edges[(level + 1) % 3];
    const bool bottom_up = E > (unsigned long long)(a.m / a.alpha);
    // Slots this level does not touch are reset for the levels ahead.
    if (tid == 0) {
      c->f_count[(level + 2) % 3] = 0;
      c->f_edges[(level + 2) % 3] = 0;
      c->touched[(level + 2) % 3] = 0;
      c->tile_next[(level + 2) % 3] = 0;
      c->q_packed[nxt] = 0;
    }

    if (!bottom_up) {
      // A frontier with many edges, early in the search, reaches many new
      // vertices: install the next frontier by one pass over all vertices
      // instead of a touched list.  After a bottom-up level (or a dense
      // install) most targets are visited already, so the list is small
      // unless the frontier's degree sum exceeds n.
      const bool dense = E > (unsigned long long)(have_queue ? a.n >> 4 : a.n);
      if (!have_queue) {
        // The frontier was written densely (bottom-up or dense install):
        // queue it from its fbits.  (q_packed[cur] was reset a level ago.)
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
            warp_queue(&c->q_packed[cur], q, qe, a.shift, keep, v, deg);
          }
        }
        mark(kPhInstall);
        if (!barrier()) return;
      }
      const unsigned long long qp = __ldcg(&c->q_packed[cur]);
      const uint64_t EQ = qp & emask;             // edges of the queued vertices
      const int64_t Q = (int64_t)(qp >> a.shift);
      if (!dense) {
        // The next frontier buffers are written sparsely: clear them first.
        for (int64_t v = tid; v < a.n; v += nthreads) frn[v] = 0;
        for (int64_t w = tid; w < a.W; w += nthreads) fbn[w] = 0;
        mark(kPhClear);
      }
      // Top-down, edge-balanced: warp spans of consecutive edges of
      // the queue's concatenated adjacency.  Lane j of the warp holds queue
      // entry base + j (its first edge, adjacency start and frontier word);
      // the window slides so that entry `base` holds the round's first edge,
      // and since every entry has an edge, the round's 32 edges lie in the
      // window.
      // Spans shrink (to 32 edges at least) until every warp has one.
      uint64_t span = (EQ + nwarps - 1) / nwarps;
      span = span < 32 ? 32 : span > kMsTdSpan ? kMsTdSpan : (span + 31) & ~31ull;
      const int64_t nspans = (int64_t)((EQ + span - 1) / span);
      for (int64_t sp = warp; sp < nspans; sp += nwarps) {
        const uint64_t e_lo = (uint64_t)sp * span;
        const uint64_t e_hi = e_lo + span < EQ ? e_lo + span : EQ;
        int64_t lo = 0, hi = Q - 1;
        while (lo < hi) {
          const int64_t mid = (lo + hi + 1) >> 1;
          if (__ldcg(qe + mid) <= e_lo) lo = mid; else hi = mid - 1;
        }
        int64_t base = lo;
        uint64_t pre = ~0ull, ob = 0;
        LaneT f = 0;
        auto load_entry = [&](int64_t j) {
          if (j < Q) {
            pre = __ldcg(qe + j);
            const int32_t u = __ldcg(q + j);
            ob = (uint64_t)a.off[u];
            f = ld_frontier(fr + u);
          } else {
            pre = ~0ull;
            ob = 0;
            f = 0;
          }
        };
        load_entry(base + lane);
        for (uint64_t e0 = e_lo; e0 < e_hi; e0 += 32) {
          for (;;) {
            const unsigned le = __ballot_sync(kFull, pre <= e0);
            const int s = 31 - __clz(le);
            if (s <= 0) break;
            const int src = lane + s;
            const uint64_t pre2 = shfl(pre, src & 31), ob2 = shfl(ob, src & 31);
            const LaneT f2 = shfl(f, src & 31);
            if (src < 32) {
              pre = pre2;
              ob = ob2;
              f = f2;
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
          const LaneT f_s = shfl(f, seg);
          bool first = false;
          int32_t v = 0;
          if (e < e_hi) {
            v = ld_stream(a.nbr + ob_s + (e - pre_s));
            if (dense) {
              // No visit test: the install pass masks visited bits anyway,
              // and the OR needs no result, so nothing waits on a load.
              atomic_or_lane(a.acc + v, f_s);
            } else {
              const LaneT nb = f_s & ~ld_lane(a.visit + v);
              if (nb) first = touch_or(a.acc, a.tflag, v, nb);
            }
          }
          if (!dense) warp_append(touched, a.tq, first, v);
        }
      }
      mark(kPhTopDown);
      if (!barrier()) return;
      if (dense) {
        // Every vertex: bits that arrived and were not yet visited.
        if (threadIdx.x == 0) {
          blk_count = 0;
          blk_edges = 0;
        }
        __syncthreads();
        unsigned long long my_count = 0, my_edges = 0;
        for (int64_t v0 = warp << 5; v0 < a.n; v0 += nwarps << 5) {
          const int64_t v = v0 + lane;
          LaneT nb = 0;
          if (v < a.n) {
            const LaneT x = ld_lane(a.acc + v);
            if (x) {
              a.acc[v] = 0;
              const LaneT vis = a.visit[v];
              nb = x & ~vis;
              if (nb) {
                a.visit[v] = vis | nb;
                my_count++;
                my_edges += (unsigned long long)(a.off[v + 1] - a.off[v]);
              }
            }
            frn[v] = nb;
          }
          const unsigned nm = __ballot_sync(kFull, nb != 0);
          if (lane == 0) fbn[v0 >> 5] = nm;
          LaneT over = 0;
          if (nb && log_found(a.lvl, a.lmask, v, nb, level)) {
            over = nb;
            a.spill[v] = 1;
          }
          write_depths(a.depth, a.dstride, v, over, level);
        }
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
        have_queue = false;
      } else {
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
            a.tflag[v] = 0;
            const LaneT vis = a.visit[v];
            nb &= ~vis;
            if (nb) {
              a.visit[v] = vis | nb;
              if (log_found(a.lvl, a.lmask, v, nb, level)) {
                a.spill[v] = 1;
                for (LaneT x = nb; x; x = clear_lowest(x))
                  a.depth[(int64_t)lowest_bit(x) * a.dstride + v] = (DepthT)level;
              }
              frn[v] = nb;
              atomicOr(fbn + (v >> 5), 1u << (v & 31));
              deg = (unsigned long long)(a.off[v + 1] - a.off[v]);
            }
          }
          warp_enqueue(&c->q_packed[nxt], qn, qen, nf_count, nf_edges, a.shift, nb != 0, v, deg);
        }
        have_queue = true;
      }
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
      const int wib = threadIdx.x >> 5;
      uint8_t* own = tile_owner[wib];
      int64_t* nbase = tile_base[wib];
      LaneT* tacc = tile_acc[wib];
      // When most edge endpoints are frontier vertices, the fbits test
      // filters little and costs a load of its own: read fr[u] directly.
      const bool filter = 2 * E < (unsigned long long)a.m;
      const int64_t ngroups = a.nunits;
      unsigned long long* next_unit = &c->tile_next[level % 3];
      for (;;) {
        // Work units from a level-wide counter: the hub chunks first, then
        // groups of kMsGrab tiles.
        unsigned long long u0 = 0;
        if (lane == 0) u0 = atomicAdd(next_unit, 1ull);
        u0 = shfl(u0, 0);
        if ((int64_t)u0 >= hub_chunks + ngroups) break;
        if ((int64_t)u0 < hub_chunks) {
          // A hub's adjacency cut into work items, merged by atomicOr.
          const int64_t hc = (int64_t)u0;
          int64_t lo = 0, hi = a.nhubs - 1;
          while (lo < hi) {
            const int64_t mid = (lo + hi + 1) >> 1;
            if ((int64_t)a.hub_chunk[mid] <= hc) lo = mid; else hi = mid - 1;
          }
          const int32_t v = a.hubs[lo];
          const LaneT vis = ld_lane(a.visit + v);
          if ((vis & all) != all) {
            const uint64_t b = (uint64_t)a.off[v] + (uint64_t)(hc - a.hub_chunk[lo]) * kMsHubChunk;
            const uint64_t ve = (uint64_t)a.off[v + 1];
            const uint64_t e = b + kMsHubChunk < ve ? b + kMsHubChunk : ve;
            const LaneT got = warp_gather_or(a.nbr, fb, fr, b, e, vis, all, filter);
            const LaneT part = got & ~vis & all;
            bool first = false;
            if (lane == 0 && part) first = touch_or(a.acc, a.tflag, v, part);
            warp_append(touched, a.tq, first, v);
          }
          mark(kPhHub);
          continue;
        }
        const int64_t unit = (int64_t)u0 - hub_chunks;
        const int64_t v_begin = (int64_t)a.unit_tile[unit] << 5;
        const int64_t v_end = (int64_t)a.unit_tile[unit + 1] << 5;
        const int64_t v_stop = v_end < a.n ? v_end : a.n;
      for (int64_t v0 = v_begin; v0 < v_stop; v0 += 32) {
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
        // Vertices of degree below kMsSmall: the warp streams their
        // concatenated adjacency, kBatchN/2 x 32 edges per round with the
        // loads of a round issued together.  own[t] names the tile lane that
        // edge t of the stream belongs to; lanes of one owner combine their
        // bits (match + warp reduction) and one of them ORs them into the
        // owner's word in shared memory.
        const bool small = need && deg < (uint64_t)kMsSmall;
        const unsigned sd = small ? (unsigned)deg : 0u;
        const unsigned sincl = warp_inclusive_sum(sd, lane);
        const unsigned sstart = sincl - sd;
        const unsigned stotal = __shfl_sync(kFull, sincl, 31);
        tacc[lane] = 0;
        nbase[lane] = (int64_t)b - (int64_t)sstart;
        for (unsigned t = sstart; t < sincl; t++) own[t] = (uint8_t)lane;
        __syncwarp();
        constexpr int kR = kBatchN / 2 > 0 ? kBatchN / 2 : 1;
        for (unsigned t0 = 0; t0 < stotal; t0 += 32 * kR) {
          unsigned o[kR];
          int32_t u[kR];
#pragma unroll
          for (int r = 0; r < kR; r++) {
            const unsigned t = t0 + 32 * r + lane;
            o[r] = t < stotal ? own[t] : 32u;
            u[r] = t < stotal ? ld_stream(a.nbr + nbase[o[r]] + t) : -1;
          }
          bool in[kR];
#pragma unroll
          for (int r = 0; r < kR; r++) in[r] = u[r] >= 0 && (!filter || in_frontier(fb, u[r]));
#pragma unroll
          for (int r = 0; r < kR; r++) {
            const LaneT x = in[r] ? ld_frontier(fr + u[r]) : (LaneT)0;
            const unsigned grp = __match_any_sync(kFull, o[r]);
            const LaneT red = group_or(grp, x);
            if (o[r] < 32u && red && lane == __ffs(grp) - 1) tacc[o[r]] |= red;
          }
        }
        __syncwarp();
        if (small) nb = tacc[lane] & ~vis & all;
        mark(kPhSmall);
        unsigned mids = __ballot_sync(kFull, need && deg >= kMsSmall && deg <= kMsHubDeg);
        while (mids) {
          const int t = __ffs(mids) - 1;
          mids &= mids - 1;
          const LaneT vt = shfl(vis, t);
          const uint64_t bt = shfl(b, t), et = shfl(e, t);
          const LaneT got = warp_gather_or(a.nbr, fb, fr, bt, et, vt, all, filter);
          if (lane == t) nb = got & ~vt & all;
        }
        mark(kPhMid);
        // Dense writes of this tile: visit, depths, next frontier and fbits.
        if (nb) a.visit[v] = vis | nb;
        if (v < a.n) frn[v] = nb;
        const unsigned nm = __ballot_sync(kFull, nb != 0);
        if (lane == 0 && (v0 >> 5) < a.W) fbn[v0 >> 5] = nm;
        LaneT over = 0;
        if (nb && log_found(a.lvl, a.lmask, v, nb, level)) {
          over = nb;
          a.spill[v] = 1;
        }
        write_depths(a.depth, a.dstride, v, over, level);
        if (nb) {
          my_count++;
          my_edges += deg;
        }
        mark(kPhWrite);
      }
      }
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
          a.tflag[v] = 0;
          const LaneT vis = a.visit[v];
          nb &= ~vis;
          if (nb) {
            a.visit[v] = vis | nb;
            if (log_found(a.lvl, a.lmask, v, nb, level)) {
              a.spill[v] = 1;
              for (LaneT x = nb; x; x = clear_lowest(x))
                a.depth[(int64_t)lowest_bit(x) * a.dstride + v] = (DepthT)level;
            }
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
        c->level_f[level] = (unsigned long long)F;
        c->level_e[level] = E;
      }
    }
  }
  if (tid == 0) c->t_end = globaltimer();
  __syncthreads();
  if (threadIdx.x < kMsPhases) atomicAdd(&c->phase_cycles[threadIdx.x], ph_acc[threadIdx.x]);
}

// Keys of the search-ordered CSR: (perm[u] << bits) | perm[v] for every
// directed edge (u, v), at u's edge positions.  Sorted, they list every new
// vertex's neighbours in new-id order (highest degree first).  A warp per
// original vertex.
template <typename OffT>
__global__ void __launch_bounds__(kThreads) k_relabel_keys(const OffT* off, const int32_t* nbr,
                                                           const int32_t* perm, int64_t n,
                                                           int bits, uint64_t* keys) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t u = warp; u < n; u += nwarps) {
    const uint64_t b = (uint64_t)off[u], e = (uint64_t)off[u + 1];
    const uint64_t hi = (uint64_t)(uint32_t)perm[u] << bits;
    for (uint64_t j = b + lane; j < e; j += 32) keys[j] = hi | (uint32_t)perm[nbr[j]];
  }
}

static __global__ void k_low_bits(const uint64_t* keys, int64_t len, uint64_t mask, int32_t* out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < len;
       i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (int32_t)(keys[i] & mask);
}

// Transpose of a 4x4 byte block: word j of the result holds byte j of each of
// w[0..3] (w[0]'s in the low byte).
__device__ __forceinline__ void transpose4x4(const uint32_t w[4], uint32_t r[4]) {
  const uint32_t lo01 = __byte_perm(w[0], w[1], 0x5140), hi01 = __byte_perm(w[0], w[1], 0x7362);
  const uint32_t lo23 = __byte_perm(w[2], w[3], 0x5140), hi23 = __byte_perm(w[2], w[3], 0x7362);
  r[0] = __byte_perm(lo01, lo23, 0x5410);
  r[1] = __byte_perm(lo01, lo23, 0x7632);
  r[2] = __byte_perm(hi01, hi23, 0x5410);
  r[3] = __byte_perm(hi01, hi23, 0x7632);
}

// Bits 0..7 of x to bits 0, 4, ..., 28 (nibble spacing).
__device__ __forceinline__ uint32_t spread_byte(uint32_t x) {
  x = (x | (x << 12)) & 0x000f000fu;
  x = (x | (x << 6)) & 0x03030303u;
  return (x | (x << 3)) & 0x11111111u;
}

// Depth rows in original vertex order from the per-vertex logs.  A block
// takes kTileV consecutive original vertices, reads each one's log through
// perm (a few contiguous words), builds its record of depths in shared
// memory, and then writes every row's segment coalesced (uint8 rows as 4x4
// byte blocks).  For uint8, 4 lanes' depths come from one __byte_perm of the
// log's level word: the selector nibble of a lane is the index of the log
// entry holding it (bit planes b0 = entry 1 or 3, b1 = entry 2 or 3,
// b2 = none, which selects 0xff).  Lanes of a flagged vertex that the log
// does not hold but visit has are read from the rows.
template <typename LaneT, typename DepthT>
__global__ void __launch_bounds__(kThreads) k_depth_decode(
    const uint32_t* lvl, const LaneT* lmask, const uint8_t* spill, const LaneT* visit,
    const DepthT* rows, int64_t stride, const int32_t* perm, DepthT* out, int64_t n,
    const int32_t* nsrc) {
  const int k = *nsrc;
  constexpr int kTileV = kDecodeTile / (int)sizeof(DepthT);  // vertices per block
  constexpr int kRecWords = kMsMaxLanes * sizeof(DepthT) / 4 + 1;
  __shared__ uint32_t tile[kTileV * kRecWords];    // [vertex][row], padded records
  const int64_t v0 = (int64_t)blockIdx.x * kTileV;
  if constexpr (sizeof(DepthT) == 1) {
    const int words = (k + 31) / 32;                 // 32-lane words of the lane word in use
    for (int t = threadIdx.x; t < kTileV * words; t += blockDim.x) {
      const int q = t / words, h = t % words;
      const int64_t v = v0 + q;
      if (v >= n) continue;
      const int64_t p = perm[v];
      // Every slot's mask is loaded with the level word (unused slots are
      // masked out after), so only perm -> log is a dependent chain.
      const uint32_t lw = lvl[p];
      uint32_t W[kLogSlots];
#pragma unroll
      for (int j = 0; j < kLogSlots; j++)
        W[j] = reinterpret_cast<const uint32_t*>(lmask + p * kLogSlots + j)[h];
#pragma unroll
      for (int j = 0; j < kLogSlots; j++)
        if (((lw >> (8 * j)) & 0xffu) == 0xffu) W[j] = 0u;
      const uint32_t reach = W[0] | W[1] | W[2] | W[3];
      const uint32_t b0 = W[1] | W[3], b1 = W[2] | W[3], b2 = ~reach;
      uint32_t sel[4];
#pragma unroll
      for (int y = 0; y < 4; y++)
        sel[y] = spread_byte((b0 >> (8 * y)) & 0xffu) | (spread_byte((b1 >> (8 * y)) & 0xffu) << 1) |
                 (spread_byte((b2 >> (8 * y)) & 0xffu) << 2);
      const uint32_t extra = spill[p] ? word32(visit[p], h) & ~reach : 0u;
      uint32_t* rec = tile + q * kRecWords + 8 * h;
#pragma unroll
      for (int g = 0; g < 8; g++) {
        uint32_t d = __byte_perm(lw, 0xffffffffu, (sel[g >> 1] >> (16 * (g & 1))) & 0xffffu);
        for (uint32_t e = (extra >> (4 * g)) & 0xfu; e; e &= e - 1) {
          const int r = __ffs(e) - 1;
          const int i = 32 * h + 4 * g + r;
          const uint32_t b = (uint8_t)rows[(int64_t)i * stride + p];
          d = (d & ~(0xffu << (8 * r))) | (b << (8 * r));
        }
        rec[g] = d;
      }
    }
  } else {
    for (int t = threadIdx.x; t < kTileV * k; t += blockDim.x) {
      const int q = t / k, i = t % k;
      const int64_t v = v0 + q;
      if (v >= n) continue;
      const int64_t p = perm[v];
      const uint32_t lw = lvl[p];
      DepthT d = (DepthT)-1;
      bool found = false;
      for (int j = 0; j < kLogSlots; j++) {
        const uint32_t L = (lw >> (8 * j)) & 0xffu;
        if (L == 0xffu) break;
        if (lane_test(lmask[p * kLogSlots + j], i)) {
          d = (DepthT)L;
          found = true;
          break;
        }
      }
      if (!found && spill[p] && lane_test(visit[p], i)) d = rows[(int64_t)i * stride + p];
      tile[q * kRecWords + i] = (uint32_t)d;
    }
  }
  __syncthreads();
  if constexpr (sizeof(DepthT) == 1) {
    if ((n & 3) == 0 && v0 + kTileV <= n) {
      // 4 records x 4 rows per step: a word of each record, transposed into
      // a word (4 consecutive vertices) of each row.
      const int groups = (k + 3) / 4;
      for (int t = threadIdx.x; t < groups * (kTileV / 4); t += blockDim.x) {
        const int b4 = t % (kTileV / 4), a4 = t / (kTileV / 4);
        uint32_t w[4], r[4];
#pragma unroll
        for (int j = 0; j < 4; j++) w[j] = tile[(4 * b4 + j) * kRecWords + a4];
        transpose4x4(w, r);
#pragma unroll
        for (int j = 0; j < 4; j++) {
          const int i = 4 * a4 + j;
          if (i < k) *reinterpret_cast<uint32_t*>(out + (int64_t)i * n + v0 + 4 * b4) = r[j];
        }
      }
      return;
    }
  }
  const DepthT* tb = reinterpret_cast<const DepthT*>(tile);
  for (int t = threadIdx.x; t < k * kTileV; t += blockDim.x) {
    const int i = t / kTileV, q = t % kTileV;
    const int64_t v = v0 + q;
    if (v < n) out[(int64_t)i * n + v] = tb[(int64_t)q * kRecWords * (4 / sizeof(DepthT)) + i];
  }
}

}  // namespace gbbfs
