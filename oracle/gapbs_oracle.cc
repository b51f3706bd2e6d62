// ORACLE — test infrastructure, not product code.
//
// A plain C++ restatement of the reference's CPU algorithm for the BFS hot path
// (the shared-memory GAPBS copy that ships in the reference as gapbs-verify/).
// It is the checker for the CUDA path: only tests/, __graft_entry__.smoke() and
// bench.py's CPU-baseline leg load it.  The product library never links it.
//
// Parity of this restatement is pinned against the reference itself: the
// recipe in oracle/build.py compiles the reference's own gapbs-verify/bfs.cc
// into oracle/_ref/, and tests/golden/make_golden.py records its graphs,
// source sequences, step traces and depths as fixtures under tests/golden/.
//
// Every function cites the reference lines it restates.  Exported with C
// linkage so Python's ctypes can call it.

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <random>
#include <vector>

#include <omp.h>

#include <type_traits>

namespace {

// gapbs-verify/util.h:19 (src/util.h:25)
const int64_t kRandSeed = 27491095;
// gapbs-verify/generator.h:163
const int64_t kGenBlock = 1 << 18;

struct Edge { int32_t u, v; };

// gapbs-verify/generator.h:66-82.  Each 2^18-edge block reseeds mt19937 with
// kRandSeed + block.  The reference writes Edge(udist(rng), udist(rng)); g++
// evaluates those two arguments right to left, so the FIRST draw is the
// destination v and the SECOND the source u (checked against the reference
// binary built by oracle/build.py; the golden CSR hashes pin it).
void MakeUniformEL(int64_t num_nodes, int64_t num_edges, Edge* el) {
  #pragma omp parallel
  {
    std::mt19937 rng;
    std::uniform_int_distribution<int32_t> udist(0, num_nodes - 1);
    #pragma omp for schedule(static)
    for (int64_t block = 0; block < num_edges; block += kGenBlock) {
      rng.seed(kRandSeed + block / kGenBlock);
      int64_t end = std::min(block + kGenBlock, num_edges);
      for (int64_t e = block; e < end; e++) {
        int32_t v = udist(rng);
        int32_t u = udist(rng);
        el[e].u = u;
        el[e].v = v;
      }
    }
  }
}

// gapbs-verify/generator.h:54-64: identity permutation shuffled by
// std::shuffle with mt19937(kRandSeed), applied to both endpoints.
void PermuteIDs(int64_t num_nodes, int64_t num_edges, Edge* el) {
  std::vector<int32_t> perm(num_nodes);
  for (int64_t i = 0; i < num_nodes; i++) perm[i] = (int32_t)i;
  std::mt19937 rng(kRandSeed);
  std::shuffle(perm.data(), perm.data() + num_nodes, rng);
  #pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < num_edges; e++) {
    el[e].u = perm[el[e].u];
    el[e].v = perm[el[e].v];
  }
}

// gapbs-verify/generator.h:84-117: R-MAT with A=.57, B=.19, C=.19; one
// uniform_real_distribution<float> draw per recursion level.
void MakeRMatEL(int scale, int64_t num_nodes, int64_t num_edges, Edge* el) {
  const float A = 0.57f, B = 0.19f, C = 0.19f;
  #pragma omp parallel
  {
    std::mt19937 rng;
    std::uniform_real_distribution<float> udist(0, 1.0f);
    #pragma omp for schedule(static)
    for (int64_t block = 0; block < num_edges; block += kGenBlock) {
      rng.seed(kRandSeed + block / kGenBlock);
      int64_t end = std::min(block + kGenBlock, num_edges);
      for (int64_t e = block; e < end; e++) {
        int32_t src = 0, dst = 0;
        for (int depth = 0; depth < scale; depth++) {
          float p = udist(rng);
          src <<= 1;
          dst <<= 1;
          if (p < A + B) {
            if (p > A) dst++;
          } else {
            src++;
            if (p > A + B + C) dst++;
          }
        }
        el[e].u = src;
        el[e].v = dst;
      }
    }
  }
  PermuteIDs(num_nodes, num_edges, el);
}

}  // namespace

extern "C" {

void orc_free(void* p) { free(p); }

// Generator + Builder for a symmetrized synthetic graph:
// gapbs-verify/builder.h:231-252 (MakeGraph), :208-229 (MakeGraphFromEL:
// num_nodes = max ID + 1), :191-206 (MakeCSR, symmetrize => both endpoints),
// :137-183 (SquishCSR/SquishGraph: per-vertex sort, unique, drop self-loop).
// The CSR that results is a function of the edge multiset only, so this
// restatement builds it as "per vertex: sorted unique neighbours minus self".
// Returns num_nodes; *off_out (int64[n+1]) and *nbr_out (int32[m]) are malloc'd.
int64_t orc_build_synthetic(int scale, int degree, int uniform,
                            int64_t** off_out, int32_t** nbr_out) {
  int64_t gen_nodes = int64_t(1) << scale;          // generator.h:40-43
  int64_t num_edges = gen_nodes * degree;
  std::vector<Edge> el(num_edges);
  if (uniform)
    MakeUniformEL(gen_nodes, num_edges, el.data());
  else
    MakeRMatEL(scale, gen_nodes, num_edges, el.data());
  int32_t max_id = 0;                                // builder.h:62-71
  for (const Edge& e : el) max_id = std::max(max_id, std::max(e.u, e.v));
  int64_t n = int64_t(max_id) + 1;
  std::vector<int64_t> deg(n + 1, 0);
  for (const Edge& e : el) { deg[e.u]++; deg[e.v]++; }
  std::vector<int64_t> start(n + 1, 0);
  for (int64_t i = 0; i < n; i++) start[i + 1] = start[i] + deg[i];
  std::vector<int32_t> raw(start[n]);
  std::vector<int64_t> fill(start.begin(), start.end() - 1);
  for (const Edge& e : el) {
    raw[fill[e.u]++] = e.v;
    raw[fill[e.v]++] = e.u;
  }
  std::vector<int64_t> kept(n, 0);
  #pragma omp parallel for schedule(dynamic, 4096)
  for (int64_t u = 0; u < n; u++) {
    int32_t* b = raw.data() + start[u];
    int32_t* e = raw.data() + start[u + 1];
    std::sort(b, e);
    int32_t* ne = std::unique(b, e);
    ne = std::remove(b, ne, (int32_t)u);
    kept[u] = ne - b;
  }
  int64_t* off = (int64_t*)malloc(sizeof(int64_t) * (n + 1));
  off[0] = 0;
  for (int64_t u = 0; u < n; u++) off[u + 1] = off[u] + kept[u];
  int32_t* nbr = (int32_t*)malloc(sizeof(int32_t) * std::max<int64_t>(off[n], 1));
  #pragma omp parallel for schedule(dynamic, 4096)
  for (int64_t u = 0; u < n; u++)
    std::copy(raw.data() + start[u], raw.data() + start[u] + kept[u], nbr + off[u]);
  *off_out = off;
  *nbr_out = nbr;
  return n;
}

// SourcePicker: gapbs-verify/benchmark.h:46-68.  mt19937(kRandSeed), uniform
// over [0, n-1], redraw while the pick has out-degree 0; a given source (-r)
// is returned as is.
void orc_source_picker(const int64_t* off, int64_t n, int64_t given, int count,
                       int32_t* out) {
  std::mt19937 rng(kRandSeed);
  std::uniform_int_distribution<int32_t> udist(0, n - 1);
  for (int i = 0; i < count; i++) {
    if (given != -1) { out[i] = (int32_t)given; continue; }
    int32_t s;
    do { s = udist(rng); } while (off[s + 1] - off[s] == 0);
    out[i] = s;
  }
}

// Trace step kinds, in the order the reference prints them with PrintStep
// (gapbs-verify/bfs.cc:144-165): td <count>, e, bu <count>, c.
enum { ORC_TD = 1, ORC_E = 2, ORC_BU = 3, ORC_C = 4 };

// Per-step record of the serial replay: the counts the algorithmic-byte model
// needs.  frontier = |F| at step start, edges = edges examined, claimed = |N|,
// unvisited = |U| at step start (BU only).
struct OrcStep {
  int64_t kind, frontier, edges, claimed, unvisited;
};

// DOBFS: gapbs-verify/bfs.cc:122-173 with TDStep :67-89, BUStep :46-64,
// QueueToBitmap :92-98, BitmapToQueue :100-112, InitParent :114-120.
// parent encoding as in the reference: parent[x] < 0 => unvisited, holding
// -out_degree (or -1 for degree 0); the final pass maps parent < -1 to -1.
// threads == 1 runs the plain serial replay and fills `steps` (may be NULL)
// with per-step counts; threads > 1 runs the OpenMP form the reference uses.
// Returns the number of trace records written (kind/count pairs in `trace`,
// capacity trace_cap), or -1 when the capacity is too small.
// *seconds = wall time of the whole call, InitParent included
// (src/benchmark.h:127-129 brackets the kernel the same way).
int orc_dobfs(const int64_t* off, const int32_t* nbr, int64_t n, int32_t source,
              int alpha, int beta, int threads, int32_t* parent,
              int64_t* trace, int trace_cap, OrcStep* steps, double* seconds) {
  auto t0 = std::chrono::steady_clock::now();
  if (threads < 1) threads = 1;
  const int64_t words = (n + 63) / 64;
  std::vector<uint64_t> front(words, 0), curr(words, 0);
  std::vector<int32_t> queue(n > 0 ? n : 1);
  int64_t q_begin = 0, q_end = 0, q_in = 0;          // SlidingQueue window
  int ntrace = 0;
  bool overflow = false;
  auto rec = [&](int64_t kind, int64_t count, int64_t fr, int64_t ed, int64_t cl,
                 int64_t un) {
    if (ntrace >= trace_cap) { overflow = true; return; }
    trace[2 * ntrace] = kind;
    trace[2 * ntrace + 1] = count;
    if (steps) steps[ntrace] = OrcStep{kind, fr, ed, cl, un};
    ntrace++;
  };
  // InitParent
  #pragma omp parallel for num_threads(threads) schedule(static)
  for (int64_t v = 0; v < n; v++) {
    int64_t d = off[v + 1] - off[v];
    parent[v] = d != 0 ? (int32_t)-d : -1;
  }
  parent[source] = source;
  queue[q_in++] = source;
  q_begin = q_end; q_end = q_in;                     // slide_window
  int64_t visited = 1;
  int64_t edges_to_check = off[n];                   // num_edges_directed
  int64_t scout_count = off[source + 1] - off[source];
  while (q_begin != q_end) {
    if (scout_count > edges_to_check / alpha) {
      // QueueToBitmap
      int64_t qsize = q_end - q_begin;
      #pragma omp parallel for num_threads(threads) schedule(static)
      for (int64_t i = q_begin; i < q_end; i++) {
        int32_t u = queue[i];
        __atomic_fetch_or(&front[u >> 6], uint64_t(1) << (u & 63), __ATOMIC_RELAXED);
      }
      rec(ORC_E, 0, qsize, 0, 0, 0);
      int64_t awake_count = qsize, old_awake_count;
      q_begin = q_end; q_end = q_in;                 // slide_window
      do {
        old_awake_count = awake_count;
        // BUStep
        std::fill(curr.begin(), curr.end(), 0);
        int64_t awake = 0, scanned = 0;
        int64_t unvisited = n - visited;
        // The scanned-edge count of the byte model is kept only when the
        // caller asks for step records, so the timed form runs the
        // reference's loop as it is.
        auto bu_step = [&](auto counting) {
          #pragma omp parallel for num_threads(threads) schedule(dynamic, 1024) \
              reduction(+ : awake, scanned)
          for (int64_t u = 0; u < n; u++) {
            if (parent[u] < 0) {
              for (int64_t e = off[u]; e < off[u + 1]; e++) {
                int32_t v = nbr[e];
                if (decltype(counting)::value) scanned++;
                if ((front[v >> 6] >> (v & 63)) & 1) {
                  parent[u] = v;
                  awake++;
                  __atomic_fetch_or(&curr[u >> 6], uint64_t(1) << (u & 63), __ATOMIC_RELAXED);
                  break;
                }
              }
            }
          }
        };
        if (steps)
          bu_step(std::true_type());
        else
          bu_step(std::false_type());
        awake_count = awake;
        visited += awake;
        front.swap(curr);
        rec(ORC_BU, awake_count, old_awake_count, scanned, awake, unvisited);
      } while ((awake_count >= old_awake_count) || (awake_count > n / beta));
      // BitmapToQueue: per-thread buffers appended at an atomic tail, as the
      // reference's QueueBuffer does (so the queue order is not fixed; one
      // thread gives bitmap order).
      {
        std::atomic<int64_t> tail(q_in);
        #pragma omp parallel num_threads(threads)
        {
          std::vector<int32_t> local;
          local.reserve(4096);
          #pragma omp for schedule(static) nowait
          for (int64_t w = 0; w < words; w++) {
            for (uint64_t x = front[w]; x; x &= x - 1)
              local.push_back((int32_t)(64 * w + __builtin_ctzll(x)));
          }
          int64_t at = tail.fetch_add((int64_t)local.size());
          std::copy(local.begin(), local.end(), queue.begin() + at);
        }
        q_in = tail.load();
      }
      q_begin = q_end; q_end = q_in;
      std::fill(front.begin(), front.end(), 0);
      rec(ORC_C, 0, 0, 0, q_end - q_begin, 0);
      scout_count = 1;
    } else {
      // TDStep
      edges_to_check -= scout_count;
      int64_t fsize = q_end - q_begin, examined = 0, scout = 0;
      std::atomic<int64_t> tail(q_in);
      // The examined-edge count equals the frontier's degree sum; it is
      // summed per vertex, outside the edge loop.
      #pragma omp parallel num_threads(threads) reduction(+ : examined, scout)
      {
        std::vector<int32_t> local;
        local.reserve(4096);
        #pragma omp for schedule(dynamic, 64)
        for (int64_t i = q_begin; i < q_end; i++) {
          int32_t u = queue[i];
          examined += off[u + 1] - off[u];
          for (int64_t e = off[u]; e < off[u + 1]; e++) {
            int32_t v = nbr[e];
            int32_t curr_val = __atomic_load_n(&parent[v], __ATOMIC_RELAXED);
            if (curr_val < 0) {
              if (__atomic_compare_exchange_n(&parent[v], &curr_val, u, false,
                                              __ATOMIC_RELAXED, __ATOMIC_RELAXED)) {
                local.push_back(v);
                scout += -(int64_t)curr_val;
              }
            }
          }
        }
        int64_t at = tail.fetch_add((int64_t)local.size());
        std::copy(local.begin(), local.end(), queue.begin() + at);
      }
      q_in = tail.load();
      scout_count = scout;
      q_begin = q_end; q_end = q_in;
      visited += q_end - q_begin;
      rec(ORC_TD, q_end - q_begin, fsize, examined, q_end - q_begin, 0);
    }
  }
  #pragma omp parallel for num_threads(threads) schedule(static)
  for (int64_t v = 0; v < n; v++)
    if (parent[v] < -1) parent[v] = -1;
  auto t1 = std::chrono::steady_clock::now();
  if (seconds) *seconds = std::chrono::duration<double>(t1 - t0).count();
  return overflow ? -1 : ntrace;
}

// Serial queue BFS depth: gapbs-verify/bfs.cc:197-210.
void orc_depth(const int64_t* off, const int32_t* nbr, int64_t n, int32_t source,
               int32_t* depth) {
  for (int64_t v = 0; v < n; v++) depth[v] = -1;
  std::vector<int32_t> q;
  q.reserve(n);
  depth[source] = 0;
  q.push_back(source);
  for (size_t i = 0; i < q.size(); i++) {
    int32_t u = q[i];
    for (int64_t e = off[u]; e < off[u + 1]; e++) {
      int32_t v = nbr[e];
      if (depth[v] == -1) {
        depth[v] = depth[u] + 1;
        q.push_back(v);
      }
    }
  }
}

// BC's BFS phase, serial: PBFS of gapbs-verify/bc.cc:51-92 (src/bc.cc:55-102
// in the DMM copy, whose path counts are unsigned long long and add with
// wrap-around).  Level by level over the queue: an unvisited neighbour gets
// the next depth and is queued; every edge into a vertex of the next depth
// sets its successor bit (bit e of the edge bitmap) and adds the path count
// of its tail.  level_start gets levels + 1 entries; returns levels.
int32_t orc_bc_bfs(const int64_t* off, const int32_t* nbr, int64_t n, int32_t source,
                   uint64_t* sigma, int32_t* depth, uint32_t* succ, int32_t* order,
                   int64_t* level_start) {
  const int64_t m = off[n];
  for (int64_t v = 0; v < n; v++) {
    depth[v] = -1;
    sigma[v] = 0;
  }
  for (int64_t w = 0; w < (m + 31) / 32; w++) succ[w] = 0;
  depth[source] = 0;
  sigma[source] = 1;
  int64_t qs = 0, qe = 1;
  order[0] = source;
  int32_t levels = 0;
  level_start[0] = 0;
  while (qs < qe) {
    const int32_t d = levels + 1;
    int64_t tail = qe;
    for (int64_t i = qs; i < qe; i++) {
      const int32_t u = order[i];
      for (int64_t e = off[u]; e < off[u + 1]; e++) {
        const int32_t v = nbr[e];
        if (depth[v] == -1) {
          depth[v] = d;
          order[tail++] = v;
        }
        if (depth[v] == d) {
          succ[e >> 5] |= 1u << (e & 31);
          sigma[v] += sigma[u];
        }
      }
    }
    levels++;
    level_start[levels] = qe;
    qs = qe;
    qe = tail;
  }
  return levels;
}

// Brandes over k sources, serial (src/bc.cc:106-171 with the BFS phase
// above): per source, dependencies from the deepest level up, each term
// (double)path_counts[u] / (double)path_counts[v] * (1 + delta[v]) added to a
// float delta as the DMM code does, delta added to the score; the scores are
// divided by their maximum at the end.  precise != 0 keeps deltas and scores
// in double instead (the exact values the float sums approximate).
void orc_bc(const int64_t* off, const int32_t* nbr, int64_t n, const int32_t* sources,
            int64_t k, int precise, float* scores) {
  const int64_t m = off[n];
  std::vector<uint64_t> sigma(n);
  std::vector<int32_t> depth(n), order(n > 0 ? n : 1);
  std::vector<int64_t> starts(n + 2);
  std::vector<uint32_t> succ((m + 31) / 32 + 1);
  std::vector<float> delta(n);
  std::vector<double> ddelta(n), dscore(n, 0.0);
  for (int64_t v = 0; v < n; v++) scores[v] = 0.0f;
  for (int64_t i = 0; i < k; i++) {
    const int32_t levels = orc_bc_bfs(off, nbr, n, sources[i], sigma.data(), depth.data(),
                                      succ.data(), order.data(), starts.data());
    std::fill(delta.begin(), delta.end(), 0.0f);
    std::fill(ddelta.begin(), ddelta.end(), 0.0);
    for (int32_t d = levels - 1; d >= 0; d--) {
      for (int64_t it = starts[d]; it < starts[d + 1]; it++) {
        const int32_t u = order[it];
        float delta_u = 0;
        double ddelta_u = 0;
        for (int64_t e = off[u]; e < off[u + 1]; e++) {
          if ((succ[e >> 5] >> (e & 31)) & 1u) {
            const int32_t v = nbr[e];
            const double r = (double)sigma[u] / (double)sigma[v];
            delta_u += r * (1 + delta[v]);
            ddelta_u += r * (1 + ddelta[v]);
          }
        }
        delta[u] = delta_u;
        scores[u] += delta_u;
        ddelta[u] = ddelta_u;
        dscore[u] += ddelta_u;
      }
    }
  }
  if (precise) {
    double big = 0;
    for (int64_t v = 0; v < n; v++) big = std::max(big, dscore[v]);
    for (int64_t v = 0; v < n; v++) scores[v] = (float)(dscore[v] / big);
    return;
  }
  float biggest = 0;
  for (int64_t v = 0; v < n; v++) biggest = std::max(biggest, scores[v]);
  for (int64_t v = 0; v < n; v++) scores[v] = scores[v] / biggest;
}

// BFSVerifier: gapbs-verify/bfs.cc:195-241.  Returns 1 on PASS, 0 on FAIL;
// *why gets 1 "source wrong", 2 "wrong depths", 3 "no such edge",
// 4 "reachability mismatch".
int orc_verify(const int64_t* off, const int32_t* nbr, int64_t n, int32_t source,
               const int32_t* parent, int* why) {
  std::vector<int32_t> depth(n);
  orc_depth(off, nbr, n, source, depth.data());
  *why = 0;
  for (int64_t u = 0; u < n; u++) {
    if (depth[u] != -1 && parent[u] != -1) {
      if (u == source) {
        if (!(parent[u] == u && depth[u] == 0)) { *why = 1; return 0; }
        continue;
      }
      bool found = false;
      for (int64_t e = off[u]; e < off[u + 1]; e++) {
        int32_t v = nbr[e];
        if (v == parent[u]) {
          if (depth[v] != depth[u] - 1) { *why = 2; return 0; }
          found = true;
          break;
        }
      }
      if (!found) { *why = 3; return 0; }
    } else if (depth[u] != parent[u]) {
      *why = 4;
      return 0;
    }
  }
  return 1;
}

// Algorithmic bytes of one BFS under the model stated for this path:
//   InitParent 12n; TD 20|F| + 8 E_td + 8|N|;
//   BU 4n + n/4 + 8|U| + 4 E_bu + 4|N|; TD->BU switch 4|F| + n/8;
//   BU->TD switch n/8 + 4|F'|.
// `steps` are the records orc_dobfs fills in its serial form.
int64_t orc_alg_bytes(int64_t n, const OrcStep* steps, int nsteps) {
  int64_t b = 12 * n;
  for (int i = 0; i < nsteps; i++) {
    const OrcStep& s = steps[i];
    switch (s.kind) {
      case ORC_TD: b += 20 * s.frontier + 8 * s.edges + 8 * s.claimed; break;
      case ORC_BU: b += 4 * n + n / 4 + 8 * s.unvisited + 4 * s.edges + 4 * s.claimed; break;
      case ORC_E:  b += 4 * s.frontier + n / 8; break;
      case ORC_C:  b += n / 8 + 4 * s.claimed; break;
    }
  }
  return b;
}

}  // extern "C"
