// Host side of the BFS path: synthetic graph generation, CSR construction,
// source picking and the bfs_output.txt writer.
//
// The graph must be bit-identical to the one the reference's verifier
// rebuilds, so generation keeps the reference's random streams: MT19937
// reseeded with kRandSeed + block for every 2^18-edge block, the bounded
// integers and unit floats libstdc++'s uniform_int_distribution<int32_t> /
// uniform_real_distribution<float> draw from it, and std::shuffle's draws for
// the R-MAT relabelling (gapbs-verify/generator.h:54-117,
// src/generator.h:66-167).  Those distributions are implementation-defined;
// gen_rng.h restates the libstdc++ 13 algorithms, so the graphs do not depend
// on the library this is built with.
//
// The CSR is a function of the edge multiset only (per vertex: sorted,
// de-duplicated neighbours without self-loops; gapbs-verify/builder.h:137-206),
// so the construction below is free to order its work as it likes.

#include <algorithm>
#include <cerrno>
#include <climits>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include <omp.h>

#include "gbbfs.h"
#include "gen_rng.h"

namespace {

const int64_t kRandSeed = 27491095;   // src/util.h:25
const int64_t kGenBlock = int64_t(1) << 18;

struct EdgePair32 { int32_t u, v; };

void GenerateUniform(int64_t nodes, int64_t edges, EdgePair32* el) {
  const int64_t nblocks = (edges + kGenBlock - 1) / kGenBlock;
  #pragma omp parallel for schedule(dynamic, 1)
  for (int64_t b = 0; b < nblocks; b++) {
    gbbfs::Mt19937 rng(static_cast<uint32_t>(kRandSeed + b));
    const uint32_t range = static_cast<uint32_t>(nodes);
    const int64_t lo = b * kGenBlock, hi = std::min(lo + kGenBlock, edges);
    for (int64_t e = lo; e < hi; e++) {
      // The reference's Edge(udist(rng), udist(rng)) is evaluated right to
      // left by g++: the first draw lands in the destination.
      const int32_t dst = static_cast<int32_t>(gbbfs::bounded(rng, range));
      const int32_t src = static_cast<int32_t>(gbbfs::bounded(rng, range));
      el[e].u = src;
      el[e].v = dst;
    }
  }
}

void GenerateRMat(int scale, int64_t nodes, int64_t edges, EdgePair32* el) {
  const float a = 0.57f, b_ = 0.19f, c = 0.19f;
  const float ab = a + b_, abc = a + b_ + c;
  const int64_t nblocks = (edges + kGenBlock - 1) / kGenBlock;
  #pragma omp parallel for schedule(dynamic, 1)
  for (int64_t b = 0; b < nblocks; b++) {
    gbbfs::Mt19937 rng(static_cast<uint32_t>(kRandSeed + b));
    const int64_t lo = b * kGenBlock, hi = std::min(lo + kGenBlock, edges);
    for (int64_t e = lo; e < hi; e++) {
      int32_t src = 0, dst = 0;
      for (int d = 0; d < scale; d++) {
        const float p = gbbfs::unit_float(rng);
        src <<= 1;
        dst <<= 1;
        if (p < ab) {
          dst += (p > a);
        } else {
          src++;
          dst += (p > abc);
        }
      }
      el[e].u = src;
      el[e].v = dst;
    }
  }
  // Relabel every vertex through one random permutation of [0, nodes).
  std::vector<int32_t> perm(nodes);
  #pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < nodes; i++) perm[i] = static_cast<int32_t>(i);
  gbbfs::Mt19937 prng(static_cast<uint32_t>(kRandSeed));
  gbbfs::shuffle_like_libstdcxx(perm.data(), nodes, prng);
  #pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < edges; e++) {
    el[e].u = perm[el[e].u];
    el[e].v = perm[el[e].v];
  }
}

// Exclusive scan of `in` (len entries) into out[0..len], in parallel blocks.
template <typename In>
void ExclusiveScan(const In* in, int64_t len, int64_t* out) {
  const int nt = omp_get_max_threads();
  std::vector<int64_t> part(nt + 1, 0);
  #pragma omp parallel num_threads(nt)
  {
    const int t = omp_get_thread_num();
    const int64_t lo = len * t / nt, hi = len * (t + 1) / nt;
    int64_t s = 0;
    for (int64_t i = lo; i < hi; i++) s += in[i];
    part[t + 1] = s;
    #pragma omp barrier
    #pragma omp single
    for (int i = 0; i < nt; i++) part[i + 1] += part[i];
    int64_t run = part[t];
    for (int64_t i = lo; i < hi; i++) {
      out[i] = run;
      run += in[i];
    }
  }
  out[len] = part[nt];
}

}  // namespace

extern "C" {

void gbbfs_free_host(void* p) { free(p); }

int gbbfs_build_csr(int32_t* el_pairs, int64_t edges, int64_t num_nodes,
                    int64_t** offsets_out, int32_t** neigh_out, int64_t* n_out,
                    int64_t* m_dir_out) {
  if (!offsets_out || !neigh_out || !n_out || !m_dir_out || edges < 0 ||
      (edges > 0 && !el_pairs))
    return GBBFS_ERR_ARG;
  EdgePair32* el = reinterpret_cast<EdgePair32*>(el_pairs);
  // num_nodes = largest ID seen + 1 (gapbs-verify/builder.h:62-71, :213-214)
  // unless the caller fixes it.
  int64_t n = num_nodes;
  if (n < 0) {
    int32_t max_id = 0;
    bool negative = false;
    #pragma omp parallel for reduction(max : max_id) reduction(|| : negative) schedule(static)
    for (int64_t e = 0; e < edges; e++) {
      max_id = std::max(max_id, std::max(el[e].u, el[e].v));
      negative = negative || el[e].u < 0 || el[e].v < 0;
    }
    if (negative) return GBBFS_ERR_ARG;
    n = int64_t(max_id) + 1;
  }
  if (n <= 0 || n > INT32_MAX) return GBBFS_ERR_ARG;
  if (num_nodes >= 0) {
    bool bad = false;
    #pragma omp parallel for reduction(|| : bad) schedule(static)
    for (int64_t e = 0; e < edges; e++)
      bad = bad || el[e].u < 0 || el[e].v < 0 || el[e].u >= n || el[e].v >= n;
    if (bad) return GBBFS_ERR_ARG;
  }

  // Symmetrized degree count and raw (unsorted, with duplicates) adjacency.
  std::vector<int64_t> deg(n, 0);
  #pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < edges; e++) {
    __atomic_fetch_add(&deg[el[e].u], 1, __ATOMIC_RELAXED);
    __atomic_fetch_add(&deg[el[e].v], 1, __ATOMIC_RELAXED);
  }
  std::vector<int64_t> raw_off(n + 1);
  ExclusiveScan(deg.data(), n, raw_off.data());
  std::vector<int32_t> raw(static_cast<size_t>(raw_off[n]));
  std::vector<int64_t> cursor(raw_off.begin(), raw_off.end() - 1);
  #pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < edges; e++) {
    const int32_t u = el[e].u, v = el[e].v;
    raw[__atomic_fetch_add(&cursor[u], 1, __ATOMIC_RELAXED)] = v;
    raw[__atomic_fetch_add(&cursor[v], 1, __ATOMIC_RELAXED)] = u;
  }
  std::vector<int64_t>().swap(cursor);

  // Per vertex: sort, drop duplicates and the self-loop.
  std::vector<int64_t>& kept = deg;
  #pragma omp parallel for schedule(dynamic, 2048)
  for (int64_t u = 0; u < n; u++) {
    int32_t* b = raw.data() + raw_off[u];
    int32_t* e = raw.data() + raw_off[u + 1];
    std::sort(b, e);
    int32_t* w = b;
    for (int32_t* r = b; r < e; r++) {
      if (*r == u) continue;
      if (w != b && *(w - 1) == *r) continue;
      *w++ = *r;
    }
    kept[u] = w - b;
  }
  int64_t* off = static_cast<int64_t*>(malloc(sizeof(int64_t) * (n + 1)));
  if (!off) return GBBFS_ERR_NOMEM;
  ExclusiveScan(kept.data(), n, off);
  const int64_t m = off[n];
  int32_t* nbr = static_cast<int32_t*>(malloc(sizeof(int32_t) * std::max<int64_t>(m, 1)));
  if (!nbr) {
    free(off);
    return GBBFS_ERR_NOMEM;
  }
  #pragma omp parallel for schedule(dynamic, 2048)
  for (int64_t u = 0; u < n; u++)
    memcpy(nbr + off[u], raw.data() + raw_off[u], sizeof(int32_t) * kept[u]);
  *offsets_out = off;
  *neigh_out = nbr;
  *n_out = n;
  *m_dir_out = m;
  return GBBFS_OK;
}

int gbbfs_generate_edges(int scale, int degree, int uniform, int32_t** el_out,
                         int64_t* edges_out) {
  if (!el_out || !edges_out) return GBBFS_ERR_ARG;
  if (scale < 1 || scale > 30 || degree < 1) return GBBFS_ERR_ARG;
  const int64_t gen_nodes = int64_t(1) << scale;
  const int64_t edges = gen_nodes * degree;
  EdgePair32* el = static_cast<EdgePair32*>(malloc(sizeof(EdgePair32) * edges));
  if (!el) return GBBFS_ERR_NOMEM;
  if (uniform)
    GenerateUniform(gen_nodes, edges, el);
  else
    GenerateRMat(scale, gen_nodes, edges, el);
  *el_out = reinterpret_cast<int32_t*>(el);
  *edges_out = edges;
  return GBBFS_OK;
}

int gbbfs_generate(int scale, int degree, int uniform, int64_t** offsets_out,
                   int32_t** neigh_out, int64_t* n_out, int64_t* m_dir_out) {
  int32_t* el = nullptr;
  int64_t edges = 0;
  int rc = gbbfs_generate_edges(scale, degree, uniform, &el, &edges);
  if (rc != GBBFS_OK) return rc;
  rc = gbbfs_build_csr(el, edges, -1, offsets_out, neigh_out, n_out, m_dir_out);
  free(el);
  return rc;
}

int gbbfs_pick_sources(const int64_t* offsets, int64_t n, int64_t given,
                       int count, int32_t* out) {
  if (!offsets || !out || n <= 0 || count < 0) return GBBFS_ERR_ARG;
  if (given != -1) {
    if (given < 0 || given >= n) return GBBFS_ERR_ARG;
    for (int i = 0; i < count; i++) out[i] = static_cast<int32_t>(given);
    return GBBFS_OK;
  }
  if (offsets[n] == 0) return GBBFS_ERR_ARG;  // every vertex has degree 0
  gbbfs::Mt19937 rng(static_cast<uint32_t>(kRandSeed));
  for (int i = 0; i < count; i++) {
    int32_t s;
    do {
      s = static_cast<int32_t>(gbbfs::bounded(rng, static_cast<uint32_t>(n)));
    } while (offsets[s + 1] == offsets[s]);
    out[i] = s;
  }
  return GBBFS_OK;
}

int gbbfs_append_bfs_output(const char* path, const int32_t* parent, int64_t n) {
  if (!path || (!parent && n > 0) || n < 0) return GBBFS_ERR_ARG;
  // Format lines in parallel chunks (each parent is at most 11 characters
  // plus '\n'), then append the chunks in order.
  const int64_t chunk = int64_t(1) << 20;
  const int64_t nchunks = (n + chunk - 1) / chunk;
  std::vector<std::vector<char>> text(nchunks);
  #pragma omp parallel for schedule(dynamic, 1)
  for (int64_t c = 0; c < nchunks; c++) {
    const int64_t lo = c * chunk, hi = std::min(n, lo + chunk);
    std::vector<char>& buf = text[c];
    buf.resize(static_cast<size_t>((hi - lo) * 12));
    char* p = buf.data();
    for (int64_t i = lo; i < hi; i++) {
      int32_t x = parent[i] < -1 ? -1 : parent[i];
      if (x < 0) {
        *p++ = '-';
        *p++ = '1';
      } else {
        char tmp[12];
        int k = 0;
        do {
          tmp[k++] = static_cast<char>('0' + x % 10);
          x /= 10;
        } while (x);
        while (k) *p++ = tmp[--k];
      }
      *p++ = '\n';
    }
    buf.resize(static_cast<size_t>(p - buf.data()));
  }
  FILE* f = fopen(path, "ab");
  if (!f) return GBBFS_ERR_IO;
  for (auto& b : text) {
    if (!b.empty() && fwrite(b.data(), 1, b.size(), f) != b.size()) {
      fclose(f);
      return GBBFS_ERR_IO;
    }
  }
  if (fclose(f) != 0) return GBBFS_ERR_IO;
  return GBBFS_OK;
}

}  // extern "C"
