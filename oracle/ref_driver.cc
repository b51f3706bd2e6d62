// Test-infrastructure driver around the reference's own shared-memory GAPBS BFS.
//
// It is compiled here, from the reference sources where they lie
// (gapbs-verify/bfs.cc and the headers it includes), by oracle/build.py into
// oracle/_ref/.  Nothing in the product links it.  It exists to pin the oracle
// restatement (oracle/gapbs_oracle.cc) and to generate the golden fixtures
// under tests/golden/.
//
// Usage:  gapbs_ref <mode> <out-prefix> <CLApp flags ...>
//   graph   : write <prefix>.off (int64[n+1]) and <prefix>.nbr (int32[m]) of the
//             graph Builder(cli).MakeGraph() builds (gapbs-verify/builder.h:231-252)
//   sources : print -n SourcePicker picks, one per line (gapbs-verify/benchmark.h:46-68)
//   bfs     : run DOBFS (gapbs-verify/bfs.cc:122-173) for -n trials, stdout carries the
//             reference's own PrintStep trace; parents of all trials are appended
//             to <prefix>.par (int32[n] per trial)
//   time    : time DOBFS for -n trials (as src/benchmark.h:127-129 brackets it) and
//             print one "trial <source> <seconds> <reached_degree_sum>" line each
//   fixture : one graph build, then everything a golden fixture records, without
//             writing the (multi-GB) arrays out:
//               "graph <n> <m_dir> <sha256 offsets int64> <sha256 neigh int32>"
//               "sources <s0> <s1> ..."            (-n SourcePicker picks)
//             and per trial DOBFS's own PrintStep trace followed by
//               "result <source> <reached> <reached_degree_sum> <max_depth> <sha256 depth int32>"
//             where depth is the BFS depth the reference's parent tree implies.
#define main gapbs_verify_bfs_main
#include "bfs.cc"
#undef main

#include <cstdio>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>
#include <algorithm>

// SHA-256 (FIPS 180-4), streaming; test infrastructure for the fixture hashes.
struct Sha256 {
  uint32_t h[8] = {0x6a09e667u, 0xbb67ae85u, 0x3c6ef372u, 0xa54ff53au,
                   0x510e527fu, 0x9b05688cu, 0x1f83d9abu, 0x5be0cd19u};
  unsigned char buf[64];
  size_t fill = 0;
  uint64_t total = 0;
  static uint32_t rotr(uint32_t x, int r) { return (x >> r) | (x << (32 - r)); }
  void block(const unsigned char* p) {
    static const uint32_t k[64] = {
        0x428a2f98u, 0x71374491u, 0xb5c0fbcfu, 0xe9b5dba5u, 0x3956c25bu, 0x59f111f1u,
        0x923f82a4u, 0xab1c5ed5u, 0xd807aa98u, 0x12835b01u, 0x243185beu, 0x550c7dc3u,
        0x72be5d74u, 0x80deb1feu, 0x9bdc06a7u, 0xc19bf174u, 0xe49b69c1u, 0xefbe4786u,
        0x0fc19dc6u, 0x240ca1ccu, 0x2de92c6fu, 0x4a7484aau, 0x5cb0a9dcu, 0x76f988dau,
        0x983e5152u, 0xa831c66du, 0xb00327c8u, 0xbf597fc7u, 0xc6e00bf3u, 0xd5a79147u,
        0x06ca6351u, 0x14292967u, 0x27b70a85u, 0x2e1b2138u, 0x4d2c6dfcu, 0x53380d13u,
        0x650a7354u, 0x766a0abbu, 0x81c2c92eu, 0x92722c85u, 0xa2bfe8a1u, 0xa81a664bu,
        0xc24b8b70u, 0xc76c51a3u, 0xd192e819u, 0xd6990624u, 0xf40e3585u, 0x106aa070u,
        0x19a4c116u, 0x1e376c08u, 0x2748774cu, 0x34b0bcb5u, 0x391c0cb3u, 0x4ed8aa4au,
        0x5b9cca4fu, 0x682e6ff3u, 0x748f82eeu, 0x78a5636fu, 0x84c87814u, 0x8cc70208u,
        0x90befffau, 0xa4506cebu, 0xbef9a3f7u, 0xc67178f2u};
    uint32_t w[64];
    for (int i = 0; i < 16; i++)
      w[i] = (uint32_t)p[4 * i] << 24 | (uint32_t)p[4 * i + 1] << 16 |
             (uint32_t)p[4 * i + 2] << 8 | (uint32_t)p[4 * i + 3];
    for (int i = 16; i < 64; i++) {
      uint32_t s0 = rotr(w[i - 15], 7) ^ rotr(w[i - 15], 18) ^ (w[i - 15] >> 3);
      uint32_t s1 = rotr(w[i - 2], 17) ^ rotr(w[i - 2], 19) ^ (w[i - 2] >> 10);
      w[i] = w[i - 16] + s0 + w[i - 7] + s1;
    }
    uint32_t a = h[0], b = h[1], c = h[2], d = h[3], e = h[4], f = h[5], g = h[6], hh = h[7];
    for (int i = 0; i < 64; i++) {
      uint32_t t1 = hh + (rotr(e, 6) ^ rotr(e, 11) ^ rotr(e, 25)) + ((e & f) ^ (~e & g)) + k[i] + w[i];
      uint32_t t2 = (rotr(a, 2) ^ rotr(a, 13) ^ rotr(a, 22)) + ((a & b) ^ (a & c) ^ (b & c));
      hh = g; g = f; f = e; e = d + t1; d = c; c = b; b = a; a = t1 + t2;
    }
    h[0] += a; h[1] += b; h[2] += c; h[3] += d; h[4] += e; h[5] += f; h[6] += g; h[7] += hh;
  }
  void update(const void* data, size_t len) {
    const unsigned char* p = static_cast<const unsigned char*>(data);
    total += len;
    if (fill) {
      size_t take = std::min(len, 64 - fill);
      memcpy(buf + fill, p, take);
      fill += take; p += take; len -= take;
      if (fill == 64) { block(buf); fill = 0; }
    }
    for (; len >= 64; p += 64, len -= 64) block(p);
    if (len) { memcpy(buf, p, len); fill = len; }
  }
  std::string hex() {
    uint64_t bits = total * 8;
    unsigned char pad = 0x80;
    update(&pad, 1);
    unsigned char zero = 0;
    while (fill != 56) update(&zero, 1);
    unsigned char len[8];
    for (int i = 0; i < 8; i++) len[i] = (unsigned char)(bits >> (56 - 8 * i));
    update(len, 8);
    char out[65];
    for (int i = 0; i < 8; i++) snprintf(out + 8 * i, 9, "%08x", h[i]);
    return std::string(out, 64);
  }
};

// Depth of every vertex in the parent tree (-1 where parent < 0); returns
// false on a cycle or a parent chain that does not reach the source.
static bool TreeDepth(const pvector<NodeID> &parent, NodeID source, std::vector<int32_t> &depth) {
  const int64_t n = parent.size();
  depth.assign(n, -1);
  depth[source] = 0;
  std::vector<NodeID> chain;
  for (int64_t v = 0; v < n; v++) {
    if (parent[v] < 0 || depth[v] >= 0) continue;
    chain.clear();
    NodeID u = (NodeID)v;
    while (depth[u] < 0) {
      if (parent[u] < 0 || (int64_t)chain.size() > n) return false;
      chain.push_back(u);
      u = parent[u];
    }
    int32_t d = depth[u];
    for (size_t i = chain.size(); i-- > 0;) depth[chain[i]] = ++d;
  }
  return true;
}

static int64_t ReachedDegreeSum(const Graph &g, const pvector<NodeID> &parent) {
  int64_t s = 0;
  for (NodeID v = 0; v < g.num_nodes(); v++)
    if (parent[v] >= 0) s += g.out_degree(v);
  return s;
}

int main(int argc, char* argv[]) {
  if (argc < 3) {
    fprintf(stderr, "usage: %s graph|sources|bfs|time <out-prefix> <flags>\n", argv[0]);
    return 2;
  }
  std::string mode = argv[1];
  std::string prefix = argv[2];
  argv[2] = argv[0];
  CLApp cli(argc - 2, argv + 2, "breadth-first search (reference driver)");
  if (!cli.ParseArgs())
    return 3;
  Builder b(cli);
  Graph g = b.MakeGraph();
  g.PrintStats();
  if (mode == "graph") {
    pvector<SGOffset> off = g.VertexOffsets(false);
    std::ofstream fo(prefix + ".off", std::ios::binary);
    fo.write(reinterpret_cast<const char*>(off.data()), sizeof(SGOffset) * (g.num_nodes() + 1));
    std::ofstream fn(prefix + ".nbr", std::ios::binary);
    for (NodeID u = 0; u < g.num_nodes(); u++)
      for (NodeID v : g.out_neigh(u))
        fn.write(reinterpret_cast<const char*>(&v), sizeof(NodeID));
    return 0;
  }
  SourcePicker<Graph> sp(g, cli.start_vertex());
  if (mode == "sources") {
    for (int i = 0; i < cli.num_trials(); i++)
      printf("%d\n", sp.PickNext());
    return 0;
  }
  if (mode == "bfs") {
    std::ofstream fp(prefix + ".par", std::ios::binary);
    for (int i = 0; i < cli.num_trials(); i++) {
      pvector<NodeID> parent = DOBFS(g, sp.PickNext());
      fp.write(reinterpret_cast<const char*>(parent.data()), sizeof(NodeID) * g.num_nodes());
    }
    return 0;
  }
  if (mode == "time") {
    for (int i = 0; i < cli.num_trials(); i++) {
      NodeID s = sp.PickNext();
      Timer t;
      t.Start();
      pvector<NodeID> parent = DOBFS(g, s);
      t.Stop();
      printf("trial %d %.9f %lld\n", s, t.Seconds(), (long long)ReachedDegreeSum(g, parent));
    }
    return 0;
  }
  if (mode == "fixture") {
    pvector<SGOffset> off = g.VertexOffsets(false);
    Sha256 ho, hn;
    ho.update(off.data(), sizeof(SGOffset) * (g.num_nodes() + 1));
    for (NodeID u = 0; u < g.num_nodes(); u++)
      hn.update(g.out_neigh(u).begin(), sizeof(NodeID) * g.out_degree(u));
    printf("graph %lld %lld %s %s\n", (long long)g.num_nodes(),
           (long long)g.num_edges_directed(), ho.hex().c_str(), hn.hex().c_str());
    SourcePicker<Graph> picks(g, cli.start_vertex());
    printf("sources");
    for (int i = 0; i < cli.num_trials(); i++)
      printf(" %d", picks.PickNext());
    printf("\n");
    std::vector<int32_t> depth;
    for (int i = 0; i < cli.num_trials(); i++) {
      NodeID s = sp.PickNext();
      pvector<NodeID> parent = DOBFS(g, s);
      if (!TreeDepth(parent, s, depth)) {
        fprintf(stderr, "parent tree of source %d is not a tree\n", s);
        return 4;
      }
      int64_t reached = 0;
      int32_t max_depth = 0;
      for (int64_t v = 0; v < g.num_nodes(); v++)
        if (parent[v] >= 0) {
          reached++;
          max_depth = std::max(max_depth, depth[v]);
        }
      Sha256 hd;
      hd.update(depth.data(), sizeof(int32_t) * depth.size());
      printf("result %d %lld %lld %d %s\n", s, (long long)reached,
             (long long)ReachedDegreeSum(g, parent), max_depth, hd.hex().c_str());
      fflush(stdout);
    }
    return 0;
  }
  fprintf(stderr, "unknown mode %s\n", mode.c_str());
  return 2;
}
