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
//             print one "trial <source> <seconds> <reached_degree_sum>" line each;
//             here <out-prefix> is a count c: the trials cycle over the first c
//             SourcePicker picks (0: a fresh pick per trial)
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
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>
#include <algorithm>

#include "sha256.h"

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
    // The out-prefix argument names how many SourcePicker picks the trials
    // cycle over (0: a fresh pick per trial).
    const int cycle = atoi(prefix.c_str());
    std::vector<NodeID> picks;
    for (int i = 0; i < cycle; i++) picks.push_back(sp.PickNext());
    for (int i = 0; i < cli.num_trials(); i++) {
      NodeID s = cycle > 0 ? picks[i % cycle] : sp.PickNext();
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
