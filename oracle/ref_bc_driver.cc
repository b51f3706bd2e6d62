// Test-infrastructure driver around the reference's shared-memory BC BFS phase.
//
// Compiled by oracle/build.py from the reference's own gapbs-verify/bc.cc
// (and the headers it includes) into oracle/_ref/gapbs_ref_bc.  Nothing in
// the product links it.  It pins the oracle's restatement of BC's BFS phase
// (oracle/gapbs_oracle.cc, orc_bc_bfs) and, through the fixtures it writes,
// the GPU's gbbfs_bc_bfs, to PBFS itself (gapbs-verify/bc.cc:51-92).
//
// Usage:  gapbs_ref_bc <CLApp flags: -g/-u/-k/-f/-s, -n trials>
// For each of the -n SourcePicker sources it runs PBFS and prints
//   "bcbfs <source> <reached> <levels> <counts_exact> <sha256 depth int32[n]>
//    <sha256 path counts uint64[n]> <sha256 successor bits> <level sizes,...>"
// The depth of a vertex is its level in PBFS's depth_index (-1 when not
// reached); path counts are the reference's doubles as unsigned 64-bit
// integers, exact while every count stays below 2^53 (counts_exact = 1);
// the successor bits are the first ceil(m/8) bytes of the succ bitmap (bit e
// of byte e/8 for the directed edge at CSR position e).
#define main gapbs_verify_bc_main
#include "bc.cc"
#undef main

#include <cstdio>
#include <string>
#include <vector>

#include "sha256.h"

int main(int argc, char* argv[]) {
  CLApp cli(argc, argv, "BC BFS phase (reference driver)");
  if (!cli.ParseArgs())
    return 3;
  Builder b(cli);
  Graph g = b.MakeGraph();
  g.PrintStats();
  SourcePicker<Graph> sp(g, cli.start_vertex());
  const int64_t n = g.num_nodes(), m = g.num_edges_directed();
  pvector<CountT> path_counts(n);
  Bitmap succ(m);
  vector<SlidingQueue<NodeID>::iterator> depth_index;
  SlidingQueue<NodeID> queue(n);
  std::vector<int32_t> depth(n);
  std::vector<uint64_t> counts(n);
  for (int t = 0; t < cli.num_trials(); t++) {
    const NodeID source = sp.PickNext();
    path_counts.fill(0);
    depth_index.resize(0);
    queue.reset();
    succ.reset();
    PBFS(g, source, path_counts, succ, depth_index, queue);
    std::fill(depth.begin(), depth.end(), -1);
    std::string sizes;
    // depth_index opens with an empty range (the source's window is pushed
    // twice); a vertex's depth is the number of non-empty ranges before its own.
    const int levels = (int)depth_index.size() - 1;
    int lvl = 0;
    for (int d = 0; d < levels; d++) {
      if (depth_index[d + 1] == depth_index[d]) continue;
      for (auto it = depth_index[d]; it < depth_index[d + 1]; it++) depth[*it] = lvl;
      lvl++;
      sizes += (sizes.empty() ? "" : ",") + std::to_string(depth_index[d + 1] - depth_index[d]);
    }
    int exact = 1;
    for (int64_t v = 0; v < n; v++) {
      if (path_counts[v] >= 9007199254740992.0) exact = 0;
      counts[v] = (uint64_t)path_counts[v];
    }
    const int64_t reached = depth_index.back() - depth_index.front();
    Sha256 hd, hc, hs;
    hd.update(depth.data(), sizeof(int32_t) * n);
    hc.update(counts.data(), sizeof(uint64_t) * n);
    std::vector<unsigned char> bits((m + 7) / 8, 0);
    for (int64_t e = 0; e < m; e++)
      if (succ.get_bit(e)) bits[e >> 3] |= (unsigned char)(1u << (e & 7));
    hs.update(bits.data(), bits.size());
    int nonempty = 0;
    for (int d = 0; d < levels; d++) nonempty += depth_index[d + 1] != depth_index[d];
    printf("bcbfs %d %lld %d %d %s %s %s %s\n", source, (long long)reached, nonempty, exact,
           hd.hex().c_str(), hc.hex().c_str(), hs.hex().c_str(), sizes.c_str());
    fflush(stdout);
  }
  return 0;
}
