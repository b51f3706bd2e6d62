// Test driver for the query server's batching policy (serve_policy.h), run by
// tests/test_serve_policy.py.  Reads one case per line from stdin and prints
// one answer per line:
//   pick <lanes> <W> <key_0> ... <key_{W-1}>   ->  chosen positions, ascending
//   plain <k> <plain_ms> <batch_ms> <batches_in_flight>   ->  0 or 1
#include <cstdio>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "serve_policy.h"

int main() {
  std::string line;
  while (std::getline(std::cin, line)) {
    std::istringstream in(line);
    std::string op;
    in >> op;
    if (op == "pick") {
      size_t lanes = 0, w = 0;
      in >> lanes >> w;
      std::vector<int> keys(w);
      for (size_t i = 0; i < w; i++) in >> keys[i];
      const std::vector<uint32_t> got = gbbfs::pick_group(keys, lanes);
      for (size_t i = 0; i < got.size(); i++) std::printf(i ? " %u" : "%u", got[i]);
      std::printf("\n");
    } else if (op == "plain") {
      int k = 0, busy = 0;
      double p = 0, b = 0;
      in >> k >> p >> b >> busy;
      std::printf("%d\n", gbbfs::plain_is_cheaper(k, p, b, busy) ? 1 : 0);
    } else {
      std::printf("?\n");
    }
  }
  return 0;
}
