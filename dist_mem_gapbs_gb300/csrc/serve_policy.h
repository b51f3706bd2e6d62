// Batching policy of the query server, as plain host functions (no CUDA), so
// that it can be tested on its own: which waiting queries form a graph's next
// batch, and whether a launch runs as plain single-source searches.
#pragma once

#include <algorithm>
#include <cstddef>
#include <cstdint>
#include <numeric>
#include <vector>

namespace gbbfs {

constexpr size_t kGroupWindow = 4;   // batches' worth of the oldest queries a batch is chosen from
constexpr int kPlainBusy = 3;        // plain searches only while fewer batches are in flight

// The waiting queries of one graph that form its next batch, as positions in
// arrival order (0 = oldest), ascending.  keys[i] is the batching key of the
// source of waiting query i, for the first min(waiting, kGroupWindow * lanes)
// queries (the caller passes that window).  A window that fits one batch
// goes whole.  Otherwise the window is sorted stably by key, and the batch is
// the run of `lanes` consecutive queries in that order with the smallest key
// spread among the runs that hold the oldest query (the earliest such run on
// ties).  The oldest query always goes, so a query waits for at most as many
// launches of its graph as there are queries ahead of it.
inline std::vector<uint32_t> pick_group(const std::vector<int>& keys, size_t lanes) {
  const size_t W = keys.size();
  std::vector<uint32_t> idx(W);
  std::iota(idx.begin(), idx.end(), 0u);
  if (W <= lanes) return idx;
  std::stable_sort(idx.begin(), idx.end(),
                   [&](uint32_t a, uint32_t b) { return keys[a] < keys[b]; });
  const size_t p = (size_t)(std::find(idx.begin(), idx.end(), 0u) - idx.begin());
  const size_t lo = p + 1 >= lanes ? p + 1 - lanes : 0;
  const size_t hi = std::min(p, W - lanes);
  size_t best = lo;
  int best_spread = keys[idx[lo + lanes - 1]] - keys[idx[lo]];
  for (size_t st = lo + 1; st <= hi; st++) {
    const int spread = keys[idx[st + lanes - 1]] - keys[idx[st]];
    if (spread < best_spread) {
      best_spread = spread;
      best = st;
    }
  }
  std::vector<uint32_t> out(idx.begin() + (std::ptrdiff_t)best,
                            idx.begin() + (std::ptrdiff_t)(best + lanes));
  std::sort(out.begin(), out.end());
  return out;
}

// Whether a launch of k queries runs as k plain searches: when both costs are
// measured (device ms of one plain search and of one batch at the launch's
// lane width), k plain searches are estimated to take less than the batch,
// and fewer than kPlainBusy batches are in flight.  Under load the step
// kernels of a plain search queue behind other graphs' batches, which hold
// the whole GPU, so there a batch answers sooner.
inline bool plain_is_cheaper(int k, double plain_ms, double batch_ms, int batches_in_flight) {
  return batches_in_flight < kPlainBusy && plain_ms > 0 && batch_ms > 0 &&
         (double)k * plain_ms < batch_ms;
}

}  // namespace gbbfs
