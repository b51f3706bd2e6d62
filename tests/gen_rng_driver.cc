// Test driver for the restated random streams (gen_rng.h), run by
// tests/test_gen_rng.py: each check draws the same stream through libstdc++
// (std::mt19937 and its distributions, as the reference calls them) and
// through gen_rng.h, and prints one line per check: its name and 1 if every
// value agreed.
#include <algorithm>
#include <cstdio>
#include <cstdint>
#include <numeric>
#include <random>
#include <vector>

#include "gen_rng.h"

static bool raw_stream(uint32_t seed, int count) {
  std::mt19937 a(seed);
  gbbfs::Mt19937 b(seed);
  for (int i = 0; i < count; i++)
    if ((uint32_t)a() != b()) return false;
  return true;
}

static bool bounded_ints(uint32_t seed, uint32_t range, int count) {
  std::mt19937 a(seed);
  gbbfs::Mt19937 b(seed);
  std::uniform_int_distribution<int64_t> d(0, (int64_t)range - 1);
  for (int i = 0; i < count; i++)
    if ((uint64_t)d(a) != gbbfs::bounded(b, range)) return false;
  return true;
}

static bool unit_floats(uint32_t seed, int64_t count) {
  std::mt19937 a(seed);
  gbbfs::Mt19937 b(seed);
  std::uniform_real_distribution<float> d(0, 1.0f);
  for (int64_t i = 0; i < count; i++)
    if (d(a) != gbbfs::unit_float(b)) return false;
  return true;
}

// The first draw of the stream at or above 2^32 - 128 (such a draw rounds to
// 2^32 as a float, so the unit float is clamped below 1), or -1.
static int64_t first_top_draw(uint32_t seed, int64_t limit) {
  gbbfs::Mt19937 g(seed);
  for (int64_t i = 0; i < limit; i++)
    if (g() >= 0xffffff80u) return i;
  return -1;
}

// Both streams through the first top draw, and its float from both.
static bool clamped_float(uint32_t seed, int64_t at) {
  std::mt19937 a(seed);
  gbbfs::Mt19937 b(seed);
  std::uniform_real_distribution<float> d(0, 1.0f);
  float x = 0, y = 0;
  for (int64_t i = 0; i <= at; i++) {
    x = d(a);
    y = gbbfs::unit_float(b);
    if (x != y) return false;
  }
  return x == y && x < 1.0f && x == 0.99999994f;
}

static bool shuffled(uint32_t seed, int64_t n) {
  std::vector<int32_t> x(n), y(n);
  std::iota(x.begin(), x.end(), 0);
  std::iota(y.begin(), y.end(), 0);
  std::mt19937 a(seed);
  gbbfs::Mt19937 b(seed);
  std::shuffle(x.begin(), x.end(), a);
  gbbfs::shuffle_like_libstdcxx(y.data(), n, b);
  return x == y && a() == b();   // and the streams end in the same place
}

int main() {
  std::printf("raw %d\n", raw_stream(27491095u, 2000000) && raw_stream(0u, 5000) &&
                              raw_stream(0xffffffffu, 5000));
  const uint32_t ranges[] = {1u, 2u, 3u, 7u, 1000u, 65536u, 1u << 20, (1u << 26) + 1,
                             1u << 31, (1u << 31) + 12345u, 0xfffffff0u, 0xffffffffu};
  bool ok = true;
  for (uint32_t r : ranges) ok = ok && bounded_ints(27491095u + r, r, 200000);
  std::printf("bounded %d\n", ok);
  std::printf("float %d\n", unit_floats(27491095u, 20000000));
  const int64_t at = first_top_draw(27491095u, 1ll << 31);
  std::printf("float_top_at %lld\n", (long long)at);
  std::printf("float_clamped %d\n", at >= 0 && clamped_float(27491095u, at));
  ok = true;
  const int64_t sizes[] = {0, 1, 2, 3, 4, 5, 6, 31, 32, 1000, 1001, 65535, 65536, 65537, 1 << 20};
  for (int64_t n : sizes) ok = ok && shuffled(27491095u, n);
  std::printf("shuffle %d\n", ok);
  return 0;
}
