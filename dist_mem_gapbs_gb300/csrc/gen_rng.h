// The random streams of the reference's graph generator and source picker,
// restated in plain integer and float arithmetic, so that generated graphs
// do not depend on the C++ library they are built with.
//
// The reference (gapbs-verify/generator.h:54-117, gapbs-verify/benchmark.h:
// 46-68, src/generator.h:66-167) draws from std::mt19937 through libstdc++'s
// uniform_int_distribution, uniform_real_distribution<float> and
// std::shuffle.  The distributions are implementation-defined; the graphs the
// reference's verifier rebuilds are those of libstdc++ 13 (GCC 13.3), whose
// published algorithms are restated here:
//   - MT19937, the 32-bit Mersenne Twister of Matsumoto and Nishimura (1998),
//     with the standard's seeding (multiplier 1812433253);
//   - bounded integers in [0, range) from a 32-bit generator by Lemire's
//     nearly divisionless method ("Fast Random Integer Generation in an
//     Interval", 2019): the high half of draw * range, redrawn while the low
//     half falls below (2^32 - range) mod range, which libstdc++ applies
//     whenever the generator's range is exactly 2^32;
//   - a float in [0, 1) from one draw: the draw converted to float (round to
//     nearest) times 2^-32, with 1.0 replaced by the largest float below 1
//     (generate_canonical<float, 24> from a 32-bit generator);
//   - the shuffle: for i = 1 .. n-1, swap element i with one drawn from
//     [0, i]; when (2^32 - 1) / n >= n, the draws are taken two at a time,
//     one bounded integer x in [0, (i+1)(i+2)) giving positions x / (i+2)
//     and x % (i+2) for elements i and i+1, after a first draw in [0, 2) for
//     element 1 when n is even.
// Bit identity with the reference's graphs is checked against fixtures the
// reference binary produced (tests/golden).
#pragma once

#include <cstdint>

#if defined(__CUDACC__)
#define GBBFS_HD __host__ __device__
#else
#define GBBFS_HD
#endif

namespace gbbfs {

struct Mt19937 {
  static constexpr int kN = 624, kM = 397;
  uint32_t mt[kN];
  int idx;

  GBBFS_HD explicit Mt19937(uint32_t seed) {
    mt[0] = seed;
    for (int i = 1; i < kN; i++) mt[i] = 1812433253u * (mt[i - 1] ^ (mt[i - 1] >> 30)) + (uint32_t)i;
    idx = kN;
  }

  // Word i from words i, i+1 and i+m (indices mod n), in place and in order.
  GBBFS_HD static uint32_t mix(uint32_t hi, uint32_t lo, uint32_t far) {
    const uint32_t y = (hi & 0x80000000u) | (lo & 0x7fffffffu);
    return far ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
  }

  GBBFS_HD void twist() {
    int i = 0;
    for (; i < kN - kM; i++) mt[i] = mix(mt[i], mt[i + 1], mt[i + kM]);
    for (; i < kN - 1; i++) mt[i] = mix(mt[i], mt[i + 1], mt[i + kM - kN]);
    mt[kN - 1] = mix(mt[kN - 1], mt[0], mt[kM - 1]);
    idx = 0;
  }

  GBBFS_HD uint32_t operator()() {
    if (idx >= kN) twist();
    uint32_t y = mt[idx++];
    y ^= y >> 11;
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= y >> 18;
    return y;
  }
};

// An integer in [0, range), 1 <= range <= 2^32 - 1 (Lemire's method).
template <typename Rng>
GBBFS_HD inline uint32_t bounded(Rng& g, uint32_t range) {
  uint64_t product = (uint64_t)g() * range;
  uint32_t low = (uint32_t)product;
  if (low < range) {
    const uint32_t threshold = (uint32_t)(0u - range) % range;
    while (low < threshold) {
      product = (uint64_t)g() * range;
      low = (uint32_t)product;
    }
  }
  return (uint32_t)(product >> 32);
}

// A float in [0, 1) from one draw.
template <typename Rng>
GBBFS_HD inline float unit_float(Rng& g) {
  const float r = (float)g() * (1.0f / 4294967296.0f);
  return r >= 1.0f ? 0.99999994f : r;   // 0.99999994f = 1 - 2^-24
}

// Shuffle of a[0..n) in place, drawing as std::shuffle does (host only:
// one sequential stream).
template <typename T, typename Rng>
inline void shuffle_like_libstdcxx(T* a, int64_t n, Rng& g) {
  if (n < 2) return;
  auto swap = [&](int64_t i, int64_t j) {
    const T t = a[i];
    a[i] = a[j];
    a[j] = t;
  };
  const uint64_t range = (uint64_t)n;
  if (0xffffffffull / range >= range) {
    int64_t i = 1;
    if ((range & 1) == 0) {
      swap(i, (int64_t)bounded(g, 2u));
      i++;
    }
    while (i != n) {
      const uint64_t b0 = (uint64_t)i + 1, b1 = b0 + 1;
      const uint32_t x = bounded(g, (uint32_t)(b0 * b1));
      swap(i, (int64_t)(x / b1));
      i++;
      swap(i, (int64_t)(x % b1));
      i++;
    }
    return;
  }
  for (int64_t i = 1; i < n; i++) swap(i, (int64_t)bounded(g, (uint32_t)(i + 1)));
}

}  // namespace gbbfs
