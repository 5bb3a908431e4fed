// The FP32X fixed-point conversion (csrc/spc_fixed.h) against the C library:
// fixed_to_double(v, q) must equal RN(v 2^-q), which is ldexp((double)v, -q)
// (the int64 -> double conversion rounds to nearest even; the power-of-two
// scaling is exact for normal results), bit for bit, and pow2i(k) must equal
// ldexp(1.0, k).  Prints "ok <n>" with the number of values compared.
#include <cfenv>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <random>

#include "spc_fixed.h"

static std::uint64_t bits_of(double d) {
  std::uint64_t b;
  std::memcpy(&b, &d, sizeof b);
  return b;
}

int main() {
  if (std::fegetround() != FE_TONEAREST) {
    std::printf("rounding mode is not to-nearest\n");
    return 2;
  }
  long long checked = 0, bad = 0;
  auto check = [&](long long v, int q) {
    const double want = std::ldexp(static_cast<double>(v), -q);
    const double got = spc::fixed_to_double(v, q);
    ++checked;
    if (bits_of(want) != bits_of(got)) {
      if (++bad <= 10) std::printf("mismatch v=%lld q=%d want=%a got=%a\n", v, q, want, got);
    }
  };
  for (int k = -1022; k <= 1023; ++k) {
    if (bits_of(spc::pow2i(k)) != bits_of(std::ldexp(1.0, k))) {
      std::printf("pow2i(%d) wrong\n", k);
      return 1;
    }
  }
  std::mt19937_64 rng(20260);
  for (int q = 0; q <= 64; ++q) {
    // edges
    const long long edges[] = {0, 1, -1, 2, -2, 3, (1ll << 53) - 1, 1ll << 53, (1ll << 53) + 1,
                               -(1ll << 53) - 1, (1ll << 62), INT64_MAX, INT64_MIN, INT64_MIN + 1,
                               INT64_MAX - 1024, INT64_MAX - 1023};
    for (long long v : edges) check(v, q);
    // every magnitude, with the 11 dropped bits at the rounding boundaries
    for (int top = 0; top < 63; ++top) {
      for (int t = 0; t < 64; ++t) {
        std::uint64_t m = (1ull << top) | (rng() & ((1ull << top) - 1));
        if (top >= 53 && (t & 3) != 3) {
          // the bits below the 53 kept: exactly half an ulp, just below, just above
          const int drop = top - 52;
          const std::uint64_t dm = (1ull << drop) - 1, half = 1ull << (drop - 1);
          const std::uint64_t r = (t & 3) == 0 ? half : ((t & 3) == 1 ? half - 1 : half + 1);
          m = (m & ~dm) | (r & dm);
        }
        const long long v = static_cast<long long>(m);
        check(v, q);
        check(-v, q);
      }
    }
    // random 64-bit values
    for (int t = 0; t < 20000; ++t) {
      const long long v = static_cast<long long>(rng() >> (rng() % 64));
      check(v, q);
      check(-v, q);
    }
  }
  if (bad) {
    std::printf("%lld of %lld wrong\n", bad, checked);
    return 1;
  }
  std::printf("ok %lld\n", checked);
  return 0;
}
