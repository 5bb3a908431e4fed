// FP32X fixed point <-> double, by integer arithmetic.
//
// A neighbour sum of the FP32X form is an exact integer v in units of 2^-q.
// Its value as a double is RN(v 2^-q), round to nearest, ties to even.  The
// conversion below builds that double's bit pattern from the integer alone
// (IEEE 754 binary64: sign, 11-bit exponent biased by 1023, 52 fraction bits):
// normalise |v| so its leading one sits at bit 63, keep the top 53 bits,
// round on the 11 bits dropped, and add the rounded significand into the
// exponent field, where a carry out of the significand (rounding up to 2^53)
// raises the exponent by one as it should.  It runs on the integer pipes,
// where the int64 -> double conversion instruction and a scaling by 2^-q
// would take the FP64 pipe (1/64 of the FP32 rate on GB300), which the
// FP32X neighbour kernels otherwise hardly use.
//
// Valid for results in the normal range, 2^-1022 <= |v 2^-q| < 2^1024, which
// holds for every q the FP32X form uses (11 <= q <= 52) and any nonzero v.
// Plain C++ as well, so the host test compares it with the C conversion.
#pragma once

#include <cstdint>

#if defined(__CUDACC__)
#define SPC_FIXED_FN __host__ __device__ __forceinline__
#else
#define SPC_FIXED_FN inline
#endif

namespace spc {

SPC_FIXED_FN int clz_u64(std::uint64_t m) {
#if defined(__CUDA_ARCH__)
  return __clzll(static_cast<long long>(m));
#else
  return m == 0 ? 64 : __builtin_clzll(m);
#endif
}

SPC_FIXED_FN double bits_to_double(std::uint64_t b) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double(static_cast<long long>(b));
#else
  double d;
  __builtin_memcpy(&d, &b, sizeof d);
  return d;
#endif
}

// 2^k exactly, for -1022 <= k <= 1023.
SPC_FIXED_FN double pow2i(int k) {
  return bits_to_double(static_cast<std::uint64_t>(k + 1023) << 52);
}

// RN(v 2^-q) for a 64-bit integer v.
SPC_FIXED_FN double fixed_to_double(long long v, int q) {
  if (v == 0) return 0.0;
  const std::uint64_t sign = v < 0 ? (1ull << 63) : 0ull;
  std::uint64_t m = v < 0 ? 0ull - static_cast<std::uint64_t>(v) : static_cast<std::uint64_t>(v);
  const int lz = clz_u64(m);
  m <<= lz;                              // leading one at bit 63
  const int e = 63 - lz - q;             // exponent of the leading one in the result
  std::uint64_t sig = m >> 11;           // 53 significant bits, leading one at bit 52
  const std::uint64_t rest = m & 0x7ffull;  // the 11 bits dropped
  sig += (rest > 0x400ull || (rest == 0x400ull && (sig & 1ull))) ? 1ull : 0ull;
  // the leading one (bit 52) adds one to the exponent field: bias 1023 - 1
  return bits_to_double(sign | ((static_cast<std::uint64_t>(e + 1022) << 52) + sig));
}

}  // namespace spc
