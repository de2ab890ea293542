// FP64 values handled on their bit patterns (integer pipes), shared by the
// packing kernels and the tensor-core GEMM epilogue.
//
// GB300 executes FP64 at about 2 operations per clock per SM, so a kernel that
// spends two FP64 instructions per 8-byte element is bound by the FP64 pipe
// rather than by HBM.  Scaling by a power of two and changing a sign are
// therefore done on the bit pattern; only sums use FP64 adds.
#pragma once

#include <cstdint>

namespace gbcc {

// Magnitude bits of |x| 2^k for the magnitude bits m of a finite nonzero x
// whose scaled exponent leaves the normal range or that is subnormal (the
// rare case of scale_pow2), in integer arithmetic: IEEE round to nearest even
// for results below the normal range, infinity above it.
__device__ __forceinline__ unsigned long long scale_pow2_rare(unsigned long long m, int k) {
  const int e = static_cast<int>(m >> 52);
  // significand s and exponent q with |x| = s 2^(q - 1074), s < 2^53
  unsigned long long s = e ? ((m & 0xFFFFFFFFFFFFFull) | (1ull << 52)) : m;
  int q = (e ? e - 1 : 0) + k;
  // normalise so that bit 52 of s is set (subnormal inputs)
  const int lz = __clzll(static_cast<long long>(s)) - 11;  // leading zeros within 53 bits
  s <<= lz;
  q -= lz;
  if (q >= 0x7FE) return 0x7FFull << 52;                    // overflow: infinity
  if (q >= 0) return (static_cast<unsigned long long>(q + 1) << 52) | (s & 0xFFFFFFFFFFFFFull);
  // subnormal result: s 2^q in units of 2^-1074, shift right by -q with RNE
  const int sh = -q;
  if (sh > 54) return 0ull;
  const unsigned long long r = s >> sh, rem = s & ((1ull << sh) - 1), half = 1ull << (sh - 1);
  return r + ((rem > half || (rem == half && (r & 1ull))) ? 1ull : 0ull);
}

// x * 2^k (|k| <= 64) on the bit pattern, exact as the IEEE product: the
// exponent field shifts when x is normal and the result stays normal; zeros,
// infinities and NaN pass through; the rest goes to scale_pow2_rare.  No FP64
// instruction is issued.
__device__ __forceinline__ double scale_pow2(double x, int k) {
  // common case on the high word: exponent field (bits 20-30) + k
  const int hi = __double2hiint(x);
  const int e = (hi >> 20) & 0x7FF;
  const int ek = e + k;
  if (e != 0 && e != 0x7FF && ek >= 1 && ek <= 0x7FE) return __hiloint2double(hi + k * (1 << 20), __double2loint(x));
  const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(x));
  const unsigned long long m = b & 0x7FFFFFFFFFFFFFFFull;
  if (m == 0ull || e == 0x7FF) return x;
  return __longlong_as_double(static_cast<long long>((b & 0x8000000000000000ull) | scale_pow2_rare(m, k)));
}

// -x when neg (sign bit flip), x otherwise
__device__ __forceinline__ double flip_sign(double x, bool neg) {
  return __longlong_as_double(__double_as_longlong(x) ^ (neg ? static_cast<long long>(1ull << 63) : 0ll));
}

// float -> double by rewriting the bit pattern (exact), integer operations
// only.  GB300 runs FP64 arithmetic and FP64 conversions at ~2 per clock per
// SM, and the epilogue of a short-K contraction is bound by them (ncu: FP64
// pipe 64 % busy, DRAM 14 % at K = 32).  Every class of input is handled
// without a hardware conversion (a rare-case fallback would be evaluated for
// every element once the compiler turns the branch into a select).
__device__ __forceinline__ double f2d_exact(float f) {
  const uint32_t b = __float_as_uint(f);
  const uint32_t e = (b >> 23) & 0xFFu, m = b & 0x7FFFFFu;
  const uint64_t sign = static_cast<uint64_t>(b >> 31) << 63;
  uint64_t d;
  if (e == 0xFFu) {
    d = sign | (0x7FFull << 52) | (static_cast<uint64_t>(m) << 29);  // inf / nan
  } else if (e != 0u) {
    d = sign | (static_cast<uint64_t>(e + 896u) << 52) | (static_cast<uint64_t>(m) << 29);
  } else if (m == 0u) {
    d = sign;
  } else {  // subnormal: m 2^-149 with leading bit p
    const int p = 31 - __clz(static_cast<int>(m));
    d = sign | (static_cast<uint64_t>(p + 874) << 52) | ((static_cast<uint64_t>(m) << (52 - p)) & 0xFFFFFFFFFFFFFull);
  }
  return __longlong_as_double(static_cast<long long>(d));
}

}  // namespace gbcc
