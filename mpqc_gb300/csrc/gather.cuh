// Device helpers of the gather / pack kernels (kernels.cu: FP64 outputs and
// BF16 splits; pack_fixed.cu: the fixed-point slices of GBCC_PREC_FP64_TC).
// Everything here has internal linkage in each translation unit.
#pragma once

#include <cuda_bf16.h>

#include <algorithm>

#include "fp_bits.cuh"
#include "kernels.h"

namespace gbcc {
namespace {

// q = x / d and r = x % d for 0 <= x, d < 2^32 (every index split in these
// kernels: x < v^2, v o, o^2).  32-bit division is a few integer and FP32
// instructions; 64-bit integer division is a long sequence that also occupies
// the FP64 pipe, which measurably slowed the elementwise kernels.
__device__ __forceinline__ void divmod32(int64_t x, int64_t d, int64_t& q, int64_t& r) {
  const unsigned xx = static_cast<unsigned>(x), dd = static_cast<unsigned>(d);
  const unsigned qq = xx / dd;
  q = qq;
  r = xx - qq * dd;
}

// BF16 bits of a finite float, rounded to nearest even (integer operations only)
__device__ __forceinline__ unsigned bf16_rne(float f) {
  const unsigned b = __float_as_uint(f);
  return (b + 0x7FFFu + ((b >> 16) & 1u)) >> 16;
}

// Split of an FP64 value into nslices (<= 3) BF16 slices, x ~ s1 + s2 + s3.
// The value is first taken apart without FP64 arithmetic (GB300 runs FP64
// and its conversions at ~2 per clock per SM): hi = x truncated to 24
// significant bits, exact, from the bit pattern; lo = the remaining 29
// mantissa bits, one integer-to-float conversion (relative error 2^-24 of lo,
// i.e. 2^-47 of x).  Each slice is then the remainder rounded to BF16 (nearest
// even), remainders in FP32: s1 = bf16(hi), r = (hi - s1) + lo, s2 = bf16(r),
// r -= s2, s3 = bf16(r); hi - s1 and r - s2 are exact, so
// |x - s1 - s2 - s3| <= 2^-24 |x| (plus 2^-33 |x| from absorbing lo).
// |x| >= 2^128 gives infinity, |x| < 2^-126 signed zeros, nan stays nan.
// The numpy emulation in the tests follows these steps bit for bit.
__device__ __forceinline__ void split_bits(double x, unsigned short* out, int nslices) {
  const unsigned long long u = static_cast<unsigned long long>(__double_as_longlong(x));
  const unsigned sign = static_cast<unsigned>(u >> 63);
  const int E = static_cast<int>((u >> 52) & 0x7FFull);
  out[0] = out[1] = out[2] = 0;
  const int e32 = E - 896;  // biased FP32 exponent of x
  if (E == 0x7FF) {
    out[0] = static_cast<unsigned short>((sign << 15) | ((u & 0xFFFFFFFFFFFFFull) ? 0x7FC0u : 0x7F80u));
    return;
  }
  if (e32 >= 255) {
    out[0] = static_cast<unsigned short>((sign << 15) | 0x7F80u);
    return;
  }
  if (e32 <= 0) {  // zero, FP64 subnormals and magnitudes below FP32's normal range
    out[0] = static_cast<unsigned short>(sign << 15);
    return;
  }
  const float hi = __uint_as_float((sign << 31) | (static_cast<unsigned>(e32) << 23) |
                                   (static_cast<unsigned>(u >> 29) & 0x7FFFFFu));
  const unsigned lo_int = static_cast<unsigned>(u) & 0x1FFFFFFFu;  // value lo_int * 2^(E - 1075)
  const int es = E - 948;                                           // biased FP32 exponent of 2^(E - 1075)
  float lo = 0.f;
  if (lo_int != 0u) {
    // 2^(E - 1075) is below FP32's normal range for |x| < 2^-74: scale in two steps
    lo = es >= 1 ? __uint2float_rn(lo_int) * __uint_as_float(static_cast<unsigned>(es) << 23)
                 : (__uint2float_rn(lo_int) * 0x1p-64f) * __uint_as_float(static_cast<unsigned>(es + 64) << 23);
    if (sign) lo = -lo;
  }
  const unsigned b1 = bf16_rne(hi);
  out[0] = static_cast<unsigned short>(b1);
  if (nslices < 2) return;
  float r = __fadd_rn(__fsub_rn(hi, __uint_as_float(b1 << 16)), lo);
  const unsigned b2 = bf16_rne(r);
  out[1] = static_cast<unsigned short>(b2);
  if (nslices < 3) return;
  r = __fsub_rn(r, __uint_as_float(b2 << 16));
  out[2] = static_cast<unsigned short>(bf16_rne(r));
}

// ---- fixed-point slices (GatherArgs.fixed; constants in kernels.h) ----

// biased FP64 exponent of x; 0 for zeros, subnormals, infinities and NaN (they
// do not set a row's scale)
__device__ __forceinline__ unsigned exp_field(double x) {
  const unsigned e = (static_cast<unsigned>(__double2hiint(x)) >> 20) & 0x7FFu;
  return e == 0x7FFu ? 0u : e;
}

// BF16 bits of I 2^k for |I| <= 256, the biased BF16 exponent of 2^k being
// `base` (exact: |I| has at most 8 significant bits); flushed to zero below
// BF16's normal range
__device__ __forceinline__ unsigned short bf16_int_pow2(int I, int base) {
  if (I == 0) return 0;
  const unsigned sign = I < 0 ? 0x8000u : 0u;
  const unsigned a = static_cast<unsigned>(I < 0 ? -I : I);
  const int L = 31 - __clz(static_cast<int>(a));  // 0..8
  const int be = base + L;
  if (be <= 0) return static_cast<unsigned short>(sign);
  if (be >= 255) return static_cast<unsigned short>(sign | 0x7F80u);
  const unsigned mant = (L <= 7 ? (a << (7 - L)) : (a >> (L - 7))) & 0x7Fu;
  return static_cast<unsigned short>(sign | (static_cast<unsigned>(be) << 7) | mant);
}

// x as n fixed-point digits under the row exponent eb (the biased FP64
// exponent of the row's largest |x|, so |x| < 2^(E-1) with E = eb - 1021: one
// bit of headroom keeps the leading digit within [-128, 128]), integer
// operations only: X = round(x 2^(8n - E)) from the 53-bit significand (|X| <=
// 2^(8n-1)), then balanced base-256 digits from the least significant up;
// slice p = I_p 2^(E - 8(p+1)), whose biased BF16 exponent base is
// eb - 902 - 8p.  Zeros and subnormals give zero slices; infinities and NaN
// pass to slice 0.
__device__ __forceinline__ void fixed_split(double x, unsigned eb, int n, unsigned short* out) {
#pragma unroll
  for (int p = 0; p < kFixedSlices; ++p) out[p] = 0;
  const unsigned long long u = static_cast<unsigned long long>(__double_as_longlong(x));
  const int e = static_cast<int>((u >> 52) & 0x7FFull);
  if (e == 0x7FF) {
    out[0] = static_cast<unsigned short>((u & 0xFFFFFFFFFFFFFull) ? 0x7FC0u : ((u >> 63) ? 0xFF80u : 0x7F80u));
    return;
  }
  if (e == 0 || eb == 0u) return;
  const int sh = 54 + (static_cast<int>(eb) - e) - kFixedBits * n;  // >= 54 - 8n >= 6
  if (sh > 62) return;
  const long long m = static_cast<long long>((u & 0xFFFFFFFFFFFFFull) | (1ull << 52));
  long long X = (m + (1ll << (sh - 1))) >> sh;
  if (u >> 63) X = -X;
  int d[kFixedSlices];
#pragma unroll
  for (int p = kFixedSlices - 1; p >= 1; --p) {
    if (p >= n) continue;
    const long long r = ((X + 128) & 255) - 128;
    d[p] = static_cast<int>(r);
    X = (X - r) >> 8;
  }
  d[0] = static_cast<int>(X);
#pragma unroll
  for (int p = 0; p < kFixedSlices; ++p)
    if (p < n) out[p] = bf16_int_pow2(d[p], static_cast<int>(eb) - 902 - kFixedBits * p);
}

// Element (r, c) of a BF16 slice panel, k-block major: [Cpad / 64][Rpad][64]
// per slice, so that a 64-wide k-block of consecutive rows (one TMA box of
// the tensor-core GEMM) is a contiguous run of memory.  Cpad is a multiple of 64.
__device__ __forceinline__ int64_t panel_index(const GatherArgs& g, int64_t r, int64_t c) {
  return (c >> 6) * (g.Rpad << 6) + (r << 6) + (c & 63);
}

__device__ __forceinline__ void split_store(double x, __nv_bfloat16* out, int nslices,
                                            int64_t slice_stride, int64_t idx) {
  unsigned short b[3];
  split_bits(x, b, nslices);
  for (int s = 0; s < nslices; ++s) out[s * slice_stride + idx] = __ushort_as_bfloat16(b[s]);
}

// One packed element (r, c) of a slice panel: FIX 0, the BF16 split; the
// fixed-point passes (GatherArgs.fixed) 1, exponent (an atomic max per
// nonzero element), and 2, the digits.  A template parameter, so that the
// BF16 path keeps its registers.
template <int FIX>
__device__ __forceinline__ void pack_store(const GatherArgs& g, int64_t r, int64_t c, double x) {
  if constexpr (FIX == 1) {
    const unsigned e = exp_field(x);
    if (e) atomicMax(g.rowexp + r, e);
  } else if constexpr (FIX == 2) {
    unsigned short b[kFixedSlices];
    fixed_split(x, g.rowexp[r], g.nslices, b);
    const int64_t idx = panel_index(g, r, c);
#pragma unroll
    for (int s = 0; s < kFixedSlices; ++s)
      if (s < g.nslices) g.outs[s * g.slice_stride + idx] = __ushort_as_bfloat16(b[s]);
  } else {
    split_store(x, g.outs, g.nslices, g.slice_stride, panel_index(g, r, c));
  }
}


// coef * x for one gather term whose coefficient is +-2^k (GatherTerm.pow2)
__device__ __forceinline__ double term_scale(const GatherTerm& T, double x) {
  return flip_sign(scale_pow2(x, T.pow2_k), T.pow2_sign != 0ull);
}

// Value of one packed element from NT terms: NT = 0 is a plain load (a single
// unscaled term whose coefficient was folded into the GEMM's alpha), otherwise
// the sum of the scaled terms, one FP64 add per term after the first.  PROD:
// some terms carry a second factor.  The term count, PROD and the
// read-modify-write of the output are template parameters, dispatched once per
// launch: as runtime conditions inside the element loop the compiler
// if-converts them, and the predicated FP64 instructions still occupy the FP64
// pipe.
// NT = -1: any coefficients (GatherArgs.general), an FP64 multiply-add per term.
template <int NT, bool PROD>
__device__ __forceinline__ double gather_value(const GatherArgs& g, int64_t r, int64_t c) {
  if constexpr (NT == 0) {
    return g.t[0].a[g.t[0].ra[r] + g.t[0].ca[c]];
  } else if constexpr (NT < 0) {
    double val = 0.0;
    for (int t = 0; t < g.nterms; ++t) {
      const GatherTerm& T = g.t[t];
      double x = T.a[T.ra[r] + T.ca[c]];
      if (T.b) x *= T.b[T.rb[r] + T.cb[c]];
      val = fma(T.coef, x, val);
    }
    return val;
  } else {
    double x[NT];
#pragma unroll
    for (int t = 0; t < NT; ++t) {
      const GatherTerm& T = g.t[t];
      x[t] = T.a[T.ra[r] + T.ca[c]];
      if constexpr (PROD) {
        if (T.b) x[t] *= T.b[T.rb[r] + T.cb[c]];
      }
    }
    double val = term_scale(g.t[0], x[0]);
#pragma unroll
    for (int t = 1; t < NT; ++t) val += term_scale(g.t[t], x[t]);
    return val;
  }
}

// calls BODY(NT, PROD) for the launch's term count and product flag
#define GBCC_GATHER_DISPATCH(g, BODY)                        \
  do {                                                       \
    const int nt_ = (g).plain ? 0 : (g).nterms;              \
    if ((g).general && nt_ > 0) {                            \
      BODY(-1, true);                                        \
    } else if ((g).products) {                               \
      switch (nt_) {                                         \
        case 1: BODY(1, true); break;                        \
        case 2: BODY(2, true); break;                        \
        case 3: BODY(3, true); break;                        \
        default: BODY(4, true); break;                       \
      }                                                      \
    } else {                                                 \
      switch (nt_) {                                         \
        case 0: BODY(0, false); break;                       \
        case 1: BODY(1, false); break;                       \
        case 2: BODY(2, false); break;                       \
        case 3: BODY(3, false); break;                       \
        default: BODY(4, false); break;                      \
      }                                                      \
    }                                                        \
  } while (0)

// blockDim = (bx, by): threads along C, rows along R.  Each thread takes
// kGatherRows rows per step and issues all their loads (and the old output
// values when beta != 0) before its stores, so that several DRAM loads per
// thread are in flight; one load at a time leaves a pass latency-bound.
constexpr int kGatherRows = 4;

template <int NT, bool PROD, bool RMW, int FIX>
__device__ __forceinline__ void gather_rows(const GatherArgs& g) {
  const int64_t c0 = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  const int64_t cstep = static_cast<int64_t>(gridDim.x) * blockDim.x;
  const int64_t r0 = static_cast<int64_t>(blockIdx.y) * blockDim.y + threadIdx.y;
  const int64_t rstep = static_cast<int64_t>(gridDim.y) * blockDim.y;
  for (int64_t c = c0; c < g.Cpad; c += cstep) {
    const bool cin = c < g.C;
    for (int64_t r = r0; r < g.Rpad; r += kGatherRows * rstep) {
      double val[kGatherRows], old[kGatherRows];
#pragma unroll
      for (int u = 0; u < kGatherRows; ++u) {
        const int64_t ru = r + u * rstep;
        val[u] = (cin && ru < g.R) ? gather_value<NT, PROD>(g, ru, c) : 0.0;
        if constexpr (RMW) old[u] = ru < g.Rpad ? g.out[ru * g.ldo + c] : 0.0;
      }
#pragma unroll
      for (int u = 0; u < kGatherRows; ++u) {
        const int64_t ru = r + u * rstep;
        if (ru >= g.Rpad) break;
        if (g.out) {
          if constexpr (RMW) g.out[ru * g.ldo + c] = fma(g.beta, old[u], val[u]);
          else g.out[ru * g.ldo + c] = val[u];
        } else {
          pack_store<FIX>(g, ru, c, val[u]);
        }
      }
    }
  }
}


// Packs into BF16 slices, 4 consecutive K elements of kSplitRows rows per
// thread step, all loads issued before the stores, any number of terms.  A
// term whose K offsets run in contiguous, even-aligned groups of four (c4) is
// read with two 16-byte vector loads per group where its row offset is even;
// otherwise its K offsets are read as 16-byte vectors and the elements one by
// one.  Every slice gets one 8-byte store per thread and row; the launcher
// checks Cpad, ldo and slice_stride are multiples of 4 (K is padded to 64) so
// the stores are 8-byte aligned.
constexpr int kSplitRows = 2;

// x[0..3] = the term's source at row offset rb and K elements c..c+3
__device__ __forceinline__ void load4(const GatherTerm& T, int64_t rb, int64_t c, int64_t C, double x[4]) {
  const double* __restrict__ a = T.a;
  const int64_t* __restrict__ ca = T.ca;
  if (c + 3 < C) {
    if (T.c4 && (rb & 1) == 0) {
      const int64_t o = ca[c];
      const double2 v01 = *reinterpret_cast<const double2*>(a + rb + o);
      const double2 v23 = *reinterpret_cast<const double2*>(a + rb + o + 2);
      x[0] = v01.x;
      x[1] = v01.y;
      x[2] = v23.x;
      x[3] = v23.y;
    } else {
      const longlong2 o01 = *reinterpret_cast<const longlong2*>(ca + c);
      const longlong2 o23 = *reinterpret_cast<const longlong2*>(ca + c + 2);
      x[0] = a[rb + o01.x];
      x[1] = a[rb + o01.y];
      x[2] = a[rb + o23.x];
      x[3] = a[rb + o23.y];
    }
  } else {
#pragma unroll
    for (int j = 0; j < 4; ++j) x[j] = c + j < C ? a[rb + ca[c + j]] : 0.0;
  }
}

// values of K elements c..c+3 of row r (0 outside R x C), NT terms as in gather_value
template <int NT, bool PROD>
__device__ __forceinline__ void split4_values(const GatherArgs& g, int64_t r, int64_t c, double v[4]) {
  if (r >= g.R) {
#pragma unroll
    for (int j = 0; j < 4; ++j) v[j] = 0.0;
    return;
  }
  if constexpr (NT == 0) {
    load4(g.t[0], g.t[0].ra[r], c, g.C, v);
  } else if constexpr (NT < 0) {
#pragma unroll
    for (int j = 0; j < 4; ++j) v[j] = c + j < g.C ? gather_value<NT, PROD>(g, r, c + j) : 0.0;
  } else {
    double x[NT][4];
#pragma unroll
    for (int t = 0; t < NT; ++t) {
      const GatherTerm& T = g.t[t];
      load4(T, T.ra[r], c, g.C, x[t]);
      if constexpr (PROD) {
        if (T.b) {
          double y[4];
          GatherTerm U = T;
          U.a = T.b;
          U.ca = T.cb;
          U.c4 = 0;
          load4(U, T.rb[r], c, g.C, y);
#pragma unroll
          for (int j = 0; j < 4; ++j) x[t][j] *= y[j];
        }
      }
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      double val = term_scale(g.t[0], x[0][j]);
#pragma unroll
      for (int t = 1; t < NT; ++t) val += term_scale(g.t[t], x[t][j]);
      v[j] = val;
    }
  }
}

// the 4 values split into BF16 slices, one 8-byte store per slice
__device__ __forceinline__ void split4_store(const GatherArgs& g, int64_t r, int64_t c, const double v[4]) {
  unsigned short* o4 = reinterpret_cast<unsigned short*>(g.outs) + panel_index(g, r, c);
  unsigned short b[4][3];
#pragma unroll
  for (int j = 0; j < 4; ++j) split_bits(v[j], b[j], g.nslices);
#pragma unroll
  for (int s = 0; s < 3; ++s) {
    if (s >= g.nslices) break;
    uint2 w;
    w.x = static_cast<unsigned>(b[0][s]) | (static_cast<unsigned>(b[1][s]) << 16);
    w.y = static_cast<unsigned>(b[2][s]) | (static_cast<unsigned>(b[3][s]) << 16);
    *reinterpret_cast<uint2*>(o4 + s * g.slice_stride) = w;
  }
}

// the 4 values of row r in fixed-point digits (GatherArgs.fixed == 2), one
// 8-byte store per slice
__device__ __forceinline__ void fixed4_store(const GatherArgs& g, int64_t r, int64_t c, const double v[4]) {
  unsigned short* o4 = reinterpret_cast<unsigned short*>(g.outs) + panel_index(g, r, c);
  unsigned short b[4][kFixedSlices];
  const unsigned eb = g.rowexp[r];
#pragma unroll
  for (int j = 0; j < 4; ++j) fixed_split(v[j], eb, g.nslices, b[j]);
#pragma unroll
  for (int s = 0; s < kFixedSlices; ++s) {
    if (s >= g.nslices) break;
    uint2 w;
    w.x = static_cast<unsigned>(b[0][s]) | (static_cast<unsigned>(b[1][s]) << 16);
    w.y = static_cast<unsigned>(b[2][s]) | (static_cast<unsigned>(b[3][s]) << 16);
    *reinterpret_cast<uint2*>(o4 + s * g.slice_stride) = w;
  }
}

__device__ __forceinline__ unsigned exp_max4(const double v[4]) {
  return max(max(exp_field(v[0]), exp_field(v[1])), max(exp_field(v[2]), exp_field(v[3])));
}

// OUT 0: BF16 slices; 1: FP64 stores; 2: FP64 read-modify-write (beta);
// 3: fixed-point exponent pass; 4: fixed-point digits
template <int NT, bool PROD, int OUT>
__device__ __forceinline__ void split4_rows(const GatherArgs& g) {
  const int64_t nq = g.Cpad / 4;
  const int64_t q0 = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  const int64_t qstep = static_cast<int64_t>(gridDim.x) * blockDim.x;
  const int64_t r0 = static_cast<int64_t>(blockIdx.y) * blockDim.y + threadIdx.y;
  const int64_t rstep = static_cast<int64_t>(gridDim.y) * blockDim.y;
  for (int64_t r = r0; r < g.Rpad; r += kSplitRows * rstep) {
    // fixed-point exponent pass: the lanes of a warp share their rows (the
    // block is at least 32 wide along C, and the row loop is uniform over a
    // warp), so a warp reduces its maxima and issues one atomic per row
    unsigned emax[kSplitRows];
#pragma unroll
    for (int u = 0; u < kSplitRows; ++u) emax[u] = 0u;
    for (int64_t q = q0; q < nq; q += qstep) {
      const int64_t c = 4 * q;
      double v[kSplitRows][4];
      double2 old[kSplitRows][2];
#pragma unroll
      for (int u = 0; u < kSplitRows; ++u) {
        const int64_t ru = r + u * rstep;
        split4_values<NT, PROD>(g, ru, c, v[u]);
        if constexpr (OUT == 2) {
          if (ru < g.Rpad) {
            const double2* po = reinterpret_cast<const double2*>(g.out + ru * g.ldo + c);
            old[u][0] = po[0];
            old[u][1] = po[1];
          }
        }
      }
#pragma unroll
      for (int u = 0; u < kSplitRows; ++u) {
        const int64_t ru = r + u * rstep;
        if (ru >= g.Rpad) break;
        if constexpr (OUT == 0) {
          split4_store(g, ru, c, v[u]);
        } else if constexpr (OUT == 3) {
          emax[u] = max(emax[u], exp_max4(v[u]));
        } else if constexpr (OUT == 4) {
          fixed4_store(g, ru, c, v[u]);
        } else {
          double2* po = reinterpret_cast<double2*>(g.out + ru * g.ldo + c);
          if constexpr (OUT == 2) {
            po[0] = make_double2(fma(g.beta, old[u][0].x, v[u][0]), fma(g.beta, old[u][0].y, v[u][1]));
            po[1] = make_double2(fma(g.beta, old[u][1].x, v[u][2]), fma(g.beta, old[u][1].y, v[u][3]));
          } else {
            po[0] = make_double2(v[u][0], v[u][1]);
            po[1] = make_double2(v[u][2], v[u][3]);
          }
        }
      }
    }
    if constexpr (OUT == 3) {
#pragma unroll
      for (int u = 0; u < kSplitRows; ++u) {
        const unsigned e = __reduce_max_sync(0xFFFFFFFFu, emax[u]);
        const int64_t ru = r + u * rstep;
        if ((threadIdx.x & 31) == 0 && e != 0u && ru < g.Rpad) atomicMax(g.rowexp + ru, e);
      }
    }
  }
}


// Same contract as gather_kernel for sources contiguous along R: a 32 x 32
// tile is read with the lanes along R (coalesced), transposed through shared
// memory and written with the lanes along C (coalesced).  Block 32 x 8.
template <int NT, bool PROD, bool RMW, int FIX>
__device__ __forceinline__ void gather_tiles(const GatherArgs& g, double (*tile)[33]) {
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int64_t nrt = (g.Rpad + 31) / 32, nct = (g.Cpad + 31) / 32;
  // BF16-slice output with 4-aligned rows: each thread writes 4 consecutive
  // columns of one row (one 8-byte store per slice) instead of one column
  const bool wide = g.outs && ((g.Cpad | g.ldo | g.slice_stride) & 3) == 0 &&
                    (reinterpret_cast<uintptr_t>(g.outs) & 7) == 0;
  for (int64_t t = blockIdx.x; t < nrt * nct; t += gridDim.x) {
    int64_t tr, tc;
    divmod32(t, nct, tr, tc);
    const int64_t r0 = tr * 32, c0 = tc * 32;
    // read: lanes along r
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int64_t r = r0 + tx, c = c0 + ty + 8 * k;
      tile[ty + 8 * k][tx] = (r < g.R && c < g.C) ? gather_value<NT, PROD>(g, r, c) : 0.0;
    }
    __syncthreads();
    if (wide) {
      // thread (row rl, columns cg..cg+3); a warp covers 4 rows x 32 columns
      const int t = ty * 32 + tx, rl = t >> 3, cg = (t & 7) * 4;
      const int64_t r = r0 + rl, c = c0 + cg;
      if (r < g.Rpad && c < g.Cpad) {
        double v[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) v[j] = tile[cg + j][rl];
        if constexpr (FIX == 1) {
          const unsigned e = exp_max4(v);
          if (e) atomicMax(g.rowexp + r, e);
        } else if constexpr (FIX == 2) {
          fixed4_store(g, r, c, v);
        } else {
          split4_store(g, r, c, v);
        }
      }
      __syncthreads();
      continue;
    }
    // write: lanes along c
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int64_t r = r0 + ty + 8 * k, c = c0 + tx;
      if (r < g.Rpad && c < g.Cpad) {
        const double val = tile[tx][ty + 8 * k];
        if (g.out) {
          double* p = g.out + r * g.ldo + c;
          if constexpr (RMW) *p = fma(g.beta, *p, val);
          else *p = val;
        } else {
          pack_store<FIX>(g, r, c, val);
        }
      }
    }
    __syncthreads();
  }
}


// Launch geometry of a gather, shared by the BF16 / FP64 and fixed-point
// launchers: 32 x 32 transposed tiles when the sources run along R; 4 K
// elements per thread when tables, panel strides and output allow 8- or
// 16-byte accesses; otherwise one element per thread.
struct GatherShape {
  enum Kind { kRows, kFour, kTiles } kind;
  dim3 grid, block;
};

inline GatherShape gather_shape(const GatherArgs& g) {
  GatherShape s{};
  if (g.transpose) {
    const int64_t tiles = ((g.Rpad + 31) / 32) * ((g.Cpad + 31) / 32);
    s.kind = GatherShape::kTiles;
    s.grid = dim3(static_cast<unsigned>(std::min<int64_t>(tiles, 152LL * 16)));
    s.block = dim3(32, 8);
    return s;
  }
  bool tables16 = true;
  for (int t = 0; t < g.nterms; ++t)
    tables16 = tables16 && reinterpret_cast<uintptr_t>(g.t[t].ca) % 16 == 0 &&
               (!g.t[t].b || reinterpret_cast<uintptr_t>(g.t[t].cb) % 16 == 0);
  const bool split_ok = g.outs && g.slice_stride % 4 == 0 && reinterpret_cast<uintptr_t>(g.outs) % 8 == 0;
  const bool fp64_ok = g.out && reinterpret_cast<uintptr_t>(g.out) % 16 == 0;
  if ((split_ok || fp64_ok) && tables16 && g.Cpad % 4 == 0 && g.ldo % 4 == 0) {
    const int64_t nq = g.Cpad / 4;
    int bx = 32;
    while (bx < nq && bx < 256) bx <<= 1;
    const int by = 256 / bx;
    const int64_t gx = std::min<int64_t>((nq + bx - 1) / bx, 152LL * 64);
    const int64_t gy = std::min<int64_t>({(g.Rpad + by - 1) / by, std::max<int64_t>(1, 152LL * 64 / gx), 65535LL});
    s.kind = GatherShape::kFour;
    s.grid = dim3(static_cast<unsigned>(gx), static_cast<unsigned>(gy));
    s.block = dim3(bx, by);
    return s;
  }
  int bx = 1;
  while (bx < g.Cpad && bx < 256) bx <<= 1;
  if (bx < 32) bx = 32;
  const int by = 256 / bx;
  int64_t gx = (g.Cpad + bx - 1) / bx;
  int64_t gy = (g.Rpad + by - 1) / by;
  // cap the grid; the kernel loops over the remainder
  const int64_t cap_total = 152LL * 64;
  if (gx > cap_total) gx = cap_total;
  const int64_t gy_cap = std::max<int64_t>(1, cap_total / gx);
  if (gy > gy_cap) gy = gy_cap;
  if (gy > 65535) gy = 65535;
  s.kind = GatherShape::kRows;
  s.grid = dim3(static_cast<unsigned>(gx), static_cast<unsigned>(gy));
  s.block = dim3(bx, by);
  return s;
}

}  // namespace
}  // namespace gbcc
