// Plain-FP64 GEMM with a scattered epilogue (the plain-FP64 residual path).
//
//   C[cm[m] + cn[n]] = beta * C[...] + alpha * sum_k A[m*lda + k] * B[n*ldb + k]
//
// Both operands are K-contiguous panels.  64x64 output tile per 256-thread
// block, 4x4 register tile per thread, BK = 16, register-staged double
// buffering.  FP64 FMA throughput, not memory, bounds this kernel on GB300.
#include "kernels.h"

#include <algorithm>

namespace gbcc {
namespace {

constexpr int BM = 64, BN = 64, BK = 16, NT = 256;

__global__ void __launch_bounds__(NT) gemm_f64_kernel(GemmF64Args g) {
  __shared__ double As[2][BK][BM + 1];
  __shared__ double Bs[2][BK][BN + 1];
  const int tid = threadIdx.x;
  const int tx = tid % 16, ty = tid / 16;
  const int64_t m0 = static_cast<int64_t>(blockIdx.y) * BM;
  const int64_t n0 = static_cast<int64_t>(blockIdx.x) * BN;
  // K range of this block (blockIdx.z selects the K split)
  const int64_t kbeg = g.ksplit > 1 ? static_cast<int64_t>(blockIdx.z) * g.k_per_split : 0;
  const int64_t kend = g.ksplit > 1 ? min(g.K, kbeg + g.k_per_split) : g.K;

  double ra[4], rb[4];
  auto load_regs = [&](int64_t k0) {
#pragma unroll
    for (int l = 0; l < 4; ++l) {
      const int idx = tid + NT * l;
      const int row = idx / BK, kk = idx % BK;
      const int64_t m = m0 + row, n = n0 + row, k = k0 + kk;
      ra[l] = (m < g.M && k < kend) ? g.A[m * g.lda + k] : 0.0;
      rb[l] = (n < g.N && k < kend) ? g.B[n * g.ldb + k] : 0.0;
    }
  };
  auto store_smem = [&](int buf) {
#pragma unroll
    for (int l = 0; l < 4; ++l) {
      const int idx = tid + NT * l;
      const int row = idx / BK, kk = idx % BK;
      As[buf][kk][row] = ra[l];
      Bs[buf][kk][row] = rb[l];
    }
  };

  double acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0.0;

  const int64_t nk = (kend - kbeg + BK - 1) / BK;
  load_regs(kbeg);
  store_smem(0);
  __syncthreads();
  for (int64_t kt = 0; kt < nk; ++kt) {
    const int buf = kt & 1;
    if (kt + 1 < nk) load_regs(kbeg + (kt + 1) * BK);
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      double a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[buf][kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[buf][kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
    }
    if (kt + 1 < nk) store_smem(buf ^ 1);
    __syncthreads();
  }

  if (g.ksplit > 1) {
    double* P = g.partial + static_cast<int64_t>(blockIdx.z) * g.M * g.N;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int64_t m = m0 + ty + 16 * i;
      if (m >= g.M) continue;
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int64_t n = n0 + tx + 16 * j;
        if (n < g.N) P[m * g.N + n] = acc[i][j];
      }
    }
    return;
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int64_t m = m0 + ty + 16 * i;
    if (m >= g.M) continue;
    const int64_t om = g.cm[m];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int64_t n = n0 + tx + 16 * j;
      if (n >= g.N) continue;
      double* p = g.C + om + g.cn[n];
      const double v = g.alpha * acc[i][j];
      *p = (g.beta == 0.0) ? v : fma(g.beta, *p, v);
    }
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// short-K contraction on CUDA cores (see kernels.h)

// double -> float, rounded to nearest (one FP32 addition of an exact head and
// a rounded tail taken from the bit pattern; no FP64 instruction).  |x| below
// FP32's normal range gives zero, beyond it infinity.
__device__ __forceinline__ float d2f_rn(double x) {
  const unsigned long long u = static_cast<unsigned long long>(__double_as_longlong(x));
  const unsigned sign = static_cast<unsigned>(u >> 63);
  const int E = static_cast<int>((u >> 52) & 0x7FFull);
  const int e32 = E - 896;
  if (E == 0x7FF) return __uint_as_float((sign << 31) | 0x7F800000u | ((u & 0xFFFFFFFFFFFFFull) ? 0x400000u : 0u));
  if (e32 >= 255) return __uint_as_float((sign << 31) | 0x7F800000u);
  if (e32 <= 0) return __uint_as_float(sign << 31);
  const float hi = __uint_as_float((sign << 31) | (static_cast<unsigned>(e32) << 23) |
                                   (static_cast<unsigned>(u >> 29) & 0x7FFFFFu));
  const unsigned lo_int = static_cast<unsigned>(u) & 0x1FFFFFFFu;
  if (lo_int == 0u) return hi;
  const int es = E - 948;
  float lo = es >= 1 ? __uint2float_rn(lo_int) * __uint_as_float(static_cast<unsigned>(es) << 23)
                     : (__uint2float_rn(lo_int) * 0x1p-64f) * __uint_as_float(static_cast<unsigned>(es + 64) << 23);
  if (sign) lo = -lo;
  return __fadd_rn(hi, lo);
}

// float -> double from the bit pattern (integer operations only)
__device__ __forceinline__ double f2d_bits(float f) {
  const unsigned b = __float_as_uint(f);
  const unsigned e = (b >> 23) & 0xFFu, m = b & 0x7FFFFFu;
  const unsigned long long sign = static_cast<unsigned long long>(b >> 31) << 63;
  unsigned long long d;
  if (e == 0xFFu) {
    d = sign | (0x7FFull << 52) | (static_cast<unsigned long long>(m) << 29);
  } else if (e != 0u) {
    d = sign | (static_cast<unsigned long long>(e + 896u) << 52) | (static_cast<unsigned long long>(m) << 29);
  } else if (m == 0u) {
    d = sign;
  } else {
    const int p = 31 - __clz(static_cast<int>(m));
    d = sign | (static_cast<unsigned long long>(p + 874) << 52) |
        ((static_cast<unsigned long long>(m) << (52 - p)) & 0xFFFFFFFFFFFFFull);
  }
  return __longlong_as_double(static_cast<long long>(d));
}

// TM x TN output tiles (64 x 64, or 128 x 32 for N <= 32), 256 threads, 16
// outputs per thread.  MMAJOR: lanes along M (C unit-stride in M), else along
// N.  Threads (u, w) = (tid % 16, tid / 16) own rows u + 16 i and columns
// w + 16 j (roles swapped for !MMAJOR), so 16 lanes touch 16 consecutive
// elements of C.  The tile's reads of C are issued first, so their latency
// overlaps the operand loads and the FMAs (the kernel is bound by the FP64
// read-modify-write of C, not by arithmetic).
template <bool MMAJOR, int TM, int TN>
__global__ void __launch_bounds__(256, 2) gemm_smallk_kernel(GemmF64Args g) {
  constexpr int IM = TM / 16, JN = TN / 16;
  static_assert(IM * JN == 16, "16 outputs per thread");
  __shared__ float As[kSmallK][TM + 1];
  __shared__ float Bs[kSmallK][TN + 1];
  const int tid = threadIdx.x;
  const int K = static_cast<int>(g.K);
  const int64_t mt = (g.M + TM - 1) / TM, nt = (g.N + TN - 1) / TN;
  const int u = tid % 16, w = tid / 16;
  const bool has_c = g.beta != 0.0;
  for (int64_t tile = blockIdx.x; tile < mt * nt; tile += gridDim.x) {
    const int64_t m0 = (tile / nt) * TM, n0 = (tile % nt) * TN;
    int64_t om[IM], on[JN];  // -1 outside C
#pragma unroll
    for (int i = 0; i < IM; ++i) {
      const int64_t m = m0 + (MMAJOR ? u : w) + 16 * i;
      om[i] = m < g.M ? g.cm[m] : -1;
    }
#pragma unroll
    for (int j = 0; j < JN; ++j) {
      const int64_t n = n0 + (MMAJOR ? w : u) + 16 * j;
      on[j] = n < g.N ? g.cn[n] : -1;
    }
    double c[IM][JN];
#pragma unroll
    for (int i = 0; i < IM; ++i)
#pragma unroll
      for (int j = 0; j < JN; ++j) c[i][j] = (has_c && om[i] >= 0 && on[j] >= 0) ? g.C[om[i] + on[j]] : 0.0;
    for (int e = tid; e < TM * K; e += blockDim.x) {
      const int r = e / K, k = e % K;
      const int64_t m = m0 + r;
      As[k][r] = m < g.M ? d2f_rn(g.A[m * g.lda + k]) : 0.f;
    }
    for (int e = tid; e < TN * K; e += blockDim.x) {
      const int r = e / K, k = e % K;
      const int64_t n = n0 + r;
      Bs[k][r] = n < g.N ? d2f_rn(g.B[n * g.ldb + k]) : 0.f;
    }
    __syncthreads();
    float acc[IM][JN];
#pragma unroll
    for (int i = 0; i < IM; ++i)
#pragma unroll
      for (int j = 0; j < JN; ++j) acc[i][j] = 0.f;
    for (int k = 0; k < K; ++k) {
      float a[IM], b[JN];
#pragma unroll
      for (int i = 0; i < IM; ++i) a[i] = As[k][(MMAJOR ? u : w) + 16 * i];
#pragma unroll
      for (int j = 0; j < JN; ++j) b[j] = Bs[k][(MMAJOR ? w : u) + 16 * j];
#pragma unroll
      for (int i = 0; i < IM; ++i)
#pragma unroll
        for (int j = 0; j < JN; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    // one FP64 operation per element; the beta cases in separate loops so no
    // multiply by beta is evaluated where beta is 0 or 1
    if (!has_c) {
#pragma unroll
      for (int i = 0; i < IM; ++i)
#pragma unroll
        for (int j = 0; j < JN; ++j)
          if (om[i] >= 0 && on[j] >= 0) g.C[om[i] + on[j]] = g.alpha * f2d_bits(acc[i][j]);
    } else if (g.beta == 1.0) {
#pragma unroll
      for (int i = 0; i < IM; ++i)
#pragma unroll
        for (int j = 0; j < JN; ++j)
          if (om[i] >= 0 && on[j] >= 0) g.C[om[i] + on[j]] = fma(g.alpha, f2d_bits(acc[i][j]), c[i][j]);
    } else {
#pragma unroll
      for (int i = 0; i < IM; ++i)
#pragma unroll
        for (int j = 0; j < JN; ++j)
          if (om[i] >= 0 && on[j] >= 0)
            g.C[om[i] + on[j]] = fma(g.alpha, f2d_bits(acc[i][j]), g.beta * c[i][j]);
    }
    __syncthreads();
  }
}

// Short contractions whose C is contiguous along M (every short-K site of the
// CCSD residual): B (N x K, rounded to FP32, K padded to KS = 32 or 64) stays
// in shared memory, each thread owns one row m of C and keeps that row of A
// in registers, and walks C eight columns at a time.  The eight C loads of a
// group are issued before its dot products (which do not need them), and
// three CTAs per SM (two at KS = 64) keep enough of them in flight to stream
// C, the dominant traffic (16 bytes per output against 8 per A element).
// With a_ra set, A is read in place through its row and column offsets (the
// K offsets staged in shared memory): for a source contiguous along M the
// lanes of a warp read consecutive elements, and no packed panel is written.
// BETA 0: C = alpha acc, 1: C += alpha acc, 2: C = beta C + alpha acc, one
// FP64 FMA per output where beta is 0 or 1.
constexpr int kStreamCols = 8;

__device__ __forceinline__ void prefetch_l2(const double* p) {
  asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

template <int BETA, int KS, bool INPLACE>
__global__ void __launch_bounds__(256, KS == 32 ? 3 : 2) gemm_smallk_stream_kernel(GemmF64Args g) {
  extern __shared__ float Bs[];  // [Npad][KS], then KS K offsets of A
  const int K = static_cast<int>(g.K);
  const int64_t npad = (g.N + kStreamCols - 1) / kStreamCols * kStreamCols;
  int64_t* aca = reinterpret_cast<int64_t*>(Bs + npad * KS);
  for (int64_t e = threadIdx.x; e < npad * KS; e += blockDim.x) {
    const int64_t n = e / KS;
    const int k = static_cast<int>(e % KS);
    Bs[e] = (n < g.N && k < K) ? d2f_rn(g.B[n * g.ldb + k]) : 0.f;
  }
  if constexpr (INPLACE)
    for (int k = threadIdx.x; k < KS; k += blockDim.x) aca[k] = k < K ? g.a_ca[k] : 0;
  __syncthreads();
  const int64_t mtiles = (g.M + blockDim.x - 1) / blockDim.x;
  for (int64_t t = blockIdx.x; t < mtiles; t += gridDim.x) {
    const int64_t m = t * blockDim.x + threadIdx.x;
    if (m >= g.M) continue;
    float a[KS];
    if constexpr (INPLACE) {
      const double* arow = g.A + g.a_ra[m];
#pragma unroll
      for (int k = 0; k < KS; ++k) a[k] = k < K ? d2f_rn(arow[aca[k]]) : 0.f;
    } else {
#pragma unroll
      for (int k = 0; k < KS; ++k) a[k] = k < K ? d2f_rn(g.A[m * g.lda + k]) : 0.f;
    }
    double* crow = g.C + g.cm[m];
    if constexpr (BETA != 0) {
#pragma unroll
      for (int j = kStreamCols; j < 2 * kStreamCols; ++j)
        if (j < g.N) prefetch_l2(crow + g.cn[j]);
    }
    for (int64_t n0 = 0; n0 < g.N; n0 += kStreamCols) {
      // (the column offsets are read again at the store, from L1, rather
      // than held: 8 live 64-bit offsets pushed the kernel into spills)
      double c[kStreamCols];
      if constexpr (BETA != 0) {
        // C two groups ahead into L2, so that each group's loads hit L2
#pragma unroll
        for (int j = 0; j < kStreamCols; ++j) {
          const int64_t n = n0 + 2 * kStreamCols + j;
          if (n < g.N) prefetch_l2(crow + g.cn[n]);
        }
#pragma unroll
        for (int j = 0; j < kStreamCols; ++j) c[j] = n0 + j < g.N ? crow[g.cn[n0 + j]] : 0.0;
      }
      float acc[kStreamCols];
#pragma unroll
      for (int j = 0; j < kStreamCols; ++j) {
        const float4* b4 = reinterpret_cast<const float4*>(Bs + (n0 + j) * KS);
        float s = 0.f;
#pragma unroll
        for (int q = 0; q < KS / 4; ++q) {
          const float4 b = b4[q];
          s = fmaf(a[4 * q], b.x, s);
          s = fmaf(a[4 * q + 1], b.y, s);
          s = fmaf(a[4 * q + 2], b.z, s);
          s = fmaf(a[4 * q + 3], b.w, s);
        }
        acc[j] = s;
      }
#pragma unroll
      for (int j = 0; j < kStreamCols; ++j) {
        if (n0 + j >= g.N) continue;
        double* p = crow + g.cn[n0 + j];
        const double y = f2d_bits(acc[j]);
        if constexpr (BETA == 0) *p = g.alpha * y;
        else if constexpr (BETA == 1) *p = fma(g.alpha, y, c[j]);
        else *p = fma(g.alpha, y, g.beta * c[j]);
      }
    }
  }
}

template <int TM, int TN>
void launch_smallk_tiles(const GemmF64Args& g, cudaStream_t st) {
  const int64_t tiles = ((g.M + TM - 1) / TM) * ((g.N + TN - 1) / TN);
  const unsigned grid = static_cast<unsigned>(std::min<int64_t>(tiles, static_cast<int64_t>(num_sms()) * 2));
  if (g.m_major)
    gemm_smallk_kernel<true, TM, TN><<<grid, 256, 0, st>>>(g);
  else
    gemm_smallk_kernel<false, TM, TN><<<grid, 256, 0, st>>>(g);
}

// The stream kernels take at most 64 KB of dynamic shared memory; the limit
// is raised once to that bound (not to each launch's size) so that launches
// from concurrent solves never see another thread's smaller limit.
template <typename K>
bool allow_stream_smem(K kernel) {
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 64 * 1024) == cudaSuccess;
}

template <int BETA, int KS, bool INPLACE>
void launch_stream_k(const GemmF64Args& g, unsigned grid, size_t smem, cudaStream_t st) {
  static const bool attr = allow_stream_smem(gemm_smallk_stream_kernel<BETA, KS, INPLACE>);
  (void)attr;
  gemm_smallk_stream_kernel<BETA, KS, INPLACE><<<grid, 256, smem, st>>>(g);
}

template <int KS, bool INPLACE>
void launch_stream(const GemmF64Args& g, size_t smem, cudaStream_t st) {
  const int64_t mtiles = (g.M + 255) / 256;
  const unsigned grid =
      static_cast<unsigned>(std::min<int64_t>(mtiles, static_cast<int64_t>(num_sms()) * (KS == 32 ? 3 : 2)));
  if (g.beta == 0.0) launch_stream_k<0, KS, INPLACE>(g, grid, smem, st);
  else if (g.beta == 1.0) launch_stream_k<1, KS, INPLACE>(g, grid, smem, st);
  else launch_stream_k<2, KS, INPLACE>(g, grid, smem, st);
}

size_t stream_smem(int64_t N, int64_t K) {
  const int64_t npad = (N + kStreamCols - 1) / kStreamCols * kStreamCols;
  const int64_t ks = K <= 32 ? 32 : 64;
  return static_cast<size_t>(npad * ks) * sizeof(float) + static_cast<size_t>(ks) * sizeof(int64_t);
}

bool smallk_streams(int64_t N, int64_t K, bool m_major) {
  return m_major && K <= 64 && stream_smem(N, K) <= 64 * 1024;
}

bool launch_gemm_smallk(const GemmF64Args& g, cudaStream_t st) {
  if (g.M <= 0 || g.N <= 0) return true;
  if (smallk_streams(g.N, g.K, g.m_major != 0)) {
    const size_t smem = stream_smem(g.N, g.K);
    if (g.K <= 32) {
      if (g.a_ra) launch_stream<32, true>(g, smem, st);
      else launch_stream<32, false>(g, smem, st);
    } else {
      if (g.a_ra) launch_stream<64, true>(g, smem, st);
      else launch_stream<64, false>(g, smem, st);
    }
    return true;
  }
  if (g.a_ra) return false;  // A in place: stream kernel only
  if (g.N <= 32)
    launch_smallk_tiles<128, 32>(g, st);
  else
    launch_smallk_tiles<64, 64>(g, st);
  return true;
}

void launch_gemm_f64(const GemmF64Args& g, cudaStream_t st) {
  if (g.M <= 0 || g.N <= 0) return;
  dim3 grid(static_cast<unsigned>((g.N + BN - 1) / BN), static_cast<unsigned>((g.M + BM - 1) / BM),
            static_cast<unsigned>(g.ksplit > 1 ? g.ksplit : 1));
  gemm_f64_kernel<<<grid, NT, 0, st>>>(g);
  if (g.ksplit > 1)
    launch_splitk_reduce(g.M, g.N, g.ksplit, g.partial, g.M, g.N, g.C, g.cm, g.cn, g.alpha, g.beta, st);
}

}  // namespace gbcc
