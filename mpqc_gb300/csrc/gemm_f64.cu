// Plain-FP64 GEMM with a scattered epilogue (the plain-FP64 residual path).
//
//   C[cm[m] + cn[n]] = beta * C[...] + alpha * sum_k A[m*lda + k] * B[n*ldb + k]
//
// Both operands are K-contiguous panels.  64x64 output tile per 256-thread
// block, 4x4 register tile per thread, BK = 16, register-staged double
// buffering.  FP64 FMA throughput, not memory, bounds this kernel on GB300.
#include "kernels.h"

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

void launch_gemm_f64(const GemmF64Args& g, cudaStream_t st) {
  if (g.M <= 0 || g.N <= 0) return;
  dim3 grid(static_cast<unsigned>((g.N + BN - 1) / BN), static_cast<unsigned>((g.M + BM - 1) / BM),
            static_cast<unsigned>(g.ksplit > 1 ? g.ksplit : 1));
  gemm_f64_kernel<<<grid, NT, 0, st>>>(g);
  if (g.ksplit > 1)
    launch_splitk_reduce(g.M, g.N, g.ksplit, g.partial, g.M, g.N, g.C, g.cm, g.cn, g.alpha, g.beta, st);
}

}  // namespace gbcc
