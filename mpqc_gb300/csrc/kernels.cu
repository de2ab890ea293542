// Elementwise, gather/pack, reduction and DIIS kernels of the CCSD engine.
//
// Everything here is FP64 and HBM-bound: the amplitude-sized arrays
// (o^2 v^2 doubles) are streamed once per kernel with coalesced accesses.
#include "kernels.h"

#include <algorithm>

namespace gbcc {

namespace {

constexpr int kThreads = 256;

inline unsigned grid_for(int64_t n, int threads, int64_t cap = 152 * 32) {
  int64_t b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  if (b > cap) b = cap;
  return static_cast<unsigned>(b);
}

// Split a value into nslices BF16 pieces x = s0 + s1 + ... (each the
// round-to-nearest BF16 of what the previous slices left over).
__device__ __forceinline__ void split_store(double x, __nv_bfloat16* out, int nslices,
                                            int64_t slice_stride, int64_t idx) {
  for (int s = 0; s < nslices; ++s) {
    __nv_bfloat16 h = __double2bfloat16(x);
    out[s * slice_stride + idx] = h;
    x -= static_cast<double>(__bfloat162float(h));
  }
}

__global__ void __launch_bounds__(kThreads) gather_kernel(GatherArgs g) {
  // blockDim = (bx, by): threads along C, rows along R.
  const int64_t c0 = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  const int64_t cstep = static_cast<int64_t>(gridDim.x) * blockDim.x;
  const int64_t r0 = static_cast<int64_t>(blockIdx.y) * blockDim.y + threadIdx.y;
  const int64_t rstep = static_cast<int64_t>(gridDim.y) * blockDim.y;
  for (int64_t r = r0; r < g.Rpad; r += rstep) {
    const bool rin = r < g.R;
    for (int64_t c = c0; c < g.Cpad; c += cstep) {
      double val = 0.0;
      if (rin && c < g.C) {
#pragma unroll
        for (int t = 0; t < kMaxTerms; ++t) {
          if (t < g.nterms) {
            const GatherTerm& T = g.t[t];
            double x = T.a[T.ra[r] + T.ca[c]];
            if (T.b) x *= T.b[T.rb[r] + T.cb[c]];
            val = fma(T.coef, x, val);
          }
        }
      }
      if (g.out) {
        double* p = g.out + r * g.ldo + c;
        *p = (g.beta == 0.0) ? val : fma(g.beta, *p, val);
      } else {
        split_store(val, g.outs, g.nslices, g.slice_stride, r * g.ldo + c);
      }
    }
  }
}

// Same contract as gather_kernel for sources contiguous along R: a 32 x 32
// tile is read with the lanes along R (coalesced), transposed through shared
// memory and written with the lanes along C (coalesced).  Block 32 x 8.
__global__ void __launch_bounds__(256) gather_t_kernel(GatherArgs g) {
  __shared__ double tile[32][33];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int64_t nrt = (g.Rpad + 31) / 32, nct = (g.Cpad + 31) / 32;
  for (int64_t t = blockIdx.x; t < nrt * nct; t += gridDim.x) {
    const int64_t r0 = (t / nct) * 32, c0 = (t % nct) * 32;
    // read: lanes along r
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int64_t r = r0 + tx, c = c0 + ty + 8 * k;
      double val = 0.0;
      if (r < g.R && c < g.C) {
#pragma unroll
        for (int q = 0; q < kMaxTerms; ++q) {
          if (q < g.nterms) {
            const GatherTerm& T = g.t[q];
            double x = T.a[T.ra[r] + T.ca[c]];
            if (T.b) x *= T.b[T.rb[r] + T.cb[c]];
            val = fma(T.coef, x, val);
          }
        }
      }
      tile[ty + 8 * k][tx] = val;
    }
    __syncthreads();
    // write: lanes along c
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int64_t r = r0 + ty + 8 * k, c = c0 + tx;
      if (r < g.Rpad && c < g.Cpad) {
        const double val = tile[tx][ty + 8 * k];
        if (g.out) {
          double* p = g.out + r * g.ldo + c;
          *p = (g.beta == 0.0) ? val : fma(g.beta, *p, val);
        } else {
          split_store(val, g.outs, g.nslices, g.slice_stride, r * g.ldo + c);
        }
      }
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------

__device__ __forceinline__ double block_sum(double v, double* sh) {
  // fixed-order tree reduction over the block (deterministic)
  const int tid = threadIdx.x;
  sh[tid] = v;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (tid < s) sh[tid] += sh[tid + s];
    __syncthreads();
  }
  double r = sh[0];
  __syncthreads();
  return r;
}

__global__ void __launch_bounds__(kThreads) energy_partial_kernel(
    int64_t o, int64_t v, const double* __restrict__ r1, const double* __restrict__ r2,
    const double* __restrict__ f_ai, const double* __restrict__ g_abij,
    const double* __restrict__ t1, const double* __restrict__ tau, double* __restrict__ partial) {
  __shared__ double sh[kThreads];
  const int64_t o2 = o * o;
  double s_r1 = 0.0, s_r2 = 0.0, s_e1 = 0.0, s_e2 = 0.0;
  for (int64_t p = blockIdx.x; p < v * v; p += gridDim.x) {
    const int64_t a = p / v, b = p % v;
    const double* r2p = r2 + p * o2;
    const double* gp = g_abij + p * o2;
    const double* tp = tau + p * o2;
    const double* tq = tau + (b * v + a) * o2;
    for (int64_t ij = threadIdx.x; ij < o2; ij += blockDim.x) {
      const double r = r2p[ij];
      s_r2 = fma(r, r, s_r2);
      s_e2 = fma(gp[ij] + r, 2.0 * tp[ij] - tq[ij], s_e2);
    }
  }
  const int64_t n1 = v * o;
  for (int64_t e = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; e < n1;
       e += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const double r = r1[e];
    s_r1 = fma(r, r, s_r1);
    s_e1 = fma(f_ai[e] + r, t1[e], s_e1);
  }
  s_r1 = block_sum(s_r1, sh);
  s_r2 = block_sum(s_r2, sh);
  s_e1 = block_sum(s_e1, sh);
  s_e2 = block_sum(s_e2, sh);
  if (threadIdx.x == 0) {
    partial[blockIdx.x * 4 + 0] = s_r1;
    partial[blockIdx.x * 4 + 1] = s_r2;
    partial[blockIdx.x * 4 + 2] = s_e1;
    partial[blockIdx.x * 4 + 3] = s_e2;
  }
}

__global__ void __launch_bounds__(kThreads) reduce_partials_kernel(const double* __restrict__ partial,
                                                                   int nblocks, int nq, double* out) {
  __shared__ double sh[kThreads];
  for (int q = 0; q < nq; ++q) {
    double s = 0.0;
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x) s += partial[b * nq + q];
    s = block_sum(s, sh);
    if (threadIdx.x == 0) out[q] = s;
  }
}

__global__ void __launch_bounds__(kThreads) make_tau_kernel(int64_t o, int64_t v,
                                                            const double* __restrict__ t1,
                                                            const double* __restrict__ t2,
                                                            double* __restrict__ tau) {
  const int64_t o2 = o * o;
  for (int64_t p = blockIdx.x; p < v * v; p += gridDim.x) {
    const int64_t a = p / v, b = p % v;
    for (int64_t ij = threadIdx.x; ij < o2; ij += blockDim.x) {
      const int64_t i = ij / o, j = ij % o;
      tau[p * o2 + ij] = fma(t1[a * o + i], t1[b * o + j], t2[p * o2 + ij]);
    }
  }
}

// ---------------------------------------------------------------------------
// DIIS

constexpr int kDiisMax = 16;

__global__ void __launch_bounds__(kThreads) diis_jacobi_dots_kernel(DiisArgs d) {
  __shared__ double sh[kThreads];
  const int64_t o = d.o, v = d.v, o2 = o * o, n2 = v * v * o2, n1 = v * o;
  double acc[kDiisMax];
#pragma unroll
  for (int q = 0; q < kDiisMax; ++q) acc[q] = 0.0;
  double* x2n = d.x2 + static_cast<int64_t>(d.slot) * n2;
  double* e2n = d.e2 + static_cast<int64_t>(d.slot) * n2;
  for (int64_t p = blockIdx.x; p < v * v; p += gridDim.x) {
    const int64_t a = p / v, b = p % v;
    const double eab = d.eps_v[a] + d.eps_v[b];
    for (int64_t ij = threadIdx.x; ij < o2; ij += blockDim.x) {
      const int64_t i = ij / o, j = ij % o;
      const int64_t e = p * o2 + ij;
      const double r = d.r2[e];
      const double den = d.eps_o[i] + d.eps_o[j] - eab;
      x2n[e] = d.t2[e] + r / den;
      e2n[e] = r;
#pragma unroll
      for (int q = 0; q < kDiisMax; ++q) {
        if (q < d.nvec) {
          const double eq = (d.slots[q] == d.slot) ? r : d.e2[static_cast<int64_t>(d.slots[q]) * n2 + e];
          acc[q] = fma(r, eq, acc[q]);
        }
      }
    }
  }
  double* x1n = d.x1 + static_cast<int64_t>(d.slot) * n1;
  double* e1n = d.e1 + static_cast<int64_t>(d.slot) * n1;
  for (int64_t e = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; e < n1;
       e += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t a = e / o, i = e % o;
    const double r = d.r1[e];
    x1n[e] = d.t1[e] + r / (d.eps_o[i] - d.eps_v[a]);
    e1n[e] = r;
#pragma unroll
    for (int q = 0; q < kDiisMax; ++q) {
      if (q < d.nvec) {
        const double eq = (d.slots[q] == d.slot) ? r : d.e1[static_cast<int64_t>(d.slots[q]) * n1 + e];
        acc[q] = fma(r, eq, acc[q]);
      }
    }
  }
  for (int q = 0; q < d.nvec; ++q) {
    const double s = block_sum(acc[q], sh);
    if (threadIdx.x == 0) d.partial[blockIdx.x * kDiisMax + q] = s;
  }
}

// Gaussian elimination with partial pivoting; returns false on a pivot below
// tol * max|A|.  Same operation order as the FP64 oracle's gepp_solve.
__device__ bool gepp(double* A, double* b, double* x, int n) {
  double scale = 0.0;
  for (int i = 0; i < n * n; ++i) scale = fmax(scale, fabs(A[i]));
  for (int col = 0; col < n; ++col) {
    int p = col;
    double best = fabs(A[col * n + col]);
    for (int r = col + 1; r < n; ++r) {
      if (fabs(A[r * n + col]) > best) { best = fabs(A[r * n + col]); p = r; }
    }
    if (best <= 1e-14 * scale) return false;
    if (p != col) {
      for (int c = 0; c < n; ++c) { double t = A[col * n + c]; A[col * n + c] = A[p * n + c]; A[p * n + c] = t; }
      double t = b[col]; b[col] = b[p]; b[p] = t;
    }
    for (int r = col + 1; r < n; ++r) {
      const double f = A[r * n + col] / A[col * n + col];
      for (int c = col; c < n; ++c) A[r * n + c] -= f * A[col * n + c];
      b[r] -= f * b[col];
    }
  }
  for (int r = n - 1; r >= 0; --r) {
    double s = b[r];
    for (int c = r + 1; c < n; ++c) s -= A[r * n + c] * x[c];
    x[r] = s / A[r * n + r];
  }
  return true;
}

__global__ void __launch_bounds__(kThreads) diis_solve_kernel(DiisArgs d) {
  __shared__ double sh[kThreads];
  __shared__ double dots[kDiisMax];
  for (int q = 0; q < d.nvec; ++q) {
    double s = 0.0;
    for (int b = threadIdx.x; b < kReduceBlocks; b += blockDim.x) s += d.partial[b * kDiisMax + q];
    s = block_sum(s, sh);
    if (threadIdx.x == 0) dots[q] = s;
  }
  __syncthreads();
  if (threadIdx.x != 0) return;
  const int nd = d.ndiis;
  for (int q = 0; q < d.nvec; ++q) {
    d.Bmat[d.slot * nd + d.slots[q]] = dots[q];
    d.Bmat[d.slots[q] * nd + d.slot] = dots[q];
  }
  for (int s = 0; s < nd; ++s) d.coef[s] = 0.0;
  const int n = d.nvec;
  if (!d.extrapolate) {
    d.coef[d.slot] = 1.0;
    *d.nskip_out = -1;
    return;
  }
  const double b00 = d.Bmat[d.slots[0] * nd + d.slots[0]];
  const double bnn = d.Bmat[d.slots[n - 1] * nd + d.slots[n - 1]];
  double norm = 1.0;
  if (fabs(b00) > 1e-10 && fabs(bnn) > 1e-10) norm = 1.0 / fabs(b00);
  double A[(kDiisMax + 1) * (kDiisMax + 1)];
  double rhs[kDiisMax + 1];
  double sol[kDiisMax + 1];
  for (int nskip = 0; nskip < n; ++nskip) {
    const int m = n - nskip;
    const int w = m + 1;
    for (int r = 0; r < w; ++r) {
      rhs[r] = (r == 0) ? -1.0 : 0.0;
      for (int c = 0; c < w; ++c) {
        double val;
        if (r == 0 && c == 0) val = 0.0;
        else if (r == 0 || c == 0) val = -1.0;
        else val = d.Bmat[d.slots[nskip + r - 1] * nd + d.slots[nskip + c - 1]] * norm;
        if (r > 0 && r == c) val *= 1.0 + d.damping;
        A[r * w + c] = val;
      }
    }
    if (gepp(A, rhs, sol, w)) {
      for (int q = 0; q < m; ++q) d.coef[d.slots[nskip + q]] = sol[q + 1];
      *d.nskip_out = nskip;
      return;
    }
  }
  d.coef[d.slot] = 1.0;
  *d.nskip_out = n - 1;
}

struct ExtrapArgs {
  int64_t o, v;
  const double* x1;
  const double* x2;
  const double* coef;
  int nvec;
  int slots[kDiisMax];
  double* t1;
  double* t2;
  double* tau;
};

__global__ void __launch_bounds__(kThreads) extrapolate_t1_kernel(ExtrapArgs x) {
  const int64_t n1 = x.v * x.o;
  for (int64_t e = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; e < n1;
       e += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    double acc = 0.0;
    for (int q = 0; q < x.nvec; ++q) acc = fma(x.coef[x.slots[q]], x.x1[x.slots[q] * n1 + e], acc);
    x.t1[e] = acc;
  }
}

__global__ void __launch_bounds__(kThreads) extrapolate_t2_tau_kernel(ExtrapArgs x) {
  const int64_t o = x.o, v = x.v, o2 = o * o, n2 = v * v * o2;
  double c[kDiisMax];
  for (int q = 0; q < kDiisMax; ++q) c[q] = (q < x.nvec) ? x.coef[x.slots[q]] : 0.0;
  for (int64_t p = blockIdx.x; p < v * v; p += gridDim.x) {
    const int64_t a = p / v, b = p % v;
    for (int64_t ij = threadIdx.x; ij < o2; ij += blockDim.x) {
      const int64_t i = ij / o, j = ij % o;
      const int64_t e = p * o2 + ij;
      double acc = 0.0;
      for (int q = 0; q < x.nvec; ++q) acc = fma(c[q], x.x2[x.slots[q] * n2 + e], acc);
      x.t2[e] = acc;
      x.tau[e] = fma(x.t1[a * o + i], x.t1[b * o + j], acc);
    }
  }
}

__global__ void __launch_bounds__(kThreads) splitk_reduce_kernel(int64_t M, int64_t N, int ksplit,
                                                                 const double* __restrict__ partial,
                                                                 int64_t rows, int64_t ldp, double* C,
                                                                 const int64_t* __restrict__ cm,
                                                                 const int64_t* __restrict__ cn,
                                                                 double alpha, double beta) {
  const int64_t total = M * N;
  const int64_t split_stride = rows * ldp;
  for (int64_t e = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; e < total;
       e += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t m = e / N, n = e - m * N;
    const double* p = partial + m * ldp + n;
    double acc = 0.0;
    for (int s = 0; s < ksplit; ++s) acc += p[s * split_stride];
    double* c = C + cm[m] + cn[n];
    *c = (beta == 0.0) ? alpha * acc : fma(beta, *c, alpha * acc);
  }
}

}  // namespace

int num_sms() {
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
  }
  return sms;
}

void launch_splitk_reduce(int64_t M, int64_t N, int ksplit, const double* partial, int64_t rows,
                          int64_t ldp, double* C, const int64_t* cm, const int64_t* cn, double alpha,
                          double beta, cudaStream_t st) {
  if (M <= 0 || N <= 0) return;
  splitk_reduce_kernel<<<grid_for(M * N, kThreads), kThreads, 0, st>>>(M, N, ksplit, partial, rows, ldp, C,
                                                                      cm, cn, alpha, beta);
}

// ---------------------------------------------------------------------------
// launchers

void launch_gather(const GatherArgs& g, cudaStream_t st) {
  if (g.Rpad <= 0 || g.Cpad <= 0) return;
  if (g.transpose) {
    const int64_t tiles = ((g.Rpad + 31) / 32) * ((g.Cpad + 31) / 32);
    const int64_t grid = std::min<int64_t>(tiles, 152LL * 16);
    gather_t_kernel<<<static_cast<unsigned>(grid), dim3(32, 8), 0, st>>>(g);
    return;
  }
  int bx = 1;
  while (bx < g.Cpad && bx < kThreads) bx <<= 1;
  if (bx < 32) bx = 32;
  const int by = kThreads / bx;
  int64_t gx = (g.Cpad + bx - 1) / bx;
  int64_t gy = (g.Rpad + by - 1) / by;
  // cap the grid; the kernel loops over the remainder
  const int64_t cap_total = 152LL * 64;
  if (gx > cap_total) gx = cap_total;
  int64_t gy_cap = std::max<int64_t>(1, cap_total / gx);
  if (gy > gy_cap) gy = gy_cap;
  if (gy > 65535) gy = 65535;
  dim3 grid(static_cast<unsigned>(gx), static_cast<unsigned>(gy));
  dim3 block(bx, by);
  gather_kernel<<<grid, block, 0, st>>>(g);
}

void launch_energy_terms(int64_t o, int64_t v, const double* r1, const double* r2,
                         const double* f_ai, const double* g_abij, const double* t1,
                         const double* tau, double* partial, double* out, cudaStream_t st) {
  energy_partial_kernel<<<kReduceBlocks, kThreads, 0, st>>>(o, v, r1, r2, f_ai, g_abij, t1, tau,
                                                           partial);
  reduce_partials_kernel<<<1, kThreads, 0, st>>>(partial, kReduceBlocks, 4, out);
}

void launch_make_tau(int64_t o, int64_t v, const double* t1, const double* t2, double* tau,
                     cudaStream_t st) {
  make_tau_kernel<<<grid_for(v * v, 1), kThreads, 0, st>>>(o, v, t1, t2, tau);
}

void launch_diis_step(const DiisArgs& d, cudaStream_t st) {
  diis_jacobi_dots_kernel<<<kReduceBlocks, kThreads, 0, st>>>(d);
  diis_solve_kernel<<<1, kThreads, 0, st>>>(d);
}

void launch_diis_extrapolate(int64_t o, int64_t v, const double* x1, const double* x2,
                             const double* coef, int ndiis, const int* slots, int nvec,
                             double* t1, double* t2, double* tau, cudaStream_t st) {
  (void)ndiis;
  ExtrapArgs x;
  x.o = o;
  x.v = v;
  x.x1 = x1;
  x.x2 = x2;
  x.coef = coef;
  x.nvec = nvec;
  for (int q = 0; q < kDiisMax; ++q) x.slots[q] = (q < nvec) ? slots[q] : 0;
  x.t1 = t1;
  x.t2 = t2;
  x.tau = tau;
  extrapolate_t1_kernel<<<grid_for(v * o, kThreads), kThreads, 0, st>>>(x);
  extrapolate_t2_tau_kernel<<<grid_for(v * v, 1), kThreads, 0, st>>>(x);
}

}  // namespace gbcc
