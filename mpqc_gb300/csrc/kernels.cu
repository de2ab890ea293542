// Elementwise, gather/pack, reduction and DIIS kernels of the CCSD engine.
//
// The amplitude-sized arrays (o^2 v^2 doubles) are streamed once per kernel
// with coalesced accesses, so HBM bandwidth is the bound these kernels aim at.
// GB300 executes FP64 arithmetic and FP64 conversions at ~2 per clock per SM
// (1/64 of FP32), so per-element FP64 work is kept to a few operations: the
// BF16 split works on bit patterns and FP32 remainders, and single-term packs
// are plain copies (their coefficient scales the GEMM instead).
#include "fp_bits.cuh"
#include "gather.cuh"
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

__global__ void __launch_bounds__(kThreads, 4) gather_kernel(GatherArgs g) {
  const bool rmw = g.out && g.beta != 0.0;
#define GBCC_ROWS(N, P) (rmw ? gather_rows<N, P, true, 0>(g) : gather_rows<N, P, false, 0>(g))
  GBCC_GATHER_DISPATCH(g, GBCC_ROWS);
#undef GBCC_ROWS
}

// 4 K elements per thread into BF16 slices
__global__ void __launch_bounds__(kThreads, 4) gather_split4_kernel(GatherArgs g) {
#define GBCC_SPLIT4(N, P) split4_rows<N, P, 0>(g)
  GBCC_GATHER_DISPATCH(g, GBCC_SPLIT4);
#undef GBCC_SPLIT4
}


// 4 columns per thread into 16-byte aligned FP64 rows (assignments, FP64 panels)
__global__ void __launch_bounds__(kThreads, 3) gather4_f64_kernel(GatherArgs g) {
  const bool rmw = g.beta != 0.0;
#define GBCC_F64X4(N, P) (rmw ? split4_rows<N, P, 2>(g) : split4_rows<N, P, 1>(g))
  GBCC_GATHER_DISPATCH(g, GBCC_F64X4);
#undef GBCC_F64X4
}

__global__ void __launch_bounds__(256) gather_t_kernel(GatherArgs g) {
  __shared__ double tile[32][33];
  const bool rmw = g.out && g.beta != 0.0;
#define GBCC_TILES(N, P) (rmw ? gather_tiles<N, P, true, 0>(g, tile) : gather_tiles<N, P, false, 0>(g, tile))
  GBCC_GATHER_DISPATCH(g, GBCC_TILES);
#undef GBCC_TILES
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
    int64_t a, b;
    divmod32(p, v, a, b);
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
    int64_t a, b;
    divmod32(p, v, a, b);
    for (int64_t ij = threadIdx.x; ij < o2; ij += blockDim.x) {
      int64_t i, j;
      divmod32(ij, o, i, j);
      tau[p * o2 + ij] = fma(t1[a * o + i], t1[b * o + j], t2[p * o2 + ij]);
    }
  }
}

// ---------------------------------------------------------------------------
// Particle-particle ladder over pair-(anti)symmetric combinations.
//
// B(a,b,i,j) = sum_cd G(a,b,c,d) tau(c,d,i,j) splits, with G+ = G_abcd + G_abdc
// (G_abcc on the diagonal), G- = G_abcd - G_abdc, tau+ = (tau_cdij + tau_dcij)/2
// (tau_ccij on the diagonal), tau- = (tau_cdij - tau_dcij)/2, into
//   B = sum_{c<=d} G+ tau+ + sum_{c<d} G- tau-.
// <ab|cd> = <ba|dc> makes G+ symmetric and G- antisymmetric under a<->b, and
// pair-symmetric amplitudes (tau(c,d,i,j) = tau(d,c,j,i)) make tau+ symmetric,
// tau- antisymmetric under i<->j, so the two products are needed for a <= b,
// i <= j (a < b, i < j) only: a quarter of the FLOPs of the plain contraction.
// Pair indices, row-major over the upper triangle:
//   sym(a,b)  = a n - a(a-1)/2 + (b - a)      a <= b < n
//   anti(a,b) = a (n-1) - a(a-1)/2 + (b-a-1)  a < b < n

__device__ __forceinline__ int64_t pair_sym(int64_t a, int64_t b, int64_t n) {
  return a * n - a * (a - 1) / 2 + (b - a);
}
__device__ __forceinline__ int64_t pair_anti(int64_t a, int64_t b, int64_t n) {
  return a * (n - 1) - a * (a - 1) / 2 + (b - a - 1);
}

// One block per (a, b): Gp[sym(a,b)][sym(c,d)], Gm[anti(a,b)][anti(c,d)].  Also
// used for o v^3 blocks (rows = any leading index pair, cols = c <= d) when
// ab_pairs is false: then row r = a*v + b of G maps to row r of the outputs.
__global__ void __launch_bounds__(kThreads) build_gpm_kernel(int64_t rows_v, int64_t v, bool ab_pairs,
                                                             const double* __restrict__ G, double* __restrict__ Gp,
                                                             double* __restrict__ Gm) {
  const int64_t np = v * (v + 1) / 2, nm = v * (v - 1) / 2;
  for (int64_t row = blockIdx.x; row < rows_v * v; row += gridDim.x) {
    int64_t a, b;
    divmod32(row, v, a, b);
    int64_t rp = row, rm = row;
    if (ab_pairs) {
      if (a > b) continue;
      rp = pair_sym(a, b, v);
      rm = a < b ? pair_anti(a, b, v) : -1;
    }
    const double* g = G + row * v * v;
    double* gp = Gp + rp * np;
    double* gm = rm >= 0 ? Gm + rm * nm : nullptr;
    for (int64_t c = 0; c < v; ++c) {
      for (int64_t d = c + threadIdx.x; d < v; d += blockDim.x) {
        const double x = g[c * v + d], y = g[d * v + c];
        gp[pair_sym(c, d, v)] = c < d ? x + y : x;
        if (gm && c < d) gm[pair_anti(c, d, v)] = x - y;
      }
    }
  }
}

// The rows a in [a0, a1) of G+ / G- (pairs a <= b / a < b), from the block
// Gblk[a - a0][b - a0][c][d] = <ab|cd> (b >= a0 only); output rows counted
// from the block's first pair: sym(a,b) - sym(a0,a0) and anti(a,b) - anti(a0,a0+1).
__global__ void __launch_bounds__(kThreads) build_gpm_rows_kernel(int64_t a0, int64_t a1, int64_t v,
                                                                  const double* __restrict__ Gblk,
                                                                  double* __restrict__ Gp, double* __restrict__ Gm) {
  const int64_t np = v * (v + 1) / 2, nm = v * (v - 1) / 2, w = v - a0;
  const int64_t p0 = pair_sym(a0, a0, v), m0 = a0 * (v - 1) - a0 * (a0 - 1) / 2;
  for (int64_t row = blockIdx.x; row < (a1 - a0) * w; row += gridDim.x) {
    int64_t al, bl;
    divmod32(row, w, al, bl);
    const int64_t a = a0 + al, b = a0 + bl;
    if (a > b) continue;
    double* gp = Gp + (pair_sym(a, b, v) - p0) * np;
    double* gm = a < b ? Gm + (pair_anti(a, b, v) - m0) * nm : nullptr;
    const double* g = Gblk + row * v * v;
    for (int64_t c = 0; c < v; ++c) {
      for (int64_t d = c + threadIdx.x; d < v; d += blockDim.x) {
        const double x = g[c * v + d], y = g[d * v + c];
        gp[pair_sym(c, d, v)] = c < d ? x + y : x;
        if (gm && c < d) gm[pair_anti(c, d, v)] = x - y;
      }
    }
  }
}

// G+ / G- over atomic-orbital pairs from (pq|rs) in chemists' order:
// <pr|qs> = G[p][q][r][s], so Gp[sym(p,r)][sym(q,s)] = (pq|rs) + (ps|rq) and
// Gm[anti(p,r)][anti(q,s)] = (pq|rs) - (ps|rq) (one block per p <= r).
__global__ void __launch_bounds__(kThreads) build_gpm_chem_kernel(int64_t n, const double* __restrict__ G,
                                                                  double* __restrict__ Gp, double* __restrict__ Gm) {
  const int64_t np = n * (n + 1) / 2, nm = n * (n - 1) / 2;
  for (int64_t row = blockIdx.x; row < n * n; row += gridDim.x) {
    int64_t p, r;
    divmod32(row, n, p, r);
    if (p > r) continue;
    double* gp = Gp + pair_sym(p, r, n) * np;
    double* gm = p < r ? Gm + pair_anti(p, r, n) * nm : nullptr;
    for (int64_t q = 0; q < n; ++q) {
      const double* gq = G + ((p * n + q) * n + r) * n;  // (pq|r .)
      for (int64_t s = q + threadIdx.x; s < n; s += blockDim.x) {
        const double x = gq[s];                            // <pr|qs> = (pq|rs)
        const double y = G[((p * n + s) * n + r) * n + q];  // <pr|sq> = (ps|rq)
        gp[pair_sym(q, s, n)] = q < s ? x + y : x;
        if (gm && q < s) gm[pair_anti(q, s, n)] = x - y;
      }
    }
  }
}

// Hole-hole ladder over pair combinations.  With W(k,l,i,j) = W(l,k,j,i) and
// pair-symmetric tau, sum_kl tau(a,b,k,l) W(k,l,i,j) splits like the
// particle-particle ladder: over k <= l into tau+(ab,kl) W+(kl,ij) and over
// k < l into tau-(ab,kl) W-(kl,ij), where tau+- are the ladder's taup / taum
// (tau(a,b,l,k) = tau(b,a,k,l)) and W+ = W(kl,ij) + W(lk,ij) (W(kk,ij) on the
// diagonal), W- = W(kl,ij) - W(lk,ij); the products are symmetric /
// antisymmetric in a <-> b and in i <-> j, so they add to the ladder's Bp / Bm.
// The part sum_cd Gijab(k,l,c,d) tau(c,d,i,j) of W+- is itself a pair
// product: <lk|cd> = <kl|dc> gives W+ = c_kl G+(kl,cd) tau+(cd,ij) and
// W- = 2 G-(kl,cd) tau-(cd,ij), with G+- = G(kl,cd) +- G(kl,dc) (G(kl,cc) on
// the diagonal) and c_kl = 2 (k < l) or 1 (k = l).
//
// Gtp[sym(k,l)][sym(c,d)] = c_kl G+, Gtm[anti(k,l)][anti(c,d)] = 2 G- from
// Gijab[k][l][c][d]; one block per k <= l.
__global__ void __launch_bounds__(kThreads) build_gpm_oo_kernel(int64_t o, int64_t v, const double* __restrict__ G,
                                                                double* __restrict__ Gtp,
                                                                double* __restrict__ Gtm) {
  const int64_t np = v * (v + 1) / 2, nm = v * (v - 1) / 2;
  for (int64_t row = blockIdx.x; row < o * o; row += gridDim.x) {
    int64_t k, l;
    divmod32(row, o, k, l);
    if (k > l) continue;
    const double* g = G + row * v * v;
    double* gp = Gtp + pair_sym(k, l, o) * np;
    double* gm = (Gtm && k < l) ? Gtm + pair_anti(k, l, o) * nm : nullptr;
    const int sk = k < l ? 1 : 0;  // c_kl = 2^sk
    for (int64_t c = 0; c < v; ++c) {
      for (int64_t d = c + threadIdx.x; d < v; d += blockDim.x) {
        const double x = g[c * v + d], y = g[d * v + c];
        gp[pair_sym(c, d, v)] = scale_pow2(c < d ? x + y : x, sk);
        if (gm && c < d) gm[pair_anti(c, d, v)] = scale_pow2(x - y, 1);
      }
    }
  }
}

// Wt[sym(k,l)][sym(i,j)] = W(k,l,i,j) + W(l,k,i,j) (W(k,k,i,j) for k = l) and
// Wm[anti(k,l)][anti(i,j)] = W(k,l,i,j) - W(l,k,i,j), from W[o][o][o][o];
// one block per k <= l.
__global__ void __launch_bounds__(kThreads) pair_combine_oo_kernel(int64_t o, const double* __restrict__ W,
                                                                   double* __restrict__ Wt,
                                                                   double* __restrict__ Wm) {
  const int64_t o2 = o * o, sp = o * (o + 1) / 2, sm = o * (o - 1) / 2;
  for (int64_t row = blockIdx.x; row < o2; row += gridDim.x) {
    int64_t k, l;
    divmod32(row, o, k, l);
    if (k > l) continue;
    const double* x = W + (k * o + l) * o2;
    const double* y = W + (l * o + k) * o2;
    double* wt = Wt + pair_sym(k, l, o) * sp;
    double* wm = (Wm && k < l) ? Wm + pair_anti(k, l, o) * sm : nullptr;
    for (int64_t ij = threadIdx.x; ij < o2; ij += blockDim.x) {
      int64_t i, j;
      divmod32(ij, o, i, j);
      if (i > j) continue;
      wt[pair_sym(i, j, o)] = k < l ? x[ij] + y[ij] : x[ij];
      if (wm && i < j) wm[pair_anti(i, j, o)] = x[ij] - y[ij];
    }
  }
}

// One block per (c <= d): taup[sym(c,d)][sym(i,j)], taum[anti(c,d)][anti(i,j)].
__global__ void __launch_bounds__(kThreads) tau_pm_kernel(int64_t o, int64_t v, const double* __restrict__ tau,
                                                          double* __restrict__ taup, double* __restrict__ taum) {
  const int64_t o2 = o * o, sp = o * (o + 1) / 2, sm = o * (o - 1) / 2;
  for (int64_t p = blockIdx.x; p < v * v; p += gridDim.x) {
    int64_t c, d;
    divmod32(p, v, c, d);
    if (c > d) continue;
    const double* x = tau + (c * v + d) * o2;
    const double* y = tau + (d * v + c) * o2;
    double* tp = taup + pair_sym(c, d, v) * sp;
    double* tm = c < d ? taum + pair_anti(c, d, v) * sm : nullptr;
    for (int64_t ij = threadIdx.x; ij < o2; ij += blockDim.x) {
      int64_t i, j;
      divmod32(ij, o, i, j);
      if (i > j) continue;
      if (c == d) {
        tp[pair_sym(i, j, o)] = x[ij];
      } else {
        tp[pair_sym(i, j, o)] = scale_pow2(x[ij] + y[ij], -1);
        if (i < j) tm[pair_anti(i, j, o)] = scale_pow2(x[ij] - y[ij], -1);
      }
    }
  }
}

// out(a,b,i,j) (+)= Bp[sym(ab)][sym(ij)] + s_ab s_ij Bm[anti(ab)][anti(ij)], s = +1 for an
// ordered pair, -1 for a swapped one, 0 on the diagonal.  With ab_pairs false the
// row index r = a*v + b addresses Bp / Bm directly (no symmetry in the row pair).
// ACC: add to out (beta = 1) rather than overwrite it.
template <bool ACC>
__global__ void __launch_bounds__(kThreads) pair_unpack_kernel(int64_t rows_v, int64_t v, int64_t o, bool ab_pairs,
                                                               const double* __restrict__ Bp,
                                                               const double* __restrict__ Bm,
                                                               double* __restrict__ out) {
  const int64_t o2 = o * o, sp = o * (o + 1) / 2, sm = o * (o - 1) / 2;
  for (int64_t row = blockIdx.x; row < rows_v * v; row += gridDim.x) {
    int64_t a, b;
    divmod32(row, v, a, b);
    int64_t rp = row, rm = row;
    bool sab_pos = true;  // s_ab = +1
    if (ab_pairs) {
      const int64_t lo = a < b ? a : b, hi = a < b ? b : a;
      rp = pair_sym(lo, hi, v);
      rm = lo < hi ? pair_anti(lo, hi, v) : -1;
      sab_pos = a < b;
    }
    const double* bp = Bp + rp * sp;
    const double* bm = (Bm && rm >= 0) ? Bm + rm * sm : nullptr;
    double* op = out + row * o2;
    for (int64_t ij = threadIdx.x; ij < o2; ij += blockDim.x) {
      int64_t i, j;
      divmod32(ij, o, i, j);
      const int64_t li = i < j ? i : j, hj = i < j ? j : i;
      double val = bp[pair_sym(li, hj, o)];
      if (bm && li < hj) val += flip_sign(bm[pair_anti(li, hj, o)], (i < j) != sab_pos);
      if constexpr (ACC) op[ij] += val;
      else op[ij] = val;
    }
  }
}

// The last pass of r2 (ccsd_r1_r2.h:254-262 and the ladder's unpack):
//   r2(a,b,i,j) (+)= Q(a,b,i,j) + g_abij(a,b,i,j) + P(a,b,i,j),
//   Q(a,b,i,j) = q(a,b,i,j) + q(b,a,j,i),  q = r2u - 0.5 tmp - tmp(b,a,i,j),
// i.e. the symmetrisation r2u(a,b,i,j) + r2u(b,a,j,i) after r2u -= 0.5
// tmp(a,b,i,j) + tmp(b,a,i,j), with P the unpack of pair_unpack_kernel (Bp
// null: none).  Q(b,a,j,i) = Q(a,b,i,j) operand for operand, so one block
// per pair a <= b and 32 x 32 tile (I, J) of (i, j) stages q of the tile
// [a][b][I][J] and of [b][a][J][I] in shared memory (coalesced along j and
// along i) and adds the same Q to r2[a][b][I][J] and to r2[b][a][J][I]: every
// r2u, tmp and g element is read once, r2 read and written once.  On the
// diagonal a = b only tiles I <= J are taken, and a tile I = J once.
__global__ void __launch_bounds__(256) r2_assemble_kernel(int64_t o, int64_t v, const double* __restrict__ r2u,
                                                          const double* __restrict__ tmp,
                                                          const double* __restrict__ g,
                                                          const double* __restrict__ Bp,
                                                          const double* __restrict__ Bm, bool accumulate,
                                                          double* __restrict__ r2) {
  __shared__ double sq[32][33];  // [i][j] of q(a,b,.,.)
  __shared__ double sr[32][33];  // [j][i] of q(b,a,.,.)
  const int64_t o2 = o * o, nt = (o + 31) / 32, nt2 = nt * nt;
  const int64_t sp = o * (o + 1) / 2, sm = o * (o - 1) / 2;
  const int tx = threadIdx.x, ty = threadIdx.y;
  for (int64_t x = blockIdx.x; x < v * v * nt2; x += gridDim.x) {
    int64_t p, t, a, b, I, J;
    divmod32(x, nt2, p, t);
    divmod32(p, v, a, b);
    if (a > b) continue;
    divmod32(t, nt, I, J);
    if (a == b && I > J) continue;
    const int64_t i0 = I * 32, j0 = J * 32;
    const int64_t ab = (a * v + b) * o2, ba = (b * v + a) * o2;
    for (int k = ty; k < 32; k += 8) {
      const int64_t i = i0 + k, j = j0 + tx;
      if (i < o && j < o) {
        const int64_t e = i * o + j;
        sq[k][tx] = fma(-0.5, tmp[ab + e], r2u[ab + e]) - tmp[ba + e];
      }
      const int64_t jj = j0 + k, ii = i0 + tx;
      if (jj < o && ii < o) {
        const int64_t e = jj * o + ii;
        sr[k][tx] = fma(-0.5, tmp[ba + e], r2u[ba + e]) - tmp[ab + e];
      }
    }
    __syncthreads();
    const double* bp = Bp ? Bp + pair_sym(a, b, v) * sp : nullptr;
    const double* bm = (Bp && Bm && a < b) ? Bm + pair_anti(a, b, v) * sm : nullptr;
    // P(a,b,i,j) = P(b,a,j,i): the B- term changes sign with i > j (a < b)
    auto unpack = [&](int64_t i, int64_t j) {
      const int64_t li = i < j ? i : j, hj = i < j ? j : i;
      double val = bp[pair_sym(li, hj, o)];
      if (bm && li < hj) val += flip_sign(bm[pair_anti(li, hj, o)], i > j);
      return val;
    };
    // r2[a][b][I][J], lanes along j
    for (int k = ty; k < 32; k += 8) {
      const int64_t i = i0 + k, j = j0 + tx;
      if (i < o && j < o) {
        double val = (sq[k][tx] + sr[tx][k]) + g[ab + i * o + j];
        if (bp) val += unpack(i, j);
        double* out = r2 + ab + i * o + j;
        *out = accumulate ? *out + val : val;
      }
    }
    // r2[b][a][J][I], lanes along i
    if (a != b || I != J) {
      for (int k = ty; k < 32; k += 8) {
        const int64_t j = j0 + k, i = i0 + tx;
        if (i < o && j < o) {
          double val = (sq[tx][k] + sr[k][tx]) + g[ba + j * o + i];
          if (bp) val += unpack(i, j);
          double* out = r2 + ba + j * o + i;
          *out = accumulate ? *out + val : val;
        }
      }
    }
    __syncthreads();
  }
}

// g_ac's Giabc term (ccsd_intermediates.h F_VV) read off the diagonals i = k
// of two contractions the residual performs anyway: with
//   Z(k,a,c,i) = sum_d Giabc(k,a,d,c) t1(d,i)   (added to K(k,a,i,c))
//   Q(k,a,c,i) = sum_d (2 Giabc(k,a,c,d) - Giabc(k,a,d,c)) t1(d,i)   (added to P(a,k,i,c))
// sum_kd (2 Giabc(k,a,d,c) - Giabc(k,a,c,d)) t1(d,k) = sum_k 1.5 Z(k,a,c,k) - 0.5 Q(k,a,c,k).
// The increments are the differences of the diagonals after and before
// those contractions: diag_snapshot stores K(k,a,k,c) (which = 0) or
// P(a,k,k,c) (which = 1) as d[k][a][c]; gac_from_diagonals adds the sum.
__global__ void __launch_bounds__(kThreads) diag_snapshot_kernel(int64_t o, int64_t v, int which,
                                                                 const double* __restrict__ X,
                                                                 double* __restrict__ d) {
  const int64_t n = o * v * v;
  for (int64_t e = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; e < n;
       e += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    int64_t ka, c, k, a;
    divmod32(e, v, ka, c);
    divmod32(ka, v, k, a);
    d[e] = which == 0 ? X[((k * v + a) * o + k) * v + c] : X[((a * o + k) * o + k) * v + c];
  }
}

__global__ void __launch_bounds__(kThreads) gac_from_diagonals_kernel(int64_t o, int64_t v,
                                                                      const double* __restrict__ K,
                                                                      const double* __restrict__ P,
                                                                      const double* __restrict__ dK,
                                                                      const double* __restrict__ dP,
                                                                      double* __restrict__ gac) {
  for (int64_t e = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; e < v * v;
       e += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    int64_t a, c;
    divmod32(e, v, a, c);
    double s = 0.0;
    for (int64_t k = 0; k < o; ++k) {
      const int64_t kac = (k * v + a) * v + c;
      const double z = K[((k * v + a) * o + k) * v + c] - dK[kac];
      const double q = P[((a * o + k) * o + k) * v + c] - dP[kac];
      s = fma(1.5, z, fma(-0.5, q, s));
    }
    gac[e] += s;
  }
}

// r1(a,i) += sum_k 2 tmp2(k,a,k,i) - tmp2(k,a,i,k) with tmp2[o][v][o][o]: the
// (2 Giabc(k,a,c,d) - Giabc(k,a,d,c)) tau(c,d,k,i) term of r1 read off the
// ladder's tmp2(k,a,i,j) = Giabc(k,a,c,d) tau(c,d,i,j), using
// tau(c,d,k,i) = tau(d,c,i,k)
__global__ void __launch_bounds__(kThreads) r1_from_tmp2_kernel(int64_t o, int64_t v,
                                                                const double* __restrict__ tmp2,
                                                                double* __restrict__ r1) {
  const int64_t n = v * o;
  for (int64_t e = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; e < n;
       e += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    int64_t a, i;
    divmod32(e, o, a, i);
    double s = 0.0;
    for (int64_t k = 0; k < o; ++k) {
      const double* p = tmp2 + (k * v + a) * o * o;
      s = fma(2.0, p[k * o + i], s);
      s -= p[i * o + k];
    }
    r1[e] += s;
  }
}

// t += r / D in place (the Jacobi step of lcao/cc/solvers.h:165-258 without
// DIIS), used to build probe amplitudes for the slice calibration
__global__ void __launch_bounds__(kThreads) jacobi_inplace_kernel(int64_t o, int64_t v, const double* eps_o,
                                                                  const double* eps_v, const double* r1,
                                                                  const double* r2, double* t1, double* t2) {
  const int64_t o2 = o * o;
  for (int64_t p = blockIdx.x; p < v * v; p += gridDim.x) {
    int64_t a, b;
    divmod32(p, v, a, b);
    const double eab = eps_v[a] + eps_v[b];
    for (int64_t ij = threadIdx.x; ij < o2; ij += blockDim.x) {
      int64_t i, j;
      divmod32(ij, o, i, j);
      t2[p * o2 + ij] += r2[p * o2 + ij] / (eps_o[i] + eps_o[j] - eab);
    }
  }
  for (int64_t e = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; e < v * o;
       e += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    int64_t a, i;
    divmod32(e, o, a, i);
    t1[e] += r1[e] / (eps_o[i] - eps_v[a]);
  }
}

// dinv2[a][b][i][j] = 1 / (eps_o[i] + eps_o[j] - eps_v[a] - eps_v[b]),
// dinv1[a][i] = 1 / (eps_o[i] - eps_v[a])
__global__ void __launch_bounds__(kThreads) denominators_kernel(int64_t o, int64_t v, const double* eps_o,
                                                                const double* eps_v, double* dinv1,
                                                                double* dinv2) {
  const int64_t o2 = o * o;
  for (int64_t p = blockIdx.x; p < v * v; p += gridDim.x) {
    int64_t a, b;
    divmod32(p, v, a, b);
    const double eab = eps_v[a] + eps_v[b];
    for (int64_t ij = threadIdx.x; ij < o2; ij += blockDim.x) {
      int64_t i, j;
      divmod32(ij, o, i, j);
      dinv2[p * o2 + ij] = 1.0 / (eps_o[i] + eps_o[j] - eab);
    }
  }
  for (int64_t e = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; e < v * o;
       e += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    int64_t a, i;
    divmod32(e, o, a, i);
    dinv1[e] = 1.0 / (eps_o[i] - eps_v[a]);
  }
}

// |x| as its bit pattern: for non-negative doubles the unsigned order of the
// bits is the order of the values (NaN above infinity), so maxima of |x| are
// integer maxima and take no FP64 instruction
__device__ __forceinline__ unsigned long long abs_bits(double x) {
  return static_cast<unsigned long long>(__double_as_longlong(x)) & 0x7FFFFFFFFFFFFFFFull;
}

// block maxima of two bit patterns, combined into out[0..1] with atomicMax
__device__ __forceinline__ void block_max2_bits(unsigned long long md, unsigned long long mb,
                                                unsigned long long* out) {
  __shared__ unsigned long long sd[kThreads], sb[kThreads];
  sd[threadIdx.x] = md;
  sb[threadIdx.x] = mb;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      sd[threadIdx.x] = max(sd[threadIdx.x], sd[threadIdx.x + w]);
      sb[threadIdx.x] = max(sb[threadIdx.x], sb[threadIdx.x + w]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    atomicMax(out, sd[0]);
    atomicMax(out + 1, sb[0]);
  }
}

// out[0] = bits of max |t2(a,b,i,j) - t2(b,a,j,i)|, out[1] = bits of max |t2|
// (out zeroed by the caller); a NaN anywhere makes the maximum a NaN
__global__ void __launch_bounds__(kThreads) pair_asym_kernel(int64_t o, int64_t v, const double* t2,
                                                             unsigned long long* out) {
  const int64_t o2 = o * o;
  unsigned long long md = 0ull, mb = 0ull;
  for (int64_t p = blockIdx.x; p < v * v; p += gridDim.x) {
    int64_t a, b;
    divmod32(p, v, a, b);
    const double* x = t2 + p * o2;
    const double* y = t2 + (b * v + a) * o2;
    for (int64_t ij = threadIdx.x; ij < o2; ij += blockDim.x) {
      int64_t i, j;
      divmod32(ij, o, i, j);
      const double xv = x[ij];
      md = max(md, abs_bits(xv - y[j * o + i]));
      mb = max(mb, abs_bits(xv));
    }
  }
  block_max2_bits(md, mb, out);
}

// out[0] = bits of max |a - b|, out[1] = bits of max |b| (out zeroed by the caller): block
// maxima combined with atomicMax on the bit patterns, which order like the
// values for non-negative doubles
__global__ void __launch_bounds__(kThreads) maxabs_diff_kernel(int64_t n, const double* a, const double* b,
                                                               unsigned long long* out) {
  unsigned long long md = 0ull, mb = 0ull;
  for (int64_t e = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; e < n;
       e += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const double bv = b[e];
    md = max(md, abs_bits(a[e] - bv));
    mb = max(mb, abs_bits(bv));
  }
  block_max2_bits(md, mb, out);
}

// ---------------------------------------------------------------------------
// DIIS

constexpr int kDiisMax = 16;

// slot, nvec, slots and the extrapolation flag of this DIIS step, from the
// launch arguments or (graph solve) from device memory, into shared memory
struct DiisMeta {
  int slot, nvec, extrapolate;
  int slots[kDiisMax];
};

__device__ __forceinline__ void load_diis_meta(const DiisArgs& d, DiisMeta* m) {
  const DiisDyn* y = d.dyn;
  if (threadIdx.x < kDiisMax) m->slots[threadIdx.x] = y ? y->slots[threadIdx.x] : d.slots[threadIdx.x];
  if (threadIdx.x == 0) {
    m->slot = y ? y->slot : d.slot;
    m->nvec = y ? y->nvec : d.nvec;
    m->extrapolate = y ? y->extrapolate : d.extrapolate;
  }
  __syncthreads();
}

__global__ void __launch_bounds__(kThreads) diis_jacobi_dots_kernel(DiisArgs d) {
  __shared__ double sh[kThreads];
  __shared__ DiisMeta meta;
  load_diis_meta(d, &meta);
  const int slot = meta.slot, nvec = meta.nvec;
  const int64_t o = d.o, v = d.v, o2 = o * o, n2 = v * v * o2, n1 = v * o;
  double acc[kDiisMax];
#pragma unroll
  for (int q = 0; q < kDiisMax; ++q) acc[q] = 0.0;
  double* x2n = d.x2 + static_cast<int64_t>(slot) * n2;
  double* e2n = d.e2 + static_cast<int64_t>(slot) * n2;
  for (int64_t p = blockIdx.x; p < v * v; p += gridDim.x) {
    for (int64_t ij = threadIdx.x; ij < o2; ij += blockDim.x) {
      const int64_t e = p * o2 + ij;
      const double r = d.r2[e];
      x2n[e] = fma(r, d.dinv2[e], d.t2[e]);
      e2n[e] = r;
#pragma unroll
      for (int q = 0; q < kDiisMax; ++q) {
        if (q < nvec) {
          const int sq = meta.slots[q];
          const double eq = (sq == slot) ? r : d.e2[static_cast<int64_t>(sq) * n2 + e];
          acc[q] = fma(r, eq, acc[q]);
        }
      }
    }
  }
  double* x1n = d.x1 + static_cast<int64_t>(slot) * n1;
  double* e1n = d.e1 + static_cast<int64_t>(slot) * n1;
  for (int64_t e = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; e < n1;
       e += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const double r = d.r1[e];
    x1n[e] = fma(r, d.dinv1[e], d.t1[e]);
    e1n[e] = r;
#pragma unroll
    for (int q = 0; q < kDiisMax; ++q) {
      if (q < nvec) {
        const int sq = meta.slots[q];
        const double eq = (sq == slot) ? r : d.e1[static_cast<int64_t>(sq) * n1 + e];
        acc[q] = fma(r, eq, acc[q]);
      }
    }
  }
  for (int q = 0; q < nvec; ++q) {
    const double s = block_sum(acc[q], sh);
    if (threadIdx.x == 0) d.partial[blockIdx.x * kDiisMax + q] = s;
  }
}

// |det| of the normalised bordered DIIS matrix below which the oldest stored
// vector is dropped (TiledArray's TA::DIIS test, threshold fixed by the water
// 6-31G iteration trace MPQC records in its validation outputs).
constexpr double kDiisDetMin = 1.0e-15;

// Gaussian elimination with partial pivoting on a row-major n x n system;
// returns |det A| (product of the pivots), 0 with x unset if a pivot is zero.
__device__ double gepp(double* A, double* b, double* x, int n) {
  double det = 1.0;
  for (int col = 0; col < n; ++col) {
    int p = col;
    double best = fabs(A[col * n + col]);
    for (int r = col + 1; r < n; ++r) {
      if (fabs(A[r * n + col]) > best) { best = fabs(A[r * n + col]); p = r; }
    }
    if (best == 0.0) return 0.0;
    det *= best;
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
  return det;
}

// DIIS coefficients (TiledArray's TA::DIIS extrapolation, cc/solvers.h:112-121)
// from the B matrix of the n stored vectors (slots, oldest first, B by slot
// with leading dimension nd): the bordered system [[0, -1], [-1, B]] on the
// newest n - nskip vectors, normalised by the oldest kept <e, e>, damped on
// the diagonal; the oldest vectors are dropped while |det| < kDiisDetMin (a
// singular or near-singular B), the newest alone as the last resort.  coef
// (by slot, nd entries) is written; returns nskip.
__device__ int diis_coefficients(const double* Bmat, int nd, const int* slots, int n, double damping,
                                 double* coef) {
  for (int s = 0; s < nd; ++s) coef[s] = 0.0;
  double A[(kDiisMax + 1) * (kDiisMax + 1)];
  double rhs[kDiisMax + 1];
  double sol[kDiisMax + 1];
  for (int nskip = 0; nskip < n; ++nskip) {
    const int m = n - nskip;
    const int w = m + 1;
    // normalise by the oldest kept vector's <e, e>
    const double b0 = fabs(Bmat[slots[nskip] * nd + slots[nskip]]);
    const double norm = b0 > 0.0 ? 1.0 / b0 : 1.0;
    for (int r = 0; r < w; ++r) {
      rhs[r] = (r == 0) ? -1.0 : 0.0;
      for (int c = 0; c < w; ++c) {
        double val;
        if (r == 0 && c == 0) val = 0.0;
        else if (r == 0 || c == 0) val = -1.0;
        else val = Bmat[slots[nskip + r - 1] * nd + slots[nskip + c - 1]] * norm;
        if (r > 0 && r == c) val *= 1.0 + damping;
        A[r * w + c] = val;
      }
    }
    const double det = gepp(A, rhs, sol, w);
    if (det > 0.0 && (det >= kDiisDetMin || nskip == n - 1)) {
      for (int q = 0; q < m; ++q) coef[slots[nskip + q]] = sol[q + 1];
      return nskip;
    }
  }
  coef[slots[n - 1]] = 1.0;
  return n - 1;
}

// test hook: diis_coefficients on a given B (slots 0..n-1 in order)
__global__ void diis_coefficients_test_kernel(const double* Bmat, int n, double damping, double* coef,
                                              int* nskip) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  int slots[kDiisMax];
  for (int q = 0; q < n; ++q) slots[q] = q;
  *nskip = diis_coefficients(Bmat, n, slots, n, damping, coef);
}

__global__ void __launch_bounds__(kThreads) diis_solve_kernel(DiisArgs d) {
  __shared__ double sh[kThreads];
  __shared__ double dots[kDiisMax];
  __shared__ DiisMeta meta;
  load_diis_meta(d, &meta);
  const int slot = meta.slot;
  for (int q = 0; q < meta.nvec; ++q) {
    double s = 0.0;
    for (int b = threadIdx.x; b < kReduceBlocks; b += blockDim.x) s += d.partial[b * kDiisMax + q];
    s = block_sum(s, sh);
    if (threadIdx.x == 0) dots[q] = s;
  }
  __syncthreads();
  if (threadIdx.x != 0) return;
  const int nd = d.ndiis;
  const int* slots = meta.slots;
  for (int q = 0; q < meta.nvec; ++q) {
    d.Bmat[slot * nd + slots[q]] = dots[q];
    d.Bmat[slots[q] * nd + slot] = dots[q];
  }
  if (!meta.extrapolate) {
    for (int s = 0; s < nd; ++s) d.coef[s] = 0.0;
    d.coef[slot] = 1.0;
    *d.nskip_out = -1;
    return;
  }
  *d.nskip_out = diis_coefficients(d.Bmat, nd, slots, meta.nvec, d.damping, d.coef);
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
  const DiisDyn* dyn;  // non-NULL: nvec and slots from device memory
};

__device__ __forceinline__ void load_extrap_meta(const ExtrapArgs& x, int* s_slots, int* s_nvec) {
  if (threadIdx.x < kDiisMax) s_slots[threadIdx.x] = x.dyn ? x.dyn->slots[threadIdx.x] : x.slots[threadIdx.x];
  if (threadIdx.x == 0) *s_nvec = x.dyn ? x.dyn->nvec : x.nvec;
  __syncthreads();
}

__global__ void __launch_bounds__(kThreads) extrapolate_t1_kernel(ExtrapArgs x) {
  __shared__ int slots[kDiisMax];
  __shared__ int nvec;
  load_extrap_meta(x, slots, &nvec);
  const int64_t n1 = x.v * x.o;
  for (int64_t e = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; e < n1;
       e += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    double acc = 0.0;
    for (int q = 0; q < nvec; ++q) acc = fma(x.coef[slots[q]], x.x1[slots[q] * n1 + e], acc);
    x.t1[e] = acc;
  }
}

__global__ void __launch_bounds__(kThreads) extrapolate_t2_tau_kernel(ExtrapArgs x) {
  __shared__ int slots[kDiisMax];
  __shared__ int s_nvec;
  load_extrap_meta(x, slots, &s_nvec);
  const int nvec = s_nvec;
  const int64_t o = x.o, v = x.v, o2 = o * o, n2 = v * v * o2;
  double c[kDiisMax];
  for (int q = 0; q < kDiisMax; ++q) c[q] = (q < nvec) ? x.coef[slots[q]] : 0.0;
  for (int64_t p = blockIdx.x; p < v * v; p += gridDim.x) {
    int64_t a, b;
    divmod32(p, v, a, b);
    for (int64_t ij = threadIdx.x; ij < o2; ij += blockDim.x) {
      int64_t i, j;
      divmod32(ij, o, i, j);
      const int64_t e = p * o2 + ij;
      double acc = 0.0;
      for (int q = 0; q < nvec; ++q) acc = fma(c[q], x.x2[slots[q] * n2 + e], acc);
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

__global__ void split_test_kernel(const double* x, int64_t n, int nslices, unsigned short* out) {
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    unsigned short b[3];
    split_bits(x[i], b, nslices);
    for (int s = 0; s < nslices; ++s) out[s * n + i] = b[s];
  }
}

__global__ void scale_test_kernel(const double* x, int64_t n, GatherTerm T, double* out) {
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    out[i] = T.pow2 ? term_scale(T, x[i]) : x[i] * T.coef;  // as the gathers dispatch
}

}  // namespace

void launch_scale_test(const double* x, int64_t n, double coef, double* out, cudaStream_t st) {
  if (n <= 0) return;
  GatherTerm T{};
  gather_set_coef(T, coef);
  scale_test_kernel<<<static_cast<unsigned>(std::min<int64_t>((n + 255) / 256, 4096)), 256, 0, st>>>(x, n, T, out);
}

void launch_split_test(const double* x, int64_t n, int nslices, unsigned short* out, cudaStream_t st) {
  if (n <= 0) return;
  split_test_kernel<<<static_cast<unsigned>(std::min<int64_t>((n + 255) / 256, 4096)), 256, 0, st>>>(
      x, n, nslices, out);
}

int num_sms() {
  static const int sms = [] {
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n > 0 ? n : 1;
  }();
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
  if (g.outs && g.fixed) {
    launch_gather_fixed(g, st);
    return;
  }
  const GatherShape sh = gather_shape(g);
  if (sh.kind == GatherShape::kTiles) gather_t_kernel<<<sh.grid, sh.block, 0, st>>>(g);
  else if (sh.kind == GatherShape::kFour && g.outs) gather_split4_kernel<<<sh.grid, sh.block, 0, st>>>(g);
  else if (sh.kind == GatherShape::kFour) gather4_f64_kernel<<<sh.grid, sh.block, 0, st>>>(g);
  else gather_kernel<<<sh.grid, sh.block, 0, st>>>(g);
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

void launch_build_gpm(int64_t rows_v, int64_t v, bool ab_pairs, const double* G, double* Gp, double* Gm,
                      cudaStream_t st) {
  build_gpm_kernel<<<grid_for(rows_v * v, 1), kThreads, 0, st>>>(rows_v, v, ab_pairs, G, Gp, Gm);
}

void launch_build_gpm_oo(int64_t o, int64_t v, const double* Gijab, double* Gtp, double* Gtm, cudaStream_t st) {
  build_gpm_oo_kernel<<<grid_for(o * o, 1), kThreads, 0, st>>>(o, v, Gijab, Gtp, Gtm);
}

void launch_pair_combine_oo(int64_t o, const double* W, double* Wt, double* Wm, cudaStream_t st) {
  pair_combine_oo_kernel<<<grid_for(o * o, 1), kThreads, 0, st>>>(o, W, Wt, Wm);
}

void launch_build_gpm_chem(int64_t n, const double* G, double* Gp, double* Gm, cudaStream_t st) {
  build_gpm_chem_kernel<<<grid_for(n * n, 1), kThreads, 0, st>>>(n, G, Gp, Gm);
}

void launch_build_gpm_rows(int64_t a0, int64_t a1, int64_t v, const double* Gblk, double* Gp, double* Gm,
                           cudaStream_t st) {
  if (a1 <= a0) return;
  build_gpm_rows_kernel<<<grid_for((a1 - a0) * (v - a0), 1), kThreads, 0, st>>>(a0, a1, v, Gblk, Gp, Gm);
}

void launch_tau_pm(int64_t o, int64_t v, const double* tau, double* taup, double* taum, cudaStream_t st) {
  tau_pm_kernel<<<grid_for(v * v, 1), kThreads, 0, st>>>(o, v, tau, taup, taum);
}

void launch_pair_unpack(int64_t rows_v, int64_t v, int64_t o, bool ab_pairs, const double* Bp, const double* Bm,
                        double beta, double* out, cudaStream_t st) {
  if (beta == 0.0)
    pair_unpack_kernel<false><<<grid_for(rows_v * v, 1), kThreads, 0, st>>>(rows_v, v, o, ab_pairs, Bp, Bm, out);
  else
    pair_unpack_kernel<true><<<grid_for(rows_v * v, 1), kThreads, 0, st>>>(rows_v, v, o, ab_pairs, Bp, Bm, out);
}

void launch_r2_assemble(int64_t o, int64_t v, const double* r2u, const double* tmp, const double* g,
                        const double* Bp, const double* Bm, bool accumulate, double* r2, cudaStream_t st) {
  const int64_t nt = (o + 31) / 32;
  const unsigned grid = static_cast<unsigned>(std::min<int64_t>(v * v * nt * nt, 152LL * 16));
  r2_assemble_kernel<<<grid, dim3(32, 8), 0, st>>>(o, v, r2u, tmp, g, Bp, Bm, accumulate, r2);
}

void launch_diag_snapshot(int64_t o, int64_t v, int which, const double* X, double* d, cudaStream_t st) {
  diag_snapshot_kernel<<<grid_for(o * v * v, kThreads), kThreads, 0, st>>>(o, v, which, X, d);
}

void launch_gac_from_diagonals(int64_t o, int64_t v, const double* K, const double* P, const double* dK,
                               const double* dP, double* gac, cudaStream_t st) {
  gac_from_diagonals_kernel<<<grid_for(v * v, kThreads), kThreads, 0, st>>>(o, v, K, P, dK, dP, gac);
}

void launch_r1_from_tmp2(int64_t o, int64_t v, const double* tmp2, double* r1, cudaStream_t st) {
  r1_from_tmp2_kernel<<<grid_for(v * o, kThreads), kThreads, 0, st>>>(o, v, tmp2, r1);
}

void launch_denominators(int64_t o, int64_t v, const double* eps_o, const double* eps_v, double* dinv1,
                         double* dinv2, cudaStream_t st) {
  denominators_kernel<<<grid_for(v * v, 1), kThreads, 0, st>>>(o, v, eps_o, eps_v, dinv1, dinv2);
}

void launch_jacobi_inplace(int64_t o, int64_t v, const double* eps_o, const double* eps_v, const double* r1,
                           const double* r2, double* t1, double* t2, cudaStream_t st) {
  jacobi_inplace_kernel<<<grid_for(v * v, 1), kThreads, 0, st>>>(o, v, eps_o, eps_v, r1, r2, t1, t2);
}

void launch_pair_asym(int64_t o, int64_t v, const double* t2, unsigned long long* out, cudaStream_t st) {
  pair_asym_kernel<<<grid_for(v * v, 1), kThreads, 0, st>>>(o, v, t2, out);
}

void launch_maxabs_diff(int64_t n, const double* a, const double* b, unsigned long long* out, cudaStream_t st) {
  if (n <= 0) return;
  maxabs_diff_kernel<<<grid_for(n, kThreads, 1216), kThreads, 0, st>>>(n, a, b, out);
}

void launch_diis_step(const DiisArgs& d, cudaStream_t st) {
  diis_jacobi_dots_kernel<<<kReduceBlocks, kThreads, 0, st>>>(d);
  diis_solve_kernel<<<1, kThreads, 0, st>>>(d);
}

void launch_diis_coefficients_test(const double* Bmat, int n, double damping, double* coef, int* nskip,
                                   cudaStream_t st) {
  diis_coefficients_test_kernel<<<1, 32, 0, st>>>(Bmat, n, damping, coef, nskip);
}

void launch_diis_extrapolate(int64_t o, int64_t v, const double* x1, const double* x2,
                             const double* coef, int ndiis, const int* slots, int nvec,
                             double* t1, double* t2, double* tau, cudaStream_t st, const DiisDyn* dyn) {
  (void)ndiis;
  ExtrapArgs x;
  x.o = o;
  x.v = v;
  x.x1 = x1;
  x.x2 = x2;
  x.coef = coef;
  x.nvec = nvec;
  for (int q = 0; q < kDiisMax; ++q) x.slots[q] = (slots && q < nvec) ? slots[q] : 0;
  x.t1 = t1;
  x.t2 = t2;
  x.tau = tau;
  x.dyn = dyn;
  extrapolate_t1_kernel<<<grid_for(v * o, kThreads), kThreads, 0, st>>>(x);
  extrapolate_t2_tau_kernel<<<grid_for(v * v, 1), kThreads, 0, st>>>(x);
}

}  // namespace gbcc
