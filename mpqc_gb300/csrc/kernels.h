// Device kernels of the CCSD engine and their host-side launchers.
#pragma once

#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <stdint.h>

#include <cmath>

namespace gbcc {

// Error word written by bounded device-side waits; read by the host after a step.
enum DeviceError : int { kDevOk = 0, kDevTimeout = 1, kDevBadArg = 2 };

// ---------------------------------------------------------------------------
// Gather / linear-combination kernel.
//
// The output is viewed as a 2-D array [R][C].  Element (r, c) of the result is
//   sum_t coef_t * a_t[ra_t[r] + ca_t[c]] * (b_t ? b_t[rb_t[r] + cb_t[c]] : 1)
// where ra/ca (rb/cb) are offset tables built on the host from the index
// labels.  The same kernel permutes tensors, forms linear combinations such as
// 2 G(k,l,c,d) - G(k,l,d,c), outer products t1(a,i) t1(b,j), and packs GEMM
// operands as K-contiguous [M][K] panels (FP64 or split BF16 slices).
// ---------------------------------------------------------------------------
constexpr int kMaxTerms = 4;

struct GatherTerm {
  double coef;
  const double* a;
  const int64_t* ra;
  const int64_t* ca;
  const double* b;   // nullptr: single factor
  const int64_t* rb;
  const int64_t* cb;
  // coef = (-1)^sign 2^pow2_k exactly (pow2 != 0): the kernels scale by
  // exponent arithmetic instead of an FP64 multiply (set by gather_set_coef)
  int pow2;
  int pow2_k;
  unsigned long long pow2_sign;
  // 1: ca runs in contiguous groups of four starting at even offsets and a is
  // 16-byte aligned (vector loads of 4 K elements; set by gather_set_c4)
  int c4;
};

// true when c = (-1)^neg 2^k exactly with |k| <= 64
inline bool pow2_parts(double c, int& k, bool& neg) {
  int e = 0;
  const double m = std::frexp(c, &e);  // c = m 2^e, 0.5 <= |m| < 1
  k = e - 1;
  neg = c < 0;
  return (m == 0.5 || m == -0.5) && k >= -64 && k <= 64;
}

inline void gather_set_coef(GatherTerm& T, double coef) {
  T.coef = coef;
  bool neg = false;
  T.pow2 = pow2_parts(coef, T.pow2_k, neg) ? 1 : 0;
  T.pow2_sign = neg ? (1ull << 63) : 0ull;
}

struct GatherArgs {
  int nterms;
  GatherTerm t[kMaxTerms];
  int64_t R, C;        // logical extent
  int64_t Rpad, Cpad;  // written extent (zero outside R x C)
  // FP64 output (out != nullptr): out[r*ldo + c] = beta*out + value
  double* out;
  int64_t ldo;
  double beta;
  // split output (outs != nullptr): nslices BF16 slices, slice s at
  // outs + s*slice_stride, each k-block major ([Cpad/64][Rpad][64], Cpad a
  // multiple of 64: the tensor-core GEMM's operand layout; ldo unused)
  __nv_bfloat16* outs;
  int nslices;
  int64_t slice_stride;
  // 1: the sources are contiguous along R, not C -- read 32 x 32 tiles along R
  // and transpose them through shared memory (set by the planner)
  int transpose;
  // 1: one term, no second factor, coefficient 1 -- a plain load (set by the planner)
  int plain;
  // 1: some term has a second factor (b != nullptr)
  int products;
  // 1: some coefficient is not +-2^k (set by gather_finish)
  int general;
  // split output in fixed point (GBCC_PREC_FP64_TC): 1, the exponent pass --
  // rowexp[r] = max over the row of the biased FP64 exponent of the packed
  // value (rowexp zeroed first; nothing stored); 2, the split pass -- every
  // element of row r in nslices 8-bit digits under that exponent
  int fixed;
  unsigned* rowexp;
};

// Fixed-point slices of the FP64-grade tensor-core contractions.  A row with
// largest |x| < 2^(E-1) is held as X = round(x 2^(8n - E)), |X| <= 2^(8n-1),
// in n balanced base-256 digits, every one in [-128, 128]; slice p stores
// I_p 2^(E - 8(p+1)) exactly in BF16 (at most 8 significant bits).  Every
// product of slices p of A and q of B with p + q = w is then an integer
// multiple of 2^(E_A + E_B - 8(w + 2)) of magnitude at most 2^14 of it, so
// FP32 sums of up to 2^10 of them stay within 2^24 units and are exact: one
// TMEM chunk (8 (k-block, pair) steps, 512 products) and the FP32 register
// sum of two chunks before each float-float fold.
constexpr int kFixedBits = 8;
constexpr int kFixedSlices = 6;   // 47 bits below the row's leading power of two
constexpr int kFixedChunk = 8;    // (k-block, pair) steps per TMEM accumulation: 512 products
constexpr int kFixedFold = 2;     // chunks summed in FP32 registers before the float-float fold
// The pairs (p, w - p), both below n, of weight class w; returns their number.
inline int fixed_class_pairs(int n, int w, int* pa, int* pb) {
  int k = 0;
  for (int p = 0; p < n; ++p)
    if (w - p >= 0 && w - p < n) {
      pa[k] = p;
      pb[k] = w - p;
      ++k;
    }
  return k;
}

inline void gather_set_c4(GatherTerm& T, const int64_t* hca, int64_t n) {
  bool ok = reinterpret_cast<uintptr_t>(T.a) % 16 == 0;
  for (int64_t q = 0; ok && q + 3 < n; q += 4)
    ok = hca[q] % 2 == 0 && hca[q + 1] == hca[q] + 1 && hca[q + 2] == hca[q] + 2 && hca[q + 3] == hca[q] + 3;
  T.c4 = ok ? 1 : 0;
}

// derived flags of a filled GatherArgs (call after its terms are set)
inline void gather_finish(GatherArgs& g) {
  g.general = 0;
  for (int t = 0; t < g.nterms; ++t)
    if (!g.t[t].pow2) g.general = 1;
}

void launch_gather(const GatherArgs& args, cudaStream_t st);
// one fixed-point pass (args.fixed 1 or 2) of a split pack (pack_fixed.cu);
// launch_gather forwards to it
void launch_gather_fixed(const GatherArgs& args, cudaStream_t st);

// out[i] = coef * x[i] as the gather kernels scale a term (exponent arithmetic
// for power-of-two coefficients)
void launch_scale_test(const double* x, int64_t n, double coef, double* out, cudaStream_t st);

// FP64 -> nslices BF16 bit patterns (out[s*n + i]) with the packing kernels' split
void launch_split_test(const double* x, int64_t n, int nslices, unsigned short* out, cudaStream_t st);

// ---------------------------------------------------------------------------
// FP64 GEMM with scattered epilogue:
//   C[cm[m] + cn[n]] = beta * C[...] + alpha * sum_k A[m*lda + k] * B[n*ldb + k]
// for m < M, n < N (bounds-checked; operands need no padding).
// ---------------------------------------------------------------------------
struct GemmF64Args {
  int64_t M, N, K;
  int ksplit;            // >1: blockIdx.z covers K range z; partials [ksplit][M][N]
  int64_t k_per_split;
  double* partial;
  const double* A;
  int64_t lda;
  const double* B;
  int64_t ldb;
  double* C;
  const int64_t* cm;
  const int64_t* cn;
  double alpha, beta;
  int m_major;           // C unit-stride along M (small-K kernel: lanes along M)
  // small-K stream kernel: A read in place, A[m][k] = A[a_ra[m] + a_ca[k]]
  // (null: A is an lda-strided panel)
  const int64_t* a_ra;
  const int64_t* a_ca;
};
void launch_gemm_f64(const GemmF64Args& g, cudaStream_t st);

// Short contractions (K <= kSmallK) with large outputs on CUDA cores: FP64
// panels rounded to FP32, FP32 products and sums, one FP64 FMA per output.
// Memory-bound on the FP64 read-modify-write of C; used in mixed precision
// instead of the tensor-core pipeline, whose per-tile handshakes leave such
// outputs latency-bound.  Same argument conventions as launch_gemm_f64 (no K split).
constexpr int64_t kSmallK = 64;
// whether launch_gemm_smallk takes the stream kernel (C contiguous along M,
// K <= 64, B within 64 KB of shared memory): the only one that reads A in place
bool smallk_streams(int64_t N, int64_t K, bool m_major);
// false (nothing launched) when A is read in place and the stream kernel does not apply
bool launch_gemm_smallk(const GemmF64Args& g, cudaStream_t st);

// ---------------------------------------------------------------------------
// Split-BF16 tcgen05 GEMM (sm_103a):
//   C[cm[m] + cn[n]] = beta*C + alpha * sum_{(p,q) in pairs} A_p[m][:] . B_q[n][:]
// A_p: slice p of A, [Mpad][Kpad] bf16 K-contiguous; B_q likewise [Npad][Kpad].
// Each TMEM (FP32) accumulation covers `chunk` k-blocks; chunks are summed in
// float-float registers and converted to FP64 in the epilogue.
// ---------------------------------------------------------------------------
constexpr int kMaxPairs = 9;
struct GemmTcArgs {
  int64_t M, N;          // logical
  int64_t Mpad, Npad, Kpad;
  const __nv_bfloat16* A; int a_slices;  // [a_slices][Mpad][Kpad]
  const __nv_bfloat16* B; int b_slices;  // [b_slices][Npad][Kpad]
  int npairs;
  int pa[kMaxPairs], pb[kMaxPairs];
  double* C;
  const int64_t* cm;
  const int64_t* cn;
  double alpha, beta;
  int bn;                // N tile (32, 64, 128 or 256)
  int chunk;             // k-blocks per TMEM accumulation (0: default 4)
  int fold;              // chunks summed in FP32 before a float-float fold (0: default 16)
  int ksplit;            // >1: K split over CTAs; partial tiles go to `partial`
  int kb_per_split;      // k-blocks per split (every split gets at least one)
  double* partial;       // [ksplit][Mpad][Npad] FP64 partial tiles (ksplit > 1)
  int m_major;           // C is contiguous along M: epilogue lanes run along M
  int cta2;              // CTA pairs (tcgen05 cta_group::2, 256-row tiles); Mpad % 256 == 0, bn >= 64
  int* err;              // device error word
  // rows per slice of the A / B panels as stored (0: Mpad / Npad); a panel may
  // hold more rows than the launch covers (padded for every candidate tile)
  int64_t a_rows, b_rows;
  // slices per pipeline stage: 0 or 1, one (A, B) slice pair per stage; 2, both
  // slices of A and B of a k-block per stage (2 slices, bn 64 / 128 / 192)
  int sps;
  // > 1: output tiles run in bands of `group` M tiles, N outer within a band
  // (CTAs working at the same time then share fewer, wider operand panels in
  // L2); 0 or 1: N fastest over whole rows of tiles
  int group;
  // first row of A / B within their panels (a window of a larger panel:
  // rows past the panel's end load as zeros; 0 for whole panels)
  int64_t a_row0, b_row0;
  // test hooks: the pipeline barriers' wait limit in ns (0: 2 s), and 1 +
  // the stage (counted over a CTA's stage uses; one pair per stage) whose
  // loads the producer leaves out (0: none -- the value-initialised default)
  uint64_t wait_ns;
  int64_t skip_stage1;
};
// Deterministic K-split reduction: C[cm[m] + cn[n]] = beta*C + alpha * sum_s
// partial[s][m][n] (splits summed in order), partial rows of length ldp and
// split stride rows*ldp.
void launch_splitk_reduce(int64_t M, int64_t N, int ksplit, const double* partial, int64_t rows,
                          int64_t ldp, double* C, const int64_t* cm, const int64_t* cn, double alpha,
                          double beta, cudaStream_t st);
int num_sms();

// Returns false if the tensor maps could not be encoded (bad alignment / size).
bool launch_gemm_tc(const GemmTcArgs& g, cudaStream_t st);
// N tile for a GEMM of N columns; allow256: 256- or 192-wide tiles (faster,
// FP32 register accumulation of the chunks) for N >= 256
int gemm_tc_pick_bn(int64_t N, bool allow256);
// N tiles worth timing for a GEMM of N columns (the tuner's candidates), the
// heuristic choice first; returns their number (<= 4)
int gemm_tc_bn_candidates(int64_t N, bool allow256, int* out);
constexpr int kTcBM = 128;
constexpr int kTcBK = 64;

// ---------------------------------------------------------------------------
// Deterministic FP64 reductions for the residual-augmented energy and the
// residual norm (two passes, fixed grid, fixed order).
//   out[0] = sum r1^2, out[1] = sum r2^2,
//   out[2] = sum (f_ai + r1) t1, out[3] = sum (g_abij + r2)(2 tau - tau(b,a,i,j))
// partial: scratch of kReduceBlocks * 4 doubles.
// ---------------------------------------------------------------------------
constexpr int kReduceBlocks = 608;
void launch_energy_terms(int64_t o, int64_t v, const double* r1, const double* r2,
                         const double* f_ai, const double* g_abij, const double* t1,
                         const double* tau, double* partial, double* out, cudaStream_t st);

// tau(a,b,i,j) = t2(a,b,i,j) + t1(a,i) t1(b,j)
// Pair-(anti)symmetric ladder (see kernels.cu): G+/G- over (a <= b or any row
// pair) x (c <= d) from G[rows_v][v][v][v]; tau+/tau- over (c <= d) x (i <= j);
// out(row, i, j) = beta out + B+ +- B- unpacked from the pair products (beta 0 or 1).
void launch_build_gpm(int64_t rows_v, int64_t v, bool ab_pairs, const double* G, double* Gp, double* Gm,
                      cudaStream_t st);
// rows a in [a0, a1) of G+ / G- from Gblk[a - a0][b][c][d], rows counted from
// the block's first pair (the density-fitted ladder builds G+- block by block)
void launch_build_gpm_rows(int64_t a0, int64_t a1, int64_t v, const double* Gblk, double* Gp, double* Gm,
                           cudaStream_t st);
// G+ / G- over n atomic-orbital pairs from G[p][q][r][s] = (pq|rs) (chemists' order)
void launch_build_gpm_chem(int64_t n, const double* G, double* Gp, double* Gm, cudaStream_t st);
// Hole-hole ladder pair factors: Gtp[sym(k,l)][sym(c,d)] = c_kl (G(kl,cd) +
// G(kl,dc)) (c = d: G(kl,cc); c_kl = 2 for k < l, 1 for k = l) and
// Gtm[anti(k,l)][anti(c,d)] = 2 (G(kl,cd) - G(kl,dc)) from Gijab[k][l][c][d]
// (Gtm null: not built)
void launch_build_gpm_oo(int64_t o, int64_t v, const double* Gijab, double* Gtp, double* Gtm, cudaStream_t st);
// Wt[sym(k,l)][sym(i,j)] = W(klij) + W(lkij) (W(kkij) for k = l), Wm[anti(k,l)][anti(i,j)] =
// W(klij) - W(lkij) from W[o][o][o][o] (Wm null: not formed)
void launch_pair_combine_oo(int64_t o, const double* W, double* Wt, double* Wm, cudaStream_t st);
void launch_tau_pm(int64_t o, int64_t v, const double* tau, double* taup, double* taum, cudaStream_t st);
void launch_pair_unpack(int64_t rows_v, int64_t v, int64_t o, bool ab_pairs, const double* Bp, const double* Bm,
                        double beta, double* out, cudaStream_t st);

// r2(a,b,i,j) (+)= q(a,b,i,j) + q(b,a,j,i) + g(a,b,i,j) + unpack(Bp, Bm)(a,b,i,j),
// q = r2u - 0.5 tmp - tmp(b,a,i,j); Bp null: no unpack, Bm null: no B- part;
// accumulate: add to r2, else overwrite it
void launch_r2_assemble(int64_t o, int64_t v, const double* r2u, const double* tmp, const double* g,
                        const double* Bp, const double* Bm, bool accumulate, double* r2, cudaStream_t st);

// d[k][a][c] = K[k][a][k][c] (which 0, K[o][v][o][v]) or P[a][k][k][c] (which 1, P[v][o][o][v])
void launch_diag_snapshot(int64_t o, int64_t v, int which, const double* X, double* d, cudaStream_t st);
// gac(a,c) += sum_k 1.5 (K(k,a,k,c) - dK[k][a][c]) - 0.5 (P(a,k,k,c) - dP[k][a][c])
void launch_gac_from_diagonals(int64_t o, int64_t v, const double* K, const double* P, const double* dK,
                               const double* dP, double* gac, cudaStream_t st);
// r1(a,i) += sum_k 2 tmp2(k,a,k,i) - tmp2(k,a,i,k), tmp2[o][v][o][o], r1[v][o]
void launch_r1_from_tmp2(int64_t o, int64_t v, const double* tmp2, double* r1, cudaStream_t st);

// t1 += r1 / D1, t2 += r2 / D2 in place
void launch_jacobi_inplace(int64_t o, int64_t v, const double* eps_o, const double* eps_v, const double* r1,
                           const double* r2, double* t1, double* t2, cudaStream_t st);

// out[0] = bits of max|t2(a,b,i,j) - t2(b,a,j,i)|, out[1] = bits of max|t2|;
// out must be zeroed first
void launch_pair_asym(int64_t o, int64_t v, const double* t2, unsigned long long* out, cudaStream_t st);

// out[0] = bits of max|a - b|, out[1] = bits of max|b|; out must be zeroed first
void launch_maxabs_diff(int64_t n, const double* a, const double* b, unsigned long long* out, cudaStream_t st);

void launch_make_tau(int64_t o, int64_t v, const double* t1, const double* t2, double* tau,
                     cudaStream_t st);

// ---------------------------------------------------------------------------
// Jacobi update + DIIS bookkeeping (FP64).
//   x_new = t + r / D stored in DIIS slot `slot`, e_new = r stored likewise,
//   dots[j] = <e_new, e_j> for the nvec slots listed in `slots` (partials in
//   scratch, reduced into Bmat row/column `slot`).
// ---------------------------------------------------------------------------
// DIIS bookkeeping kept in device memory when the solve loop runs as one CUDA
// graph (the decision kernel of solve_graph.cu writes it each iteration)
struct DiisDyn {
  int slot;
  int nvec;
  int slots[16];
  int extrapolate;
};

struct DiisArgs {
  const DiisDyn* dyn;  // non-NULL: slot, nvec, slots and extrapolate are read from here
  int64_t o, v;
  const double* eps_o;
  const double* eps_v;
  // reciprocal denominators 1 / (eps_o[i] - eps_v[a]) [v][o] and
  // 1 / (eps_o[i] + eps_o[j] - eps_v[a] - eps_v[b]) [v][v][o][o]
  const double* dinv1;
  const double* dinv2;
  const double* t1;
  const double* t2;
  const double* r1;
  const double* r2;
  double* x1;          // [ndiis][v*o]
  double* x2;          // [ndiis][v*v*o*o]
  double* e1;
  double* e2;
  int ndiis;
  int slot;            // slot receiving the new pair
  int nvec;            // stored pairs after insertion
  int slots[16];       // age order, oldest first; slots[nvec-1] == slot
  double* partial;     // scratch [kReduceBlocks][16]
  double* Bmat;        // [ndiis][ndiis] by slot
  double* coef;        // [ndiis] by slot (output of the solve)
  double damping;
  int extrapolate;     // 0: coefficients select the newest vector only
  int* nskip_out;      // device int
};
void launch_diis_step(const DiisArgs& d, cudaStream_t st);
// test hook: the DIIS coefficients of a given n x n B (n <= 16), coef[n], *nskip
void launch_diis_coefficients_test(const double* Bmat, int n, double damping, double* coef, int* nskip,
                                   cudaStream_t st);

// dinv1 = 1 / D1, dinv2 = 1 / D2 (the Jacobi denominators of DiisArgs), once
// per set of orbital energies: the iteration then multiplies, and the FP64
// pipe that a division per element would occupy (a sequence of FP64
// instructions on a GPU whose FP64 rate is 1/64 of FP32) is left to the dots
void launch_denominators(int64_t o, int64_t v, const double* eps_o, const double* eps_v, double* dinv1,
                         double* dinv2, cudaStream_t st);

// t1 = sum_j coef[j] x1_j, t2 = sum_j coef[j] x2_j, tau = t2 + t1 t1
// (dyn non-NULL: nvec and slots read from device memory)
void launch_diis_extrapolate(int64_t o, int64_t v, const double* x1, const double* x2,
                             const double* coef, int ndiis, const int* slots, int nvec,
                             double* t1, double* t2, double* tau, cudaStream_t st,
                             const DiisDyn* dyn = nullptr);

// ---------------------------------------------------------------------------
// Whole-solve CUDA graph (solve_graph.cu): the convergence test of each
// iteration runs on the device and drives the graph's conditional nodes.
// ---------------------------------------------------------------------------
struct SolveState {
  // loop
  int iter, converged, stop, status;  // status: 0 ok, 1 non-finite energy or residual
  int mixed_phase, used_mixed, stalled, pending_reset;
  int fp64_resid, mixed_resid;
  double E0, E1, dE, error, best_error, best_dE;
  // DIIS bookkeeping (read by the DIIS kernels)
  int diis_iter, head;
  DiisDyn diis;
};
struct SolveParams {
  int64_t n1, n2;
  int max_iter, n_diis, diis_start, diis_ngroup, diis_group_nstart, refine_iters, reset_diis;
  double target, switch_precision;
  double* Bmat;                 // [n_diis][n_diis], cleared at a DIIS restart
  const double* sums;           // the energy reduction's four sums
  SolveState* state;
  double* history;              // [max_iter + 1][3]: E, dE, error per convergence test
  unsigned long long cond_loop, cond_update, cond_mixed, cond_fp64;  // cudaGraphConditionalHandle
};
// zero the state for a solve (mixed: start in the mixed phase)
void launch_solve_init(SolveState* s, int mixed, cudaStream_t st);
// one thread: E, error, convergence test, phase switch, DIIS bookkeeping,
// and the conditions of the loop, the update and the residual precision
void launch_solve_decide(const SolveParams& p, cudaStream_t st);
// nanosecond timestamp (globaltimer) of the current iteration's residual:
// base[2 (iter - 1) + which]
void launch_stamp(unsigned long long* base, const SolveState* s, int which, cudaStream_t st);
// the same as an explicit kernel node of graph g
cudaError_t add_stamp_node(cudaGraph_t g, const cudaGraphNode_t* deps, size_t ndeps, unsigned long long* base,
                           const SolveState* s, int which, cudaGraphNode_t* out);

}  // namespace gbcc
