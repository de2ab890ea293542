/*
 * gbcc_testing.h -- test hooks of libgbcc.  Not part of the drop-in
 * boundary (include/gbcc.h is); used by the GPU test-suite and the
 * benchmark to exercise single kernels in isolation.
 */
#ifndef GBCC_TESTING_H_
#define GBCC_TESTING_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* C[m][n] = sum_k A[m][k] B[n][k] for row-major A [M][K], B [N][K], C [M][N]
 * (host or device pointers).  slices == 0 runs the FP64 GEMM kernel;
 * slices 1..3 run the split-BF16 tcgen05 kernel with that many slices per
 * operand.  If ms is not NULL it receives the kernel time (CUDA events, ms)
 * averaged over `repeat` launches.  Returns 0 on success, else a
 * gbcc_status code. */
int gbcc_testing_gemm(int64_t M, int64_t N, int64_t K, const double* A, const double* B, double* C,
                      int slices, int repeat, float* ms);

/* As gbcc_testing_gemm with the tensor-core kernel's knobs exposed: the K
 * dimension split over `ksplit` groups of CTAs (partial tiles reduced in a
 * fixed order by a second kernel), the N tile `bn` (0: automatic; 192 and 256 sum
 * chunks in FP32 registers), CTA pairs (`cta2`, tcgen05 cta_group::2), the
 * k-blocks per TMEM accumulation (`chunk`, 0: default) and the chunks per
 * float-float fold (`fold`, 0: default).  slices == 0 runs the FP64 kernel. */
int gbcc_testing_gemm_ex(int64_t M, int64_t N, int64_t K, const double* A, const double* B, double* C,
                         int slices, int ksplit, int bn, int cta2, int chunk, int fold, int repeat, float* ms);

/* The BF16 split the packing kernels apply: x[0..n) (host) -> out[s*n + i]
 * (host), the bit patterns of slices s = 0..nslices-1 (nslices 1..3). */
int gbcc_testing_split(const double* x, int64_t n, int nslices, uint16_t* out);

/* out[i] = coef * x[i] (host arrays) as the packing kernels scale a term of a
 * linear combination: exponent arithmetic for coef = +-2^k, an FP64 multiply
 * otherwise.  Must equal the IEEE product bit for bit. */
int gbcc_testing_scale(const double* x, int64_t n, double coef, double* out);

/* As gbcc_testing_gemm_ex with the number of slices per pipeline stage:
 * sps = 1, one (A, B) slice pair per stage; 2, both slices of a k-block per
 * stage (slices = 2, bn 64 / 128 / 192). */
int gbcc_testing_gemm_ex2(int64_t M, int64_t N, int64_t K, const double* A, const double* B, double* C,
                          int slices, int ksplit, int bn, int cta2, int chunk, int fold, int sps, int repeat,
                          float* ms);

/* As gbcc_testing_gemm_ex2 with the tile order and the output form: group > 1
 * runs the output tiles in bands of `group` M tiles, N outer within a band;
 * cmode bit 0 accumulates into C (beta = 1; the timed launches add up, the
 * returned C is one product added to zeros), bit 1 stores C column-major on
 * the device (unit stride along M, the m-major epilogue).  C is returned
 * row-major either way. */
int gbcc_testing_gemm_ex3(int64_t M, int64_t N, int64_t K, const double* A, const double* B, double* C,
                          int slices, int ksplit, int bn, int cta2, int chunk, int fold, int sps, int group,
                          int cmode, int repeat, float* ms);


/* Peak probe: FP64 FMA throughput of this GPU in GFLOP/s (a register-resident
 * DFMA loop over all SMs). */
int gbcc_testing_fp64_peak(double* gflops);

/* Fixed-point slices of a row-major [rows][cols] FP64 matrix as the
 * FP64-grade contractions pack them (GBCC_PREC_FP64_TC): out[s][r][c], the
 * BF16 bits of slice s (nslices <= 6), and rowexp[r], the row's largest
 * biased FP64 exponent. */
int gbcc_testing_fixed_split(const double* x, int64_t rows, int64_t cols, int nslices, uint16_t* out,
                             uint32_t* rowexp);

/* C[M][N] = A[M][K] B[N][K]^T through the FP64-grade tensor-core path: six
 * fixed-point slices per operand row, one tcgen05 launch per weight class
 * (bn 0: the heuristic tile width; 32, 64 or 128), K split over CTAs when
 * ksplit > 1, CTA pairs (cta_group::2, 256-row tiles; bn 64 or 128) when
 * cta2.  *ms: the time of one product (all class launches). */
int gbcc_testing_gemm_fp64tc(int64_t M, int64_t N, int64_t K, const double* A, const double* B, double* C,
                             int bn, int ksplit, int cta2, int repeat, float* ms);

/* Failure detection of the tensor-core GEMM without a GPU fault: one launch
 * of C = A B^T (3 BF16 slices) whose producer leaves stage skip_stage of
 * every CTA unloaded, with the pipeline barriers' wait limit shortened to
 * wait_ns; the kernel's bounded wait runs out, it records the timeout, drains
 * its copies, waits for its MMAs, frees its tensor memory and returns.
 * *first = that launch's status (GBCC_ERR_TIMEOUT), *second = the status of
 * the same product run normally afterwards, whose result is written to C. */
int gbcc_testing_gemm_timeout(int64_t M, int64_t N, int64_t K, const double* A, const double* B, double* C,
                              uint64_t wait_ns, int64_t skip_stage, int* first, int* second);

/* Triplets per (T) batch for calls from now on (0: the default, as many as
 * keep the batch's slice of t3 in L2). */
int gbcc_testing_triples_chunk(int64_t k);

/* Peak probe: FP64 tensor-core throughput (mma.sync m8n8k4 .f64, DMMA) in
 * GFLOP/s, register operands over all SMs. */
int gbcc_testing_dmma_peak(double* gflops);

/* The solver's DIIS coefficient solve (the bordered system of the stored
 * vectors, oldest dropped while it is singular) on a given n x n B (n <= 16,
 * vectors in age order, oldest first): coef[n] and the number of oldest
 * vectors dropped. */
int gbcc_testing_diis_coefficients(int32_t n, const double* B, double damping, double* coef, int32_t* nskip);

/* Device allocations of the engine: *count (may be NULL) receives how many
 * were made so far in the process; from now on `after` more succeed and the
 * next one fails with GBCC_ERR_OOM as if the device were full (-1: none fails). */
int gbcc_testing_fail_alloc(int64_t after, int64_t* count);

/* Rows a per block of the density-fitted ladder for handles whose inputs are
 * set from now on (0: the default size, a block of (ab|cd) of at most 4 GB). */
int gbcc_testing_df_block_rows(int64_t rows);

/* Symmetric eigensolver of the RHF driver (host code, no GPU needed):
 * eigenvalues w[n] ascending, eigenvectors V[n][n] by column. */
int gbcc_testing_eigh(int32_t n, const double* A, double* w, double* V);

/* One residual on the device-resident amplitudes of handle h (t1/t2 as left
 * by the previous gbcc_residual / gbcc_solve call) with CUDA events around
 * every operation of the residual program.  For each of the first
 * max_sites operations writes: its time in ms, its algorithmic FLOPs
 * (2 M N K, 0 for elementwise operations), the number of BF16 slice
 * products it executed on the tensor cores (0: FP64 kernel or elementwise)
 * and its term class (0 ladder, 1 ring, 2 other, -1 elementwise).
 * *nsites receives the number of operations. */
struct gbcc_handle;
int gbcc_testing_profile_residual(struct gbcc_handle* h, int precision, int max_sites, double* ms,
                                  double* flops, int* pairs, int* cls, int* nsites);

/* Tensor-core GEMM launches of handle h since its creation, slice
 * calibration and tile tuning included (for choosing an ncu launch to skip to). */
int gbcc_testing_tc_launches_total(gbcc_handle* h, int64_t* launches);

/* Kernel launches of the last residual (every kernel of this library). */
int gbcc_testing_last_launches(struct gbcc_handle* h, int* launches);

/* Record timing event `slot` (0..7) on the handle's CUDA stream, and read the
 * milliseconds between two recorded slots (waits for the second). */
int gbcc_testing_record(struct gbcc_handle* h, int slot);
int gbcc_testing_elapsed(struct gbcc_handle* h, int slot0, int slot1, float* ms);

/* GEMM-kernel-only time (ms) of each operation in the last profiled residual
 * (0 for elementwise operations); same indexing as
 * gbcc_testing_profile_residual. */
int gbcc_testing_profile_gemm_ms(struct gbcc_handle* h, int max_sites, double* ms);

/* Per operation of the last profiled residual: N tile width of a tensor-core
 * contraction (-1: the short-K CUDA-core kernel, 0: FP64 / elementwise), its
 * K split, its slices per pipeline stage and the M tiles per band of its tile
 * order (1: whole rows), as tiles[4 i .. 4 i + 3]. */
int gbcc_testing_profile_tiles(gbcc_handle* h, int max_sites, int32_t* tiles);

/* GEMM shape (M, N, K) of each operation of the last profiled residual,
 * three int64 per operation (elementwise operations: rows, columns, 0). */
int gbcc_testing_profile_dims(struct gbcc_handle* h, int max_sites, int64_t* mnk);

#ifdef __cplusplus
}
#endif

#endif /* GBCC_TESTING_H_ */
