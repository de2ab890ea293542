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

/* Peak probe: FP64 FMA throughput of this GPU in GFLOP/s (a register-resident
 * DFMA loop over all SMs). */
int gbcc_testing_fp64_peak(double* gflops);

#ifdef __cplusplus
}
#endif

#endif /* GBCC_TESTING_H_ */
