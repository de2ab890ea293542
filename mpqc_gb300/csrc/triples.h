// Perturbative triples correction (T) (triples.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace gbcc {

// Device-resident inputs, MPQC annotation order (as the residual engine
// holds them): t1[a][i], t2[a][b][i][j], Gijab[i][j][a][b] = <ij|ab>,
// Gijka[i][j][k][a] = <ij|ka>, Giabc[i][a][b][c] = <ia|bc>, active orbital
// energies.
struct TriplesInputs {
  int64_t o = 0, v = 0;
  const double* t1 = nullptr;
  const double* t2 = nullptr;
  const double* Gijab = nullptr;
  const double* Gijka = nullptr;
  const double* Giabc = nullptr;
  const double* eps_o = nullptr;
  const double* eps_v = nullptr;
};

// E(T) in the given precision (GBCC_PREC_FP64: the DFMA GEMM; MIXED: three
// BF16 slices; FP64_TC: six fixed-point slices); the energy sums are FP64.
// Synchronises the stream; throws gbcc::Error.
double triples_energy(const TriplesInputs& in, int precision, cudaStream_t st, int* err);

}  // namespace gbcc
