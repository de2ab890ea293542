// Small dense host linear algebra for the RHF driver (N x N, N a few hundred).
#pragma once

#include <vector>

namespace gbcc {
namespace hostla {

// C[m x n] = A[m x k] B[k x n]
void gemm_nn(int m, int n, int k, const double* A, const double* B, double* C);
// C[m x n] = A[m x k] B[n x k]^T
void gemm_nt(int m, int n, int k, const double* A, const double* B, double* C);
// C[m x n] = A[k x m]^T B[k x n]
void gemm_tn(int m, int n, int k, const double* A, const double* B, double* C);
// A = (A + A^T) / 2
void symmetrize(int n, double* A);

// Eigenvalues w (ascending) and eigenvectors V (column j of the row-major
// n x n V belongs to w[j]) of the symmetric A: Householder reduction to
// tridiagonal form, then implicit symmetric QR steps with the Wilkinson shift
// (G. H. Golub, C. F. Van Loan, Matrix Computations, sections 8.3.1-8.3.3).
void eigh(int n, std::vector<double> A, std::vector<double>& w, std::vector<double>& V);

// x = A^{-1} b by Gaussian elimination with partial pivoting; false when a
// pivot vanishes (relative to the largest entry)
bool solve(int n, std::vector<double> A, std::vector<double> b, std::vector<double>& x);

}  // namespace hostla
}  // namespace gbcc
