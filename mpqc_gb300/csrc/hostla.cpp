// Small dense host linear algebra for the RHF driver.
#include "hostla.h"

#include <algorithm>
#include <cmath>
#include <numeric>
#include <stdexcept>

namespace gbcc {
namespace hostla {

void gemm_nn(int m, int n, int k, const double* A, const double* B, double* C) {
  for (int i = 0; i < m; ++i) {
    double* c = C + static_cast<size_t>(i) * n;
    std::fill(c, c + n, 0.0);
    for (int q = 0; q < k; ++q) {
      const double a = A[static_cast<size_t>(i) * k + q];
      if (a == 0.0) continue;
      const double* b = B + static_cast<size_t>(q) * n;
      for (int j = 0; j < n; ++j) c[j] += a * b[j];
    }
  }
}

void gemm_nt(int m, int n, int k, const double* A, const double* B, double* C) {
  for (int i = 0; i < m; ++i)
    for (int j = 0; j < n; ++j) {
      const double* a = A + static_cast<size_t>(i) * k;
      const double* b = B + static_cast<size_t>(j) * k;
      double s = 0.0;
      for (int q = 0; q < k; ++q) s += a[q] * b[q];
      C[static_cast<size_t>(i) * n + j] = s;
    }
}

void gemm_tn(int m, int n, int k, const double* A, const double* B, double* C) {
  std::fill(C, C + static_cast<size_t>(m) * n, 0.0);
  for (int q = 0; q < k; ++q) {
    const double* a = A + static_cast<size_t>(q) * m;
    const double* b = B + static_cast<size_t>(q) * n;
    for (int i = 0; i < m; ++i) {
      const double ai = a[i];
      if (ai == 0.0) continue;
      double* c = C + static_cast<size_t>(i) * n;
      for (int j = 0; j < n; ++j) c[j] += ai * b[j];
    }
  }
}

void symmetrize(int n, double* A) {
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < i; ++j) {
      const double s = 0.5 * (A[static_cast<size_t>(i) * n + j] + A[static_cast<size_t>(j) * n + i]);
      A[static_cast<size_t>(i) * n + j] = A[static_cast<size_t>(j) * n + i] = s;
    }
}

void eigh(int n, std::vector<double> A, std::vector<double>& w, std::vector<double>& V) {
  auto at = [&](int i, int j) -> double& { return A[static_cast<size_t>(i) * n + j]; };
  std::vector<double> Q(static_cast<size_t>(n) * n, 0.0);
  auto q = [&](int i, int j) -> double& { return Q[static_cast<size_t>(i) * n + j]; };
  for (int i = 0; i < n; ++i) q(i, i) = 1.0;

  // Householder: A <- H_k A H_k zeroes column k below the subdiagonal; Q <- Q H_k
  std::vector<double> v(n), p(n), wv(n);
  for (int k = 0; k + 2 < n; ++k) {
    const int m = n - k - 1;  // trailing size
    double xn = 0.0;
    for (int i = 0; i < m; ++i) xn += at(k + 1 + i, k) * at(k + 1 + i, k);
    xn = std::sqrt(xn);
    if (xn == 0.0) continue;
    const double x0 = at(k + 1, k);
    const double alpha = x0 > 0.0 ? -xn : xn;
    for (int i = 0; i < m; ++i) v[i] = at(k + 1 + i, k);
    v[0] -= alpha;
    double vn2 = 0.0;
    for (int i = 0; i < m; ++i) vn2 += v[i] * v[i];
    if (vn2 == 0.0) continue;
    const double beta = 2.0 / vn2;
    at(k + 1, k) = at(k, k + 1) = alpha;
    for (int i = 1; i < m; ++i) at(k + 1 + i, k) = at(k, k + 1 + i) = 0.0;
    // trailing block B <- H B H = B - v w^T - w v^T, w = p - (beta/2)(p.v) v, p = beta B v
    for (int i = 0; i < m; ++i) {
      double s = 0.0;
      const double* row = &at(k + 1 + i, k + 1);
      for (int j = 0; j < m; ++j) s += row[j] * v[j];
      p[i] = beta * s;
    }
    double pv = 0.0;
    for (int i = 0; i < m; ++i) pv += p[i] * v[i];
    const double kk = 0.5 * beta * pv;
    for (int i = 0; i < m; ++i) wv[i] = p[i] - kk * v[i];
    for (int i = 0; i < m; ++i) {
      double* row = &at(k + 1 + i, k + 1);
      for (int j = 0; j < m; ++j) row[j] -= v[i] * wv[j] + wv[i] * v[j];
    }
    // Q[:, k+1:] -= beta (Q[:, k+1:] v) v^T
    for (int r = 0; r < n; ++r) {
      double* row = &q(r, k + 1);
      double s = 0.0;
      for (int j = 0; j < m; ++j) s += row[j] * v[j];
      s *= beta;
      for (int j = 0; j < m; ++j) row[j] -= s * v[j];
    }
  }
  std::vector<double> d(n), e(n > 1 ? n - 1 : 1, 0.0);
  for (int i = 0; i < n; ++i) d[i] = at(i, i);
  for (int i = 0; i + 1 < n; ++i) e[i] = at(i + 1, i);

  // implicit symmetric QR on the tridiagonal (d, e), rotations accumulated in Q
  const double eps = 2.220446049250313e-16;
  auto negligible = [&](int i) { return std::fabs(e[i]) <= eps * (std::fabs(d[i]) + std::fabs(d[i + 1])); };
  int hi = n - 1;
  long steps = 0;
  while (hi > 0) {
    if (negligible(hi - 1)) {
      e[hi - 1] = 0.0;
      --hi;
      continue;
    }
    int lo = hi - 1;
    while (lo > 0 && !negligible(lo - 1)) --lo;
    if (lo > 0) e[lo - 1] = 0.0;
    if (++steps > 60L * n) throw std::runtime_error("eigh: QR iteration did not converge");
    // Wilkinson shift of the trailing 2 x 2
    const double dl = 0.5 * (d[hi - 1] - d[hi]);
    const double eh = e[hi - 1];
    const double sg = dl >= 0.0 ? 1.0 : -1.0;
    const double mu = d[hi] - eh * eh / (dl + sg * std::hypot(dl, eh));
    double x = d[lo] - mu, z = e[lo];
    for (int k = lo; k < hi; ++k) {
      const double r = std::hypot(x, z);
      const double c = r == 0.0 ? 1.0 : x / r, s = r == 0.0 ? 0.0 : z / r;
      // rows/columns k, k+1 of T rotated by R = [c s; -s c]: T <- R T R^T
      if (k > lo) e[k - 1] = r;  // the bulge of the previous step is absorbed
      const double a = d[k], b = e[k], dd = d[k + 1];
      d[k] = c * c * a + 2.0 * c * s * b + s * s * dd;
      d[k + 1] = s * s * a - 2.0 * c * s * b + c * c * dd;
      e[k] = (c * c - s * s) * b + c * s * (dd - a);
      double bulge = 0.0;
      if (k + 1 < hi) {
        bulge = s * e[k + 1];
        e[k + 1] *= c;
      }
      for (int i = 0; i < n; ++i) {
        const double qk = q(i, k), qk1 = q(i, k + 1);
        q(i, k) = c * qk + s * qk1;
        q(i, k + 1) = -s * qk + c * qk1;
      }
      x = e[k];
      z = bulge;
    }
  }
  std::vector<int> order(n);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return d[a] < d[b]; });
  w.resize(n);
  V.assign(static_cast<size_t>(n) * n, 0.0);
  for (int j = 0; j < n; ++j) {
    w[j] = d[order[j]];
    for (int i = 0; i < n; ++i) V[static_cast<size_t>(i) * n + j] = q(i, order[j]);
  }
}

bool solve(int n, std::vector<double> A, std::vector<double> b, std::vector<double>& x) {
  double amax = 0.0;
  for (double a : A) amax = std::max(amax, std::fabs(a));
  if (!(amax > 0.0)) return false;
  for (int k = 0; k < n; ++k) {
    int piv = k;
    for (int i = k + 1; i < n; ++i)
      if (std::fabs(A[static_cast<size_t>(i) * n + k]) > std::fabs(A[static_cast<size_t>(piv) * n + k])) piv = i;
    if (std::fabs(A[static_cast<size_t>(piv) * n + k]) <= 1e-300 * amax ||
        A[static_cast<size_t>(piv) * n + k] == 0.0)
      return false;
    if (piv != k) {
      for (int j = 0; j < n; ++j) std::swap(A[static_cast<size_t>(k) * n + j], A[static_cast<size_t>(piv) * n + j]);
      std::swap(b[k], b[piv]);
    }
    for (int i = k + 1; i < n; ++i) {
      const double f = A[static_cast<size_t>(i) * n + k] / A[static_cast<size_t>(k) * n + k];
      if (f == 0.0) continue;
      for (int j = k; j < n; ++j) A[static_cast<size_t>(i) * n + j] -= f * A[static_cast<size_t>(k) * n + j];
      b[i] -= f * b[k];
    }
  }
  x.assign(n, 0.0);
  for (int i = n - 1; i >= 0; --i) {
    double s = b[i];
    for (int j = i + 1; j < n; ++j) s -= A[static_cast<size_t>(i) * n + j] * x[j];
    x[i] = s / A[static_cast<size_t>(i) * n + i];
  }
  return true;
}

}  // namespace hostla
}  // namespace gbcc
