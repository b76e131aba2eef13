// hosteig.h -- small dense eigensolvers for the Ritz problems (host, FP64).
//
// The reference calls LAPACK dstevx (eigen_solver.f90:128, lanczos.f90:104)
// and zheevr (eigen_solver.f90:205) on NOM x NOM matrices.  The library needs
// no LAPACK: Ritz matrices are solved with a cyclic complex Jacobi method
// (Hermitian; high relative accuracy, ascending order) and, for the long
// tridiagonals of plain Lanczos, Sturm-sequence bisection for the lowest
// eigenvalue plus inverse iteration for its vector.
#pragma once

#include <algorithm>
#include <cmath>
#include <complex>
#include <vector>

namespace qs3g {

using zd = std::complex<double>;

// Eigen-decomposition of the Hermitian n x n matrix A (column-major, full
// storage; only the upper triangle is read).  On return w holds ascending
// eigenvalues and Z (column-major) the orthonormal eigenvectors.
inline int herm_jacobi(int n, const std::vector<zd>& Ain, std::vector<double>& w, std::vector<zd>& Z) {
  std::vector<zd> A(Ain);
  for (int j = 0; j < n; ++j)
    for (int i = j + 1; i < n; ++i) A[i + (size_t)j * n] = std::conj(A[j + (size_t)i * n]);
  for (int i = 0; i < n; ++i) A[i + (size_t)i * n] = zd(A[i + (size_t)i * n].real(), 0.0);
  Z.assign((size_t)n * n, zd(0.0, 0.0));
  for (int i = 0; i < n; ++i) Z[i + (size_t)i * n] = 1.0;
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0, tot = 0.0;
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        const double a2 = std::norm(A[i + (size_t)j * n]);
        tot += a2;
        if (i != j) off += a2;
      }
    if (off <= 1e-34 * tot || off == 0.0) break;
    for (int p = 0; p < n - 1; ++p)
      for (int q = p + 1; q < n; ++q) {
        const zd apq = A[p + (size_t)q * n];
        const double aa = std::abs(apq);
        if (aa == 0.0) continue;
        const double app = A[p + (size_t)p * n].real(), aqq = A[q + (size_t)q * n].real();
        const zd u = apq / aa;
        const double tau = (aqq - app) / (2.0 * aa);
        const double t = (tau >= 0 ? 1.0 : -1.0) / (std::fabs(tau) + std::sqrt(1.0 + tau * tau));
        const double c = 1.0 / std::sqrt(1.0 + t * t), s = t * c;
        // J = [[c, s], [-s conj(u), c conj(u)]] on (p, q); A <- J^H A J, Z <- Z J
        const zd jqp = -s * std::conj(u), jqq = c * std::conj(u);
        for (int k = 0; k < n; ++k) {  // columns
          const zd akp = A[k + (size_t)p * n], akq = A[k + (size_t)q * n];
          A[k + (size_t)p * n] = c * akp + jqp * akq;
          A[k + (size_t)q * n] = s * akp + jqq * akq;
        }
        for (int k = 0; k < n; ++k) {  // rows
          const zd apk = A[p + (size_t)k * n], aqk = A[q + (size_t)k * n];
          A[p + (size_t)k * n] = c * apk + std::conj(jqp) * aqk;
          A[q + (size_t)k * n] = s * apk + std::conj(jqq) * aqk;
        }
        A[p + (size_t)q * n] = 0.0;
        A[q + (size_t)p * n] = 0.0;
        A[p + (size_t)p * n] = zd(A[p + (size_t)p * n].real(), 0.0);
        A[q + (size_t)q * n] = zd(A[q + (size_t)q * n].real(), 0.0);
        for (int k = 0; k < n; ++k) {
          const zd zkp = Z[k + (size_t)p * n], zkq = Z[k + (size_t)q * n];
          Z[k + (size_t)p * n] = c * zkp + jqp * zkq;
          Z[k + (size_t)q * n] = s * zkp + jqq * zkq;
        }
      }
  }
  std::vector<int> idx(n);
  for (int i = 0; i < n; ++i) idx[i] = i;
  std::vector<double> d(n);
  for (int i = 0; i < n; ++i) d[i] = A[i + (size_t)i * n].real();
  std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return d[a] < d[b]; });
  w.resize(n);
  std::vector<zd> Zs((size_t)n * n);
  for (int j = 0; j < n; ++j) {
    w[j] = d[idx[j]];
    for (int i = 0; i < n; ++i) Zs[i + (size_t)j * n] = Z[i + (size_t)idx[j] * n];
  }
  Z.swap(Zs);
  return 0;
}

// Number of eigenvalues of the symmetric tridiagonal (d, e) below x (Sturm count).
inline int sturm_count(const std::vector<double>& d, const std::vector<double>& e, double x) {
  int cnt = 0;
  double q = 1.0;
  const int n = (int)d.size();
  for (int i = 0; i < n; ++i) {
    const double e2 = (i > 0) ? e[i - 1] * e[i - 1] : 0.0;
    q = d[i] - x - ((i > 0) ? e2 / q : 0.0);
    if (q == 0.0) q = -1e-300;
    if (q < 0) ++cnt;
  }
  return cnt;
}

// Lowest eigenpair of the symmetric tridiagonal matrix (diag d[0..n-1], off e[0..n-2]).
inline int tridiag_lowest(const std::vector<double>& d, const std::vector<double>& e, double& lam,
                          std::vector<double>& z) {
  const int n = (int)d.size();
  double lo = d[0], hi = d[0];
  for (int i = 0; i < n; ++i) {
    const double r = ((i > 0) ? std::fabs(e[i - 1]) : 0.0) + ((i < n - 1) ? std::fabs(e[i]) : 0.0);
    lo = std::min(lo, d[i] - r);
    hi = std::max(hi, d[i] + r);
  }
  for (int it = 0; it < 200; ++it) {
    const double mid = 0.5 * (lo + hi);
    if (mid <= lo || mid >= hi) break;
    if (sturm_count(d, e, mid) >= 1) hi = mid; else lo = mid;
  }
  lam = 0.5 * (lo + hi);
  // inverse iteration with partial pivoting (tridiagonal LU)
  z.assign(n, 1.0);
  const double shift = lam - 1e-14 * std::max(1.0, std::fabs(lam));
  for (int it = 0; it < 4; ++it) {
    // solve (T - shift I) y = z by Gaussian elimination with pivoting on a banded copy
    std::vector<double> a(n, 0.0), b(n), c(n, 0.0), c2(n, 0.0), r(z);
    for (int i = 0; i < n; ++i) b[i] = d[i] - shift;
    for (int i = 0; i < n - 1; ++i) { c[i] = e[i]; a[i + 1] = e[i]; }
    // rows: a[i] (sub), b[i] (diag), c[i] (super), c2[i] (second super after pivoting)
    for (int i = 0; i < n - 1; ++i) {
      if (std::fabs(a[i + 1]) > std::fabs(b[i])) {
        std::swap(b[i], a[i + 1]);
        std::swap(c[i], b[i + 1]);
        std::swap(c2[i], c[i + 1]);
        std::swap(r[i], r[i + 1]);
      }
      if (b[i] == 0.0) b[i] = 1e-300;
      const double f = a[i + 1] / b[i];
      b[i + 1] -= f * c[i];
      c[i + 1] -= f * c2[i];
      r[i + 1] -= f * r[i];
    }
    if (b[n - 1] == 0.0) b[n - 1] = 1e-300;
    std::vector<double> y(n);
    for (int i = n - 1; i >= 0; --i) {
      double s = r[i];
      if (i + 1 < n) s -= c[i] * y[i + 1];
      if (i + 2 < n) s -= c2[i] * y[i + 2];
      y[i] = s / b[i];
    }
    double nrm = 0.0;
    for (double v : y) nrm += v * v;
    nrm = std::sqrt(nrm);
    for (int i = 0; i < n; ++i) z[i] = y[i] / nrm;
  }
  // sign convention: largest component positive
  int im = 0;
  for (int i = 1; i < n; ++i)
    if (std::fabs(z[i]) > std::fabs(z[im])) im = i;
  if (z[im] < 0)
    for (double& v : z) v = -v;
  return 0;
}

}  // namespace qs3g
