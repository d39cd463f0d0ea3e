// mom_host.h -- the host algebra of the Robbins-Monro Method-of-Moments fit
// (R/mom.R:15-22, :173-197): inverse and pseudo-inverse, the score-function
// derivative summed over periods, the diagonalised inverse and the guarded
// step. Plain C++ (no CUDA): cusna_mom_estimate (mom_estimator.cu) uses it,
// and the CPU tests compile it alone against the Python estimator's values.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <vector>

namespace cusna {

typedef std::vector<double> Mat;  // row-major p x p

// Inverse by Gauss-Jordan elimination with partial pivoting; false when a
// pivot vanishes (R's solve() fails there).
inline bool mom_invert(const Mat &A, int p, Mat &out) {
  Mat a = A;
  out.assign((size_t)p * p, 0.0);
  for (int i = 0; i < p; ++i) out[(size_t)i * p + i] = 1.0;
  double scale = 0.0;
  for (double x : a) scale = std::max(scale, std::fabs(x));
  if (!(scale > 0.0)) return false;
  for (int c = 0; c < p; ++c) {
    int piv = c;
    for (int r = c + 1; r < p; ++r)
      if (std::fabs(a[(size_t)r * p + c]) > std::fabs(a[(size_t)piv * p + c])) piv = r;
    const double pv = a[(size_t)piv * p + c];
    if (!(std::fabs(pv) > 1e-14 * scale)) return false;
    if (piv != c)
      for (int q = 0; q < p; ++q) {
        std::swap(a[(size_t)piv * p + q], a[(size_t)c * p + q]);
        std::swap(out[(size_t)piv * p + q], out[(size_t)c * p + q]);
      }
    for (int q = 0; q < p; ++q) {
      a[(size_t)c * p + q] /= pv;
      out[(size_t)c * p + q] /= pv;
    }
    for (int r = 0; r < p; ++r) {
      if (r == c) continue;
      const double f = a[(size_t)r * p + c];
      if (f == 0.0) continue;
      for (int q = 0; q < p; ++q) {
        a[(size_t)r * p + q] -= f * a[(size_t)c * p + q];
        out[(size_t)r * p + q] -= f * out[(size_t)c * p + q];
      }
    }
  }
  return true;
}

// Moore-Penrose pseudo-inverse (R/mom.R:15-19: singular values below
// sqrt(eps) times the largest dropped) by one-sided Jacobi SVD.
inline Mat mom_pinv(const Mat &A, int p) {
  Mat U = A, V((size_t)p * p, 0.0);
  for (int i = 0; i < p; ++i) V[(size_t)i * p + i] = 1.0;
  for (int sweep = 0; sweep < 60; ++sweep) {
    double off = 0.0;
    for (int i = 0; i < p - 1; ++i)
      for (int j = i + 1; j < p; ++j) {
        double a = 0, b = 0, g = 0;
        for (int r = 0; r < p; ++r) {
          const double ui = U[(size_t)r * p + i], uj = U[(size_t)r * p + j];
          a += ui * ui;
          b += uj * uj;
          g += ui * uj;
        }
        if (std::fabs(g) <= 1e-300) continue;
        off = std::max(off, std::fabs(g) / std::sqrt(a * b + 1e-300));
        const double zeta = (b - a) / (2.0 * g);
        const double t = (zeta >= 0 ? 1.0 : -1.0) / (std::fabs(zeta) + std::sqrt(1.0 + zeta * zeta));
        const double c = 1.0 / std::sqrt(1.0 + t * t), s = c * t;
        for (int r = 0; r < p; ++r) {
          const double ui = U[(size_t)r * p + i], uj = U[(size_t)r * p + j];
          U[(size_t)r * p + i] = c * ui - s * uj;
          U[(size_t)r * p + j] = s * ui + c * uj;
          const double vi = V[(size_t)r * p + i], vj = V[(size_t)r * p + j];
          V[(size_t)r * p + i] = c * vi - s * vj;
          V[(size_t)r * p + j] = s * vi + c * vj;
        }
      }
    if (off < 1e-15) break;
  }
  std::vector<double> sv(p);
  double smax = 0.0;
  for (int j = 0; j < p; ++j) {
    double s2 = 0;
    for (int r = 0; r < p; ++r) s2 += U[(size_t)r * p + j] * U[(size_t)r * p + j];
    sv[j] = std::sqrt(s2);
    smax = std::max(smax, sv[j]);
  }
  const double tol = std::sqrt(2.220446049250313e-16) * smax;
  Mat out((size_t)p * p, 0.0);
  for (int j = 0; j < p; ++j) {
    if (!(sv[j] > tol)) continue;
    for (int r = 0; r < p; ++r)
      for (int c = 0; c < p; ++c)
        out[(size_t)r * p + c] += V[(size_t)r * p + j] * U[(size_t)c * p + j] / (sv[j] * sv[j]);
  }
  return out;
}

// R/mom.R:20-22 (.safe_solve): the inverse, or the pseudo-inverse when solve() fails
inline Mat mom_safe_solve(const Mat &A, int p) {
  Mat inv;
  if (mom_invert(A, p, inv)) return inv;
  return mom_pinv(A, p);
}

inline std::vector<double> mom_matvec(const Mat &A, const std::vector<double> &x, int p) {
  std::vector<double> y(p, 0.0);
  for (int r = 0; r < p; ++r)
    for (int c = 0; c < p; ++c) y[r] += A[(size_t)r * p + c] * x[c];
  return y;
}

// column means of an M x p row-major block
inline std::vector<double> mom_col_means(const std::vector<double> &X, int M, int p) {
  std::vector<double> mu(p, 0.0);
  for (int c = 0; c < M; ++c)
    for (int j = 0; j < p; ++j) mu[j] += X[(size_t)c * p + j];
  for (int j = 0; j < p; ++j) mu[j] /= M;
  return mu;
}

// Score-function derivative summed over periods (R/mom.R:173-182): per period
// q the cross-covariance of the statistics sp[q] and the scores scp[q] (M x p
// each), divided by M.
inline Mat mom_derivative(const std::vector<std::vector<double>> &sp,
                          const std::vector<std::vector<double>> &scp, int M, int p) {
  Mat D((size_t)p * p, 0.0);
  for (size_t q = 0; q < sp.size(); ++q) {
    const std::vector<double> ms = mom_col_means(sp[q], M, p), mc = mom_col_means(scp[q], M, p);
    for (int c = 0; c < M; ++c)
      for (int a = 0; a < p; ++a) {
        const double x = sp[q][(size_t)c * p + a] - ms[a];
        if (x == 0.0) continue;
        for (int b = 0; b < p; ++b) D[(size_t)a * p + b] += x * (scp[q][(size_t)c * p + b] - mc[b]);
      }
  }
  for (double &x : D) x /= M;
  return D;
}

// The diagonalised inverse (R/mom.R:184-187): off-diagonal entries scaled by
// 1 - w, then inverted.
inline Mat mom_dinv(const Mat &D, int p, double w) {
  Mat A = D;
  for (int a = 0; a < p; ++a)
    for (int b = 0; b < p; ++b) A[(size_t)a * p + b] *= (a == b) ? 1.0 : (1.0 - w);
  return mom_safe_solve(A, p);
}

// Step cap and rate floor (R/mom.R:189-197): every step within max(1,
// |theta|/2), and a rate (the first n_rates entries) never stepped below a
// tenth of its value (then halved instead).
inline std::vector<double> mom_guard_step(const std::vector<double> &theta, std::vector<double> step,
                                          int n_rates) {
  for (size_t j = 0; j < step.size(); ++j) {
    const double cap = std::max(1.0, 0.5 * std::fabs(theta[j]));
    step[j] = std::min(std::max(step[j], -cap), cap);
  }
  for (int j = 0; j < n_rates; ++j)
    if (theta[j] - step[j] < 0.1 * theta[j]) step[j] = 0.5 * theta[j];
  return step;
}

}  // namespace cusna
