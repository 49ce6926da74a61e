// The oracle's small least-squares solve (test infrastructure only):
// x = argmin |A x - b| for an m x m matrix A (the Anderson mixer's Gram
// matrix), minimum norm, through the singular value decomposition with
// singular values at or below machine epsilon times the largest dropped --
// what LAPACK's dgelss gives with rcond < 0, the reference's call
// (include/sl3dpp/detail/AndersonMixer.hpp:186-205). The SVD is one-sided
// Jacobi (Hestenes): plane rotations orthogonalise A's columns, A V = U S.
// Returns false on a non-finite result (the mixer then takes the Picard
// step, as the reference does on info != 0).
#pragma once

#include <cmath>
#include <limits>
#include <vector>

namespace orc {

inline bool SvdLstsq(int m, const double* A /* m x m, row-major */, const double* b, double* x) {
  std::vector<double> u(A, A + static_cast<std::size_t>(m) * m);  // columns become U S
  std::vector<double> v(static_cast<std::size_t>(m) * m, 0.0);
  for (int i = 0; i < m; ++i) v[static_cast<std::size_t>(i) * m + i] = 1.0;
  auto at = [m](std::vector<double>& a, int r, int c) -> double& { return a[static_cast<std::size_t>(r) * m + c]; };
  for (int sweep = 0; sweep < 80; ++sweep) {
    bool rotated = false;
    for (int p = 0; p < m - 1; ++p)
      for (int q = p + 1; q < m; ++q) {
        double alpha = 0.0, beta = 0.0, gamma = 0.0;
        for (int r = 0; r < m; ++r) {
          alpha += at(u, r, p) * at(u, r, p);
          beta += at(u, r, q) * at(u, r, q);
          gamma += at(u, r, p) * at(u, r, q);
        }
        if (gamma == 0.0 || std::abs(gamma) <= 1e-15 * std::sqrt(alpha * beta)) continue;
        rotated = true;
        const double zeta = (beta - alpha) / (2.0 * gamma);
        const double t = (zeta >= 0.0 ? 1.0 : -1.0) / (std::abs(zeta) + std::sqrt(1.0 + zeta * zeta));
        const double c = 1.0 / std::sqrt(1.0 + t * t), s = c * t;
        for (int r = 0; r < m; ++r) {
          const double up = at(u, r, p), uq = at(u, r, q);
          at(u, r, p) = c * up - s * uq;
          at(u, r, q) = s * up + c * uq;
          const double vp = at(v, r, p), vq = at(v, r, q);
          at(v, r, p) = c * vp - s * vq;
          at(v, r, q) = s * vp + c * vq;
        }
      }
    if (!rotated) break;
  }
  std::vector<double> sigma(m, 0.0);
  double largest = 0.0;
  for (int c = 0; c < m; ++c) {
    double n2 = 0.0;
    for (int r = 0; r < m; ++r) n2 += at(u, r, c) * at(u, r, c);
    sigma[c] = std::sqrt(n2);
    largest = std::max(largest, sigma[c]);
  }
  const double cut = std::numeric_limits<double>::epsilon() * largest;
  for (int i = 0; i < m; ++i) x[i] = 0.0;
  for (int c = 0; c < m; ++c) {
    if (!(sigma[c] > cut)) continue;
    // (u_c . b) / sigma_c^2 along v_c: u_c holds sigma_c times the unit vector
    double proj = 0.0;
    for (int r = 0; r < m; ++r) proj += at(u, r, c) * b[r];
    const double coef = proj / (sigma[c] * sigma[c]);
    for (int i = 0; i < m; ++i) x[i] += coef * at(v, i, c);
  }
  for (int i = 0; i < m; ++i)
    if (!std::isfinite(x[i])) return false;
  return true;
}

}  // namespace orc
