// The Anderson mixer's small least-squares solve, gamma = argmin |A gamma - b|
// for the symmetric positive semi-definite m x m Gram matrix A (m <= 8):
// cyclic Jacobi eigen-decomposition, directions whose |eigenvalue| is at or
// below machine epsilon times the largest dropped -- the minimum-norm
// solution LAPACK's dgelss gives with rcond < 0 (the reference's call,
// include/sl3dpp/detail/AndersonMixer.hpp:186-205), for a symmetric matrix
// whose singular values are its eigenvalues' magnitudes. Returns false when
// the decomposition produced a non-finite value (the caller then takes the
// Picard step, as the reference does on info != 0).
#pragma once

#include <cmath>

#ifdef __CUDACC__
#define SL3D_HD __host__ __device__
#else
#define SL3D_HD
#endif

namespace sl3dgpu {

SL3D_HD inline bool SymmetricLstsq(int m, const double* A /* m x m, row-major */, const double* b,
                                   double* x) {
  constexpr int kMax = 8;
  double a[kMax][kMax], v[kMax][kMax];
  for (int i = 0; i < m; ++i)
    for (int j = 0; j < m; ++j) {
      a[i][j] = 0.5 * (A[i * m + j] + A[j * m + i]);
      v[i][j] = i == j ? 1.0 : 0.0;
    }
  for (int sweep = 0; sweep < 60; ++sweep) {
    double off = 0.0, diag = 0.0;
    for (int i = 0; i < m; ++i)
      for (int j = 0; j < m; ++j) (i == j ? diag : off) += a[i][j] * a[i][j];
    if (off <= 1e-32 * diag || off == 0.0) break;
    for (int p = 0; p < m; ++p)
      for (int q = p + 1; q < m; ++q) {
        if (a[p][q] == 0.0) continue;
        const double theta = (a[q][q] - a[p][p]) / (2.0 * a[p][q]);
        const double t = (theta >= 0.0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < m; ++k) {
          const double akp = a[k][p], akq = a[k][q];
          a[k][p] = c * akp - s * akq;
          a[k][q] = s * akp + c * akq;
        }
        for (int k = 0; k < m; ++k) {
          const double apk = a[p][k], aqk = a[q][k];
          a[p][k] = c * apk - s * aqk;
          a[q][k] = s * apk + c * aqk;
        }
        for (int k = 0; k < m; ++k) {
          const double vkp = v[k][p], vkq = v[k][q];
          v[k][p] = c * vkp - s * vkq;
          v[k][q] = s * vkp + c * vkq;
        }
      }
  }
  double largest = 0.0;
  for (int i = 0; i < m; ++i) largest = fmax(largest, fabs(a[i][i]));
  const double cut = 2.220446049250313e-16 * largest;
  for (int i = 0; i < m; ++i) x[i] = 0.0;
  for (int k = 0; k < m; ++k) {
    const double lambda = a[k][k];
    if (!(fabs(lambda) > cut)) continue;
    double proj = 0.0;
    for (int i = 0; i < m; ++i) proj += v[i][k] * b[i];
    for (int i = 0; i < m; ++i) x[i] += v[i][k] * proj / lambda;
  }
  for (int i = 0; i < m; ++i)
    if (!(x[i] - x[i] == 0.0)) return false;  // NaN or infinite
  return true;
}

}  // namespace sl3dgpu
