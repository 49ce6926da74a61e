// The Anderson mixer's small least-squares solve, gamma = argmin |A gamma - b|
// for the symmetric positive semi-definite m x m Gram matrix A (m <= 16):
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

// The solve for a compile-time order M: every loop bound a constant, so the
// matrices stay in registers on the device.
template <int M>
SL3D_HD inline bool SymmetricLstsqOf(const double* A /* M x M, row-major */, const double* b, double* x) {
  double a[M][M], v[M][M];
#pragma unroll
  for (int i = 0; i < M; ++i)
#pragma unroll
    for (int j = 0; j < M; ++j) {
      a[i][j] = 0.5 * (A[i * M + j] + A[j * M + i]);
      v[i][j] = i == j ? 1.0 : 0.0;
    }
  for (int sweep = 0; sweep < 60; ++sweep) {
    double off = 0.0, diag = 0.0;
#pragma unroll
    for (int i = 0; i < M; ++i)
#pragma unroll
      for (int j = 0; j < M; ++j) (i == j ? diag : off) += a[i][j] * a[i][j];
    if (off <= 1e-32 * diag || off == 0.0) break;
#pragma unroll
    for (int p = 0; p < M; ++p)
#pragma unroll
      for (int q = p + 1; q < M; ++q) {
        if (a[p][q] == 0.0) continue;
        const double theta = (a[q][q] - a[p][p]) / (2.0 * a[p][q]);
        const double t = (theta >= 0.0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
#pragma unroll
        for (int k = 0; k < M; ++k) {
          const double akp = a[k][p], akq = a[k][q];
          a[k][p] = c * akp - s * akq;
          a[k][q] = s * akp + c * akq;
        }
#pragma unroll
        for (int k = 0; k < M; ++k) {
          const double apk = a[p][k], aqk = a[q][k];
          a[p][k] = c * apk - s * aqk;
          a[q][k] = s * apk + c * aqk;
        }
#pragma unroll
        for (int k = 0; k < M; ++k) {
          const double vkp = v[k][p], vkq = v[k][q];
          v[k][p] = c * vkp - s * vkq;
          v[k][q] = s * vkp + c * vkq;
        }
      }
  }
  double largest = 0.0;
#pragma unroll
  for (int i = 0; i < M; ++i) largest = fmax(largest, fabs(a[i][i]));
  const double cut = 2.220446049250313e-16 * largest;
  double y[M];
#pragma unroll
  for (int i = 0; i < M; ++i) y[i] = 0.0;
#pragma unroll
  for (int k = 0; k < M; ++k) {
    const double lambda = a[k][k];
    if (!(fabs(lambda) > cut)) continue;
    double proj = 0.0;
#pragma unroll
    for (int i = 0; i < M; ++i) proj += v[i][k] * b[i];
#pragma unroll
    for (int i = 0; i < M; ++i) y[i] += v[i][k] * proj / lambda;
  }
  bool finite = true;
#pragma unroll
  for (int i = 0; i < M; ++i) {
    x[i] = y[i];
    if (!(y[i] - y[i] == 0.0)) finite = false;  // NaN or infinite
  }
  return finite;
}

SL3D_HD inline bool SymmetricLstsq(int m, const double* A /* m x m, row-major */, const double* b,
                                   double* x) {
  switch (m) {
    case 0: return true;
    case 1: return SymmetricLstsqOf<1>(A, b, x);
    case 2: return SymmetricLstsqOf<2>(A, b, x);
    case 3: return SymmetricLstsqOf<3>(A, b, x);
    case 4: return SymmetricLstsqOf<4>(A, b, x);
    case 5: return SymmetricLstsqOf<5>(A, b, x);
    case 6: return SymmetricLstsqOf<6>(A, b, x);
    case 7: return SymmetricLstsqOf<7>(A, b, x);
    case 8: return SymmetricLstsqOf<8>(A, b, x);
    case 9: return SymmetricLstsqOf<9>(A, b, x);
    case 10: return SymmetricLstsqOf<10>(A, b, x);
    case 11: return SymmetricLstsqOf<11>(A, b, x);
    case 12: return SymmetricLstsqOf<12>(A, b, x);
    case 13: return SymmetricLstsqOf<13>(A, b, x);
    case 14: return SymmetricLstsqOf<14>(A, b, x);
    case 15: return SymmetricLstsqOf<15>(A, b, x);
    case 16: return SymmetricLstsqOf<16>(A, b, x);
    default: return false;
  }
}

}  // namespace sl3dgpu
