// ORACLE — test infrastructure only.
//
// A CPU FP64 restatement of sl3dpp's hot-path arithmetic, used solely as the
// checker by tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg.
// Nothing in the product library (sl3dpp_gb300/) links, imports or calls it.
//
// This file: the banded factorisations and solves, the Gauss-Legendre rule,
// the Wigner-d table and the spin-weighted spherical-harmonic transforms.
//
// Parity anchors:
//  - band solvers restate src/BandSolvers.cpp:23-139 (LAPACK's unblocked
//    dpbtf2/dpbtrs and dgbtf2/dgbtrs, same storage and pivots); pinned in the
//    tests against LAPACK itself through scipy.linalg.lapack, as
//    tests/TestBandSolvers.cpp:87-176 pins the reference;
//  - the transforms restate the basis of docs/design.md:245-250 and the
//    index layouts of include/sl3dpp/SurfaceGrid.hpp:110-118, 191-200
//    (GSHTrans itself, pinned at c71313c5, is not in the reference tree):
//    Y^N_lm = sqrt((2l+1)/4pi) d^l_{Nm}(theta) e^{i m phi} with
//    d^l_{0m} the Condon-Shortley associated Legendre function, forward
//    transform the integral of conj(Y) f. Pinned in the tests against
//    closed forms (scipy's CS spherical harmonics, exact-rational Wigner d)
//    and the reference's own properties (round trip 1e-12, reality
//    relations; tests/TestSpinMachinery.cpp:33-165).

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstddef>
#include <cstdint>
#include <vector>

#include "oracle.h"

namespace {

inline double& BandAt(double* ab, std::size_t ld, int diagonal, int i, int j) {
  return ab[static_cast<std::size_t>(j) * ld + static_cast<std::size_t>(diagonal + i - j)];
}

}  // namespace

extern "C" {

// -- band solvers (src/BandSolvers.cpp:23-139) -------------------------------

int oracle_band_cholesky_factor(double* ab, int n, int kd) {
  const auto ld = static_cast<std::size_t>(kd) + 1;
  std::vector<double> row(ld);
  for (int j = 0; j < n; ++j) {
    const double d = BandAt(ab, ld, kd, j, j);
    if (!(d > 0.0)) return j + 1;
    const double ujj = std::sqrt(d);
    BandAt(ab, ld, kd, j, j) = ujj;
    const int kn = std::min(kd, n - 1 - j);
    const double inverse = 1.0 / ujj;
    for (int c = 1; c <= kn; ++c) row[c] = (BandAt(ab, ld, kd, j, j + c) *= inverse);
    for (int c = 1; c <= kn; ++c) {
      double* column = &BandAt(ab, ld, kd, j, j + c);
      const double uc = row[c];
      for (int r = 1; r <= c; ++r) column[r] -= row[r] * uc;
    }
  }
  return 0;
}

void oracle_band_cholesky_solve(const double* ab, int n, int kd, double* b, int nrhs) {
  const auto ld = static_cast<std::size_t>(kd) + 1;
  auto at = [&](int i, int j) { return ab[static_cast<std::size_t>(j) * ld + kd + i - j]; };
  for (int k = 0; k < nrhs; ++k) {
    double* x = b + static_cast<std::size_t>(k) * n;
    for (int j = 0; j < n; ++j) {
      double sum = x[j];
      for (int i = std::max(0, j - kd); i < j; ++i) sum -= at(i, j) * x[i];
      x[j] = sum / at(j, j);
    }
    for (int j = n - 1; j >= 0; --j) {
      x[j] /= at(j, j);
      const double xj = x[j];
      for (int i = std::max(0, j - kd); i < j; ++i) x[i] -= at(i, j) * xj;
    }
  }
}

int oracle_band_lu_factor(double* ab, int n, int kl, int ku, int* pivots) {
  const int kv = kl + ku;
  const auto ld = static_cast<std::size_t>(2 * kl + ku + 1);
  auto at = [&](int i, int j) -> double& { return BandAt(ab, ld, kv, i, j); };
  for (int j = ku + 1; j < std::min(kv, n); ++j)
    for (int i = 0; i < j - ku; ++i) at(i, j) = 0.0;
  int info = 0, ju = 0;
  for (int j = 0; j < n; ++j) {
    if (j + kv < n)
      for (int i = j; i < j + kl; ++i) at(i, j + kv) = 0.0;
    const int km = std::min(kl, n - 1 - j);
    int p = j;
    for (int i = j + 1; i <= j + km; ++i)
      if (std::abs(at(i, j)) > std::abs(at(p, j))) p = i;
    pivots[j] = p;
    if (at(p, j) == 0.0) {
      if (info == 0) info = j + 1;
      continue;
    }
    ju = std::max(ju, std::min(p + ku, n - 1));
    if (p != j)
      for (int c = j; c <= ju; ++c) std::swap(at(p, c), at(j, c));
    if (km > 0) {
      const double inverse = 1.0 / at(j, j);
      for (int i = j + 1; i <= j + km; ++i) at(i, j) *= inverse;
      for (int c = j + 1; c <= ju; ++c) {
        const double ujc = at(j, c);
        for (int i = j + 1; i <= j + km; ++i) at(i, c) -= at(i, j) * ujc;
      }
    }
  }
  return info;
}

void oracle_band_lu_solve(const double* ab, int n, int kl, int ku, const int* pivots,
                          double* b, int nrhs) {
  const int kv = kl + ku;
  const auto ld = static_cast<std::size_t>(2 * kl + ku + 1);
  auto at = [&](int i, int j) { return ab[static_cast<std::size_t>(j) * ld + kv + i - j]; };
  for (int k = 0; k < nrhs; ++k) {
    double* x = b + static_cast<std::size_t>(k) * n;
    for (int j = 0; j + 1 < n; ++j) {
      if (pivots[j] != j) std::swap(x[pivots[j]], x[j]);
      const double xj = x[j];
      const int lm = std::min(kl, n - 1 - j);
      for (int i = j + 1; i <= j + lm; ++i) x[i] -= at(i, j) * xj;
    }
    for (int j = n - 1; j >= 0; --j) {
      x[j] /= at(j, j);
      const double xj = x[j];
      for (int i = std::max(0, j - kv); i < j; ++i) x[i] -= at(i, j) * xj;
    }
  }
}

// -- Gauss-Legendre rule ------------------------------------------------------

void oracle_gauss_legendre(int n, double* x, double* w) {
  // Newton on P_n from the Tricomi initial guesses; nodes returned as
  // cos(theta) for increasing theta (x decreasing), weights summing to 2.
  const double pi = 3.14159265358979323846;
  for (int i = 0; i < n; ++i) {
    double z = std::cos(pi * (i + 0.75) / (n + 0.5));
    double dp = 0.0;
    for (int it = 0; it < 100; ++it) {
      double p0 = 1.0, p1 = z;
      for (int k = 2; k <= n; ++k) {
        const double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      if (n == 1) { p1 = z; p0 = 1.0; }
      dp = n * (z * p1 - p0) / (z * z - 1.0);
      const double dz = p1 / dp;
      z -= dz;
      if (std::abs(dz) < 1e-16) break;
    }
    double p0 = 1.0, p1 = z;
    for (int k = 2; k <= n; ++k) {
      const double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
      p0 = p1;
      p1 = p2;
    }
    if (n == 1) { p1 = z; p0 = 1.0; }
    dp = n * (z * p1 - p0) / (z * z - 1.0);
    x[i] = z;
    w[i] = 2.0 / ((1.0 - z * z) * dp * dp);
  }
}

// -- Wigner d and the normalised spin-N Legendre table -----------------------

// The closed form of d^l_{Nm}(theta) (= Edmonds d^l_{mN}) at l0 = max(|m|, |N|)
// for N <= 0, from c = cos(theta/2), s = sin(theta/2): for |m| >= |N| the
// product recursion in |m| of sqrt(C(2M, M + N)) times the half-angle powers
// (each factor sqrt((2M+2)(2M+1) / ((M+1+N)(M+1-N))) c s), which neither
// overflows nor loses relative accuracy; for |m| < |N| the direct form.
static double WignerStart(int N, int m, double c, double s) {
  const int M = std::abs(m), A = -N;  // A = |N|
  if (M >= A) {
    double v = 1.0;
    for (int k = 0; k < 2 * A; ++k) v *= (m >= 0 ? s : c);
    for (int k = A; k < M; ++k)
      v *= std::sqrt((2.0 * k + 2.0) * (2.0 * k + 1.0) / ((k + 1.0 + N) * (k + 1.0 - N))) * c * s;
    if (m >= 0 && ((M - N) % 2 != 0)) v = -v;
    return v;
  }
  // l0 = A > M: (-1)^(l+m) sqrt((2l)! / ((l+m)! (l-m)!)) c^(l-m) s^(l+m)
  const int l = A;
  double fact[5] = {1.0, 1.0, 2.0, 6.0, 24.0};
  double v = std::sqrt(fact[2 * l] / (fact[l + m] * fact[l - m]));
  for (int k = 0; k < l - m; ++k) v *= c;
  for (int k = 0; k < l + m; ++k) v *= s;
  if ((l + m) % 2 != 0) v = -v;
  return v;
}

// Lambda^N_{lm}(theta) = sqrt((2l+1)/4pi) d^l_{Nm}(theta), with
// d^l_{Nm}(theta) = (Edmonds) d^l_{mN}(theta), so that d^l_{0m} is the
// Condon-Shortley associated Legendre function: the three-term recurrence in l
// from the closed form at l0 = max(|m|, |N|); for N > 0 through
// d^l_{Nm}(theta) = (-1)^(l+m) d^l_{-N,m}(pi - theta). Written into
// out[(l - l0) * ntheta + j] for l = l0..lmax.
void oracle_wigner_column(int lmax, int N, int m, int ntheta, const double* theta,
                          double* out) {
  const double pi = 3.14159265358979323846;
  const int l0 = std::max(std::abs(m), std::abs(N));
  const bool mirrored = N > 0;
  const int Nr = mirrored ? -N : N;
  for (int j = 0; j < ntheta; ++j) {
    const double t = mirrored ? pi - theta[j] : theta[j];
    const double c = std::cos(0.5 * t), s = std::sin(0.5 * t);
    double dprev = 0.0, d = WignerStart(Nr, m, c, s);
    const double ct = std::cos(t);
    for (int l = l0; l <= lmax; ++l) {
      const double sign = mirrored && ((l + m) % 2 != 0) ? -1.0 : 1.0;
      out[static_cast<std::size_t>(l - l0) * ntheta + j] =
          sign * std::sqrt((2.0 * l + 1.0) / (4.0 * pi)) * d;
      if (l == lmax) break;
      double next;
      if (l == 0) {
        next = ct;  // d^1_00
      } else {
        const double a = (l + 1.0) * (2.0 * l + 1.0) /
                         std::sqrt(((l + 1.0) * (l + 1.0) - 1.0 * m * m) *
                                   ((l + 1.0) * (l + 1.0) - 1.0 * Nr * Nr));
        const double b = 1.0 * m * Nr / (l * (l + 1.0));
        const double e = std::sqrt((1.0 * l * l - 1.0 * m * m) * (1.0 * l * l - 1.0 * Nr * Nr)) /
                         (l * (2.0 * l + 1.0));
        next = a * ((ct - b) * d - e * dprev);
      }
      dprev = d;
      d = next;
    }
  }
}

// -- spin-weighted transforms (SurfaceGrid.hpp layouts) ----------------------

// Synthesis of a complex spin-N field from coefficients at index
// l^2 - N^2 + (m + l) (l = |N|..lmax, all m), onto ntheta x nphi values
// (colatitude-major, longitudes 2 pi k / nphi from zero).
void oracle_synthesise_spin(int lmax, int N, int ntheta, int nphi, const double* theta,
                            const double* coeffs /* complex pairs */, double* field) {
  const double pi = 3.14159265358979323846;
  using C = std::complex<double>;
  const auto* c = reinterpret_cast<const C*>(coeffs);
  auto* f = reinterpret_cast<C*>(field);
  std::vector<C> F(static_cast<std::size_t>(2 * lmax + 1) * ntheta, C{});
  std::vector<double> column(static_cast<std::size_t>(lmax + 1) * ntheta);
  for (int m = -lmax; m <= lmax; ++m) {
    const int l0 = std::max(std::abs(m), std::abs(N));
    if (l0 > lmax) continue;
    oracle_wigner_column(lmax, N, m, ntheta, theta, column.data());
    for (int l = l0; l <= lmax; ++l) {
      const C a = c[static_cast<std::size_t>(l) * l - N * N + (m + l)];
      for (int j = 0; j < ntheta; ++j)
        F[static_cast<std::size_t>(m + lmax) * ntheta + j] += a * column[static_cast<std::size_t>(l - l0) * ntheta + j];
    }
  }
  for (int j = 0; j < ntheta; ++j) {
    for (int k = 0; k < nphi; ++k) {
      C sum{};
      for (int m = -lmax; m <= lmax; ++m) {
        const double ang = 2.0 * pi * static_cast<double>((static_cast<long long>(m) * k) % nphi) / nphi;
        sum += F[static_cast<std::size_t>(m + lmax) * ntheta + j] * C(std::cos(ang), std::sin(ang));
      }
      f[static_cast<std::size_t>(j) * nphi + k] = sum;
    }
  }
}

// Forward transform of a complex spin-N field: c_lm = int conj(Y^N_lm) f dOmega
// by the grid's quadrature (GL weights in cos theta, 2 pi / nphi in phi).
void oracle_expand_spin(int lmax, int N, int ntheta, int nphi, const double* theta,
                        const double* weights, const double* field, double* coeffs) {
  const double pi = 3.14159265358979323846;
  using C = std::complex<double>;
  const auto* f = reinterpret_cast<const C*>(field);
  auto* c = reinterpret_cast<C*>(coeffs);
  std::vector<C> F(static_cast<std::size_t>(2 * lmax + 1) * ntheta, C{});
  for (int j = 0; j < ntheta; ++j) {
    for (int m = -lmax; m <= lmax; ++m) {
      C sum{};
      for (int k = 0; k < nphi; ++k) {
        const double ang = -2.0 * pi * static_cast<double>((static_cast<long long>(m) * k) % nphi) / nphi;
        sum += f[static_cast<std::size_t>(j) * nphi + k] * C(std::cos(ang), std::sin(ang));
      }
      F[static_cast<std::size_t>(m + lmax) * ntheta + j] = sum * (2.0 * pi / nphi) * weights[j];
    }
  }
  const std::size_t size = static_cast<std::size_t>(lmax + 1) * (lmax + 1) - N * N;
  std::fill(c, c + size, C{});
  std::vector<double> column(static_cast<std::size_t>(lmax + 1) * ntheta);
  for (int m = -lmax; m <= lmax; ++m) {
    const int l0 = std::max(std::abs(m), std::abs(N));
    if (l0 > lmax) continue;
    oracle_wigner_column(lmax, N, m, ntheta, theta, column.data());
    for (int l = l0; l <= lmax; ++l) {
      C sum{};
      for (int j = 0; j < ntheta; ++j)
        sum += column[static_cast<std::size_t>(l - l0) * ntheta + j] * F[static_cast<std::size_t>(m + lmax) * ntheta + j];
      c[static_cast<std::size_t>(l) * l - N * N + (m + l)] = sum;
    }
  }
}

// Real spin-0 field from m >= 0 coefficients at l(l+1)/2 + m.
void oracle_synthesise_real(int lmax, int ntheta, int nphi, const double* theta,
                            const double* coeffs, double* field) {
  const double pi = 3.14159265358979323846;
  using C = std::complex<double>;
  const auto* c = reinterpret_cast<const C*>(coeffs);
  std::vector<C> F(static_cast<std::size_t>(lmax + 1) * ntheta, C{});
  std::vector<double> column(static_cast<std::size_t>(lmax + 1) * ntheta);
  for (int m = 0; m <= lmax; ++m) {
    oracle_wigner_column(lmax, 0, m, ntheta, theta, column.data());
    for (int l = m; l <= lmax; ++l) {
      const C a = c[static_cast<std::size_t>(l) * (l + 1) / 2 + m];
      for (int j = 0; j < ntheta; ++j)
        F[static_cast<std::size_t>(m) * ntheta + j] += a * column[static_cast<std::size_t>(l - m) * ntheta + j];
    }
  }
  for (int j = 0; j < ntheta; ++j) {
    for (int k = 0; k < nphi; ++k) {
      double sum = F[static_cast<std::size_t>(j)].real();
      for (int m = 1; m <= lmax; ++m) {
        const double ang = 2.0 * pi * static_cast<double>((static_cast<long long>(m) * k) % nphi) / nphi;
        sum += 2.0 * (F[static_cast<std::size_t>(m) * ntheta + j] * C(std::cos(ang), std::sin(ang))).real();
      }
      field[static_cast<std::size_t>(j) * nphi + k] = sum;
    }
  }
}

void oracle_expand_real(int lmax, int ntheta, int nphi, const double* theta,
                        const double* weights, const double* field, double* coeffs) {
  const double pi = 3.14159265358979323846;
  using C = std::complex<double>;
  auto* c = reinterpret_cast<C*>(coeffs);
  std::vector<C> F(static_cast<std::size_t>(lmax + 1) * ntheta, C{});
  for (int j = 0; j < ntheta; ++j) {
    for (int m = 0; m <= lmax; ++m) {
      C sum{};
      for (int k = 0; k < nphi; ++k) {
        const double ang = -2.0 * pi * static_cast<double>((static_cast<long long>(m) * k) % nphi) / nphi;
        sum += field[static_cast<std::size_t>(j) * nphi + k] * C(std::cos(ang), std::sin(ang));
      }
      F[static_cast<std::size_t>(m) * ntheta + j] = sum * (2.0 * pi / nphi) * weights[j];
    }
  }
  std::vector<double> column(static_cast<std::size_t>(lmax + 1) * ntheta);
  for (int m = 0; m <= lmax; ++m) {
    oracle_wigner_column(lmax, 0, m, ntheta, theta, column.data());
    for (int l = m; l <= lmax; ++l) {
      C sum{};
      for (int j = 0; j < ntheta; ++j)
        sum += column[static_cast<std::size_t>(l - m) * ntheta + j] * F[static_cast<std::size_t>(m) * ntheta + j];
      c[static_cast<std::size_t>(l) * (l + 1) / 2 + m] = sum;
    }
  }
}

}  // extern "C"
