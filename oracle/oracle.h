// ORACLE — test infrastructure only (see oracle_core.cpp's header).
// The C interface tests/ and bench.py's cpu_baseline bind through ctypes.
#pragma once

#ifdef __cplusplus
extern "C" {
#endif

int oracle_band_cholesky_factor(double* ab, int n, int kd);
void oracle_band_cholesky_solve(const double* ab, int n, int kd, double* b, int nrhs);
int oracle_band_lu_factor(double* ab, int n, int kl, int ku, int* pivots);
void oracle_band_lu_solve(const double* ab, int n, int kl, int ku, const int* pivots,
                          double* b, int nrhs);

void oracle_gauss_legendre(int n, double* x, double* w);
void oracle_wigner_column(int lmax, int N, int m, int ntheta, const double* theta, double* out);

void oracle_synthesise_spin(int lmax, int N, int ntheta, int nphi, const double* theta,
                            const double* coeffs, double* field);
void oracle_expand_spin(int lmax, int N, int ntheta, int nphi, const double* theta,
                        const double* weights, const double* field, double* coeffs);
void oracle_synthesise_real(int lmax, int ntheta, int nphi, const double* theta,
                            const double* coeffs, double* field);
void oracle_expand_real(int lmax, int ntheta, int nphi, const double* theta,
                        const double* weights, const double* field, double* coeffs);

#ifdef __cplusplus
}
#endif
