// tl_host_numerics.h -- host-side numerics of the Chebyshev / PPCG switch
// (tea_leaf_cheby.f90:46-174), computed once per solve on the CPU exactly as
// the reference does.
#pragma once

namespace tl {

// QL with implicit shifts on a symmetric tridiagonal matrix (the tqli of
// tea_leaf_cheby.f90:46-96).  d: diagonal (n), e: sub-diagonal stored in
// e[1..n-1].  Returns 0, or 1 when an eigenvalue needs more than 30 sweeps.
int tl_tqli(double *d, double *e, int n);

// Extreme eigenvalues of the Lanczos tridiagonal matrix built from the first
// n CG alphas and betas (tea_calc_eigenvalues, tea_leaf_cheby.f90:98-145).
int tl_calc_eigenvalues(const double *alphas, const double *betas, int n, double *eigmin,
                        double *eigmax);

// Chebyshev recurrence coefficients over [eigmin, eigmax]
// (tea_calc_ch_coefs, tea_leaf_cheby.f90:147-174).
void tl_calc_ch_coefs(double *alphas, double *betas, double eigmin, double eigmax, double *theta,
                      int n);

}  // namespace tl
