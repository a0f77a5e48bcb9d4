// Lowest eigenpairs of the Lanczos tridiagonal matrix, on the host CPU.
//
// The Lanczos tridiagonal T_m (m <= a few hundred) is a latency-bound chain
// of dependent FP64 operations: on GB300 the FP64 pipe is 1/64 of the FP32
// one and one SM runs such a chain at a small fraction of a Grace core's
// speed.  The solver therefore runs on the host thread that drives the
// iteration, one chunk of Lanczos steps behind the GPU, so the device never
// waits for it (ARPACK, which the reference calls, also works on T on the
// host: src/DMRG_SUPERBLOCK.f90:412-425 -> sp_eigh).
#pragma once

#include <vector>

namespace nss {

// Lowest `ne` eigenpairs of the symmetric tridiagonal matrix with diagonal
// a[0..m) and off-diagonal b[0..m-1):
//   theta[e]  ascending eigenvalues (multisection on Sturm counts, converged
//             to a few ulps of max(|theta|, ||T||_inf eps)),
//   s[e*m+i]  unit eigenvectors by inverse iteration (reorthogonalised within
//             clusters), sign fixed so the largest component is positive,
//   resid[e]  |b_last * s_e[m-1]|, the Lanczos residual norm of Ritz pair e
//             when b_last is the coupling to the next Lanczos vector.
// `upper` (may be null): upper bounds of the wanted eigenvalues from a
// smaller leading block (Cauchy interlacing), used to narrow the bracket.
void tridiag_lowest(const double *a, const double *b, int m, int ne, double b_last, double *theta,
                    double *s, double *resid, const double *upper, std::vector<double> &work);

// Lowest eigenpair of the (k+1) x (k+1) "arrowhead + tridiagonal" matrix
//     M = [ theta0  m^T ]
//         [ m       T   ]     T = tridiag(a[0..k), b[0..k-1))
// that the anchored refinement of the mixed-precision Lanczos produces (row 0
// is the FP64 anchor vector, rows 1.. its FP32 Krylov complement).  The root
// lam < min(theta0, lambda_min(T)) of the secular equation
//     f(lam) = theta0 - lam - m^T (T - lam)^{-1} m = 0
// by safeguarded Newton (T - lam I is positive definite there, so LDL^T
// needs no pivoting); c[0] = 1, c[1..] = -(T - lam)^{-1} m, normalised.
// resid = |b_last * c[k]|.  Returns false when no root is bracketed.
bool arrow_lowest(double theta0, const double *m, const double *a, const double *b, int k, double b_last,
                  double *lam, double *c, double *resid, std::vector<double> &work);

// All eigenpairs of the symmetric tridiagonal matrix with diagonal d[0..n)
// and off-diagonal e[0..n-1) (e[i] couples i and i+1): implicit QL
// iterations with Wilkinson shifts, the rotations accumulated into Z
// (column-major n x n, initialised to the identity here).  On return d
// holds the eigenvalues ascending and column j of Z the eigenvector of
// d[j].  Returns false if an eigenvalue takes more than 60 iterations.
bool tridiag_ql(int n, double *d, double *e, double *Z);

}  // namespace nss
