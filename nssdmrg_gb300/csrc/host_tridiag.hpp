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

}  // namespace nss
