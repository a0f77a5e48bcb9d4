// FP64 eigendecomposition of the reduced-density-matrix blocks, written for
// GB300's FP64 pipe (one DFMA per ~0.55 cycle and SM, 64-cycle dependent
// latency, a correctly rounded division costing ~650 cycles).
//
// The reference diagonalises every block with LAPACK dsyev
// (eigh_blocks_matrix, src/MATRIX/MATRIX_BLOCKS.f90:589-657) and keeps the
// eigenvectors of the m_s largest eigenvalues over all blocks
// (renormalize_block, src/DMRG_RDM.f90:204-221).  Here the work is split so
// that only kept eigenvectors are ever formed:
//
//   k_trd     one CTA per block: Householder reduction to tridiagonal form
//             T = Q^T rho Q (LAPACK dsytd2 order, lower triangle), the
//             reflectors kept for the back-transformation;
//   k_bisect  every eigenvalue of T by multisection on Sturm counts (16
//             shifts per eigenvalue and round, ~4 bits a round).  The count
//             uses the three-term recurrence of the leading minors,
//             p_i = (a_i - s) p_{i-1} - b_{i-1}^2 p_{i-2}, one FMA on the
//             dependent chain and no division, rescaled by exact powers of
//             two every 8 steps; it is backward stable (each step equals the
//             exact recurrence of a matrix whose a_i - s and b^2 are
//             perturbed by a few ulps).  The chunk-0 CTA of a block also
//             factors T - sigma0 I = L D L^T with sigma0 = -4 n eps ||T||
//             just below the spectrum of the positive semidefinite block.
//             Off-diagonals below 2 n eps ||T|| are set to zero first, which
//             splits T into unreduced blocks (exact eigenvalue degeneracies
//             of rho end up in different ones); each eigenvalue is computed
//             and indexed within its unreduced block;
//   (truncation over all blocks: k_clamp, k_rank, k_truncate)
//   k_vec     one warp per kept eigenvalue: the eigenvector of L D L^T from
//             the twisted factorisation (stationary and progressive
//             differential qd transforms, twist index at the smallest
//             |gamma_r|, Dhillon-Parlett), refined by Rayleigh-quotient
//             corrections, then x = Q z.  A positive definite L D L^T
//             determines its eigenvalues and eigenvectors to high relative
//             accuracy, so vectors of eigenvalues with relative gaps above
//             RELGAP_MIN come out mutually orthogonal to working accuracy
//             without Gram-Schmidt.  Kept eigenvalues closer than that
//             (near-degenerate pairs of symmetric states) form a cluster that
//             one warp handles: each member's twisted vector lies in the
//             cluster's invariant subspace up to eps / (gap to the rest), so
//             Gram-Schmidt among the cluster's kept vectors gives an
//             orthonormal basis of that subspace.  Gaps below 32 eps, a
//             factorisation that is not positive definite, an iteration that
//             does not settle or a Gram-Schmidt remainder below 1/2 mark the
//             block, and the host recomputes that block's vectors with the
//             library eigensolver.
#include "device.cuh"

#include <cfloat>
#include <cmath>

namespace nss {

namespace {

constexpr int TRD_THREADS = 512;
constexpr int BIS_EPC = 8;          // eigenvalues per CTA
constexpr int BIS_THREADS = 160;    // 4 warps x 2 eigenvalues x 16 shifts, 1 warp for L D L^T
constexpr int VEC_WARPS = 4;
constexpr double RELGAP_MIN = 1e-2;
constexpr double PIVMIN = 0x1p-900;

__device__ __forceinline__ double wsum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ double wmax(double v) {
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Householder tridiagonalisation of one block (n <= SYEV_MAX) in shared
// memory.  rho blocks are row-major and symmetric (checked before).  The
// block's rows are first reordered so that the connected components of its
// exact nonzero pattern are contiguous (perm[new] = old row): the reflectors
// of one component then never touch another's rows, T splits exactly at
// the component boundaries, and eigenvectors keep the exact zeros of the
// block structure (as a Jacobi rotation method would; later sparse
// products of the rotation matrix depend on them).  The lower triangle is
// read and updated.  Writes, for the block's eigenvalue slot eo:
// td[eo+i] = T_ii, te[eo+i] = T_{i+1,i}, tau[eo+k], perm[eo+i]; and the
// reflector v_k (v_k[k+1] = 1) as column k of the block's slot in refl.
__global__ void __launch_bounds__(TRD_THREADS, 1)
    k_trd(const double *__restrict__ rho, const int64_t *__restrict__ rho_off, const int *__restrict__ dims,
          const int *__restrict__ ev_off, const int *__restrict__ blocks, double *__restrict__ refl,
          double *__restrict__ td, double *__restrict__ te, double *__restrict__ tau, int *__restrict__ perm) {
    extern __shared__ double trd_smem[];
    constexpr int NW = TRD_THREADS / 32;
    __shared__ double sh[4];
    __shared__ int lab[SYEV_MAX], pm[SYEV_MAX];
    __shared__ int changed;
    const int q = blocks[blockIdx.x];
    const int n = dims[q];
    const int ld = n + 1;
    double *A = trd_smem;
    double *v = A + (size_t)n * ld;
    double *w = v + n;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const double *R = rho + rho_off[q];
    double *Vq = refl + rho_off[q];
    const int eo = ev_off[q];
    // components: minimum-label propagation over the nonzero pattern
    for (int i = tid; i < n; i += TRD_THREADS) lab[i] = i;
    __syncthreads();
    for (int it = 0; it <= n; ++it) {
        if (tid == 0) changed = 0;
        __syncthreads();
        for (int i = warp; i < n; i += NW) {
            int m = lab[i];
            for (int j = lane; j < n; j += 32)
                if (R[(int64_t)i * n + j] != 0.0) m = min(m, lab[j]);
            for (int o = 16; o > 0; o >>= 1) m = min(m, __shfl_xor_sync(0xffffffffu, m, o));
            if (lane == 0 && m < lab[i]) {
                lab[i] = m;
                changed = 1;
            }
        }
        __syncthreads();
        if (!changed) break;
    }
    for (int i = tid; i < n; i += TRD_THREADS) {
        const int li = lab[i];
        int p = 0;
        for (int j = 0; j < n; ++j) p += (lab[j] < li) || (lab[j] == li && j < i);
        pm[p] = i;
    }
    __syncthreads();
    for (int i = tid; i < n; i += TRD_THREADS) perm[eo + i] = pm[i];
    for (int e = tid; e < n * n; e += TRD_THREADS) {
        const int i = e / n, j = e - i * n;
        if (j <= i) A[i * ld + j] = R[(int64_t)pm[i] * n + pm[j]];
    }
    __syncthreads();
    for (int k = 0; k + 2 < n; ++k) {
        const int m = n - k - 1;                    // trailing rows k+1 .. n-1
        if (warp == 0) {
            double ss = 0.0;
            for (int i = k + 2 + lane; i < n; i += 32) {
                const double x = A[i * ld + k];
                ss = fma(x, x, ss);
            }
            ss = wsum(ss);
            if (lane == 0) {
                const double alpha = A[(k + 1) * ld + k];
                double t = 0.0, beta = alpha, scal = 0.0;
                if (ss > 0.0) {                      // dlarfg: H x = beta e_1
                    beta = -copysign(sqrt(fma(alpha, alpha, ss)), alpha);
                    t = (beta - alpha) / beta;
                    scal = 1.0 / (alpha - beta);
                }
                sh[0] = t;
                sh[2] = scal;
                td[eo + k] = A[k * ld + k];
                te[eo + k] = beta;
                tau[eo + k] = t;
            }
        }
        __syncthreads();
        const double t = sh[0];
        for (int i = tid; i < m; i += TRD_THREADS) {
            const double x = (i == 0) ? 1.0 : A[(k + 1 + i) * ld + k] * sh[2];
            v[i] = x;
            Vq[(int64_t)k * n + k + 1 + i] = x;
        }
        __syncthreads();
        if (t == 0.0) continue;                      // uniform: t is shared
        // p = t A v over the trailing block (symmetric reads of the lower triangle)
        for (int i = warp; i < m; i += NW) {
            const int r = k + 1 + i;
            double acc = 0.0;
            for (int j = lane; j < m; j += 32) {
                const int c = k + 1 + j;
                acc = fma(j <= i ? A[r * ld + c] : A[c * ld + r], v[j], acc);
            }
            acc = wsum(acc);
            if (lane == 0) w[i] = t * acc;
        }
        __syncthreads();
        if (warp == 0) {
            double s = 0.0;
            for (int i = lane; i < m; i += 32) s = fma(w[i], v[i], s);
            s = wsum(s);
            if (lane == 0) sh[3] = -0.5 * t * s;
        }
        __syncthreads();
        const double K = sh[3];
        for (int i = tid; i < m; i += TRD_THREADS) w[i] = fma(K, v[i], w[i]);   // w = p - (t/2)(p.v) v
        __syncthreads();
        for (int i = warp; i < m; i += NW) {         // A -= v w^T + w v^T (lower triangle)
            const int r = k + 1 + i;
            const double vi = v[i], wi = w[i];
            for (int j = lane; j <= i; j += 32) {
                const int c = k + 1 + j;
                A[r * ld + c] -= fma(vi, w[j], wi * v[j]);
            }
        }
        __syncthreads();
    }
    if (tid == 0) {
        if (n >= 2) {
            td[eo + n - 2] = A[(n - 2) * ld + n - 2];
            te[eo + n - 2] = A[(n - 1) * ld + n - 2];
            tau[eo + n - 2] = 0.0;
        }
        td[eo + n - 1] = A[(n - 1) * ld + n - 1];
        te[eo + n - 1] = 0.0;
        tau[eo + n - 1] = 0.0;
    }
}

// Number of eigenvalues of the scaled T below s (a: diagonal, bb[i] =
// b_{i-1}^2, bb[0] = 0; the caller passes one unreduced block).  Sign changes of the leading minors; an exact zero
// minor is replaced by -2^-100 times the previous one (a negative pivot, as
// the LDL^T count does with its pivmin).  Integer tests on the bit patterns
// keep FP64 compares off the dependent chain.
__device__ __forceinline__ int sturm_count(const double *a, const double *bb, int n, double s) {
    double pm = 0.0, pc = 1.0;
    int cnt = 0;
    for (int i = 0; i < n; ++i) {
        const double t = bb[i] * pm;
        double pn = fma(a[i] - s, pc, -t);
        long long bn = __double_as_longlong(pn);
        if ((bn << 1) == 0) {
            pn = -pc * 0x1p-100;
            bn = __double_as_longlong(pn);
        }
        cnt += (int)((unsigned long long)(bn ^ __double_as_longlong(pc)) >> 63);
        pm = pc;
        pc = pn;
        if ((i & 7) == 7) {                          // keep max(|pm|, |pc|) in [1, 2)
            const int em = (int)((__double_as_longlong(pm) >> 52) & 0x7ff);
            const int ec = (int)((__double_as_longlong(pc) >> 52) & 0x7ff);
            const int eb = max(em, ec);
            if (eb > 0) {
                const double f = __longlong_as_double((long long)(2046 - eb) << 52);
                pm *= f;
                pc *= f;
            }
        }
    }
    return cnt;
}

// Eigenvalues BIS_EPC * chunk ... of one block.  items[b] = (block, first
// eigenvalue index).  Writes evals (ascending, unscaled); the chunk-0 CTA
// also writes the block's scale, sigma0 and L D L^T (scaled) and sets bit 0
// of flags[q] when that factorisation is not positive definite.
__global__ void __launch_bounds__(BIS_THREADS)
    k_bisect(const int *__restrict__ dims, const int *__restrict__ ev_off, const int2 *__restrict__ items,
             const double *__restrict__ td, const double *__restrict__ te, double *__restrict__ evals,
             double *__restrict__ ldd, double *__restrict__ ldl, double *__restrict__ bscale,
             double *__restrict__ bsig, int *__restrict__ flags, int *__restrict__ sub) {
    __shared__ double sa[SYEV_MAX], sbb[SYEV_MAX], sb[SYEV_MAX];
    __shared__ double red[BIS_THREADS / 32];
    __shared__ double s_norm;
    const int2 it = items[blockIdx.x];
    const int q = it.x, k0 = it.y;
    const int n = dims[q], eo = ev_off[q];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    double r = 0.0;
    for (int i = tid; i < n; i += BIS_THREADS) {
        const double bl = i > 0 ? fabs(te[eo + i - 1]) : 0.0, br = i + 1 < n ? fabs(te[eo + i]) : 0.0;
        r = fmax(r, fabs(td[eo + i]) + bl + br);
    }
    r = wmax(r);
    if (lane == 0) red[warp] = r;
    __syncthreads();
    if (tid == 0) {
        double x = 0.0;
        for (int w = 0; w < BIS_THREADS / 32; ++w) x = fmax(x, red[w]);
        s_norm = x;
    }
    __syncthreads();
    const double tnorm = s_norm;
    if (!(tnorm > 0.0)) {                            // zero block: exact zeros, vectors from the library
        for (int k = k0 + tid; k < min(n, k0 + BIS_EPC); k += BIS_THREADS) {
            evals[eo + k] = 0.0;
            sub[eo + k] = (n << 16);
        }
        if (k0 == 0 && tid == 0) {
            bscale[q] = 1.0;
            bsig[q] = 0.0;
            atomicOr(&flags[q], 1);
        }
        return;
    }
    int ex;
    frexp(tnorm, &ex);
    const double scale = ldexp(1.0, -ex);            // scaled ||T||_inf in [0.5, 1)
    const double split = 2.0 * n * 0x1p-53;
    for (int i = tid; i < n; i += BIS_THREADS) {
        sa[i] = td[eo + i] * scale;
        const double b = i + 1 < n ? te[eo + i] * scale : 0.0;
        sb[i] = fabs(b) <= split ? 0.0 : b;
    }
    __syncthreads();
    for (int i = tid; i < n; i += BIS_THREADS) sbb[i] = i > 0 ? sb[i - 1] * sb[i - 1] : 0.0;
    __syncthreads();
    if (warp < 4) {
        const int g = lane >> 4, j = lane & 15;
        const int k = k0 + warp * 2 + g;
        const bool active = k < n && k < k0 + BIS_EPC;
        // unreduced block [r0, r1) holding row k; the eigenvalue is its (k - r0)-th
        int r0 = 0, r1 = 0;
        if (active) {
            r0 = k;
            while (r0 > 0 && sb[r0 - 1] != 0.0) --r0;
            r1 = k + 1;
            while (r1 < n && sb[r1 - 1] != 0.0) ++r1;
        }
        const int kl = k - r0;
        double lo = -1.0, hi = 1.0;
        // a 1 x 1 unreduced block (the split-off noise rows of a rank-deficient
        // block, mostly) is its own eigenvalue, exactly
        bool done = !active || r1 - r0 == 1;
        if (active && r1 - r0 == 1) lo = hi = sa[k];
        for (int round = 0; round < 64 && __any_sync(0xffffffffu, !done); ++round) {
            const double h = (hi - lo) * (1.0 / 17.0);
            const int c = sturm_count(sa + r0, sbb + r0, r1 - r0, lo + (double)(j + 1) * h);
            const unsigned bal = __ballot_sync(0xffffffffu, c > kl);
            const unsigned gm = (bal >> (16 * g)) & 0xffffu;
            if (!done) {
                const double wold = hi - lo;
                if (gm == 0) {
                    lo = lo + 16.0 * h;
                } else {
                    const int jj = __ffs(gm) - 1;
                    const double nh = lo + (double)(jj + 1) * h;
                    if (jj > 0) lo = lo + (double)jj * h;
                    hi = nh;
                }
                // converged, or the shifts no longer split the bracket (a few ulps)
                if (hi - lo <= fmax(0x1p-52, 0x1p-51 * fmax(fabs(lo), fabs(hi))) || hi - lo >= wold) done = true;
            }
        }
        if (active && j == 0) {
            evals[eo + k] = 0.5 * (lo + hi) / scale;
            sub[eo + k] = r0 | (r1 << 16);
        }
    } else if (k0 == 0 && lane == 0) {
        const double sig0 = -4.0 * n * 0x1p-53;
        double D = sa[0] - sig0;
        bool pd = D > 0.0;
        for (int i = 0; i + 1 < n; ++i) {
            const double L = sb[i] / D;
            ldd[eo + i] = D;
            ldl[eo + i] = L;
            D = (sa[i + 1] - sig0) - L * sb[i];
            pd = pd && D > 0.0;
        }
        ldd[eo + n - 1] = D;
        ldl[eo + n - 1] = 0.0;
        bscale[q] = scale;
        bsig[q] = sig0;
        if (!pd || !isfinite(D)) atomicOr(&flags[q], 1);
    }
}

// One warp per kept eigenvalue j < ms of one side: order[j] + ev_base is its
// position in the block-concatenated eigenvalue list, rank[pos] its rank
// within the side.
// Blocks of the library path (bmode != 0) already hold their vectors.  The
// kept eigenvalues of one relative cluster are done by the warp of the
// cluster's first kept member, in ascending order, each orthogonalised
// against the ones before it.  Output: column col of the block's
// column-major slot in vec.  Failure sets bit 1 of flags[q].
constexpr int VEC_MAXCL = 16;

__global__ void __launch_bounds__(VEC_WARPS * 32)
    k_vec(const int *__restrict__ order, const int *__restrict__ rank, int ev_base, int ms, int nblk,
          const int *__restrict__ ev_off, const int *__restrict__ dims, const int64_t *__restrict__ rho_off,
          const int *__restrict__ bmode, const int *__restrict__ sub, const double *__restrict__ evals,
          const double *__restrict__ ldd, const double *__restrict__ ldl, const double *__restrict__ bscale,
          const double *__restrict__ bsig, const double *__restrict__ tau, const double *__restrict__ refl,
          const int *__restrict__ perm, int *__restrict__ flags, double *__restrict__ vec) {
    __shared__ double sm[VEC_WARPS][7][SYEV_MAX];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int j = blockIdx.x * VEC_WARPS + warp;
    if (j >= ms) return;
    const int pos = order[j] + ev_base;
    int q = 0;
    while (q + 1 < nblk && ev_off[q + 1] <= pos) ++q;
    const int n = dims[q], eo = ev_off[q], col = pos - eo;
    if (bmode[q] != 0) return;
    double *X = vec + rho_off[q];
    if (n == 1) {
        if (lane == 0) X[0] = 1.0;
        return;
    }
    const double scale = bscale[q], sig0 = bsig[q];
    const int sr = sub[eo + col], r0 = sr & 0xffff, r1 = sr >> 16;
    auto lamS = [&](int c) { return evals[eo + c] * scale - sig0; };
    auto linked = [&](int c) {      // c and c + 1 in one relative cluster
        if (c + 1 >= r1) return false;
        const double x = lamS(c), y = lamS(c + 1);
        return y - x < RELGAP_MIN * fmax(x, y);
    };
    auto kept = [&](int c) { return rank[eo + c] < ms; };
    int c0 = col;
    while (c0 > r0 && linked(c0 - 1)) --c0;
    int c1 = col;
    while (linked(c1)) ++c1;
    for (int c = c0; c < col; ++c)
        if (kept(c)) return;                         // an earlier kept member leads
    double *dD = sm[warp][0], *dL = sm[warp][1], *lp = sm[warp][2], *um = sm[warp][3], *ss = sm[warp][4],
           *pp = sm[warp][5], *z = sm[warp][6];
    bool ok = (flags[q] & 1) == 0;
    int nm = 0;
    for (int c = col; c <= c1; ++c) nm += kept(c);
    ok = ok && nm <= VEC_MAXCL;
    for (int i = lane; i < n; i += 32) {
        dD[i] = ldd[eo + i];
        dL[i] = ldl[eo + i];
    }
    __syncwarp();
    const double *Vq = refl + rho_off[q];
    for (int c = col; ok && c <= c1; ++c) {
        if (!kept(c)) continue;
        const double lam0 = lamS(c);
        const double gap = fmin(c > r0 ? lam0 - lamS(c - 1) : INFINITY, c + 1 < r1 ? lamS(c + 1) - lam0 : INFINITY);
        if (!(gap > 32.0 * 0x1p-52)) {
            ok = false;
            break;
        }
        double lam = lam0, ztz = 1.0;
        bool conv = false;
        for (int itr = 0; itr < 8; ++itr) {
            if (lane == 0) {                         // stationary: L+ D+ L+^T = L D L^T - lam
                double s = -lam;
                for (int i = r0; i + 1 < r1; ++i) {
                    ss[i] = s;
                    double dp = dD[i] + s;
                    if (fabs(dp) < PIVMIN) dp = -PIVMIN;
                    const double l = dD[i] * dL[i] / dp;
                    lp[i] = l;
                    s = l * dL[i] * s - lam;
                }
                ss[r1 - 1] = s;
            } else if (lane == 1) {                  // progressive: U- D- U-^T = L D L^T - lam
                double p = dD[r1 - 1] - lam;
                for (int i = r1 - 2; i >= r0; --i) {
                    pp[i + 1] = p;
                    double dm = dD[i] * dL[i] * dL[i] + p;
                    if (fabs(dm) < PIVMIN) dm = -PIVMIN;
                    const double t = dD[i] / dm;
                    um[i] = dL[i] * t;
                    p = p * t - lam;
                }
                pp[r0] = p;
            }
            __syncwarp();
            double best = INFINITY;
            int bi = r1;
            for (int k = r0 + lane; k < r1; k += 32) {
                const double gk = fabs(ss[k] + pp[k] + lam);
                if (gk < best) {
                    best = gk;
                    bi = k;
                }
            }
            for (int o = 16; o > 0; o >>= 1) {
                const double ob = __shfl_xor_sync(0xffffffffu, best, o);
                const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
                if (ob < best || (ob == best && oi < bi)) {
                    best = ob;
                    bi = oi;
                }
            }
            if (bi >= r1) break;                     // every gamma NaN
            const int r = bi;
            const double gam = ss[r] + pp[r] + lam;
            __syncwarp();
            for (int i = lane; i < n; i += 32) z[i] = 0.0;
            __syncwarp();
            if (lane == 0) {
                double zz = 1.0;
                z[r] = 1.0;
                for (int i = r - 1; i >= r0; --i) {
                    zz = -lp[i] * zz;
                    z[i] = zz;
                }
            } else if (lane == 1) {
                double zz = 1.0;
                for (int i = r; i + 1 < r1; ++i) {
                    zz = -um[i] * zz;
                    z[i + 1] = zz;
                }
            }
            __syncwarp();
            double t2 = 0.0;
            for (int k = r0 + lane; k < r1; k += 32) t2 = fma(z[k], z[k], t2);
            ztz = wsum(t2);
            const double corr = gam / ztz;
            if (!isfinite(ztz) || !isfinite(corr)) break;
            if (fabs(corr) <= 0x1p-49 * lam) {
                conv = true;
                break;
            }
            lam += corr;
            if (!(fabs(lam - lam0) <= 0.25 * gap)) break;
            __syncwarp();
        }
        if (!conv) {
            ok = false;
            break;
        }
        const double inv = 1.0 / sqrt(ztz);
        for (int k = lane; k < n; k += 32) z[k] *= inv;
        __syncwarp();
        // x = H_0 H_1 ... H_{n-3} z
        for (int k = n - 3; k >= 0; --k) {
            const double t = tau[eo + k];
            if (t == 0.0) continue;
            const double *vk = Vq + (int64_t)k * n;
            double d = 0.0;
            for (int i = k + 1 + lane; i < n; i += 32) d = fma(vk[i], z[i], d);
            d = t * wsum(d);
            for (int i = k + 1 + lane; i < n; i += 32) z[i] = fma(-d, vk[i], z[i]);
            __syncwarp();
        }
        // Gram-Schmidt against the cluster's kept vectors done before (rows
        // of X in the block's own order: row perm[i] holds z[i])
        for (int cp = col; cp < c; ++cp) {
            if (!kept(cp)) continue;
            const double *Y = X + (int64_t)cp * n;
            double d = 0.0;
            for (int i = lane; i < n; i += 32) d = fma(Y[perm[eo + i]], z[i], d);
            d = wsum(d);
            for (int i = lane; i < n; i += 32) z[i] = fma(-d, Y[perm[eo + i]], z[i]);
            __syncwarp();
        }
        double nz = 0.0;
        for (int i = lane; i < n; i += 32) nz = fma(z[i], z[i], nz);
        nz = sqrt(wsum(nz));
        if (!(nz >= 0.5)) {
            ok = false;
            break;
        }
        double *Xc = X + (int64_t)c * n;
        for (int i = lane; i < n; i += 32) Xc[perm[eo + i]] = z[i] / nz;
        __syncwarp();
    }
    if (!ok && lane == 0) atomicOr(&flags[q], 2);
}

}  // namespace

int syev_trd(const double *rho, const int64_t *rho_off, const int *dims, const int *ev_off, const int *blocks,
             int nblocks, int maxn, double *refl, double *td, double *te, double *tau, int *perm, cudaStream_t st) {
    if (nblocks <= 0) return 0;
    const int smem = (int)(((size_t)maxn * (maxn + 1) + 2 * (size_t)maxn) * sizeof(double));
    cudaError_t e = cudaFuncSetAttribute(k_trd, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return (int)e;
    k_trd<<<nblocks, TRD_THREADS, smem, st>>>(rho, rho_off, dims, ev_off, blocks, refl, td, te, tau, perm);
    return (int)cudaGetLastError();
}

int syev_bisect(const int *dims, const int *ev_off, const int2 *items, int nitems, const double *td,
                const double *te, double *evals, double *ldd, double *ldl, double *bscale, double *bsig,
                int *flags, int *sub, cudaStream_t st) {
    if (nitems <= 0) return 0;
    k_bisect<<<nitems, BIS_THREADS, 0, st>>>(dims, ev_off, items, td, te, evals, ldd, ldl, bscale, bsig, flags,
                                             sub);
    return (int)cudaGetLastError();
}

int syev_vec(const int *order, const int *rank, int ev_base, int ms, int nblk, const int *ev_off, const int *dims,
             const int64_t *rho_off, const int *bmode, const int *sub, const double *evals, const double *ldd,
             const double *ldl, const double *bscale, const double *bsig, const double *tau, const double *refl,
             const int *perm, int *flags, double *vec, cudaStream_t st) {
    if (ms <= 0) return 0;
    k_vec<<<(ms + VEC_WARPS - 1) / VEC_WARPS, VEC_WARPS * 32, 0, st>>>(order, rank, ev_base, ms, nblk, ev_off,
                                                                        dims, rho_off, bmode, sub, evals, ldd, ldl,
                                                                        bscale, bsig, tau, refl, perm, flags, vec);
    return (int)cudaGetLastError();
}

int syev_eigs_per_cta() { return BIS_EPC; }

}  // namespace nss
