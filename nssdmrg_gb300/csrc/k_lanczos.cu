// Lanczos eigensolver for the lowest eigenpairs of H_sb, entirely on the GPU.
//
// Replaces SciFortran sp_eigh (ARPACK, called at src/DMRG_SUPERBLOCK.f90:
// 394-425) for the direct mode.  Algorithm: Lanczos with full
// reorthogonalisation -- the three-term recurrence first, then one classical
// Gram-Schmidt projection of the (small) residual against the whole basis,
// and a second projection only when that one removes more than half of the
// residual -- the whole Krylov basis kept resident in HBM (no restarts), and a
// convergence test every CHECK steps on the tridiagonal matrix T on the
// device: residual beta_m |s_m| <= tol |theta| for each wanted Ritz pair,
// the ARPACK criterion.  Breakdown (beta ~ 0, invariant subspace) restarts
// with a fresh random vector orthogonal to the basis.  Eigenvectors are
// gauge-dependent, so parity with the reference is on eigenvalues and on
// what the RDM derives from them.
//
// Per iteration j (m = j+1 basis vectors):
//   k_hv          w = H v_j
//   k_alpha       alpha = v_j . w
//   k_dots        w -= alpha v_j + beta_{j-1} v_{j-1};  h = V_m^T w, ww = w.w
//   k_update      w -= V_m h, beta^2 = w.w, alpha_j = alpha + h_j
//   k_dots/k_update again only if beta^2 < ww/2 (device flag)
//   k_next        v_{j+1} = w / beta
// Projecting the raw H v_j instead (one pass) lets the orthogonality error
// grow by ||H||/beta per step; the recurrence-first order keeps it at 1e-15.
// Every kernel reads the device stop flag first, so the host can enqueue a
// whole chunk of iterations ahead of the convergence test.
//
// Precision modes.  The kernels are templates over the type T of the Krylov
// vectors.  T = double is the plain method: FP64 everywhere.  T = float is
// the mixed method: H*psi in FP32 (k_hv_fp32), the basis and the projections
// in FP32 with FP64 block partial sums, while alpha/beta, the tridiagonal
// eigensolve and the Ritz vector stay FP64; it runs to a relative residual
// of MIXED_TOL, and the energy is then refined in FP64 as the Rayleigh
// quotient psi.H.psi of the FP64 Ritz vector with the FP64 H*psi (error
// quadratic in the vector error: |dE|/|E| ~ 1e-13 at MIXED_TOL = 1e-7),
// whose FP64 residual ||H psi - E psi|| is reported.  On GB300 the FP64
// pipe runs at 1/64 of the FP32 one, which is what the mixed method buys.
#include "device.cuh"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

namespace nss {

namespace {

constexpr int NBLK = 304;         // 2 CTAs per SM on the 152-SM GB300
constexpr int CHECK = 8;          // convergence test period (iterations)
constexpr int SUB = 1024;         // rows staged per shared-memory sub-chunk
constexpr double MIXED_TOL = 1e-7;

// device scalar slots (Ctx::lz.scal)
enum { S_WW = 0, S_BB = 1, S_ALPHA = 2, S_NSCAL = 4 };
// device flag slots (Ctx::lz.flags)
enum { F_STOP = 0, F_PASS2 = 1, F_M = 2, F_CONV = 3, F_BREAK = 4, F_NFLAGS = 8 };

template <class T>
__device__ __forceinline__ T warp_sum(T x) {
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    return x;
}

__device__ __forceinline__ uint64_t splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

// uniform(-1,1) start vector from a counter-based hash of (seed, stream, i)
template <class T>
__global__ void k_random(T *x, int64_t n, uint64_t seed, uint64_t stream) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        uint64_t r = splitmix64(seed ^ splitmix64(stream * 0x632BE59BD9B4E019ull + (uint64_t)i));
        x[i] = (T)(2.0 * ((double)(r >> 11) * (1.0 / 9007199254740992.0)) - 1.0);
    }
}

// Last-CTA-done grid reduction helper: every CTA writes its partials, the
// last one to arrive sees all of them.
__device__ __forceinline__ bool last_block(unsigned *counter) {
    __shared__ unsigned last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = (atomicAdd(counter, 1u) == gridDim.x - 1);
    __syncthreads();
    if (last) __threadfence();
    return last != 0;
}

// h[l] = V[l] . w for l < m, and scal[S_WW] = w . w.  With threeterm != 0
// the recurrence step w -= alpha v_{m-1} + beta v_{m-2} (alpha from
// scal[S_ALPHA], beta = betas[m-2]) is applied to w first and the updated w
// is written back.  Per-thread sums in T, block and grid sums in FP64.
template <class T>
__global__ void __launch_bounds__(256) k_dots(const T *__restrict__ V, int m, T *__restrict__ w, int64_t n,
                                              double *__restrict__ part, double *__restrict__ h,
                                              double *__restrict__ scal, unsigned *counter, const int *flags,
                                              int pass2, int threeterm, const double *__restrict__ betas) {
    if (flags[F_STOP] || (pass2 && !flags[F_PASS2])) return;
    extern __shared__ double sm[];
    double *acc = sm;                      // [m+1]
    T *ws = (T *)(sm + (m + 2));           // [SUB]
    const T a3 = threeterm ? (T)scal[S_ALPHA] : (T)0;
    const T b3 = (threeterm && m >= 2) ? (T)betas[m - 2] : (T)0;
    const T *vj = V + (int64_t)(m - 1) * n;
    const T *vjm = (m >= 2) ? V + (int64_t)(m - 2) * n : V;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int l = tid; l <= m; l += 256) acc[l] = 0.0;
    const int64_t chunk = (n + gridDim.x - 1) / gridDim.x;
    const int64_t i0 = blockIdx.x * chunk, i1 = min(n, i0 + chunk);
    for (int64_t s0 = i0; s0 < i1; s0 += SUB) {
        const int len = (int)min((int64_t)SUB, i1 - s0);
        __syncthreads();
        if (threeterm) {
            for (int e = tid; e < len; e += 256) {
                T x = w[s0 + e] - a3 * vj[s0 + e];
                if (m >= 2) x -= b3 * vjm[s0 + e];
                ws[e] = x;
                w[s0 + e] = x;
            }
        } else {
            for (int e = tid; e < len; e += 256) ws[e] = w[s0 + e];
        }
        __syncthreads();
        for (int l = warp; l <= m; l += 8) {
            T p = (T)0;
            if (l < m) {
                const T *vl = V + (int64_t)l * n + s0;
                for (int e = lane; e < len; e += 32) p += vl[e] * ws[e];
            } else {
                for (int e = lane; e < len; e += 32) p += ws[e] * ws[e];
            }
            const double pd = warp_sum<double>((double)p);
            if (lane == 0) acc[l] += pd;
        }
    }
    __syncthreads();
    for (int l = tid; l <= m; l += 256) part[(int64_t)l * gridDim.x + blockIdx.x] = acc[l];
    if (!last_block(counter)) return;
    for (int l = warp; l <= m; l += 8) {
        double p = 0.0;
        for (int b = lane; b < (int)gridDim.x; b += 32) p += part[(int64_t)l * gridDim.x + b];
        p = warp_sum<double>(p);
        if (lane == 0) {
            if (l < m) h[l] = p;
            else scal[S_WW] = p;
        }
    }
    if (tid == 0) *counter = 0u;
}

// alpha = v . w  (grid reduction by the last CTA) -> scal[S_ALPHA]
template <class T>
__global__ void __launch_bounds__(256) k_alpha(const T *__restrict__ v, const T *__restrict__ w, int64_t n,
                                               double *__restrict__ part, double *__restrict__ scal,
                                               unsigned *counter, const int *flags) {
    if (flags[F_STOP]) return;
    const int tid = threadIdx.x;
    T p = (T)0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + tid; i < n; i += (int64_t)gridDim.x * blockDim.x)
        p += v[i] * w[i];
    const double pd = warp_sum<double>((double)p);
    __shared__ double red[8];
    if ((tid & 31) == 0) red[tid >> 5] = pd;
    __syncthreads();
    if (tid == 0) {
        double t = 0.0;
        for (int q = 0; q < 8; ++q) t += red[q];
        part[blockIdx.x] = t;
    }
    if (!last_block(counter) || tid != 0) return;
    double t = 0.0;
    for (int b = 0; b < (int)gridDim.x; ++b) t += part[b];
    scal[S_ALPHA] = t;
    *counter = 0u;
}

// w -= V_m h ; beta^2 = w.w ; the last CTA records alpha_j and beta_j.
template <class T>
__global__ void __launch_bounds__(256) k_update(const T *__restrict__ V, int m, T *__restrict__ w, int64_t n,
                                                const double *__restrict__ h, double *__restrict__ part,
                                                double *__restrict__ scal, unsigned *counter, int *flags,
                                                double *alpha, double *beta, int pass2) {
    if (flags[F_STOP] || (pass2 && !flags[F_PASS2])) return;
    extern __shared__ double hsd[];
    T *hs = (T *)hsd;
    const int tid = threadIdx.x;
    for (int l = tid; l < m; l += 256) hs[l] = (T)h[l];
    __syncthreads();
    T ss = (T)0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + tid; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        T x = w[i];
        for (int l = 0; l < m; ++l) x -= V[(int64_t)l * n + i] * hs[l];
        w[i] = x;
        ss += x * x;
    }
    const double sd = warp_sum<double>((double)ss);
    __shared__ double red[8];
    if ((tid & 31) == 0) red[tid >> 5] = sd;
    __syncthreads();
    if (tid == 0) {
        double t = 0.0;
        for (int q = 0; q < 8; ++q) t += red[q];
        part[blockIdx.x] = t;
    }
    if (!last_block(counter) || tid != 0) return;
    double bb = 0.0;
    for (int b = 0; b < (int)gridDim.x; ++b) bb += part[b];
    const int j = m - 1;
    if (!pass2) {
        alpha[j] = scal[S_ALPHA] + h[j];
        flags[F_PASS2] = (bb < 0.5 * scal[S_WW]) ? 1 : 0;
    } else {
        alpha[j] += h[j];
    }
    scal[S_BB] = bb;
    beta[j] = sqrt(bb);
    *counter = 0u;
}

// v_{j+1} = w / beta_j, or flag a breakdown (invariant subspace).
template <class T>
__global__ void k_next(T *__restrict__ vnext, const T *__restrict__ w, int64_t n, int *flags,
                       const double *alpha, const double *beta, int j) {
    if (flags[F_STOP]) return;
    const double b = beta[j];
    const double scale = fmax(fabs(alpha[j]), j > 0 ? beta[j - 1] : 0.0);
    if (!(b > 1e-13 * fmax(scale, 1e-300))) {
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            flags[F_BREAK] = j + 1;
            flags[F_STOP] = 2;
        }
        return;
    }
    const T inv = (T)(1.0 / b);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        vnext[i] = w[i] * inv;
}

// x <- x / ||x|| (one CTA per launch is enough for start vectors);
// blockDim.x <= 1024, so at most 32 warp partial sums
template <class T>
__global__ void __launch_bounds__(1024) k_normalize(T *x, int64_t n) {
    __shared__ double red[32];
    double ss = 0.0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) ss += (double)x[i] * (double)x[i];
    ss = warp_sum<double>(ss);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = ss;
    __syncthreads();
    double t = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) t += red[q];
    const double inv = 1.0 / sqrt(t);
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) x[i] = (T)((double)x[i] * inv);
}

// Number of eigenvalues of T_m below x (Sturm count of the leading
// principal minors, division-free with exact power-of-two rescaling).
__device__ int sturm_count(const double *alpha, const double *beta, int m, double x) {
    double p0 = 1.0, p1 = alpha[0] - x;
    int cnt = (p1 < 0.0) ? 1 : 0;
    for (int i = 1; i < m; ++i) {
        const double b = beta[i - 1];
        double p2 = (alpha[i] - x) * p1 - b * b * p0;
        // a zero minor takes the sign opposite to its predecessor
        if (p2 == 0.0) p2 = -copysign(1e-300, p1);
        if ((p2 < 0.0) != (p1 < 0.0)) ++cnt;
        p0 = p1;
        p1 = p2;
        const double a = fmax(fabs(p0), fabs(p1));
        if (a > 0x1p+600) { p0 *= 0x1p-600; p1 *= 0x1p-600; }
        else if (a < 0x1p-600) { p0 *= 0x1p+600; p1 *= 0x1p+600; }
    }
    return cnt;
}

// Eigenvalues theta[0..ne) of T_m by 32-way multisection, one warp per
// eigenvalue (a round costs one Sturm count per lane; GB300's FP64 pipe is
// narrow, so fewer concurrent counts and more rounds is the faster trade),
// eigenvectors s by inverse iteration, residual estimates beta_{m-1} |s_{m-1}|
// and the convergence flag.
// m_arg is the basis size the chunk would reach; after a breakdown the
// kernel uses the breakdown step instead, and once a solve has converged
// (stop flag 1) later calls leave theta and s untouched.  It records the m it
// used (F_M) and sets the stop flag: 1 converged or Krylov space exhausted
// (m = n), 3 iteration cap reached.
__global__ void __launch_bounds__(128) k_tridiag(const double *alpha, const double *beta, int m_arg, int ne,
                                                 double tol, double *theta, double *resid, double *svec,
                                                 int sstride, int *flags, int mmax, int64_t nvec) {
    if (flags[F_STOP] == 1 || flags[F_STOP] == 3) return;
    const int m = (flags[F_STOP] == 2) ? flags[F_BREAK] : m_arg;
    __shared__ double lo_s, hi_s;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (tid == 0) {
        double lo = 1e300, hi = -1e300;
        for (int i = 0; i < m; ++i) {
            double r = (i > 0 ? fabs(beta[i - 1]) : 0.0) + (i < m - 1 ? fabs(beta[i]) : 0.0);
            lo = fmin(lo, alpha[i] - r);
            hi = fmax(hi, alpha[i] + r);
        }
        double pad = 1e-12 * fmax(fabs(lo), fabs(hi)) + 1e-300;
        lo_s = lo - pad;
        hi_s = hi + pad;
    }
    __syncthreads();
    const int e = warp;
    if (e < ne && e < m) {
        double a = lo_s, b = hi_s;
        for (int round = 0; round < 24; ++round) {
            if (!(b - a > 4e-16 * fmax(fabs(a), fabs(b)) + 1e-300)) break;
            const double x = a + (b - a) * (double)(lane + 1) / 33.0;
            const int cnt = sturm_count(alpha, beta, m, x);
            const unsigned over = __ballot_sync(0xffffffffu, cnt > e);
            // first point whose count exceeds e brackets eigenvalue e
            const int t = over ? __ffs(over) - 1 : 32;
            const double xt = __shfl_sync(0xffffffffu, x, t < 32 ? t : 31);
            const double xp = __shfl_sync(0xffffffffu, x, t > 0 ? t - 1 : 0);
            const double na = (t == 0) ? a : xp;
            const double nb = (t == 32) ? b : xt;
            a = na;
            b = nb;
        }
        if (lane == 0) theta[e] = 0.5 * (a + b);
    }
    __syncthreads();
    // inverse iteration, one thread per eigenvalue: (T - shift I) y = s, solved
    // by Gaussian elimination with partial pivoting (the LAPACK dgtsv scheme);
    // the factor bands live in the eigenvector's scratch row (stride 4*m+).
    if (tid < ne && tid < m) {
        const int e = tid;
        double *s = svec + (int64_t)e * sstride;
        double *D = s + m, *DU = s + 2 * m, *DL = s + 3 * m;
        const double th = theta[e];
        const double shift = th + 1e-14 * fmax(fabs(th), 1.0);
        for (int i = 0; i < m; ++i) s[i] = 1.0 + 0.01 * (double)((i * 7 + e * 3) % 11);
        for (int it = 0; it < 3; ++it) {
            for (int i = 0; i < m; ++i) {
                D[i] = alpha[i] - shift;
                DU[i] = (i < m - 1) ? beta[i] : 0.0;
                DL[i] = (i < m - 1) ? beta[i] : 0.0;
            }
            for (int i = 0; i < m - 1; ++i) {
                if (fabs(D[i]) >= fabs(DL[i])) {
                    if (D[i] == 0.0) D[i] = 1e-300;
                    const double f = DL[i] / D[i];
                    D[i + 1] -= f * DU[i];
                    s[i + 1] -= f * s[i];
                    DL[i] = 0.0;
                } else {
                    const double f = D[i] / DL[i];
                    D[i] = DL[i];
                    const double tmp = D[i + 1];
                    D[i + 1] = DU[i] - f * tmp;
                    if (i < m - 2) {
                        DL[i] = DU[i + 1];
                        DU[i + 1] = -f * DL[i];
                    } else {
                        DL[i] = 0.0;
                    }
                    DU[i] = tmp;
                    const double b0 = s[i];
                    s[i] = s[i + 1];
                    s[i + 1] = b0 - f * s[i + 1];
                }
            }
            if (D[m - 1] == 0.0) D[m - 1] = 1e-300;
            s[m - 1] /= D[m - 1];
            if (m > 1) s[m - 2] = (s[m - 2] - DU[m - 2] * s[m - 1]) / D[m - 2];
            for (int i = m - 3; i >= 0; --i) s[i] = (s[i] - DU[i] * s[i + 1] - DL[i] * s[i + 2]) / D[i];
            double nrm = 0.0;
            for (int i = 0; i < m; ++i) nrm = fma(s[i], s[i], nrm);
            nrm = 1.0 / sqrt(nrm);
            for (int i = 0; i < m; ++i) s[i] *= nrm;
        }
        // sign convention: largest component positive
        double big = 0.0;
        for (int i = 0; i < m; ++i) if (fabs(s[i]) > fabs(big)) big = s[i];
        if (big < 0.0) for (int i = 0; i < m; ++i) s[i] = -s[i];
        resid[e] = fabs(beta[m - 1] * s[m - 1]);
    }
    __syncthreads();
    if (tid == 0) {
        int conv = 0;
        for (int e = 0; e < ne && e < m; ++e)
            if (resid[e] <= tol * fmax(fabs(theta[e]), 1e-300)) ++conv;
        flags[F_CONV] = conv;
        flags[F_M] = m;
        if (conv >= min(ne, m) || (int64_t)m >= nvec) flags[F_STOP] = 1;
        else if (m >= mmax) flags[F_STOP] = 3;
    }
}

// Ritz vectors: out[e] = sum_l V[l] s_e[l]   (FP64 accumulation, FP64 out)
template <class T>
__global__ void __launch_bounds__(256) k_ritz(const T *__restrict__ V, int m, int64_t n,
                                              const double *__restrict__ svec, int sstride, int ne,
                                              double *__restrict__ out) {
    extern __shared__ double ss[];   // [ne][m]
    for (int t = threadIdx.x; t < ne * m; t += blockDim.x) ss[t] = svec[(int64_t)(t / m) * sstride + (t % m)];
    __syncthreads();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double acc[4] = {0, 0, 0, 0};
        for (int l = 0; l < m; ++l) {
            const double v = (double)V[(int64_t)l * n + i];
            for (int e = 0; e < ne && e < 4; ++e) acc[e] = fma(v, ss[e * m + l], acc[e]);
        }
        for (int e = 0; e < ne && e < 4; ++e) out[(int64_t)e * n + i] = acc[e];
    }
}

// FP64 refinement: r[0] = psi.w, r[1] = w.w, r[2] = psi.psi (grid reduction)
__global__ void __launch_bounds__(256) k_rq(const double *__restrict__ psi, const double *__restrict__ w, int64_t n,
                                            double *__restrict__ part, double *__restrict__ r, unsigned *counter) {
    const int tid = threadIdx.x;
    double a = 0.0, b = 0.0, c = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + tid; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        a = fma(psi[i], w[i], a);
        b = fma(w[i], w[i], b);
        c = fma(psi[i], psi[i], c);
    }
    a = warp_sum<double>(a);
    b = warp_sum<double>(b);
    c = warp_sum<double>(c);
    __shared__ double red[3][8];
    if ((tid & 31) == 0) { red[0][tid >> 5] = a; red[1][tid >> 5] = b; red[2][tid >> 5] = c; }
    __syncthreads();
    if (tid < 3) {
        double t = 0.0;
        for (int q = 0; q < 8; ++q) t += red[tid][q];
        part[(int64_t)tid * gridDim.x + blockIdx.x] = t;
    }
    if (!last_block(counter)) return;
    if (tid < 3) {
        double t = 0.0;
        for (int bb = 0; bb < (int)gridDim.x; ++bb) t += part[(int64_t)tid * gridDim.x + bb];
        r[tid] = t;
    }
    if (tid == 0) *counter = 0u;
}

// ||w - theta psi||^2 (grid reduction); theta = r[0]/r[2]
__global__ void __launch_bounds__(256) k_resid(const double *__restrict__ psi, const double *__restrict__ w, int64_t n,
                                               double *__restrict__ part, double *__restrict__ r, unsigned *counter) {
    const int tid = threadIdx.x;
    const double th = r[0] / r[2];
    double a = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + tid; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double d = w[i] - th * psi[i];
        a = fma(d, d, a);
    }
    a = warp_sum<double>(a);
    __shared__ double red[8];
    if ((tid & 31) == 0) red[tid >> 5] = a;
    __syncthreads();
    if (tid == 0) {
        double t = 0.0;
        for (int q = 0; q < 8; ++q) t += red[q];
        part[blockIdx.x] = t;
    }
    if (!last_block(counter) || tid != 0) return;
    double t = 0.0;
    for (int bb = 0; bb < (int)gridDim.x; ++bb) t += part[bb];
    r[3] = t;
    *counter = 0u;
}

// per-eigenvector scratch row: s[m] followed by three factor bands of m
inline int svec_stride(int cap) { return 4 * (cap + 1); }

int ensure_lanczos(Ctx &c, int64_t n, int cap, bool mixed) {
    DevLanczos &z = c.lz;
    // reuse only buffers shaped for this mode: the FP64 method needs a whole
    // FP64 basis in V, the mixed one an FP32 basis in V32
    if (z.V && z.n == n && z.cap >= cap && (mixed ? (z.V32 != nullptr) : z.full64)) return NSS_OK;
    lanczos_release(c);
    z.n = n;
    z.cap = cap;
    if (mixed) {
        NSS_CUDA_TRY(c, ctx_alloc(c, &z.V32, (size_t)(cap + 1) * n));
        NSS_CUDA_TRY(c, ctx_alloc(c, &z.w32, (size_t)n));
        NSS_CUDA_TRY(c, ctx_alloc(c, &z.V, (size_t)n));   // FP64 refinement scratch
        z.full64 = false;
    } else {
        NSS_CUDA_TRY(c, ctx_alloc(c, &z.V, (size_t)(cap + 1) * n));
        z.full64 = true;
    }
    NSS_CUDA_TRY(c, ctx_alloc(c, &z.w, (size_t)n));
    NSS_CUDA_TRY(c, ctx_alloc(c, &z.evecs, (size_t)4 * n));
    // scalars, two projection-coefficient vectors, restart scratch alpha/beta
    NSS_CUDA_TRY(c, ctx_alloc(c, &z.scal, (size_t)S_NSCAL + 4 * (cap + 2) + 8));
    NSS_CUDA_TRY(c, ctx_alloc(c, &z.part, (size_t)(cap + 2) * NBLK));
    NSS_CUDA_TRY(c, ctx_alloc(c, &z.counter, 4));
    NSS_CUDA_TRY(c, ctx_alloc(c, &z.alpha, (size_t)cap + 1));
    NSS_CUDA_TRY(c, ctx_alloc(c, &z.beta, (size_t)cap + 1));
    NSS_CUDA_TRY(c, ctx_alloc(c, &z.theta, 8));
    NSS_CUDA_TRY(c, ctx_alloc(c, &z.resid, 8));
    NSS_CUDA_TRY(c, ctx_alloc(c, &z.svec, (size_t)4 * svec_stride(cap)));
    NSS_CUDA_TRY(c, ctx_alloc(c, &z.flags, F_NFLAGS));
    NSS_CUDA_TRY(c, cudaMallocHost((void **)&z.h_flags, 2 * F_NFLAGS * sizeof(int)));
    NSS_CUDA_TRY(c, cudaMemsetAsync(z.counter, 0, 4 * sizeof(unsigned), c.stream));
    return NSS_OK;
}

template <class T>
int hv_t(Ctx &c, const T *v, T *hv, const int *stop);
template <>
int hv_t<double>(Ctx &c, const double *v, double *hv, const int *stop) { return hv_device(c, v, hv, stop); }
template <>
int hv_t<float>(Ctx &c, const float *v, float *hv, const int *stop) { return hv_device_fp32(c, v, hv, stop); }

// The Lanczos iterations on a basis of type T; leaves theta (Ritz values),
// svec (their T-eigenvectors) and the Ritz vectors (FP64) in c.lz.
template <class T>
int run_lanczos(Ctx &c, T *V, T *w, int neigen, int mmax, double tol, uint64_t seed, int *numop_out,
                int *m_out) {
    DevLanczos &z = c.lz;
    const int64_t n = c.sb.n;
    const int cap = z.cap;
    double *h1 = z.scal + S_NSCAL, *h2 = h1 + (cap + 2);
    double *rs_alpha = h2 + (cap + 2), *rs_beta = rs_alpha + (cap + 2);
    const int sstride = svec_stride(cap);
    cudaStream_t st = c.stream;
    NSS_CUDA_TRY(c, cudaMemsetAsync(z.flags, 0, F_NFLAGS * sizeof(int), st));
    NSS_CUDA_TRY(c, cudaMemsetAsync(z.beta, 0, (cap + 1) * sizeof(double), st));
    const int vb = 608;   // 4 CTAs per SM for elementwise kernels
    uint64_t restarts = 0;
    ++c.launches;
    k_random<T><<<vb, 256, 0, st>>>(V, n, seed, restarts);
    ++c.launches;
    k_normalize<T><<<1, 1024, 0, st>>>(V, n);
    int m_done = 1, numop_ = 0, rc = NSS_OK;
    bool converged = false;
    const size_t dots_smem = (size_t)(cap + 2) * sizeof(double) + SUB * sizeof(T);
    const size_t upd_smem = (size_t)(cap + 2) * sizeof(double);
    if (dots_smem > 48 * 1024)
        cudaFuncSetAttribute(k_dots<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dots_smem);
    if (upd_smem > 48 * 1024)
        cudaFuncSetAttribute(k_update<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)upd_smem);
    // Chunks of CHECK iterations, each followed by the convergence test and
    // a copy of the flags into one of two pinned slots; one chunk runs ahead
    // of the host's read of the previous one, so the stream never idles.
    // Kernels of a chunk enqueued after convergence exit at once (stop flag).
    cudaEvent_t evs[2];
    cudaEventCreateWithFlags(&evs[0], cudaEventDisableTiming);
    cudaEventCreateWithFlags(&evs[1], cudaEventDisableTiming);
    auto enqueue_chunk = [&](int j0, int slot) -> int {
        const int jend = std::min(mmax, j0 + CHECK);
        for (int jj = j0; jj < jend; ++jj) {
            const int m = jj + 1;
            int r2 = hv_t<T>(c, V + (int64_t)jj * n, w, z.flags + F_STOP);
            if (r2) return -1;
            c.launches += 5;
            k_alpha<T><<<NBLK, 256, 0, st>>>(V + (int64_t)jj * n, w, n, z.part, z.scal, z.counter, z.flags);
            k_dots<T><<<NBLK, 256, dots_smem, st>>>(V, m, w, n, z.part, h1, z.scal, z.counter, z.flags, 0, 1,
                                                    z.beta);
            k_update<T><<<NBLK, 256, upd_smem, st>>>(V, m, w, n, h1, z.part, z.scal, z.counter, z.flags,
                                                     z.alpha, z.beta, 0);
            k_dots<T><<<NBLK, 256, dots_smem, st>>>(V, m, w, n, z.part, h2, z.scal, z.counter, z.flags, 1, 0,
                                                    z.beta);
            k_update<T><<<NBLK, 256, upd_smem, st>>>(V, m, w, n, h2, z.part, z.scal, z.counter, z.flags,
                                                     z.alpha, z.beta, 1);
            if (m < mmax) {
                ++c.launches;
                k_next<T><<<vb, 256, 0, st>>>(V + (int64_t)m * n, w, n, z.flags, z.alpha, z.beta, jj);
            }
        }
        ++c.launches;
        k_tridiag<<<1, 128, 0, st>>>(z.alpha, z.beta, jend, neigen, tol, z.theta, z.resid, z.svec, sstride,
                                     z.flags, mmax, n);
        cudaMemcpyAsync(z.h_flags + slot * F_NFLAGS, z.flags, F_NFLAGS * sizeof(int), cudaMemcpyDeviceToHost, st);
        cudaEventRecord(evs[slot], st);
        return jend;
    };
    int slot = 0;
    int pend_end = enqueue_chunk(0, slot);
    bool capped = false;
    while (pend_end >= 0) {
        const int next_end = (pend_end < mmax) ? enqueue_chunk(pend_end, slot ^ 1) : -2;
        if (next_end == -1) { rc = NSS_ERR_CUDA; break; }
        cudaError_t ce = cudaEventSynchronize(evs[slot]);
        if (ce != cudaSuccess) { c.err = cudaGetErrorString(ce); rc = NSS_ERR_CUDA; break; }
        const int *f = z.h_flags + slot * F_NFLAGS;
        m_done = f[F_M];
        if (f[F_STOP] == 1) { converged = true; break; }
        if (f[F_STOP] == 3) { capped = true; break; }
        if (f[F_STOP] == 2) {
            // invariant subspace without convergence: continue from a random
            // vector orthogonal to V (the chunk run ahead has already exited)
            NSS_CUDA_TRY(c, cudaStreamSynchronize(st));
            ++restarts;
            T *vn = V + (int64_t)m_done * n;
            ++c.launches;
            k_random<T><<<vb, 256, 0, st>>>(vn, n, seed, restarts);
            NSS_CUDA_TRY(c, cudaMemsetAsync(z.flags, 0, F_NFLAGS * sizeof(int), st));
            for (int pass = 0; pass < 2; ++pass) {
                NSS_CUDA_TRY(c, cudaMemsetAsync(z.scal + S_ALPHA, 0, sizeof(double), st));
                c.launches += 2;
                k_dots<T><<<NBLK, 256, dots_smem, st>>>(V, m_done, vn, n, z.part, h1, z.scal, z.counter, z.flags,
                                                        0, 0, z.beta);
                k_update<T><<<NBLK, 256, upd_smem, st>>>(V, m_done, vn, n, h1, z.part, z.scal, z.counter, z.flags,
                                                         rs_alpha, rs_beta, 0);
            }
            ++c.launches;
            k_normalize<T><<<1, 1024, 0, st>>>(vn, n);
            NSS_CUDA_TRY(c, cudaMemsetAsync(z.beta + (m_done - 1), 0, sizeof(double), st));
            NSS_CUDA_TRY(c, cudaMemsetAsync(z.flags, 0, F_NFLAGS * sizeof(int), st));
            slot = 0;
            pend_end = enqueue_chunk(m_done, slot);
            continue;
        }
        if (next_end < 0) { capped = true; break; }
        slot ^= 1;
        pend_end = next_end;
    }
    cudaStreamSynchronize(st);
    cudaEventDestroy(evs[0]);
    cudaEventDestroy(evs[1]);
    if (rc) return rc;
    (void)capped;
    numop_ = m_done;
    *numop_out = numop_;
    *m_out = m_done;
    if (!converged) {
        c.err = "nss_eigh: no convergence within nitermax=" + std::to_string(mmax) + " iterations";
        return NSS_ERR_NOCONV;
    }
    const int ne = (int)std::min<int64_t>(neigen, m_done);
    ++c.launches;
    k_ritz<T><<<NBLK, 256, (size_t)ne * m_done * sizeof(double), st>>>(V, m_done, n, z.svec, sstride, ne, z.evecs);
    for (int e = 0; e < ne; ++e) {
        ++c.launches;
        k_normalize<double><<<1, 1024, 0, st>>>(z.evecs + (int64_t)e * n, n);
    }
    NSS_CUDA_TRY(c, cudaGetLastError());
    return NSS_OK;
}

}  // namespace

void lanczos_release(Ctx &c) {
    DevLanczos &z = c.lz;
    void *ptrs[] = {z.V, z.w, z.V32, z.w32, z.evecs, z.scal, z.part, z.counter, z.alpha, z.beta,
                    z.theta, z.resid, z.svec, z.flags};
    for (void *p : ptrs) ctx_free(c, p);
    if (z.h_flags) cudaFreeHost(z.h_flags);
    z = DevLanczos{};
}

int lanczos_eigh(Ctx &c, int neigen, int nitermax, double tol, uint64_t seed, int precision,
                 double *evals_host, int *numop) {
    DevSb &s = c.sb;
    if (!s.valid) { c.err = "nss_eigh: no superblock uploaded"; return NSS_ERR_STATE; }
    const int64_t n = s.n;
    if (neigen < 1 || neigen > 4) { c.err = "nss_eigh: neigen must be in [1,4]"; return NSS_ERR_INVALID; }
    if (neigen > n) neigen = (int)n;
    if (nitermax <= 0) nitermax = 512;
    int mmax = (int)std::min<int64_t>(n, nitermax);
    if (mmax < neigen) mmax = neigen;
    if (tol <= 0.0) tol = 1e-15;
    const bool mixed = precision == NSS_PREC_MIXED;
    int rc = ensure_lanczos(c, n, mmax + 1, mixed);
    if (rc) return rc;
    DevLanczos &z = c.lz;
    cudaStream_t st = c.stream;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, st);
    int numop_ = 0, m_done = 0;
    if (!mixed) {
        rc = run_lanczos<double>(c, z.V, z.w, neigen, mmax, tol, seed, &numop_, &m_done);
    } else {
        rc = run_lanczos<float>(c, z.V32, z.w32, neigen, mmax, std::max(tol, MIXED_TOL), seed, &numop_, &m_done);
    }
    const int ne = (int)std::min<int64_t>(neigen, std::max(m_done, 1));
    if (!rc && mixed) {
        // FP64 refinement of each eigenvalue: theta = psi.H.psi / psi.psi with
        // the FP64 H*psi, and the FP64 residual ||H psi - theta psi||.
        double *r = z.scal + S_NSCAL + 4 * (z.cap + 2);   // 8 refinement slots
        for (int e = 0; e < ne; ++e) {
            const double *psi = z.evecs + (int64_t)e * n;
            rc = hv_device(c, psi, z.w);
            ++numop_;
            if (rc) break;
            c.launches += 2;
            k_rq<<<NBLK, 256, 0, st>>>(psi, z.w, n, z.part, r, z.counter);
            k_resid<<<NBLK, 256, 0, st>>>(psi, z.w, n, z.part, r, z.counter);
            double hr[4];
            NSS_CUDA_TRY(c, cudaMemcpyAsync(hr, r, 4 * sizeof(double), cudaMemcpyDeviceToHost, st));
            NSS_CUDA_TRY(c, cudaStreamSynchronize(st));
            const double th = hr[0] / hr[2];
            z.last_resid[e] = std::sqrt(std::max(hr[3], 0.0));
            NSS_CUDA_TRY(c, cudaMemcpyAsync(z.theta + e, &th, sizeof(double), cudaMemcpyHostToDevice, st));
        }
    }
    cudaEventRecord(e1, st);
    cudaError_t ce = cudaStreamSynchronize(st);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    if (ce != cudaSuccess) { c.err = cudaGetErrorString(ce); return NSS_ERR_CUDA; }
    if (mixed && c.sb.d_tc_err) {
        int tc_err = 0;
        NSS_CUDA_TRY(c, cudaMemcpy(&tc_err, c.sb.d_tc_err, sizeof(int), cudaMemcpyDeviceToHost));
        if (tc_err) {
            c.err = "nss_eigh: a tensor-core pipeline wait timed out (results discarded)";
            return NSS_ERR_CUDA;
        }
    }
    if (evals_host) NSS_CUDA_TRY(c, cudaMemcpy(evals_host, z.theta, ne * sizeof(double), cudaMemcpyDeviceToHost));
    c.last_ms_eigh = ms;
    c.last_numop = numop_;
    z.last_iters = m_done;
    z.neigen_done = ne;
    if (numop) *numop = numop_;
    return NSS_OK;
}

}  // namespace nss
