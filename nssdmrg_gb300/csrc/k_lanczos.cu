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

// device scalar slots (Ctx::lz.scal)
enum { S_WW = 0, S_BB = 1, S_ALPHA = 2, S_NSCAL = 4 };
// device flag slots (Ctx::lz.flags)
enum { F_STOP = 0, F_PASS2 = 1, F_M = 2, F_CONV = 3, F_BREAK = 4, F_NFLAGS = 8 };

__device__ __forceinline__ double warp_sum(double x) {
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
__global__ void k_random(double *x, int64_t n, uint64_t seed, uint64_t stream) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        uint64_t r = splitmix64(seed ^ splitmix64(stream * 0x632BE59BD9B4E019ull + (uint64_t)i));
        x[i] = 2.0 * ((double)(r >> 11) * (1.0 / 9007199254740992.0)) - 1.0;
    }
}

// h[l] = V[l] . w for l < m, and h[m] = w . w (written to scal[slot_ww]).
// Grid-wide reduction by the last CTA to finish.
// With threeterm != 0 the recurrence step w -= alpha v_{m-1} + beta v_{m-2}
// (alpha from scal[S_ALPHA], beta = betas[m-2]) is applied to w first and
// the updated w is written back.
__global__ void __launch_bounds__(256) k_dots(const double *__restrict__ V, int m, double *__restrict__ w,
                                              int64_t n, double *__restrict__ part, double *__restrict__ h,
                                              double *__restrict__ scal, unsigned *counter, const int *flags,
                                              int pass2, int threeterm, const double *__restrict__ betas) {
    if (flags[F_STOP] || (pass2 && !flags[F_PASS2])) return;
    const double a3 = threeterm ? scal[S_ALPHA] : 0.0;
    const double b3 = (threeterm && m >= 2) ? betas[m - 2] : 0.0;
    const double *vj = V + (int64_t)(m - 1) * n;
    const double *vjm = (m >= 2) ? V + (int64_t)(m - 2) * n : V;
    extern __shared__ double sm[];
    double *ws = sm;             // [SUB]
    double *acc = sm + SUB;      // [m+1]
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int l = tid; l <= m; l += 256) acc[l] = 0.0;
    const int64_t chunk = (n + gridDim.x - 1) / gridDim.x;
    const int64_t i0 = blockIdx.x * chunk, i1 = min(n, i0 + chunk);
    for (int64_t s0 = i0; s0 < i1; s0 += SUB) {
        const int len = (int)min((int64_t)SUB, i1 - s0);
        __syncthreads();
        if (threeterm) {
            for (int e = tid; e < len; e += 256) {
                double x = w[s0 + e] - a3 * vj[s0 + e];
                if (m >= 2) x -= b3 * vjm[s0 + e];
                ws[e] = x;
                w[s0 + e] = x;
            }
        } else {
            for (int e = tid; e < len; e += 256) ws[e] = w[s0 + e];
        }
        __syncthreads();
        for (int l = warp; l <= m; l += 8) {
            const double *vl = (l < m) ? V + (int64_t)l * n + s0 : nullptr;
            double p = 0.0;
            if (l < m)
                for (int e = lane; e < len; e += 32) p = fma(vl[e], ws[e], p);
            else
                for (int e = lane; e < len; e += 32) p = fma(ws[e], ws[e], p);
            p = warp_sum(p);
            if (lane == 0) acc[l] += p;
        }
    }
    __syncthreads();
    for (int l = tid; l <= m; l += 256) part[(int64_t)l * gridDim.x + blockIdx.x] = acc[l];
    __threadfence();
    __shared__ unsigned last;
    if (tid == 0) last = (atomicAdd(counter, 1u) == gridDim.x - 1);
    __syncthreads();
    if (!last) return;
    __threadfence();
    for (int l = warp; l <= m; l += 8) {
        double p = 0.0;
        for (int b = lane; b < (int)gridDim.x; b += 32) p += part[(int64_t)l * gridDim.x + b];
        p = warp_sum(p);
        if (lane == 0) {
            if (l < m) h[l] = p;
            else scal[S_WW] = p;
        }
    }
    if (tid == 0) *counter = 0u;
}

// alpha = v . w  (grid reduction by the last CTA) -> scal[S_ALPHA]
__global__ void __launch_bounds__(256) k_alpha(const double *__restrict__ v, const double *__restrict__ w, int64_t n,
                                               double *__restrict__ part, double *__restrict__ scal,
                                               unsigned *counter, const int *flags) {
    if (flags[F_STOP]) return;
    const int tid = threadIdx.x;
    double p = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + tid; i < n; i += (int64_t)gridDim.x * blockDim.x)
        p = fma(v[i], w[i], p);
    p = warp_sum(p);
    __shared__ double red[8];
    if ((tid & 31) == 0) red[tid >> 5] = p;
    __syncthreads();
    if (tid == 0) {
        double t = 0.0;
        for (int q = 0; q < 8; ++q) t += red[q];
        part[blockIdx.x] = t;
    }
    __threadfence();
    __shared__ unsigned last;
    if (tid == 0) last = (atomicAdd(counter, 1u) == gridDim.x - 1);
    __syncthreads();
    if (!last || tid != 0) return;
    __threadfence();
    double t = 0.0;
    for (int b = 0; b < (int)gridDim.x; ++b) t += part[b];
    scal[S_ALPHA] = t;
    *counter = 0u;
}

// w -= V_m h ; beta^2 = w.w ; the last CTA records alpha_j and beta_j.
__global__ void __launch_bounds__(256) k_update(const double *__restrict__ V, int m, double *__restrict__ w,
                                                int64_t n, const double *__restrict__ h, double *__restrict__ part,
                                                double *__restrict__ scal, unsigned *counter, int *flags,
                                                double *alpha, double *beta, int pass2) {
    if (flags[F_STOP] || (pass2 && !flags[F_PASS2])) return;
    extern __shared__ double hs[];
    const int tid = threadIdx.x;
    for (int l = tid; l < m; l += 256) hs[l] = h[l];
    __syncthreads();
    double ss = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + tid; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double x = w[i];
        for (int l = 0; l < m; ++l) x = fma(-V[(int64_t)l * n + i], hs[l], x);
        w[i] = x;
        ss = fma(x, x, ss);
    }
    ss = warp_sum(ss);
    __shared__ double red[8];
    if ((tid & 31) == 0) red[tid >> 5] = ss;
    __syncthreads();
    if (tid == 0) {
        double t = 0.0;
        for (int q = 0; q < 8; ++q) t += red[q];
        part[blockIdx.x] = t;
    }
    __threadfence();
    __shared__ unsigned last;
    if (tid == 0) last = (atomicAdd(counter, 1u) == gridDim.x - 1);
    __syncthreads();
    if (!last || tid != 0) return;
    __threadfence();
    double bb = 0.0;
    for (int b = 0; b < (int)gridDim.x; ++b) bb += part[b];
    const int j = m - 1;
    if (!pass2) {
        alpha[j] = scal[S_ALPHA] + hs[j];
        flags[F_PASS2] = (bb < 0.5 * scal[S_WW]) ? 1 : 0;
    } else {
        alpha[j] += hs[j];
    }
    scal[S_BB] = bb;
    beta[j] = sqrt(bb);
    *counter = 0u;
}

// v_{j+1} = w / beta_j, or flag a breakdown (invariant subspace).
__global__ void k_next(double *__restrict__ vnext, const double *__restrict__ w, int64_t n, const double *scal,
                       int *flags, const double *alpha, const double *beta, int j) {
    if (flags[F_STOP]) return;
    const double b = beta[j];
    // breakdown: beta below roundoff of the projected step
    const double scale = fmax(fabs(alpha[j]), j > 0 ? beta[j - 1] : 0.0);
    if (!(b > 1e-13 * fmax(scale, 1e-300))) {
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            flags[F_BREAK] = j + 1;
            flags[F_STOP] = 2;
        }
        return;
    }
    const double inv = 1.0 / b;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        vnext[i] = w[i] * inv;
    if (blockIdx.x == 0 && threadIdx.x == 0) flags[F_M] = j + 2;
}

// x <- x / ||x|| (one CTA per launch is enough for start vectors);
// blockDim.x <= 1024, so at most 32 warp partial sums
__global__ void __launch_bounds__(1024) k_normalize(double *x, int64_t n) {
    __shared__ double red[32];
    double ss = 0.0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) ss = fma(x[i], x[i], ss);
    ss = warp_sum(ss);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = ss;
    __syncthreads();
    double t = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) t += red[q];
    const double inv = 1.0 / sqrt(t);
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) x[i] *= inv;
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

// Eigenvalues theta[0..ne) of T_m by 64-way multisection (one 64-thread group
// per eigenvalue), eigenvectors s by inverse iteration, residual estimates
// beta_{m-1} |s_{m-1}| and the convergence flag.
__global__ void __launch_bounds__(256) k_tridiag(const double *alpha, const double *beta, int m, int ne,
                                                 double tol, double *theta, double *resid, double *svec,
                                                 int sstride, int *flags, int final_pass) {
    __shared__ double lo_s, hi_s;
    __shared__ double xs[4][65];
    __shared__ int cs[4][65];
    __shared__ double ab[4][2];
    const int tid = threadIdx.x, grp = tid >> 6, g = tid & 63;
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
    for (int e0 = 0; e0 < ne; e0 += 4) {
        const int e = e0 + grp;
        const bool active = e < ne && e < m;
        if (g == 0) { ab[grp][0] = lo_s; ab[grp][1] = hi_s; }
        __syncthreads();
        for (int round = 0; round < 12; ++round) {
            double a = ab[grp][0], b = ab[grp][1];
            bool done = !(b - a > 4e-16 * fmax(fabs(a), fabs(b)) + 1e-300);
            if (active && !done) {
                double x = a + (b - a) * (double)(g + 1) / 65.0;
                xs[grp][g] = x;
                cs[grp][g] = sturm_count(alpha, beta, m, x);
            }
            __syncthreads();
            if (active && !done && g == 0) {
                // first point whose count exceeds e brackets eigenvalue e
                int t = 0;
                while (t < 64 && cs[grp][t] <= e) ++t;
                ab[grp][0] = (t == 0) ? a : xs[grp][t - 1];
                ab[grp][1] = (t == 64) ? b : xs[grp][t];
            }
            __syncthreads();
        }
        if (active && g == 0) theta[e] = 0.5 * (ab[grp][0] + ab[grp][1]);
        __syncthreads();
    }
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
        if (!final_pass && conv >= ne) flags[F_STOP] = 1;
    }
}

// Ritz vectors: out[e] = sum_l V[l] s_e[l]
__global__ void __launch_bounds__(256) k_ritz(const double *__restrict__ V, int m, int64_t n,
                                              const double *__restrict__ svec, int sstride, int ne,
                                              double *__restrict__ out) {
    extern __shared__ double ss[];   // [ne][m]
    for (int t = threadIdx.x; t < ne * m; t += blockDim.x) ss[t] = svec[(int64_t)(t / m) * sstride + (t % m)];
    __syncthreads();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double acc[4] = {0, 0, 0, 0};
        for (int l = 0; l < m; ++l) {
            const double v = V[(int64_t)l * n + i];
            for (int e = 0; e < ne && e < 4; ++e) acc[e] = fma(v, ss[e * m + l], acc[e]);
        }
        for (int e = 0; e < ne && e < 4; ++e) out[(int64_t)e * n + i] = acc[e];
    }
}

// per-eigenvector scratch row: s[m] followed by three factor bands of m
inline int svec_stride(int cap) { return 4 * (cap + 1); }

int ensure_lanczos(Ctx &c, int64_t n, int cap, int neigen) {
    DevLanczos &z = c.lz;
    if (z.V && z.n == n && z.cap >= cap) return NSS_OK;
    lanczos_release(c);
    z.n = n;
    z.cap = cap;
    NSS_CUDA_TRY(c, ctx_alloc(c, &z.V, (size_t)(cap + 1) * n));
    NSS_CUDA_TRY(c, ctx_alloc(c, &z.w, (size_t)n));
    NSS_CUDA_TRY(c, ctx_alloc(c, &z.evecs, (size_t)4 * n));
    // scalars, two projection-coefficient vectors, restart scratch alpha/beta
    NSS_CUDA_TRY(c, ctx_alloc(c, &z.scal, (size_t)S_NSCAL + 4 * (cap + 2)));
    NSS_CUDA_TRY(c, ctx_alloc(c, &z.part, (size_t)(cap + 2) * NBLK));
    NSS_CUDA_TRY(c, ctx_alloc(c, &z.counter, 4));
    NSS_CUDA_TRY(c, ctx_alloc(c, &z.alpha, (size_t)cap + 1));
    NSS_CUDA_TRY(c, ctx_alloc(c, &z.beta, (size_t)cap + 1));
    NSS_CUDA_TRY(c, ctx_alloc(c, &z.theta, 8));
    NSS_CUDA_TRY(c, ctx_alloc(c, &z.resid, 8));
    NSS_CUDA_TRY(c, ctx_alloc(c, &z.svec, (size_t)4 * svec_stride(cap)));
    NSS_CUDA_TRY(c, ctx_alloc(c, &z.flags, F_NFLAGS));
    NSS_CUDA_TRY(c, cudaMallocHost((void **)&z.h_flags, F_NFLAGS * sizeof(int)));
    NSS_CUDA_TRY(c, cudaMemsetAsync(z.counter, 0, 4 * sizeof(unsigned), c.stream));
    (void)neigen;
    return NSS_OK;
}

}  // namespace

void lanczos_release(Ctx &c) {
    DevLanczos &z = c.lz;
    void *ptrs[] = {z.V, z.w, z.evecs, z.scal, z.part, z.counter, z.alpha, z.beta,
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
    (void)precision;
    int rc = ensure_lanczos(c, n, mmax + 1, neigen);
    if (rc) return rc;
    DevLanczos &z = c.lz;
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
    k_random<<<vb, 256, 0, st>>>(z.V, n, seed, restarts);
    ++c.launches;
    k_normalize<<<1, 1024, 0, st>>>(z.V, n);
    int j = 0, m_done = 1, numop_ = 0;
    bool converged = false;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, st);
    const size_t dots_smem = (SUB + cap + 2) * sizeof(double);
    const size_t upd_smem = (cap + 2) * sizeof(double);
    if (dots_smem > 48 * 1024)
        cudaFuncSetAttribute(k_dots, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dots_smem);
    if (upd_smem > 48 * 1024)
        cudaFuncSetAttribute(k_update, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)upd_smem);
    while (!converged) {
        const int jend = std::min(mmax, j + CHECK);
        for (int jj = j; jj < jend; ++jj) {
            const int m = jj + 1;
            rc = hv_device(c, z.V + (int64_t)jj * n, z.w);
            if (rc) return rc;
            ++c.launches;
            k_alpha<<<NBLK, 256, 0, st>>>(z.V + (int64_t)jj * n, z.w, n, z.part, z.scal, z.counter, z.flags);
            ++c.launches;
            k_dots<<<NBLK, 256, dots_smem, st>>>(z.V, m, z.w, n, z.part, h1, z.scal, z.counter, z.flags, 0, 1,
                                                 z.beta);
            ++c.launches;
            k_update<<<NBLK, 256, upd_smem, st>>>(z.V, m, z.w, n, h1, z.part, z.scal, z.counter, z.flags,
                                                  z.alpha, z.beta, 0);
            ++c.launches;
            k_dots<<<NBLK, 256, dots_smem, st>>>(z.V, m, z.w, n, z.part, h2, z.scal, z.counter, z.flags, 1, 0,
                                                 z.beta);
            ++c.launches;
            k_update<<<NBLK, 256, upd_smem, st>>>(z.V, m, z.w, n, h2, z.part, z.scal, z.counter, z.flags,
                                                  z.alpha, z.beta, 1);
            if (m < mmax)
                ++c.launches;
                k_next<<<vb, 256, 0, st>>>(z.V + (int64_t)m * n, z.w, n, z.scal, z.flags, z.alpha, z.beta, jj);
        }
        NSS_CUDA_TRY(c, cudaGetLastError());
        NSS_CUDA_TRY(c, cudaMemcpyAsync(z.h_flags, z.flags, F_NFLAGS * sizeof(int), cudaMemcpyDeviceToHost, st));
        NSS_CUDA_TRY(c, cudaStreamSynchronize(st));
        // iterations that ran: up to the breakdown step, or the whole chunk
        int ran = z.h_flags[F_STOP] == 2 ? z.h_flags[F_BREAK] : jend;
        numop_ += ran - j;
        j = ran;
        m_done = j;
        const bool full = (m_done >= mmax) || (m_done >= n);
        ++c.launches;
        k_tridiag<<<1, 256, 0, st>>>(z.alpha, z.beta, m_done, neigen, tol, z.theta, z.resid, z.svec, sstride,
                                     z.flags, full ? 1 : 0);
        NSS_CUDA_TRY(c, cudaMemcpyAsync(z.h_flags, z.flags, F_NFLAGS * sizeof(int), cudaMemcpyDeviceToHost, st));
        NSS_CUDA_TRY(c, cudaStreamSynchronize(st));
        const int conv = z.h_flags[F_CONV];
        if (conv >= neigen || m_done >= n) { converged = true; break; }
        if (m_done >= mmax) break;
        if (z.h_flags[F_STOP] == 2) {
            // invariant subspace: continue from a random vector orthogonal to V
            ++restarts;
            double *vn = z.V + (int64_t)m_done * n;
            ++c.launches;
            k_random<<<vb, 256, 0, st>>>(vn, n, seed, restarts);
            NSS_CUDA_TRY(c, cudaMemsetAsync(z.flags, 0, F_NFLAGS * sizeof(int), st));
            for (int pass = 0; pass < 2; ++pass) {
                NSS_CUDA_TRY(c, cudaMemsetAsync(z.scal + S_ALPHA, 0, sizeof(double), st));
                ++c.launches;
                k_dots<<<NBLK, 256, dots_smem, st>>>(z.V, m_done, vn, n, z.part, h1, z.scal, z.counter, z.flags, 0,
                                                     0, z.beta);
                // reuse k_update on the candidate vector; alpha/beta slots of
                // m_done-1 are restored below
                ++c.launches;
                k_update<<<NBLK, 256, upd_smem, st>>>(z.V, m_done, vn, n, h1, z.part, z.scal, z.counter, z.flags,
                                                      rs_alpha, rs_beta, 0);
            }
            ++c.launches;
            k_normalize<<<1, 1024, 0, st>>>(vn, n);
            NSS_CUDA_TRY(c, cudaMemsetAsync(z.beta + (m_done - 1), 0, sizeof(double), st));
            NSS_CUDA_TRY(c, cudaMemsetAsync(z.flags, 0, F_NFLAGS * sizeof(int), st));
        }
    }
    if (!converged) {
        c.err = "nss_eigh: no convergence within nitermax=" + std::to_string(nitermax) + " iterations";
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        return NSS_ERR_NOCONV;
    }
    const int ne = std::min<int64_t>(neigen, m_done);
    ++c.launches;
    k_ritz<<<NBLK, 256, (size_t)ne * m_done * sizeof(double), st>>>(z.V, m_done, n, z.svec, sstride, ne, z.evecs);
    for (int e = 0; e < ne; ++e) {
        ++c.launches;
        k_normalize<<<1, 1024, 0, st>>>(z.evecs + (int64_t)e * n, n);
    }
    cudaEventRecord(e1, st);
    NSS_CUDA_TRY(c, cudaGetLastError());
    if (evals_host) NSS_CUDA_TRY(c, cudaMemcpyAsync(evals_host, z.theta, ne * sizeof(double), cudaMemcpyDeviceToHost, st));
    NSS_CUDA_TRY(c, cudaStreamSynchronize(st));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    c.last_ms_eigh = ms;
    c.last_numop = numop_;
    z.neigen_done = ne;
    if (numop) *numop = numop_;
    return NSS_OK;
}

}  // namespace nss
