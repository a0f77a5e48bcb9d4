// Lanczos eigensolver for the lowest eigenpairs of H_sb, on the GPU with the
// small tridiagonal problem on the host.
//
// Replaces SciFortran sp_eigh (ARPACK, called at src/DMRG_SUPERBLOCK.f90:
// 394-425) for the direct mode.  Algorithm: Lanczos with full
// reorthogonalisation -- the three-term recurrence first, then one classical
// Gram-Schmidt projection of the (small) residual against the whole basis,
// and a second projection only when that one removes more than half of the
// residual -- the whole Krylov basis kept resident in HBM (no restarts), and a
// convergence test every CHECK steps on the tridiagonal matrix T_m:
// residual beta_m |s_m| <= tol |theta| for each wanted Ritz pair, the ARPACK
// criterion.  Breakdown (beta ~ 0, invariant subspace) restarts with a fresh
// random vector orthogonal to the basis.  Eigenvectors are gauge-dependent,
// so parity with the reference is on eigenvalues and on what the RDM derives
// from them.
//
// Per iteration j (m = j+1 basis vectors) two kinds of launch:
//   sector H*psi   w = H v_j                      (k_hv_* kernels)
//   k_orth         one cooperative launch, one CTA per SM, each CTA owning a
//                  contiguous slice of the rows; grid barriers separate
//                    alpha = v_j . w
//                    w -= alpha v_j + beta_{j-1} v_{j-1};  h = V_m^T w, ww = w.w
//                    w -= V_m h, beta^2 = w.w  (again if beta^2 < ww/2)
//                    v_{j+1} = w / beta, or the breakdown flag
// Projecting the raw H v_j instead (one pass) lets the orthogonality error
// grow by ||H||/beta per step; the recurrence-first order keeps it at 1e-15.
// Every grid-level sum is reduced by every CTA in the same fixed order, so
// all CTAs hold bitwise identical scalars and take the same branches.
//
// The tridiagonal problem (m <= a few hundred) is a chain of dependent FP64
// operations, which GB300's narrow FP64 pipe runs slowly on one SM; it is
// solved on the host (host_tridiag.cpp) from alpha/beta that k_orth writes
// into host-mapped memory, while the GPU already runs the next CHECK
// iterations.  On convergence the host raises a stop request in host-mapped
// memory; the next k_orth publishes it as the device stop flag, and every
// kernel still queued returns at once.  The decision depends only on the
// checked chunk, so results do not depend on that timing.
//
// Precision modes.  The kernels are templates over the type T of the Krylov
// vectors.  T = double is the plain method: FP64 everywhere.  T = float is
// the mixed method: H*psi in FP32 (k_hv_fp32 on CUDA cores, and the
// split-TF32 tensor-core sector GEMM k_sector_mma where the plan routes
// large sectors to it), the basis and the
// projections in FP32 with FP64 block partial sums, while alpha/beta, the
// tridiagonal eigensolve and the Ritz vector stay FP64; it runs to a relative
// residual of MIXED_TOL, and the energy is then refined in FP64 as the
// Rayleigh quotient psi.H.psi of the FP64 Ritz vector with the FP64 H*psi
// (error quadratic in the vector error: |dE|/|E| ~ 1e-13 at MIXED_TOL =
// 1e-7), whose FP64 residual ||H psi - E psi|| is reported.  On GB300 the
// FP64 pipe runs at about 1/70 of the FP32 one (1.06 against 78 TFLOP/s
// measured), which is what the mixed method buys.
#include "device.cuh"
#include "host_tridiag.hpp"
#include "hv_tile.cuh"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

namespace nss {

namespace {

constexpr int NBLK = 304;         // grid of the restart-path reductions
constexpr int CHECK = 4;          // convergence test period (iterations)
constexpr int SUB = 1024;         // rows staged per shared-memory sub-chunk
constexpr double MIXED_TOL = 1e-7;

// residual target of the FP32 phase (env NSS_MIXED_TOL overrides, clamped to
// [1e-9, 1e-2]); the anchored FP64 phase then takes the vector to `tol`
double mixed_tol() {
    static const double v = [] {
        const char *e = std::getenv("NSS_MIXED_TOL");
        if (!e) return MIXED_TOL;
        const double x = std::atof(e);
        return x < 1e-9 ? 1e-9 : (x > 1e-2 ? 1e-2 : x);
    }();
    return v;
}
// Raise a kernel's dynamic shared-memory limit on the current device to at
// least `bytes`.  The attribute belongs to the kernel, shared by every
// context of the process, so it only ever grows: a context sized for a
// smaller basis must not take the room a larger one was set up with.
inline cudaError_t allow_smem(const void *fn, size_t bytes) {
    if (bytes <= 48 * 1024) return cudaSuccess;
    static std::mutex mu;
    static std::map<std::pair<int, const void *>, size_t> done;
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(mu);
    size_t &cur = done[{dev, fn}];
    if (bytes <= cur) return cudaSuccess;
    const cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e == cudaSuccess) cur = bytes;
    return e;
}

constexpr int ORTH_THREADS = 512;
constexpr int ORTH_WARPS = ORTH_THREADS / 32;

// device scalar slots (Ctx::lz.scal)
enum { S_WW = 0, S_BB = 1, S_ALPHA = 2, S_NRM = 3, S_NSCAL = 4 };
// device flag slots (Ctx::lz.flags); the host-mapped mirror uses the same
// indices and one more word, F_NFLAGS, for the host's stop request
enum { F_STOP = 0, F_PASS2 = 1, F_M = 2, F_CONV = 3, F_BREAK = 4, F_HOST = 5, F_ERR = 6, F_NFLAGS = 8 };

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
__global__ void k_seti(int *p, int v) { *p = v; }

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

// Sum of the G per-CTA partials, by every thread of the last CTA (256
// threads): a serial loop over ~300 FP64 adds would cost ~20k cycles of
// dependent 64-cycle latency on this GPU.
__device__ __forceinline__ double lastblock_sum(const double *part, int G) {
    __shared__ double red_lb[8];
    double p = 0.0;
    for (int b = threadIdx.x; b < G; b += blockDim.x) p += part[b];
    p = warp_sum<double>(p);
    if ((threadIdx.x & 31) == 0) red_lb[threadIdx.x >> 5] = p;
    __syncthreads();
    double t = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) t += red_lb[q];
    __syncthreads();
    return t;
}

// Restart path only (a fresh start vector orthogonalised against the basis):
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
    if (!last_block(counter)) return;
    const double bb = lastblock_sum(part, gridDim.x);
    if (tid != 0) return;
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

// x <- x / ||x|| over the whole GPU: k_sumsq (FP64 partial sums, the last
// CTA writes 1 / ||x||), then k_scale.
template <class T>
__global__ void __launch_bounds__(256) k_sumsq(const T *__restrict__ x, int64_t n, double *__restrict__ part,
                                               double *__restrict__ inv, unsigned *counter) {
    const int tid = threadIdx.x;
    double a = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + tid; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double v = (double)x[i];
        a = fma(v, v, a);
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
    if (!last_block(counter)) return;
    const double t = lastblock_sum(part, gridDim.x);
    if (tid != 0) return;
    *inv = 1.0 / sqrt(t);
    *counter = 0u;
}

template <class T>
__global__ void __launch_bounds__(256) k_scale(T *__restrict__ x, int64_t n, const double *__restrict__ inv) {
    const double f = *inv;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        x[i] = (T)((double)x[i] * f);
}

// ---------------------------------------------------------------------------
// Fused orthogonalisation step (cooperative launch).
//
// Reductions are carried out in the basis type T: FP32 for the mixed
// method, FP64 for the plain one.  On GB300 an FP64 add or FMA occupies a
// warp's share of the FP64 pipe for 64 cycles (a division ~650), so FP64
// reduction trees inside the FP32 method would cost more than the FP32
// vector work they sum; FP32 sums are as accurate as the FP32 vectors and
// the FP32 products they add up.

struct OrthArgs {
    void *V, *w;                 // T*: basis [cap+1][n], work vector [n]
    int64_t n;
    int j, mmax, pstride;        // step, iteration cap, column stride of partials
    double *alpha, *beta;        // device tridiagonal coefficients
    void *part;                  // T*: per-CTA partials (five regions)
    unsigned *bar;               // grid barrier: arrival count, generation
    int *flags;                  // device flags
    double *h_alpha, *h_beta;    // host-mapped mirrors of alpha, beta
    int *h_flags;                // host-mapped flag mirror + stop request
    // anchored refinement (anc_u == nullptr: plain Lanczos), T* vectors: the
    // Krylov vectors are kept orthogonal to the anchor u and to ndefl
    // vectors defl[k*n..]; m_j = r . v_j (r = H u - theta0 u) goes to h_m[j]
    const void *anc_u, *anc_r, *defl;
    int ndefl;
    double *h_m;
    uint32_t spin;               // poll limit of the grid barriers (wait_limit)
    // replayed chunks (CUDA graph): the step is read from *jdev and advanced
    // by the kernel, and the new Lanczos vector is also written to vcur, the
    // fixed input of the next H*psi (null: step a.j, no copy)
    int *jdev;
    void *vcur;
};

constexpr int PA_COLS = 8;       // per-CTA values of the first phase (alpha, u.w, r.v, y_k.w)

// Grid-wide barrier for a cooperative launch (all CTAs resident).  The
// arrival counter only grows during a launch: barrier e of the launch waits
// for e*G arrivals (`epoch`, kept by each CTA), so there is no reset on the
// critical path; grid_exit zeroes the counter when the last CTA leaves.
// Bounded: a wait that runs out sets flags[F_ERR] and every later barrier
// returns false at once, so the kernel always ends.
__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ bool grid_sync(unsigned *bar, unsigned &epoch, int *err, uint32_t spin) {
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        int good = 1;
        epoch += gridDim.x;
        __threadfence();
        atomicAdd(bar, 1u);
        uint32_t it = 0;
        while (ld_acquire_u32(bar) < epoch) {
            if (++it > spin) { atomicExch(err, 1); good = 0; break; }
            if ((it & 255u) == 0 && *(volatile int *)err) { good = 0; break; }
        }
        ok = good;
    }
    __syncthreads();
    return ok != 0;
}

// every CTA calls this once when it leaves a launch that may use grid_sync
__device__ __forceinline__ void grid_exit(unsigned *bar) {
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(bar + 1, 1u) == gridDim.x - 1) {
            atomicExch(bar, 0u);
            atomicExch(bar + 1, 0u);
        }
    }
}

// leaving after a barrier that failed: the host learns of it through the
// mapped flag mirror at its next check, before it reads any result
__device__ __forceinline__ void fail_exit(unsigned *bar, int *h_flags) {
    if (threadIdx.x == 0) {
        h_flags[F_ERR] = 1;
        __threadfence_system();
    }
    grid_exit(bar);
}

// CTA sums of NV values at once (512 threads), valid in thread 0
template <class R, int NV>
__device__ __forceinline__ void block_sums(R (&v)[NV], R *scr) {
#pragma unroll
    for (int q = 0; q < NV; ++q) v[q] = warp_sum<R>(v[q]);
    __syncthreads();
    if ((threadIdx.x & 31) == 0)
#pragma unroll
        for (int q = 0; q < NV; ++q) scr[q * ORTH_WARPS + (threadIdx.x >> 5)] = v[q];
    __syncthreads();
    if (threadIdx.x < 32) {
#pragma unroll
        for (int q = 0; q < NV; ++q) {
            R t = threadIdx.x < ORTH_WARPS ? scr[q * ORTH_WARPS + threadIdx.x] : (R)0;
            v[q] = warp_sum<R>(t);
        }
    }
}

// p[i0] + p[i0 + stride] + ... (indices below end), added in that order;
// the loads go out eight at a time, so a sum over the partials of a grid
// costs one L2 round trip instead of one per term (an add waiting for its
// load stalls the warp's next load: the loop form issued them one by one)
template <class R>
__device__ __forceinline__ R strided_sum(const R *p, int i0, int end, int stride) {
    R t = (R)0;
    for (int b0 = i0; b0 < end; b0 += 8 * stride) {
        R v[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int b = b0 + q * stride;
            v[q] = b < end ? __ldcg(p + b) : (R)0;
        }
#pragma unroll
        for (int q = 0; q < 8; ++q) t += v[q];
    }
    return t;
}

// sums of the G per-CTA partials of NV columns p[q*G + b], same order in
// every CTA; warp q reduces column q, results broadcast through bc[]
template <class R, int NV>
__device__ __forceinline__ void grid_totals(const R *p, int G, R *bc, R (&out)[NV]) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (warp < NV) {
        R t = strided_sum<R>(p + (int64_t)warp * G, lane, G, 32);
        t = warp_sum<R>(t);
        if (lane == 0) bc[warp] = t;
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < NV; ++q) out[q] = bc[q];
}

// hs[l] = sum_b p[l*G + b] for l < ncol (four columns per warp in flight;
// all their loads issued before the first add)
template <class R>
__device__ __forceinline__ void grid_columns(const R *p, int G, int ncol, R *hs) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int l0 = warp; l0 < ncol; l0 += 4 * ORTH_WARPS) {
        R t[4] = {(R)0, (R)0, (R)0, (R)0};
        for (int b0 = lane; b0 < G; b0 += 8 * 32) {
            R v[4][8];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int l = l0 + u * ORTH_WARPS;
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    const int b = b0 + 32 * q;
                    v[u][q] = (l < ncol && b < G) ? __ldcg(p + (int64_t)l * G + b) : (R)0;
                }
            }
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
                for (int q = 0; q < 8; ++q) t[u] += v[u][q];
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const R s = warp_sum<R>(t[u]);
            const int l = l0 + u * ORTH_WARPS;
            if (lane == 0 && l < ncol) hs[l] = s;
        }
    }
}

// Reduce CW per-lane values over the 32 lanes of a warp at once (butterfly
// with exchange: 31 shuffles for all CW columns); lane L ends with the sum of
// column L % CW in d[0].
template <class R, int CW>
__device__ __forceinline__ R multi_reduce(R (&d)[CW], int lane) {
    if (CW < 32) {
#pragma unroll
        for (int s = 16; s >= CW; s >>= 1)
#pragma unroll
            for (int c = 0; c < CW; ++c) d[c] += __shfl_xor_sync(0xffffffffu, d[c], s);
    }
#pragma unroll
    for (int s = CW / 2; s >= 1; s >>= 1) {
        const bool upper = (lane & s) != 0;
#pragma unroll
        for (int c = 0; c < s; ++c) {
            const R send = upper ? d[c] : d[c + s];
            const R keep = upper ? d[c + s] : d[c];
            d[c] = keep + __shfl_xor_sync(0xffffffffu, send, s);
        }
    }
    return d[0];
}

// CTA partials of h[l] = V[l] . w (l < m) over rows [i0, i1), plus w.w as
// column m when `ww`; written to out[l*G] (out = region + blockIdx.x).  Work
// items are (CW-column group, row quarter); a lane runs down the rows of its
// item accumulating CW columns in registers, then one multi_reduce.
template <class T, int CW>
__device__ __forceinline__ void cta_dots(const T *__restrict__ V, int m, const T *__restrict__ w, int64_t n,
                                         int64_t i0, int64_t i1, bool ww, T *red, T *out, int G) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int ncol = m + (ww ? 1 : 0);
    const int ng = (ncol + CW - 1) / CW;
    const int nq = ng >= ORTH_WARPS ? 1 : ORTH_WARPS / ng;
    const int rs = ng * CW;
    const int64_t len = i1 - i0, qlen = (len + nq - 1) / nq;
    for (int item = warp; item < ng * nq; item += ORTH_WARPS) {
        const int g = item % ng, q = item / ng, l0 = g * CW;
        const int64_t r0 = i0 + (int64_t)q * qlen, r1 = min(i1, r0 + qlen);
        T acc[CW];
#pragma unroll
        for (int c = 0; c < CW; ++c) acc[c] = (T)0;
        if (l0 + CW <= m) {
            for (int64_t r = r0 + lane; r < r1; r += 32) {
                const T wv = w[r];
                const T *vr = V + (int64_t)l0 * n + r;
#pragma unroll
                for (int c = 0; c < CW; ++c) acc[c] += vr[(int64_t)c * n] * wv;
            }
        } else {
            for (int64_t r = r0 + lane; r < r1; r += 32) {
                const T wv = w[r];
#pragma unroll
                for (int c = 0; c < CW; ++c) {
                    const int l = l0 + c;
                    if (l < m) acc[c] += V[(int64_t)l * n + r] * wv;
                    else if (ww && l == m) acc[c] += wv * wv;
                }
            }
        }
        const T s = multi_reduce<T, CW>(acc, lane);
        if (lane < CW && l0 + lane < ncol) red[q * rs + l0 + lane] = s;
    }
    __syncthreads();
    for (int l = threadIdx.x; l < ncol; l += ORTH_THREADS) {
        T s = (T)0;
        for (int q = 0; q < nq; ++q) s += red[q * rs + l];
        out[(int64_t)l * G] = s;
    }
}

// w -= V_m h over rows [i0, i1); returns this thread's share of w.w
template <class T>
__device__ __forceinline__ T cta_update(const T *__restrict__ V, int m, T *__restrict__ w, int64_t n, int64_t i0,
                                        int64_t i1, const T *hs) {
    T ss = (T)0;
    for (int64_t i = i0 + threadIdx.x; i < i1; i += ORTH_THREADS) {
        T x = w[i];
#pragma unroll 32
        for (int l = 0; l < m; ++l) x -= V[(int64_t)l * n + i] * hs[l];
        w[i] = x;
        ss += x * x;
    }
    return ss;
}

template <class T>
struct OrthCW { static constexpr int value = sizeof(T) == 4 ? 32 : 16; };

__host__ __device__ inline int orth_redsz(int pstride, int cw) {
    return ORTH_WARPS * cw > pstride + cw ? ORTH_WARPS * cw : pstride + cw;
}

// shared memory of k_orth, in elements of T: hs, red, scratch
__host__ __device__ inline size_t orth_smem(int pstride, int cw, size_t tsize) {
    return (size_t)(pstride + orth_redsz(pstride, cw) + 8 * ORTH_WARPS + 16) * tsize;
}

template <class T, int CW>
__global__ void __launch_bounds__(ORTH_THREADS, 1) k_orth(OrthArgs a) {
    int *flags = a.flags;
    unsigned epoch = 0;
    if (*(volatile int *)&flags[F_STOP]) {           // set before this launch: uniform
        grid_exit(a.bar);
        return;
    }
    extern __shared__ __align__(16) unsigned char osm_raw[];
    T *osm = (T *)osm_raw;
    const int ps = a.pstride;
    T *hs = osm;
    T *red = hs + ps;
    T *scr = red + orth_redsz(ps, CW);               // [8 x 16] block sums, then [16] broadcasts
    T *bc = scr + 8 * ORTH_WARPS;
    const int G = gridDim.x, blk = blockIdx.x, tid = threadIdx.x;
    const int64_t n = a.n;
    const int64_t chunk = (n + G - 1) / G;
    const int64_t i0 = min(n, (int64_t)blk * chunk), i1 = min(n, i0 + chunk);
    T *V = (T *)a.V, *w = (T *)a.w;
    const int j = a.jdev ? *(volatile const int *)a.jdev : a.j, m = j + 1;
    const T *vj = V + (int64_t)j * n;
    const T *vjm = V + (int64_t)(j > 0 ? j - 1 : 0) * n;
    T *pA = (T *)a.part, *pH = pA + PA_COLS * G, *pB = pH + (int64_t)ps * G, *pH2 = pB + G,
      *pB2 = pH2 + (int64_t)ps * G;
    int *err = flags + F_ERR;
    const T *au = (const T *)a.anc_u, *ar = (const T *)a.anc_r, *ay = (const T *)a.defl;
    const bool anc = au != nullptr;
    const int nd = anc ? a.ndefl : 0;

    // the host's stop request (host memory: issued first, consumed just
    // before the first barrier so the read overlaps the first phase)
    int host_stop = 0;
    if (blk == 0 && tid == 0) host_stop = *(volatile const int *)(a.h_flags + F_NFLAGS);
    // alpha = v_j . w; anchored also u.w, r.v_j and y_k.w
    T av[PA_COLS];
#pragma unroll
    for (int q = 0; q < PA_COLS; ++q) av[q] = (T)0;
    for (int64_t i = i0 + tid; i < i1; i += ORTH_THREADS) {
        const T wi = w[i], vi = vj[i];
        av[0] += vi * wi;
        if (anc) {
            av[1] += au[i] * wi;
            av[2] += ar[i] * vi;
#pragma unroll
            for (int k = 0; k < 4; ++k)
                if (k < nd) av[3 + k] += ay[(int64_t)k * n + i] * wi;
        }
    }
    if (anc) {
        block_sums<T, PA_COLS>(av, scr);
        if (tid == 0)
#pragma unroll
            for (int q = 0; q < PA_COLS; ++q) pA[q * G + blk] = av[q];
    } else {
        T a1[1] = {av[0]};
        block_sums<T, 1>(a1, scr);
        if (tid == 0) pA[blk] = a1[0];
    }
    if (blk == 0 && tid == 0) flags[F_HOST] = host_stop;
    if (!grid_sync(a.bar, epoch, err, a.spin)) { fail_exit(a.bar, a.h_flags); return; }
    if (__ldcg(&flags[F_HOST])) {
        if (blk == 0 && tid == 0) flags[F_STOP] = 1;
        grid_exit(a.bar);
        return;
    }
    T tot[PA_COLS];
    if (anc) {
        grid_totals<T, PA_COLS>(pA, G, bc, tot);
        if (blk == 0 && tid == 0) a.h_m[j] = (double)tot[2];
    } else {
        T t1[1];
        grid_totals<T, 1>(pA, G, bc, t1);
#pragma unroll
        for (int q = 0; q < PA_COLS; ++q) tot[q] = (T)0;
        tot[0] = t1[0];
    }
    const T alpha0 = tot[0];
    {   // three-term step (and the anchor projections), then h = V_m^T w and ww = w.w
        const T b3 = j > 0 ? (T)a.beta[j - 1] : (T)0;
        for (int64_t i = i0 + tid; i < i1; i += ORTH_THREADS) {
            T x = w[i] - alpha0 * vj[i];
            if (j > 0) x -= b3 * vjm[i];
            if (anc) {
                x -= tot[1] * au[i];
#pragma unroll
                for (int k = 0; k < 4; ++k)
                    if (k < nd) x -= tot[3 + k] * ay[(int64_t)k * n + i];
            }
            w[i] = x;
        }
        __syncthreads();
        cta_dots<T, CW>(V, m, w, n, i0, i1, true, red, pH + blk, G);
    }
    if (!grid_sync(a.bar, epoch, err, a.spin)) { fail_exit(a.bar, a.h_flags); return; }
    grid_columns<T>(pH, G, m + 1, hs);
    __syncthreads();
    const T ww = hs[m];
    T hj = hs[j];
    {
        T s1[1] = {cta_update<T>(V, m, w, n, i0, i1, hs)};
        block_sums<T, 1>(s1, scr);
        if (tid == 0) pB[blk] = s1[0];
    }
    if (!grid_sync(a.bar, epoch, err, a.spin)) { fail_exit(a.bar, a.h_flags); return; }
    T bb[1];
    grid_totals<T, 1>(pB, G, bc + 8, bb);
    if (bb[0] < (T)0.5 * ww) {   // second projection (same decision in every CTA)
        cta_dots<T, CW>(V, m, w, n, i0, i1, false, red, pH2 + blk, G);
        if (!grid_sync(a.bar, epoch, err, a.spin)) { fail_exit(a.bar, a.h_flags); return; }
        grid_columns<T>(pH2, G, m, hs);
        __syncthreads();
        hj += hs[j];
        T s1[1] = {cta_update<T>(V, m, w, n, i0, i1, hs)};
        block_sums<T, 1>(s1, scr);
        if (tid == 0) pB2[blk] = s1[0];
        if (!grid_sync(a.bar, epoch, err, a.spin)) { fail_exit(a.bar, a.h_flags); return; }
        grid_totals<T, 1>(pB2, G, bc + 9, bb);
    }
    const T alpha_j = alpha0 + hj;
    const T beta_j = sqrt(bb[0]);
    bool brk = false;
    if (m < a.mmax) {
        const T scale = fmax(fabs(alpha_j), j > 0 ? (T)a.beta[j - 1] : (T)0);
        brk = !(beta_j > (T)1e-13 * fmax(scale, (T)1e-30));
        if (!brk) {
            const T inv = (T)1 / beta_j;
            T *vn = V + (int64_t)m * n;
            T *vc = (T *)a.vcur;
            for (int64_t i = i0 + tid; i < i1; i += ORTH_THREADS) {
                const T x = w[i] * inv;
                vn[i] = x;
                if (vc) vc[i] = x;
            }
        }
    }
    if (blk == 0 && tid == 0) {
        if (a.jdev) *a.jdev = j + 1;   // every CTA read j before the first barrier
        a.alpha[j] = (double)alpha_j;
        a.beta[j] = (double)beta_j;
        a.h_alpha[j] = (double)alpha_j;
        a.h_beta[j] = (double)beta_j;
        if (brk) {
            flags[F_BREAK] = m;
            flags[F_STOP] = 2;
            a.h_flags[F_BREAK] = m;
            a.h_flags[F_STOP] = 2;
        }
        __threadfence_system();
    }
    grid_exit(a.bar);
}

// ---------------------------------------------------------------------------
// Persistent chunk kernel of the mixed method (FP32 basis, all sectors on
// FP32 CUDA-core tiles): one cooperative launch runs iterations
// [j0, jend), each as
//   H*psi          work items (32x32 tiles, the long ones split into an H_L
//                  and an H_R + A x B part written to two slot vectors)
//                  shared out over the CTAs, two items per CTA at a time (two
//                  256-thread groups, named barriers); the input is the
//                  previous w'' scaled by 1/beta, the alpha partials come out
//                  of the item epilogues
//   barrier
//   three-term step on the CTA's rows (w = slot0 + slot1 - alpha v_j -
//   beta v_{j-1}) and the CGS dots, with the anchored refinement's extra
//   columns (u.w, r.v_j, y_k.w)
//   barrier, column sums, update w -= V h, beta^2 partials
//   barrier, (second projection when needed), next step
// so an iteration costs three grid barriers and no launch.  V rows are only
// touched by the CTA that owns them; the work vectors alternate between two
// buffers so that the items reading w''_{j-1} (all rows) never race with the
// writes of w''_j.  The normalisation v_j = w''_{j-1} / beta_{j-1} is written
// into V[j] by the owner CTA in iteration j.  alpha, beta, the anchor
// couplings and the flags reach the host-visible arrays when the launch ends.

struct ChunkArgs {
    OrthArgs o;                  // V, n, mmax, pstride, alpha/beta, part, bar, flags, mirrors, anchors
    float *buf[2];               // w buffers, iteration j reads buf[j & 1], writes buf[(j+1) & 1]
    float *slot[3];              // H v_j parts
    int j0, jend;
    int first_from_v;            // iteration j0 reads V[j0] itself (start or restart)
    const ItemRec *items;
    int nitems;
    Hv32Ops op;
    // shared-memory copy of the CTA's rows: basis vectors V[l < vc] and the
    // work vector, `cs` floats per vector (0: everything from global memory)
    int vc = 0, cs = 0;
};

constexpr int CHUNK_EXTRA = 8;   // extra partial columns of the anchored refinement
constexpr int CHUNK_MAXIT = 16;  // iterations per launch (>= CHECK)

__host__ __device__ inline size_t chunk_smem(int pstride) {
    return 2 * sizeof(Item32Smem) + orth_smem(pstride, OrthCW<float>::value, sizeof(float));
}

// offset of the row cache in k_chunk32's dynamic shared memory
__host__ __device__ inline size_t chunk_cache_off(int pstride) { return (chunk_smem(pstride) + 15) & ~(size_t)15; }

// dynamic shared memory k_chunk32 may take: the 227 KB of one CTA less room
// for its static arrays
constexpr size_t CHUNK_SMEM_MAX = 232448 - 2048;

// NSS_CHUNK_CACHE=0 turns the row cache off (comparisons, experiments)
inline bool chunk_cache_enabled() {
    const char *e = std::getenv("NSS_CHUNK_CACHE");
    return !(e && std::atoi(e) == 0);
}

__device__ __forceinline__ void cp_async4(float *dst, const float *src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)), "l"(src)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// cta_dots on the row cache: the CTA's rows of V[l] (l < vc) at vs[l*cs + r]
// and of w at ws[r] (r = row - i0).  Cached columns: one warp per column,
// the lanes down the rows, one warp sum (shared-memory operands need no
// loads in flight; the multi-column form below measured 3-5 us here against
// 1.5 us).  Columns l >= vc stream from global memory in the multi-column
// form of cta_dots (CW columns per lane, to keep enough loads in flight).
template <int CW>
__device__ __forceinline__ void cta_dots_vc(const float *__restrict__ vs, int vc, int cs, const float *__restrict__ V,
                                            int m, const float *__restrict__ ws, int64_t n, int64_t i0, int64_t i1,
                                            bool ww, float *red, float *out, int G) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int len = (int)(i1 - i0);
    const int mc = min(m, vc);
    const int n1 = mc + ((ww && m <= vc) ? 1 : 0);   // the w.w column here when nothing is left beyond the cache
    for (int l = warp; l < n1; l += ORTH_WARPS) {
        const float *src = l < mc ? vs + (int64_t)l * cs : ws;
        float acc = 0.f;
#pragma unroll 8
        for (int r = lane; r < len; r += 32) acc += src[r] * ws[r];
        acc = warp_sum<float>(acc);
        if (lane == 0) out[(int64_t)l * G] = acc;
    }
    if (m <= vc) return;
    const int ncol = m - vc + (ww ? 1 : 0);
    const int ng = (ncol + CW - 1) / CW;
    const int nq = ng >= ORTH_WARPS ? 1 : ORTH_WARPS / ng;
    const int rs = ng * CW;
    const int qlen = (len + nq - 1) / nq;
    const float *Vg = V + i0;
    for (int item = warp; item < ng * nq; item += ORTH_WARPS) {
        const int g = item % ng, q = item / ng, l0 = vc + g * CW;
        const int r0 = q * qlen, r1 = min(len, r0 + qlen);
        float acc[CW];
#pragma unroll
        for (int c = 0; c < CW; ++c) acc[c] = 0.f;
        if (l0 + CW <= m) {
            const float *vr = Vg + (int64_t)l0 * n;
            for (int r = r0 + lane; r < r1; r += 32) {
                const float wv = ws[r];
#pragma unroll
                for (int c = 0; c < CW; ++c) acc[c] += vr[(int64_t)c * n + r] * wv;
            }
        } else {
            for (int r = r0 + lane; r < r1; r += 32) {
                const float wv = ws[r];
#pragma unroll
                for (int c = 0; c < CW; ++c) {
                    const int l = l0 + c;
                    if (l < m) acc[c] += Vg[(int64_t)l * n + r] * wv;
                    else if (ww && l == m) acc[c] += wv * wv;
                }
            }
        }
        const float s = multi_reduce<float, CW>(acc, lane);
        if (lane < CW && l0 - vc + lane < ncol) red[q * rs + l0 - vc + lane] = s;
    }
    __syncthreads();
    for (int l = threadIdx.x; l < ncol; l += ORTH_THREADS) {
        float s = 0.f;
        for (int q = 0; q < nq; ++q) s += red[q * rs + l];
        out[(int64_t)(vc + l) * G] = s;
    }
}

__global__ void __launch_bounds__(ORTH_THREADS, 1) k_chunk32(ChunkArgs a) {
    constexpr int CW = OrthCW<float>::value;
    int *flags = a.o.flags;
    unsigned epoch = 0;
    if (*(volatile int *)&flags[F_STOP]) {           // set before this launch: uniform
        grid_exit(a.o.bar);
        return;
    }
    extern __shared__ __align__(16) unsigned char chunk_raw[];
    Item32Smem *ism = (Item32Smem *)chunk_raw;
    float *osm = (float *)(chunk_raw + 2 * sizeof(Item32Smem));
    __shared__ float rec_a[CHUNK_MAXIT], rec_b[CHUNK_MAXIT], rec_m[CHUNK_MAXIT];
    const int ps = a.o.pstride;
    float *hs = osm;
    float *red = hs + ps;
    float *scr = red + orth_redsz(ps, CW);
    float *bc = scr + 8 * ORTH_WARPS;
    const int G = gridDim.x, blk = blockIdx.x, tid = threadIdx.x, grp = tid >> 8, lt = tid & 255;
    const int64_t n = a.o.n;
    const int64_t chunk = (n + G - 1) / G;
    const int64_t i0 = min(n, (int64_t)blk * chunk), i1 = min(n, i0 + chunk);
    float *V = (float *)a.o.V;
    float *pA = (float *)a.o.part, *pH = pA + PA_COLS * G, *pB = pH + (int64_t)ps * G, *pH2 = pB + G,
          *pB2 = pH2 + (int64_t)ps * G;
    int *err = flags + F_ERR;
    const float *au = (const float *)a.o.anc_u, *ar = (const float *)a.o.anc_r, *ay = (const float *)a.o.defl;
    const bool anc = au != nullptr;
    const int nd = anc ? a.o.ndefl : 0;
    const int nx = anc ? 3 + nd : 0;                 // extra columns: u.w, r.v_j, y_k.w
    // row cache: the dots and updates of every iteration read the CTA's rows
    // of V and of w from shared memory instead of L2 (a round of dependent
    // loads less per phase); global V and w stay complete (other CTAs read
    // w, the host-side steps read V).  The basis vectors of earlier launches
    // are copied in asynchronously, behind the first H*psi items.
    const bool yc = a.vc > 0;
    const int vc = a.vc, cs = a.cs;
    float *vcache = (float *)(chunk_raw + chunk_cache_off(ps));
    float *ycache = vcache + (size_t)vc * cs;
    if (yc) {
        const int rows = (int)(i1 - i0);
        const int npre = min(vc, a.first_from_v ? a.j0 + 1 : a.j0);
        for (int e = tid; e < npre * rows; e += ORTH_THREADS) {
            const int l = e / rows, r = e - l * rows;
            cp_async4(vcache + l * cs + r, V + (int64_t)l * n + i0 + r);
        }
        cp_async_commit();
    }
    float beta_prev = a.j0 > 0 ? (float)a.o.beta[a.j0 - 1] : 0.f;
    int done = 0, brk_m = 0;
    // CTA 0 publishes the completed iterations (device arrays, host mirrors)
    auto publish = [&]() {
        if (tid == 0 && *(volatile int *)err) {
            a.o.h_flags[F_ERR] = 1;
            __threadfence_system();
        }
        if (blk == 0 && tid == 0) {
            for (int q = 0; q < done; ++q) {
                const int j = a.j0 + q;
                a.o.alpha[j] = (double)rec_a[q];
                a.o.beta[j] = (double)rec_b[q];
                a.o.h_alpha[j] = (double)rec_a[q];
                a.o.h_beta[j] = (double)rec_b[q];
                if (anc) a.o.h_m[j] = (double)rec_m[q];
            }
            if (brk_m) {
                flags[F_BREAK] = brk_m;
                flags[F_STOP] = 2;
                a.o.h_flags[F_BREAK] = brk_m;
                a.o.h_flags[F_STOP] = 2;
            }
            __threadfence_system();
        }
        grid_exit(a.o.bar);
    };
    for (int jj = a.j0; jj < a.jend; ++jj) {
        const int m = jj + 1;
        const bool first = jj == a.j0 && a.first_from_v;
        const float *x = first ? V + (int64_t)jj * n : a.buf[jj & 1];
        const float sc = first ? 1.f : 1.f / beta_prev;
        float *y = a.buf[(jj + 1) & 1];
        int host_stop = 0;
        if (blk == 0 && tid == 0) host_stop = *(volatile const int *)(a.o.h_flags + F_NFLAGS);
        // H v_j into the slots, alpha partials from the items
        float ap = 0.f;
        for (int ti = 2 * blk + grp; ti < a.nitems; ti += 2 * G)
            ap += hv32_item(a.items[ti], x, a.slot, a.op, ism[grp], lt, GroupSync{1 + grp}, sc);
        if (yc && jj == a.j0) cp_async_wait_all();   // the row cache (published by the barriers below)
        {
            float a1[1] = {ap};
            block_sums<float, 1>(a1, scr);
            if (tid == 0) pA[blk] = a1[0];
        }
        if (blk == 0 && tid == 0) flags[F_HOST] = host_stop;
        if (!grid_sync(a.o.bar, epoch, err, a.o.spin)) { publish(); return; }
        if (__ldcg(&flags[F_HOST])) {
            if (blk == 0 && tid == 0) flags[F_STOP] = 1;
            publish();
            return;
        }
        const float *s0 = a.slot[0], *s1 = a.slot[1], *s2 = a.slot[2];
        // the three-term step's H v_j of the thread's first row, loaded before
        // the alpha total so that the two L2 round trips overlap
        const int64_t if0 = i0 + tid;
        float hv0 = 0.f;
        if (if0 < i1) hv0 = s0[if0] + s1[if0] + s2[if0];
        float alpha0;
        {
            float t1[1];
            grid_totals<float, 1>(pA, G, bc, t1);
            alpha0 = t1[0];
        }
        // v_j into V (own rows), three-term step, anchor extras
        float ex[CHUNK_EXTRA];
#pragma unroll
        for (int q = 0; q < CHUNK_EXTRA; ++q) ex[q] = 0.f;
        {
            float *vj = V + (int64_t)jj * n;
            const float *vjm = V + (int64_t)(jj > 0 ? jj - 1 : 0) * n;
            // own rows of x: the cached w of the previous iteration of this launch
            const bool xc = yc && jj > a.j0;
            const bool jc = jj < vc, jmc = jj > 0 && jj - 1 < vc;
            for (int64_t i = if0; i < i1; i += ORTH_THREADS) {
                const int r = (int)(i - i0);
                const float v = (xc ? ycache[r] : x[i]) * sc;
                if (!first) vj[i] = v;
                if (jc) vcache[jj * cs + r] = v;
                float w = (i == if0 ? hv0 : (s0[i] + s1[i] + s2[i])) - alpha0 * v;
                if (jj > 0) w -= beta_prev * (jmc ? vcache[(jj - 1) * cs + r] : vjm[i]);
                y[i] = w;
                if (yc) ycache[r] = w;
                if (anc) {
                    ex[0] += au[i] * w;
                    ex[1] += ar[i] * v;
#pragma unroll
                    for (int k = 0; k < 4; ++k)
                        if (k < nd) ex[2 + k] += ay[(int64_t)k * n + i] * w;
                }
            }
        }
        __syncthreads();
        if (yc) cta_dots_vc<CW>(vcache, vc, cs, V, m, ycache, n, i0, i1, true, red, pH + blk, G);
        else cta_dots<float, CW>(V, m, y, n, i0, i1, true, red, pH + blk, G);
        if (anc) {
            block_sums<float, CHUNK_EXTRA>(ex, scr);
            if (tid == 0) {
                pH[(int64_t)(m + 1) * G + blk] = ex[0];
                pH[(int64_t)(m + 2) * G + blk] = ex[1];
#pragma unroll
                for (int k = 0; k < 4; ++k)
                    if (k < nd) pH[(int64_t)(m + 3 + k) * G + blk] = ex[2 + k];
            }
        }
        if (!grid_sync(a.o.bar, epoch, err, a.o.spin)) { publish(); return; }
        grid_columns<float>(pH, G, m + 1 + nx, hs);
        __syncthreads();
        const float ww = hs[m];
        float hj = hs[jj];
        const float mj = anc ? hs[m + 2] : 0.f;
        // w -= V h (+ the anchor and deflation components)
        auto update = [&](int xoff) -> float {
            float ss = 0.f;
            const int mc = min(m, vc);
            for (int64_t i = i0 + tid; i < i1; i += ORTH_THREADS) {
                const int r = (int)(i - i0);
                float w = yc ? ycache[r] : y[i];
#pragma unroll 8
                for (int l = 0; l < mc; ++l) w -= vcache[l * cs + r] * hs[l];
#pragma unroll 32
                for (int l = mc; l < m; ++l) w -= V[(int64_t)l * n + i] * hs[l];
                if (anc) {
                    w -= hs[xoff] * au[i];
                    for (int k = 0; k < nd; ++k) w -= hs[xoff + 2 + k] * ay[(int64_t)k * n + i];
                }
                y[i] = w;
                if (yc) ycache[r] = w;
                ss += w * w;
            }
            return ss;
        };
        {
            float s1[1] = {update(m + 1)};
            block_sums<float, 1>(s1, scr);
            if (tid == 0) pB[blk] = s1[0];
        }
        if (!grid_sync(a.o.bar, epoch, err, a.o.spin)) { publish(); return; }
        float bb;
        {
            float t1[1];
            grid_totals<float, 1>(pB, G, bc + 8, t1);
            bb = t1[0];
        }
        if (bb < 0.5f * ww) {   // second projection (same decision in every CTA)
            if (yc) cta_dots_vc<CW>(vcache, vc, cs, V, m, ycache, n, i0, i1, false, red, pH2 + blk, G);
            else cta_dots<float, CW>(V, m, y, n, i0, i1, false, red, pH2 + blk, G);
            if (anc) {
#pragma unroll
                for (int q = 0; q < CHUNK_EXTRA; ++q) ex[q] = 0.f;
                for (int64_t i = i0 + tid; i < i1; i += ORTH_THREADS) {
                    const float w = yc ? ycache[i - i0] : y[i];
                    ex[0] += au[i] * w;
#pragma unroll
                    for (int k = 0; k < 4; ++k)
                        if (k < nd) ex[2 + k] += ay[(int64_t)k * n + i] * w;
                }
                block_sums<float, CHUNK_EXTRA>(ex, scr);
                if (tid == 0) {
                    pH2[(int64_t)m * G + blk] = ex[0];
                    pH2[(int64_t)(m + 1) * G + blk] = 0.f;
#pragma unroll
                    for (int k = 0; k < 4; ++k)
                        if (k < nd) pH2[(int64_t)(m + 2 + k) * G + blk] = ex[2 + k];
                }
            }
            if (!grid_sync(a.o.bar, epoch, err, a.o.spin)) { publish(); return; }
            grid_columns<float>(pH2, G, m + (anc ? 2 + nd : 0), hs);
            __syncthreads();
            hj += hs[jj];
            float s1[1] = {update(m)};
            block_sums<float, 1>(s1, scr);
            if (tid == 0) pB2[blk] = s1[0];
            if (!grid_sync(a.o.bar, epoch, err, a.o.spin)) { publish(); return; }
            float t1[1];
            grid_totals<float, 1>(pB2, G, bc + 9, t1);
            bb = t1[0];
        }
        const float alpha_j = alpha0 + hj;
        const float beta_j = sqrtf(bb);
        bool brk = false;
        if (m < a.o.mmax) {
            const float scale = fmaxf(fabsf(alpha_j), jj > 0 ? beta_prev : 0.f);
            brk = !(beta_j > 1e-13f * fmaxf(scale, 1e-30f));
        }
        if (blk == 0 && tid == 0) {
            rec_a[done] = alpha_j;
            rec_b[done] = beta_j;
            rec_m[done] = mj;
        }
        ++done;
        if (brk) {
            brk_m = m;
            publish();
            return;
        }
        beta_prev = beta_j;
        __syncthreads();
    }
    publish();
}

// ---------------------------------------------------------------------------
// Batched persistent kernel: several independent mixed-precision solves (one
// context each) advance together, one launch per chunk of iterations.  The
// H*psi work items of all solves are shared out over all CTAs (longest
// first); each solve's rows belong to its own range of CTAs, which run its
// three-term step, projections and updates.  The grid barriers are global,
// so every CTA takes the same barrier sequence: the per-solve decisions that
// change it (second projection, breakdown, end of the chunk) are recomputed
// by every CTA from the solves' partial sums, in the same order, so all CTAs
// agree.  Solves stop within a launch only at their chunk end or at a
// breakdown; the host checks convergence between launches.

struct BatchSolve {
    ChunkArgs c;                 // per-solve arguments (c.o.bar unused)
    float *pitem;                // [c.nitems] alpha partials of the solve's items
    int cta0, ncta;              // CTAs owning the solve's rows
    int active;                  // takes part in this launch
    int pad;
};

struct BatchArgs {
    const BatchSolve *s;
    int ns;
    int nitems;                  // items of all active solves
    const int2 *gitems;          // (solve, item) in processing order
    float *st;                   // [4 ns] per-solve scalars published inside an iteration
    unsigned *bar;               // global barrier
    int *err;
    int steps;                   // iterations of this launch
    uint32_t spin;               // poll limit of the grid barriers (wait_limit)
    unsigned *qcnt;              // [CHUNK_MAXIT] item queue heads, zero at launch
};

constexpr int BATCH_MAX = 160;   // solves per launch (each needs a CTA)

__global__ void __launch_bounds__(ORTH_THREADS, 1) k_batch32(BatchArgs B) {
    constexpr int CW = OrthCW<float>::value;
    extern __shared__ __align__(16) unsigned char batch_raw[];
    Item32Smem *ism = (Item32Smem *)batch_raw;
    float *osm = (float *)(batch_raw + 2 * sizeof(Item32Smem));
    __shared__ float rec_a[CHUNK_MAXIT], rec_b[CHUNK_MAXIT], rec_m[CHUNK_MAXIT];
    __shared__ float bprev[BATCH_MAX], balpha[BATCH_MAX], bbb[BATCH_MAX];
    __shared__ int alive[BATCH_MAX], p2[BATCH_MAX], brkm[BATCH_MAX];
    __shared__ int my_s, any_p2;
    __shared__ int qn[2];
    const int blk = blockIdx.x, tid = threadIdx.x, grp = tid >> 8, lt = tid & 255;
    const int ns = B.ns;
    unsigned epoch = 0;
    if (tid == 0) {
        my_s = -1;
        for (int s = 0; s < ns; ++s)
            if (B.s[s].active && blk >= B.s[s].cta0 && blk < B.s[s].cta0 + B.s[s].ncta) my_s = s;
    }
    for (int s = tid; s < ns; s += ORTH_THREADS) {
        const BatchSolve &S = B.s[s];
        const int j0 = S.c.j0;
        alive[s] = S.active && !*(volatile int *)&S.c.o.flags[F_STOP] && S.c.jend > j0;
        bprev[s] = j0 > 0 ? (float)S.c.o.beta[j0 - 1] : 0.f;
        brkm[s] = 0;
    }
    __syncthreads();
    const int me = my_s;
    // this CTA's own solve (if any)
    const BatchSolve *Mp = me >= 0 ? &B.s[me] : nullptr;
    const int Gs = Mp ? Mp->ncta : 1, lb = Mp ? blk - Mp->cta0 : 0;
    const int ps = Mp ? Mp->c.o.pstride : 8;
    float *hs = osm;
    float *red = hs + ps;
    float *scr = red + orth_redsz(ps, CW);
    float *bc = scr + 8 * ORTH_WARPS;
    const int64_t n = Mp ? Mp->c.o.n : 0;
    const int64_t chunk = (n + Gs - 1) / Gs;
    const int64_t i0 = min(n, (int64_t)lb * chunk), i1 = min(n, i0 + chunk);
    float *V = Mp ? (float *)Mp->c.o.V : nullptr;
    float *pA = Mp ? (float *)Mp->c.o.part : nullptr;
    float *pH = pA + PA_COLS * Gs, *pB = pH + (int64_t)ps * Gs, *pH2 = pB + Gs, *pB2 = pH2 + (int64_t)ps * Gs;
    const float *au = Mp ? (const float *)Mp->c.o.anc_u : nullptr;
    const float *ar = Mp ? (const float *)Mp->c.o.anc_r : nullptr;
    const float *ay = Mp ? (const float *)Mp->c.o.defl : nullptr;
    const bool anc = au != nullptr;
    const int nd = anc ? Mp->c.o.ndefl : 0;
    const int nx = anc ? 3 + nd : 0;
    int done = 0;
    for (int step = 0; step < B.steps; ++step) {
        // ---- H*psi of every running solve, all items over all CTAs: each
        // thread group takes the next item off a global queue (longest
        // first), fetching the index after next while it works on one
        if (lt == 0) qn[grp] = (int)atomicAdd(B.qcnt + step, 1u);
        GroupSync{1 + grp}();
        for (int gi = qn[grp]; gi < B.nitems;) {
            int nxt = 0;
            if (lt == 0) nxt = (int)atomicAdd(B.qcnt + step, 1u);
            const int2 g = B.gitems[gi];
            const BatchSolve &S = B.s[g.x];
            const int tj = S.c.j0 + step;
            if (alive[g.x] && tj < S.c.jend) {
                const bool first = tj == S.c.j0 && S.c.first_from_v;
                const float *x = first ? (const float *)S.c.o.V + (int64_t)tj * S.c.o.n : S.c.buf[tj & 1];
                const float sc = first ? 1.f : 1.f / bprev[g.x];
                float ap = hv32_item(S.c.items[g.y], x, S.c.slot, S.c.op, ism[grp], lt, GroupSync{1 + grp}, sc);
                // group sum of the alpha partial (named barrier of the group)
                ap = warp_sum<float>(ap);
                if ((lt & 31) == 0) scr[grp * 8 + (lt >> 5)] = ap;
                GroupSync{1 + grp}();
                if (lt == 0) {
                    float t = 0.f;
                    for (int q = 0; q < 8; ++q) t += scr[grp * 8 + q];
                    S.pitem[g.y] = t;
                }
            }
            GroupSync{1 + grp}();
            if (lt == 0) qn[grp] = nxt;
            GroupSync{1 + grp}();
            gi = qn[grp];
        }
        if (!grid_sync(B.bar, epoch, B.err, B.spin)) break;
        const bool run = me >= 0 && alive[me] && Mp->c.j0 + step < Mp->c.jend;
        const int jj = Mp ? Mp->c.j0 + step : 0, m = jj + 1;
        const bool first = run && jj == Mp->c.j0 && Mp->c.first_from_v;
        const float *x = run ? (first ? V + (int64_t)jj * n : Mp->c.buf[jj & 1]) : nullptr;
        const float sc = first ? 1.f : (me >= 0 ? 1.f / bprev[me] : 1.f);
        float *y = run ? Mp->c.buf[(jj + 1) & 1] : nullptr;
        float ex[CHUNK_EXTRA];
#pragma unroll
        for (int q = 0; q < CHUNK_EXTRA; ++q) ex[q] = 0.f;
        float alpha0 = 0.f;
        if (run) {
            {   // alpha from the item partials, fixed order
                float t = 0.f;
                if (tid < 32) {
                    t = strided_sum<float>(Mp->pitem, tid, Mp->c.nitems, 32);
                    t = warp_sum<float>(t);
                    if (tid == 0) bc[0] = t;
                }
                __syncthreads();
                alpha0 = bc[0];
            }
            float *vj = V + (int64_t)jj * n;
            const float *vjm = V + (int64_t)(jj > 0 ? jj - 1 : 0) * n;
            const float *s0 = Mp->c.slot[0], *s1 = Mp->c.slot[1], *s2 = Mp->c.slot[2];
            for (int64_t i = i0 + tid; i < i1; i += ORTH_THREADS) {
                const float v = x[i] * sc;
                if (!first) vj[i] = v;
                float w = (s0[i] + s1[i] + s2[i]) - alpha0 * v;
                if (jj > 0) w -= bprev[me] * vjm[i];
                y[i] = w;
                if (anc) {
                    ex[0] += au[i] * w;
                    ex[1] += ar[i] * v;
#pragma unroll
                    for (int k = 0; k < 4; ++k)
                        if (k < nd) ex[2 + k] += ay[(int64_t)k * n + i] * w;
                }
            }
            __syncthreads();
            cta_dots<float, CW>(V, m, y, n, i0, i1, true, red, pH + lb, Gs);
            if (anc) {
                block_sums<float, CHUNK_EXTRA>(ex, scr);
                if (tid == 0) {
                    pH[(int64_t)(m + 1) * Gs + lb] = ex[0];
                    pH[(int64_t)(m + 2) * Gs + lb] = ex[1];
#pragma unroll
                    for (int k = 0; k < 4; ++k)
                        if (k < nd) pH[(int64_t)(m + 3 + k) * Gs + lb] = ex[2 + k];
                }
            }
        }
        if (!grid_sync(B.bar, epoch, B.err, B.spin)) break;
        float hj = 0.f, mj = 0.f;
        auto update = [&](int xoff) -> float {
            float ss = 0.f;
            for (int64_t i = i0 + tid; i < i1; i += ORTH_THREADS) {
                float w = y[i];
#pragma unroll 32
                for (int l = 0; l < m; ++l) w -= V[(int64_t)l * n + i] * hs[l];
                if (anc) {
                    w -= hs[xoff] * au[i];
                    for (int k = 0; k < nd; ++k) w -= hs[xoff + 2 + k] * ay[(int64_t)k * n + i];
                }
                y[i] = w;
                ss += w * w;
            }
            return ss;
        };
        if (run) {
            grid_columns<float>(pH, Gs, m + 1 + nx, hs);
            __syncthreads();
            hj = hs[jj];
            mj = anc ? hs[m + 2] : 0.f;
            if (lb == 0 && tid == 0) {
                B.st[4 * me + 0] = alpha0 + hj;
                B.st[4 * me + 1] = hs[m];
                B.st[4 * me + 2] = 0.f;
            }
            float s1[1] = {update(m + 1)};
            block_sums<float, 1>(s1, scr);
            if (tid == 0) pB[lb] = s1[0];
        }
        if (!grid_sync(B.bar, epoch, B.err, B.spin)) break;
        // every CTA: beta^2 and the second-projection decision of every solve
        if (tid == 0) any_p2 = 0;
        __syncthreads();
        for (int s = tid; s < ns; s += ORTH_THREADS) {
            const BatchSolve &S = B.s[s];
            p2[s] = 0;
            if (!alive[s] || S.c.j0 + step >= S.c.jend) continue;
            const float *pBs = (const float *)S.c.o.part + (PA_COLS + (int64_t)S.c.o.pstride) * S.ncta;
            float t = 0.f;
            t = strided_sum<float>(pBs, 0, S.ncta, 1);
            bbb[s] = t;
            balpha[s] = __ldcg(B.st + 4 * s + 0);
            if (t < 0.5f * __ldcg(B.st + 4 * s + 1)) {
                p2[s] = 1;
                any_p2 = 1;
            }
        }
        __syncthreads();
        if (any_p2) {
            const bool mine = run && p2[me];
            if (mine) {
                cta_dots<float, CW>(V, m, y, n, i0, i1, false, red, pH2 + lb, Gs);
                if (anc) {
#pragma unroll
                    for (int q = 0; q < CHUNK_EXTRA; ++q) ex[q] = 0.f;
                    for (int64_t i = i0 + tid; i < i1; i += ORTH_THREADS) {
                        const float w = y[i];
                        ex[0] += au[i] * w;
#pragma unroll
                        for (int k = 0; k < 4; ++k)
                            if (k < nd) ex[2 + k] += ay[(int64_t)k * n + i] * w;
                    }
                    block_sums<float, CHUNK_EXTRA>(ex, scr);
                    if (tid == 0) {
                        pH2[(int64_t)m * Gs + lb] = ex[0];
                        pH2[(int64_t)(m + 1) * Gs + lb] = 0.f;
#pragma unroll
                        for (int k = 0; k < 4; ++k)
                            if (k < nd) pH2[(int64_t)(m + 2 + k) * Gs + lb] = ex[2 + k];
                    }
                }
            }
            if (!grid_sync(B.bar, epoch, B.err, B.spin)) break;
            if (mine) {
                grid_columns<float>(pH2, Gs, m + (anc ? 2 + nd : 0), hs);
                __syncthreads();
                if (lb == 0 && tid == 0) B.st[4 * me + 2] = hs[jj];
                float s1[1] = {update(m)};
                block_sums<float, 1>(s1, scr);
                if (tid == 0) pB2[lb] = s1[0];
            }
            if (!grid_sync(B.bar, epoch, B.err, B.spin)) break;
            for (int s = tid; s < ns; s += ORTH_THREADS) {
                if (!p2[s]) continue;
                const BatchSolve &S = B.s[s];
                const float *pB2s = (const float *)S.c.o.part + (PA_COLS + 2 * (int64_t)S.c.o.pstride + 1) * S.ncta;
                float t = 0.f;
                t = strided_sum<float>(pB2s, 0, S.ncta, 1);
                bbb[s] = t;
                balpha[s] += __ldcg(B.st + 4 * s + 2);
            }
            __syncthreads();
        }
        // every CTA: beta, breakdown, next scale of every solve that ran
        for (int s = tid; s < ns; s += ORTH_THREADS) {
            const BatchSolve &S = B.s[s];
            if (!alive[s] || S.c.j0 + step >= S.c.jend) continue;
            const float beta = sqrtf(bbb[s]);
            const int ms = S.c.j0 + step + 1;
            if (ms < S.c.o.mmax) {
                const float scale = fmaxf(fabsf(balpha[s]), S.c.j0 + step > 0 ? bprev[s] : 0.f);
                if (!(beta > 1e-13f * fmaxf(scale, 1e-30f))) {
                    brkm[s] = ms;
                    alive[s] = 0;
                }
            }
            bprev[s] = beta;
        }
        __syncthreads();
        if (run) {
            if (lb == 0 && tid == 0) {
                rec_a[done] = balpha[me];
                rec_b[done] = bprev[me];
                rec_m[done] = mj;
            }
            ++done;
        }
    }
    // publish the completed iterations of the own solve
    if (me >= 0 && lb == 0 && tid == 0) {
        const ChunkArgs &a = Mp->c;
        for (int q = 0; q < done; ++q) {
            const int j = a.j0 + q;
            a.o.alpha[j] = (double)rec_a[q];
            a.o.beta[j] = (double)rec_b[q];
            a.o.h_alpha[j] = (double)rec_a[q];
            a.o.h_beta[j] = (double)rec_b[q];
            if (anc) a.o.h_m[j] = (double)rec_m[q];
        }
        if (brkm[me]) {
            a.o.flags[F_BREAK] = brkm[me];
            a.o.flags[F_STOP] = 2;
            a.o.h_flags[F_BREAK] = brkm[me];
            a.o.h_flags[F_STOP] = 2;
        }
        __threadfence_system();
    }
    grid_exit(B.bar);
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
    for (int q = 0; q < 3; ++q) {
        const double t = lastblock_sum(part + (int64_t)q * gridDim.x, gridDim.x);
        if (tid == 0) r[q] = t;
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
    if (!last_block(counter)) return;
    const double t = lastblock_sum(part, gridDim.x);
    if (tid != 0) return;
    r[3] = t;
    *counter = 0u;
}

// Anchor residual: w <- w - theta0 psi with theta0 = r[0]/r[2] (from k_rq),
// and r[4] = ||w||^2 (grid reduction)
__global__ void __launch_bounds__(256) k_anchor_r(const double *__restrict__ psi, double *__restrict__ w, int64_t n,
                                                  double *__restrict__ part, double *__restrict__ r, unsigned *counter) {
    const int tid = threadIdx.x;
    const double th = r[0] / r[2];
    double a = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + tid; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double d = w[i] - th * psi[i];
        w[i] = d;
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
    if (!last_block(counter)) return;
    const double t = lastblock_sum(part, gridDim.x);
    if (tid != 0) return;
    r[4] = t;
    *counter = 0u;
}

// Gram matrix of k <= 4 FP64 vectors against k others: r[i*k+j] = U_i . W_j
// (grid reduction; part holds k*k columns of gridDim.x partials)
__global__ void __launch_bounds__(256) k_gram(const double *__restrict__ U, const double *__restrict__ W, int k,
                                              int64_t n, double *__restrict__ part, double *__restrict__ r,
                                              unsigned *counter) {
    const int tid = threadIdx.x;
    double acc[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) acc[q] = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + tid; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double u[4], w[4];
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            u[a] = a < k ? U[(int64_t)a * n + i] : 0.0;
            w[a] = a < k ? W[(int64_t)a * n + i] : 0.0;
        }
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int b = 0; b < 4; ++b) acc[a * 4 + b] = fma(u[a], w[b], acc[a * 4 + b]);
    }
    __shared__ double red[16][8];
#pragma unroll
    for (int q = 0; q < 16; ++q) {
        const double v = warp_sum<double>(acc[q]);
        if ((tid & 31) == 0) red[q][tid >> 5] = v;
    }
    __syncthreads();
    if (tid < k * k) {
        const int a = tid / k, b = tid % k;
        double t = 0.0;
        for (int q = 0; q < 8; ++q) t += red[a * 4 + b][q];
        part[(int64_t)tid * gridDim.x + blockIdx.x] = t;
    }
    if (!last_block(counter)) return;
    for (int q = 0; q < k * k; ++q) {
        const double t = lastblock_sum(part + (int64_t)q * gridDim.x, gridDim.x);
        if (tid == 0) r[q] = t;
    }
    if (tid == 0) *counter = 0u;
}

// X <- X Q for k <= 4 FP64 vectors (Q column-major k x k)
struct Rot4 {
    double q[16];
};
__global__ void __launch_bounds__(256) k_rot(double *__restrict__ X, int k, int64_t n, Rot4 Q) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double x[4], y[4];
#pragma unroll
        for (int a = 0; a < 4; ++a) x[a] = a < k ? X[(int64_t)a * n + i] : 0.0;
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            double t = 0.0;
#pragma unroll
            for (int a = 0; a < 4; ++a) t = fma(x[a], Q.q[b * 4 + a], t);
            y[b] = t;
        }
#pragma unroll
        for (int b = 0; b < 4; ++b)
            if (b < k) X[(int64_t)b * n + i] = y[b];
    }
}

// Eigenvalues (ascending) and orthonormal eigenvectors (columns of q,
// column-major k x k) of a symmetric k x k matrix a (row-major, destroyed),
// k <= 4, by cyclic Jacobi rotations.
void sym_eig_small(int k, double *a, double *lam, double *q) {
    if (k < 1 || k > 4) return;   // callers pass 1..4
    for (int i = 0; i < k; ++i)
        for (int j = 0; j < k; ++j) q[j * k + i] = i == j ? 1.0 : 0.0;
    for (int sweep = 0; sweep < 50; ++sweep) {
        double off = 0.0, tot = 0.0;
        for (int i = 0; i < k; ++i)
            for (int j = 0; j < k; ++j) {
                tot += a[i * k + j] * a[i * k + j];
                if (i != j) off += a[i * k + j] * a[i * k + j];
            }
        if (off <= 1e-34 * tot) break;
        for (int p = 0; p < k; ++p)
            for (int r = p + 1; r < k; ++r) {
                const double apr = a[p * k + r];
                if (apr == 0.0) continue;
                const double tau = (a[r * k + r] - a[p * k + p]) / (2.0 * apr);
                const double t = (tau >= 0.0 ? 1.0 : -1.0) / (std::fabs(tau) + std::sqrt(1.0 + tau * tau));
                const double cs = 1.0 / std::sqrt(1.0 + t * t), sn = t * cs;
                for (int i = 0; i < k; ++i) {   // columns p, r
                    const double x = a[i * k + p], y = a[i * k + r];
                    a[i * k + p] = cs * x - sn * y;
                    a[i * k + r] = sn * x + cs * y;
                }
                for (int j = 0; j < k; ++j) {   // rows p, r
                    const double x = a[p * k + j], y = a[r * k + j];
                    a[p * k + j] = cs * x - sn * y;
                    a[r * k + j] = sn * x + cs * y;
                }
                for (int i = 0; i < k; ++i) {
                    const double x = q[p * k + i], y = q[r * k + i];
                    q[p * k + i] = cs * x - sn * y;
                    q[r * k + i] = sn * x + cs * y;
                }
            }
    }
    // ascending by the diagonal: insertion sort (equal values keep their order)
    int ord[4] = {0, 1, 2, 3};
    for (int j = 1; j < k; ++j) {
        const int x = ord[j];
        int i = j;
        for (; i > 0 && a[x * k + x] < a[ord[i - 1] * k + ord[i - 1]]; --i) ord[i] = ord[i - 1];
        ord[i] = x;
    }
    double qs[16];
    for (int j = 0; j < k; ++j) {
        lam[j] = a[ord[j] * k + ord[j]];
        for (int i = 0; i < k; ++i) qs[j * k + i] = q[ord[j] * k + i];
    }
    for (int t = 0; t < k * k; ++t) q[t] = qs[t];
}

// out = (float)(x * s)
__global__ void k_to32(float *__restrict__ out, const double *__restrict__ x, double s, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = (float)(x[i] * s);
}

// x <- x / ||x|| on stream st (two launches)
template <class T>
void normalize_dev(DevLanczos &z, T *x, int64_t n, cudaStream_t st, int64_t &launches) {
    k_sumsq<T><<<NBLK, 256, 0, st>>>(x, n, z.part, z.scal + S_NRM, z.counter);
    k_scale<T><<<NBLK, 256, 0, st>>>(x, n, z.scal + S_NRM);
    launches += 1;   // the caller counted one launch for the normalisation
}

// per-eigenvector scratch row of svec
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
        NSS_CUDA_TRY(c, ctx_alloc(c, &z.anc32, (size_t)6 * n));   // FP32 anchor, residual, deflation set
        NSS_CUDA_TRY(c, ctx_alloc(c, &z.V, (size_t)n));   // FP64 refinement scratch
        z.full64 = false;
    } else {
        NSS_CUDA_TRY(c, ctx_alloc(c, &z.V, (size_t)(cap + 1) * n));
        z.full64 = true;
    }
    int dev = 0, nsm = 0;
    NSS_CUDA_TRY(c, cudaGetDevice(&dev));
    NSS_CUDA_TRY(c, cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    const int pstride = cap + 8;   // m+1 columns plus the anchored refinement's extras
    const int cw = mixed ? OrthCW<float>::value : OrthCW<double>::value;
    const size_t smem = orth_smem(pstride, cw, mixed ? sizeof(float) : sizeof(double));
    const void *fn = mixed ? (const void *)k_orth<float, OrthCW<float>::value>
                           : (const void *)k_orth<double, OrthCW<double>::value>;
    NSS_CUDA_TRY(c, allow_smem(fn, smem));
    int occ = 0;
    NSS_CUDA_TRY(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, ORTH_THREADS, smem));
    if (occ < 1) {
        c.err = "nss_eigh: Krylov basis too large for the orthogonalisation kernel's shared memory";
        return NSS_ERR_INVALID;
    }
    z.orth_grid = nsm;      // one CTA per SM, all resident (cooperative launch)
    z.orth_smem = smem;
    z.chunk_ok = false;
    if (mixed) {
        // the persistent chunk kernel of the mixed method
        const size_t csm = chunk_smem(pstride);
        // the row cache takes what one CTA per SM leaves: the CTA's rows of
        // the work vector and of as many basis vectors as fit
        const int64_t rows = (n + nsm - 1) / nsm;
        const int cs = (int)((rows + 3) & ~(int64_t)3);
        const size_t coff = chunk_cache_off(pstride), vbytes = (size_t)cs * sizeof(float);
        int vc = 0;
        if (chunk_cache_enabled() && coff + 2 * vbytes <= CHUNK_SMEM_MAX)
            vc = (int)std::min<int64_t>(cap + 1, (int64_t)((CHUNK_SMEM_MAX - coff - vbytes) / vbytes));
        const size_t csm_vc = vc > 0 ? coff + (size_t)(vc + 1) * vbytes : csm;
        NSS_CUDA_TRY(c, allow_smem((const void *)k_chunk32, std::max(csm, csm_vc)));
        int occ2 = 0;
        NSS_CUDA_TRY(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ2, (const void *)k_chunk32, ORTH_THREADS,
                                                                      csm_vc));
        if (occ2 < 1 && vc > 0) {   // no room for the cache after all: run without it
            vc = 0;
            NSS_CUDA_TRY(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ2, (const void *)k_chunk32, ORTH_THREADS,
                                                                          csm));
        }
        if (occ2 >= 1) {
            NSS_CUDA_TRY(c, ctx_alloc(c, &z.wbuf32, (size_t)2 * n));
            NSS_CUDA_TRY(c, ctx_alloc(c, &z.slot32, (size_t)3 * n));
            z.chunk_smem = csm;
            z.chunk_vc = vc;
            z.chunk_cs = vc > 0 ? cs : 0;
            z.chunk_smem_vc = vc > 0 ? csm_vc : csm;
            z.chunk_ok = true;
        }
    }
    NSS_CUDA_TRY(c, ctx_alloc(c, &z.w, (size_t)n));
    {
        double *vc = nullptr;
        NSS_CUDA_TRY(c, ctx_alloc(c, &vc, (size_t)n));
        z.vcur = vc;
    }
    NSS_CUDA_TRY(c, ctx_alloc(c, &z.jdev, 1));
    NSS_CUDA_TRY(c, ctx_alloc(c, &z.evecs, (size_t)4 * n));
    // scalars, projection coefficients, restart scratch alpha/beta, refinement
    NSS_CUDA_TRY(c, ctx_alloc(c, &z.scal, (size_t)S_NSCAL + 4 * (cap + 2) + 8));
    const size_t part = std::max((size_t)(cap + 2) * NBLK, (size_t)(2 * pstride + PA_COLS + 2) * (size_t)nsm);
    NSS_CUDA_TRY(c, ctx_alloc(c, &z.part, part));
    NSS_CUDA_TRY(c, ctx_alloc(c, &z.counter, 4));
    NSS_CUDA_TRY(c, ctx_alloc(c, &z.alpha, (size_t)cap + 1));
    NSS_CUDA_TRY(c, ctx_alloc(c, &z.beta, (size_t)cap + 1));
    NSS_CUDA_TRY(c, ctx_alloc(c, &z.theta, 8));
    NSS_CUDA_TRY(c, ctx_alloc(c, &z.resid, 8));
    NSS_CUDA_TRY(c, ctx_alloc(c, &z.svec, (size_t)4 * svec_stride(cap)));
    NSS_CUDA_TRY(c, ctx_alloc(c, &z.flags, F_NFLAGS));
    // host-mapped mirrors: alpha, beta, anchor couplings m; flags + the host's stop request
    NSS_CUDA_TRY(c, cudaHostAlloc((void **)&z.h_ab, 3 * (size_t)(cap + 1) * sizeof(double), cudaHostAllocMapped));
    NSS_CUDA_TRY(c, cudaHostAlloc((void **)&z.h_flags, (F_NFLAGS + 8) * sizeof(int), cudaHostAllocMapped));
    NSS_CUDA_TRY(c, cudaHostGetDevicePointer((void **)&z.d_h_ab, z.h_ab, 0));
    NSS_CUDA_TRY(c, cudaHostGetDevicePointer((void **)&z.d_h_flags, z.h_flags, 0));
    NSS_CUDA_TRY(c, cudaMemsetAsync(z.counter, 0, 4 * sizeof(unsigned), c.stream));
    return NSS_OK;
}

// the FP64 scratch of the mixed refinement's Rayleigh-Ritz step (4 vectors)
int ensure_rrw(Ctx &c, int64_t n) {
    DevLanczos &z = c.lz;
    if (z.rrw) return NSS_OK;
    NSS_CUDA_TRY(c, ctx_alloc(c, &z.rrw, (size_t)4 * n));
    return NSS_OK;
}

template <class T>
int hv_t(Ctx &c, const T *v, T *hv, const int *stop);
template <>
int hv_t<double>(Ctx &c, const double *v, double *hv, const int *stop) { return hv_device(c, v, hv, stop); }
template <>
int hv_t<float>(Ctx &c, const float *v, float *hv, const int *stop) { return hv_device_fp32(c, v, hv, stop); }

// Anchored refinement of one eigenvector (mixed precision, second phase):
// the FP64 anchor u with theta0 = u.H.u and r = H u - theta0 u; the caller
// has put r/|r| (FP32) into V[0].  The result c0 u + sum_l c_l V[l] goes to
// `out` (may alias u).
struct AnchorSpec {
    const double *u;             // FP64 anchor (the combination uses it)
    const float *u32, *r32, *defl32;   // FP32 copies for the projections in k_orth
    int ndefl;
    double theta0;
    double *out;
};

// out = c[0] u + sum_l c[l+1] V[l]   (FP64 accumulation)
template <class T>
__global__ void __launch_bounds__(256) k_ritz_anchor(const T *__restrict__ V, int m, int64_t n,
                                                     const double *__restrict__ cvec, const double *u, double *out) {
    extern __shared__ double cs[];   // [m+1]
    for (int t = threadIdx.x; t <= m; t += blockDim.x) cs[t] = cvec[t];
    __syncthreads();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double acc = cs[0] * u[i];
        for (int l = 0; l < m; ++l) acc = fma((double)V[(int64_t)l * n + i], cs[l + 1], acc);
        out[i] = acc;
    }
}

// The Lanczos iterations on a basis of type T; leaves theta (Ritz values),
// svec (their T_m eigenvectors, stride m) and the Ritz vectors (FP64) in c.lz.
// With `anc` it runs the anchored refinement instead (one eigenvector).
// cluster_max > neigen (mixed first phase): the Ritz pairs just above the
// wanted ones whose values lie within CLUSTER_GAP (relative) of their lower
// neighbour are returned as well, up to cluster_max in all; *ne_out gets the
// number of Ritz vectors left in evecs.
constexpr double CLUSTER_GAP = 1e-4;
template <class T>
int run_lanczos(Ctx &c, T *V, T *w, int neigen, int mmax, double tol, uint64_t seed, int *numop_out,
                int *m_out, const AnchorSpec *anc = nullptr, int cluster_max = 0, int *ne_out = nullptr,
                const double *start = nullptr) {
    DevLanczos &z = c.lz;
    const int64_t n = c.sb.n;
    const int cap = z.cap;
    double *h1 = z.scal + S_NSCAL;
    double *rs_alpha = h1 + 2 * (cap + 2), *rs_beta = rs_alpha + (cap + 2);
    cudaStream_t st = c.stream;
    volatile int *hf = z.h_flags;
    double *ha = z.h_ab, *hb = z.h_ab + (cap + 1);
    // no kernel of this context is running: the previous solve synchronised
    for (int i = 0; i < F_NFLAGS + 8; ++i) hf[i] = 0;
    for (int i = 0; i <= cap; ++i) ha[i] = hb[i] = 0.0;
    NSS_CUDA_TRY(c, cudaMemsetAsync(z.flags, 0, F_NFLAGS * sizeof(int), st));
    NSS_CUDA_TRY(c, cudaMemsetAsync(z.beta, 0, (cap + 1) * sizeof(double), st));
    NSS_CUDA_TRY(c, cudaMemsetAsync(z.counter, 0, 4 * sizeof(unsigned), st));
    const int vb = 608;   // 4 CTAs per SM for elementwise kernels
    uint64_t restarts = 0;
    if (anc) {
        neigen = 1;
    } else {
        ++c.launches;
        if (start && sizeof(T) == sizeof(float))   // a given FP64 start vector (mixed refinement)
            k_to32<<<vb, 256, 0, st>>>((float *)(void *)V, start, 1.0, n);
        else
            k_random<T><<<vb, 256, 0, st>>>(V, n, seed, restarts);
        ++c.launches;
        normalize_dev<T>(z, V, n, st, c.launches);
    }
    const size_t dots_smem = (size_t)(cap + 2) * sizeof(double) + SUB * sizeof(T);
    const size_t upd_smem = (size_t)(cap + 2) * sizeof(double);
    allow_smem((const void *)k_dots<T>, dots_smem);
    allow_smem((const void *)k_update<T>, upd_smem);
    constexpr int CW = OrthCW<T>::value;
    OrthArgs oa;
    oa.V = V;
    oa.w = w;
    oa.n = n;
    oa.j = 0;
    oa.mmax = mmax;
    oa.pstride = cap + 8;
    oa.alpha = z.alpha;
    oa.beta = z.beta;
    oa.part = z.part;
    oa.bar = z.counter + 2;
    oa.flags = z.flags;
    oa.h_alpha = z.d_h_ab;
    oa.h_beta = z.d_h_ab + (cap + 1);
    oa.h_flags = z.d_h_flags;
    oa.anc_u = anc ? (const void *)anc->u32 : nullptr;
    oa.anc_r = anc ? (const void *)anc->r32 : nullptr;
    oa.defl = anc ? (const void *)anc->defl32 : nullptr;
    oa.ndefl = anc ? anc->ndefl : 0;
    oa.h_m = z.d_h_ab + 2 * (cap + 1);
    oa.spin = wait_limit();
    oa.jdev = nullptr;
    // the launched chunks keep vcur current too, so that a replayed chunk
    // can follow one
    oa.vcur = c.use_graphs ? z.vcur : nullptr;
    const double *hm = z.h_ab + 2 * (cap + 1);
    std::vector<double> cvec;
    // Chunks of CHECK iterations, each ending with an event; the host checks
    // chunk k on T_m while the GPU runs chunk k+1.
    cudaEvent_t evs[2];
    cudaEventCreateWithFlags(&evs[0], cudaEventDisableTiming);
    cudaEventCreateWithFlags(&evs[1], cudaEventDisableTiming);
    // mixed method without tensor-core sectors: one persistent launch per chunk
    const bool use_chunk = sizeof(T) == sizeof(float) && z.chunk_ok && c.sb.mma_nitems == 0;
    struct ChunkTiming {
        cudaEvent_t a, b;
        int j0, jend;
    };
    std::vector<ChunkTiming> ctime;
    if (use_chunk)   // slot 1 and 2 regions that no item writes must read as zero
        NSS_CUDA_TRY(c, cudaMemsetAsync(z.slot32 + n, 0, (size_t)2 * n * sizeof(float), st));
    bool from_v = true;   // the next chunk starts from V[j0] (start, restart)
    auto enqueue_chunk = [&](int j0, int slot) -> int {
        const int jend = std::min(mmax, j0 + CHECK);
        if (use_chunk && jend > j0) {
            ChunkArgs ca;
            ca.o = oa;
            ca.buf[0] = z.wbuf32;
            ca.buf[1] = z.wbuf32 + n;
            ca.j0 = j0;
            ca.jend = jend;
            ca.first_from_v = from_v ? 1 : 0;
            ca.slot[0] = z.slot32;
            ca.slot[1] = z.slot32 + n;
            ca.slot[2] = z.slot32 + 2 * n;
            ca.items = c.sb.d_items32;
            ca.nitems = c.sb.nitems32;
            ca.op = hv32_ops(c.sb);
            ca.vc = z.chunk_vc;
            ca.cs = z.chunk_cs;
            from_v = false;
            void *args[] = {&ca};
            ChunkTiming ct{nullptr, nullptr, j0, jend};
            if (c.time_chunks) {
                cudaEventCreate(&ct.a);
                cudaEventCreate(&ct.b);
                cudaEventRecord(ct.a, st);
            }
            cudaError_t e = cudaLaunchCooperativeKernel((const void *)k_chunk32, dim3(z.orth_grid),
                                                        dim3(ORTH_THREADS), args, z.chunk_smem_vc, st);
            if (c.time_chunks) {
                cudaEventRecord(ct.b, st);
                ctime.push_back(ct);
            }
            ++c.launches;
            if (e != cudaSuccess) {
                c.err = std::string("nss_eigh: cooperative launch failed: ") + cudaGetErrorString(e);
                return -1;
            }
            cudaEventRecord(evs[slot], st);
            return jend;
        }
        // a whole chunk of a plain (not anchored) Lanczos run replays the
        // CUDA graph of CHECK iterations captured for this superblock,
        // precision and iteration cap (the step and the input vector live on
        // the device); the first chunk of a key runs as launches and captures
        // the graph for the next ones
        const int prec = sizeof(T) == sizeof(float) ? 1 : 0;
        const bool key_ok = z.gx && z.gx_gen == c.sb.gen && z.gx_prec == prec && z.gx_mmax == mmax &&
                            z.gx_anc == oa.anc_u && z.gx_ndefl == oa.ndefl && z.gx_spin == oa.spin;
        const bool graphable = c.use_graphs && !z.gx_failed && jend - j0 == CHECK && oa.anc_u == nullptr;
        if (graphable && key_ok) {
            if (from_v)
                NSS_CUDA_TRY_R(c, cudaMemcpyAsync(z.vcur, V + (int64_t)j0 * n, (size_t)n * sizeof(T),
                                                  cudaMemcpyDeviceToDevice, st), -1);
            k_seti<<<1, 1, 0, st>>>(z.jdev, j0);
            NSS_CUDA_TRY_R(c, cudaGraphLaunch(z.gx, st), -1);
            c.launches += 1 + z.gx_launches;
            ++c.graph_replays;
            from_v = false;
            cudaEventRecord(evs[slot], st);
            return jend;
        }
        for (int jj = j0; jj < jend; ++jj) {
            if (hv_t<T>(c, V + (int64_t)jj * n, w, z.flags + F_STOP)) return -1;
            oa.j = jj;
            void *args[] = {&oa};
            cudaError_t e = cudaLaunchCooperativeKernel((const void *)k_orth<T, CW>, dim3(z.orth_grid),
                                                        dim3(ORTH_THREADS), args, z.orth_smem, st);
            ++c.launches;
            if (e != cudaSuccess) {
                c.err = std::string("nss_eigh: cooperative launch failed: ") + cudaGetErrorString(e);
                return -1;
            }
        }
        from_v = false;
        cudaEventRecord(evs[slot], st);
        if (graphable && !key_ok) {
            // record (not run) the iterations of a chunk: H*psi of vcur, then
            // k_orth stepping *jdev and writing the next vector to vcur
            if (z.gx) {
                cudaGraphExecDestroy(z.gx);
                z.gx = nullptr;
            }
            OrthArgs og = oa;
            og.jdev = z.jdev;
            og.vcur = z.vcur;
            const int64_t l0 = c.launches;
            cudaGraph_t g = nullptr;
            bool ok = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
            for (int it = 0; ok && it < CHECK; ++it) {
                if (hv_t<T>(c, (const T *)z.vcur, w, z.flags + F_STOP)) ok = false;
                void *args[] = {&og};
                if (ok && cudaLaunchCooperativeKernel((const void *)k_orth<T, CW>, dim3(z.orth_grid),
                                                      dim3(ORTH_THREADS), args, z.orth_smem, st) != cudaSuccess)
                    ok = false;
            }
            const cudaError_t ee = cudaStreamEndCapture(st, &g);
            ok = ok && ee == cudaSuccess && g && cudaGraphInstantiate(&z.gx, g, 0) == cudaSuccess;
            if (g) cudaGraphDestroy(g);
            cudaGetLastError();                      // a failed capture leaves nothing behind
            if (ok) {
                z.gx_gen = c.sb.gen;
                z.gx_prec = prec;
                z.gx_mmax = mmax;
                z.gx_anc = oa.anc_u;
                z.gx_ndefl = oa.ndefl;
                z.gx_spin = oa.spin;
                z.gx_launches = (int)(c.launches - l0);
                ++c.graph_captures;
            } else {
                if (z.gx) cudaGraphExecDestroy(z.gx);
                z.gx = nullptr;
                z.gx_failed = true;
                c.err.clear();
            }
            c.launches = l0;
        }
        return jend;
    };
    std::vector<double> theta(4, 0.0), resid(4, 0.0), upper(4, 0.0), svec, work;
    bool have_upper = false;
    int m_done = 1, rc = NSS_OK, ne_done = 1;
    bool converged = false;
    int slot = 0;
    int pend_end = enqueue_chunk(0, slot);
    if (pend_end < 0) rc = NSS_ERR_CUDA;
    while (pend_end >= 0) {
        const int next_end = (pend_end < mmax) ? enqueue_chunk(pend_end, slot ^ 1) : -2;
        if (next_end == -1) { rc = NSS_ERR_CUDA; break; }
        cudaError_t ce = cudaEventSynchronize(evs[slot]);
        if (ce != cudaSuccess) { c.err = cudaGetErrorString(ce); rc = NSS_ERR_CUDA; break; }
        if (hf[F_ERR]) {   // a bounded barrier wait ran out: nothing of this solve is trusted
            c.err = "nss_eigh: a grid barrier of the orthogonalisation kernel timed out (results discarded)";
            rc = NSS_ERR_CUDA;
            break;
        }
        // a breakdown inside this chunk ends it early; one flagged by the
        // chunk running ahead belongs to the next check
        int m = pend_end;
        const bool brk = hf[F_STOP] == 2 && hf[F_BREAK] <= pend_end;
        if (brk) m = hf[F_BREAK];
        const int ne = std::min(neigen, m);
        int conv = 0;
        if (anc) {
            // lowest eigenpair of [[theta0, m^T], [m, T_m]]
            cvec.resize((size_t)m + 1);
            double lam = 0.0, res = 0.0;
            if (arrow_lowest(anc->theta0, hm, ha, hb, m, hb[m - 1], &lam, cvec.data(), &res, work)) {
                theta[0] = lam;
                resid[0] = res;
                if (res <= tol * std::max(std::fabs(lam), 1e-300) || brk) conv = 1;
            }
        } else {
            svec.resize((size_t)ne * m);
            tridiag_lowest(ha, hb, m, ne, hb[m - 1], theta.data(), svec.data(), resid.data(),
                           (have_upper && ne == neigen) ? upper.data() : nullptr, work);
            for (int e = 0; e < ne; ++e) upper[e] = theta[e];
            have_upper = ne == neigen;
            for (int e = 0; e < ne; ++e)
                if (resid[e] <= tol * std::max(std::fabs(theta[e]), 1e-300)) ++conv;
        }
        m_done = m;
        ne_done = ne;
        if (conv >= ne || (int64_t)m >= n) {
            hf[F_NFLAGS] = 1;                        // stop request for the queued kernels
            std::atomic_thread_fence(std::memory_order_seq_cst);
            converged = true;
            break;
        }
        if (brk) {
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
            normalize_dev<T>(z, vn, n, st, c.launches);
            NSS_CUDA_TRY(c, cudaMemsetAsync(z.beta + (m_done - 1), 0, sizeof(double), st));
            NSS_CUDA_TRY(c, cudaMemsetAsync(z.flags, 0, F_NFLAGS * sizeof(int), st));
            NSS_CUDA_TRY(c, cudaStreamSynchronize(st));
            hb[m_done - 1] = 0.0;
            hf[F_STOP] = 0;
            hf[F_BREAK] = 0;
            from_v = true;
            slot = 0;
            pend_end = enqueue_chunk(m_done, slot);
            if (pend_end < 0) { rc = NSS_ERR_CUDA; break; }
            continue;
        }
        if (next_end < 0) break;   // iteration cap reached without convergence
        slot ^= 1;
        pend_end = next_end;
    }
    cudaError_t ce = cudaStreamSynchronize(st);
    cudaEventDestroy(evs[0]);
    cudaEventDestroy(evs[1]);
    for (const ChunkTiming &ct : ctime) {
        // launches that completed iterations of the basis the solve kept
        if (ce == cudaSuccess && ct.j0 < m_done) {
            float ms = 0.f;
            cudaEventElapsedTime(&ms, ct.a, ct.b);
            const int je = std::min(ct.jend, m_done);
            c.chunk_ms += ms;
            ++c.chunk_launches;
            c.chunk_iters += je - ct.j0;
            for (int jj = ct.j0; jj < je; ++jj) c.chunk_cols += jj + 1;
        }
        cudaEventDestroy(ct.a);
        cudaEventDestroy(ct.b);
    }
    if ((rc || ce != cudaSuccess) && z.gx) {   // a failed run keeps no graph
        cudaGraphExecDestroy(z.gx);
        z.gx = nullptr;
    }
    if (rc) return rc;
    if (ce != cudaSuccess) { c.err = cudaGetErrorString(ce); return NSS_ERR_CUDA; }
    int dflags[F_NFLAGS];
    NSS_CUDA_TRY(c, cudaMemcpy(dflags, z.flags, sizeof(dflags), cudaMemcpyDeviceToHost));
    if (dflags[F_ERR]) {
        c.err = "nss_eigh: a grid barrier of the orthogonalisation kernel timed out (results discarded)";
        return NSS_ERR_CUDA;
    }
    *numop_out = m_done;
    *m_out = m_done;
    if (!converged) {
        c.err = "nss_eigh: no convergence within nitermax=" + std::to_string(mmax) + " iterations";
        return NSS_ERR_NOCONV;
    }
    if (anc) {
        if (cvec.size() != (size_t)m_done + 1) {
            c.err = "nss_eigh: the anchored refinement found no eigenpair";
            return NSS_ERR_NOCONV;
        }
        NSS_CUDA_TRY(c, cudaMemcpyAsync(z.svec, cvec.data(), cvec.size() * sizeof(double), cudaMemcpyHostToDevice, st));
        c.launches += 2;
        k_ritz_anchor<T><<<NBLK, 256, cvec.size() * sizeof(double), st>>>(V, m_done, n, z.svec, anc->u, anc->out);
        normalize_dev<double>(z, anc->out, n, st, c.launches);
        NSS_CUDA_TRY(c, cudaGetLastError());
        NSS_CUDA_TRY(c, cudaStreamSynchronize(st));
        z.last_anchor_theta = theta[0];
        return NSS_OK;
    }
    if (cluster_max > ne_done && m_done > ne_done && (int64_t)cluster_max * cluster_max <= cap + 2) {
        // near-degenerate partners of the wanted pairs (see cluster_max)
        const int ntry = std::min(cluster_max, m_done);
        std::vector<double> th2(ntry), sv2((size_t)ntry * m_done), rs2(ntry);
        tridiag_lowest(ha, hb, m_done, ntry, hb[m_done - 1], th2.data(), sv2.data(), rs2.data(), nullptr, work);
        double scale = 0.0;
        for (int e = 0; e < ntry; ++e) scale = std::max(scale, std::fabs(th2[e]));
        int k = ne_done;
        while (k < ntry && th2[k] - th2[k - 1] <= CLUSTER_GAP * scale) ++k;
        if (k > ne_done) {
            for (int e = 0; e < k; ++e) {
                theta[e] = th2[e];
                resid[e] = rs2[e];
            }
            svec.assign(sv2.begin(), sv2.begin() + (size_t)k * m_done);
            ne_done = k;
        }
    }
    if (ne_out) *ne_out = ne_done;
    const int ne = ne_done;
    NSS_CUDA_TRY(c, cudaMemcpyAsync(z.theta, theta.data(), ne * sizeof(double), cudaMemcpyHostToDevice, st));
    NSS_CUDA_TRY(c, cudaMemcpyAsync(z.resid, resid.data(), ne * sizeof(double), cudaMemcpyHostToDevice, st));
    NSS_CUDA_TRY(c, cudaMemcpyAsync(z.svec, svec.data(), (size_t)ne * m_done * sizeof(double),
                                    cudaMemcpyHostToDevice, st));
    ++c.launches;
    k_ritz<T><<<NBLK, 256, (size_t)ne * m_done * sizeof(double), st>>>(V, m_done, n, z.svec, m_done, ne, z.evecs);
    for (int e = 0; e < ne; ++e) {
        ++c.launches;
        normalize_dev<double>(z, z.evecs + (int64_t)e * n, n, st, c.launches);
    }
    NSS_CUDA_TRY(c, cudaGetLastError());
    // the pageable sources above are consumed before this returns
    NSS_CUDA_TRY(c, cudaStreamSynchronize(st));
    return NSS_OK;
}

}  // namespace

void lanczos_release(Ctx &c) {
    DevLanczos &z = c.lz;
    void *ptrs[] = {z.V, z.w, z.V32, z.w32, z.anc32, z.wbuf32, z.slot32, z.evecs, z.rrw, z.scal, z.part, z.counter,
                    z.alpha, z.beta, z.theta, z.resid, z.svec, z.flags, z.pitem, z.vcur, z.jdev};
    if (z.gx) cudaGraphExecDestroy(z.gx);
    for (void *p : ptrs) ctx_free(c, p);
    if (z.h_flags) cudaFreeHost(z.h_flags);
    if (z.h_ab) cudaFreeHost(z.h_ab);
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
    c.chunk_ms = 0.0;
    c.graph_replays = 0;
    c.graph_captures = 0;
    c.chunk_launches = 0;
    c.chunk_iters = 0;
    c.chunk_cols = 0.0;
    cudaStream_t st = c.stream;
    // the tensor-core pipeline's error word belongs to this solve
    if (mixed && s.d_tc_err) NSS_CUDA_TRY(c, cudaMemsetAsync(s.d_tc_err, 0, sizeof(int), st));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, st);
    int numop_ = 0, m_done = 0, kcl = 1;
    if (!mixed) {
        rc = run_lanczos<double>(c, z.V, z.w, neigen, mmax, tol, seed, &numop_, &m_done);
    } else {
        // after a solve that needed a near-degenerate partner (consecutive
        // DMRG steps have alike spectra) the FP32 phase also converges the
        // next Ritz pair, so that the pair is resolved when it stops
        const int want32 = std::min(4, neigen + (c.last_pair ? 1 : 0));
        rc = run_lanczos<float>(c, z.V32, z.w32, want32, mmax, std::max(tol, mixed_tol()), seed, &numop_, &m_done,
                                nullptr, std::min(4, want32 + 2), &kcl);
        if (rc == NSS_ERR_NOCONV && want32 > neigen) {
            // the extra pair did not converge within nitermax: the wanted ones alone
            int it0 = numop_;
            rc = run_lanczos<float>(c, z.V32, z.w32, neigen, mmax, std::max(tol, mixed_tol()), seed, &numop_, &m_done,
                                    nullptr, std::min(4, neigen + 2), &kcl);
            numop_ += it0;
        }
    }
    const int ne = (int)std::min<int64_t>(neigen, std::max(m_done, 1));
    if (!rc && mixed) {
        // Iterative refinement of the FP32 Ritz vectors to FP64 quality.  Each
        // pass takes every vector u (deflated against the ones before it) as
        // an FP64 anchor: theta0 = u.H.u and r = H u - theta0 u in FP64; a
        // vector with ||r|| <= tol |theta0| is final, any other gets an FP32
        // Lanczos run on the complement of u started from r/|r|, with the
        // couplings u.H.v = r.v in FP64, solved on the host.  The FP32 errors
        // then only touch the correction, which shrinks by about
        // eps32 ||H|| / gap per pass, gap the distance to the nearest other
        // eigenvalue.  Near-degenerate partners (within CLUSTER_GAP of the
        // wanted pairs, e.g. the singlet and Sz=0 triplet of a spin-1
        // chain's edge spins, split by ~1e-7 relative) would make that factor
        // ~1: they are refined along, and before every later pass an FP64
        // Rayleigh-Ritz step on the cluster resolves the mixing among them
        // exactly, so only the gap to the rest of the spectrum matters.  The
        // passes end when every wanted vector meets the FP64 residual test;
        // after MAX_PASSES without that the solve is redone in FP64.
        constexpr int MAX_PASSES = 8;
        double *r = z.scal + S_NSCAL + 4 * (z.cap + 2);   // 8 refinement slots
        double *h1 = z.scal + S_NSCAL;
        double *rs_alpha = h1 + 2 * (z.cap + 2), *rs_beta = rs_alpha + (z.cap + 2);
        const size_t dots_smem = (size_t)(z.cap + 2) * sizeof(double) + SUB * sizeof(double);
        const size_t upd_smem = (size_t)(z.cap + 2) * sizeof(double);
        allow_smem((const void *)k_dots<double>, dots_smem);
        allow_smem((const void *)k_update<double>, upd_smem);
        // w -= Y (Y^T w) against the e vectors before it; returns via scal[S_BB]
        auto deflate = [&](double *vec, int e) -> int {
            NSS_CUDA_TRY(c, cudaMemsetAsync(z.flags, 0, F_NFLAGS * sizeof(int), st));
            NSS_CUDA_TRY(c, cudaMemsetAsync(z.scal + S_ALPHA, 0, sizeof(double), st));
            c.launches += 2;
            k_dots<double><<<NBLK, 256, dots_smem, st>>>(z.evecs, e, vec, n, z.part, h1, z.scal, z.counter, z.flags,
                                                         0, 0, z.beta);
            k_update<double><<<NBLK, 256, upd_smem, st>>>(z.evecs, e, vec, n, h1, z.part, z.scal, z.counter, z.flags,
                                                          rs_alpha, rs_beta, 0);
            return NSS_OK;
        };
        double th[4] = {0, 0, 0, 0}, res[4] = {0, 0, 0, 0};
        // FP64 check of wanted vector e (deflated against the ones before it
        // and normalised): th[e] = u.H.u, res[e] = ||H u - th u||; leaves
        // r = H u - th u in z.w (deflated for e > 0) and its norm in *beta0
        double rr_lam[4] = {0, 0, 0, 0};
        int rr_k = 0;                                // cluster size of the last Rayleigh-Ritz step
        bool rr_fresh = false;                       // rrw holds H U of the current U
        auto check = [&](int e, double *beta0) -> int {
            double *u = z.evecs + (int64_t)e * n;
            if (e > 0) {
                if (int rc2 = deflate(u, e)) return rc2;
                ++c.launches;
                normalize_dev<double>(z, u, n, st, c.launches);
            }
            if (e == 0 && rr_fresh) {
                // right after a Rayleigh-Ritz step H u_0 is known
                NSS_CUDA_TRY(c, cudaMemcpyAsync(z.w, z.rrw, (size_t)n * sizeof(double), cudaMemcpyDeviceToDevice, st));
            } else {
                if (int rc2 = hv_device(c, u, z.w)) return rc2;
                ++numop_;
            }
            rr_fresh = false;
            c.launches += 2;
            k_rq<<<NBLK, 256, 0, st>>>(u, z.w, n, z.part, r, z.counter);
            k_anchor_r<<<NBLK, 256, 0, st>>>(u, z.w, n, z.part, r, z.counter);
            double hr[8];
            NSS_CUDA_TRY(c, cudaMemcpyAsync(hr, r, 8 * sizeof(double), cudaMemcpyDeviceToHost, st));
            NSS_CUDA_TRY(c, cudaStreamSynchronize(st));
            th[e] = hr[0] / hr[2];
            res[e] = std::sqrt(std::max(hr[4], 0.0));
            double rr = hr[4];
            if (e > 0) {
                if (int rc2 = deflate(z.w, e)) return rc2;
                NSS_CUDA_TRY(c, cudaMemcpyAsync(&rr, z.scal + S_BB, sizeof(double), cudaMemcpyDeviceToHost, st));
                NSS_CUDA_TRY(c, cudaStreamSynchronize(st));
            }
            *beta0 = std::sqrt(std::max(rr, 0.0));
            return NSS_OK;
        };
        // anchored FP32 correction of wanted vector e, right after check(e)
        auto refine = [&](int e, double beta0) -> int {
            double *u = z.evecs + (int64_t)e * n;
            float *u32 = z.anc32, *r32 = z.anc32 + n, *y32 = z.anc32 + 2 * n;
            c.launches += 3 + e;
            k_to32<<<608, 256, 0, st>>>(z.V32, z.w, 1.0 / beta0, n);
            k_to32<<<608, 256, 0, st>>>(u32, u, 1.0, n);
            k_to32<<<608, 256, 0, st>>>(r32, z.w, 1.0, n);
            for (int f = 0; f < e; ++f)
                k_to32<<<608, 256, 0, st>>>(y32 + (int64_t)f * n, z.evecs + (int64_t)f * n, 1.0, n);
            AnchorSpec as{u, u32, r32, y32, e, th[e], u};
            int it2 = 0, m2 = 0;
            // the anchored problem is solved to 1e-6 of the vector's residual
            // (from the FP32 phase's 1e-7 that is the final tolerance: one
            // pass; a stalled pass cannot gain more than its FP32 floor)
            const double tol_pass = std::max(tol, 1e-6 * beta0 / std::max(std::fabs(th[e]), 1e-300));
            if (int rc2 = run_lanczos<float>(c, z.V32, z.w32, 1, mmax, tol_pass, seed, &it2, &m2, &as)) return rc2;
            numop_ += it2;
            return NSS_OK;
        };
        // FP64 Rayleigh-Ritz on the k cluster vectors: orthonormalise them,
        // W = H U (into the FP64 scratch), G = U^T W, U <- U Q with G's
        // eigenvectors Q in ascending order
        auto rayleigh_ritz = [&](int k) -> int {
            if (k < 1 || k > 4) { c.err = "nss_eigh: Rayleigh-Ritz over 1 to 4 vectors"; return NSS_ERR_INVALID; }
            ++c.launches;
            normalize_dev<double>(z, z.evecs, n, st, c.launches);
            for (int e = 1; e < k; ++e) {
                double *u = z.evecs + (int64_t)e * n;
                if (int rc2 = deflate(u, e)) return rc2;
                ++c.launches;
                normalize_dev<double>(z, u, n, st, c.launches);
            }
            for (int e = 0; e < k; ++e) {
                if (int rc2 = hv_device(c, z.evecs + (int64_t)e * n, z.rrw + (int64_t)e * n)) return rc2;
                ++numop_;
            }
            ++c.launches;
            k_gram<<<NBLK, 256, 0, st>>>(z.evecs, z.rrw, k, n, z.part, h1, z.counter);
            double g[16];
            NSS_CUDA_TRY(c, cudaMemcpyAsync(g, h1, (size_t)k * k * sizeof(double), cudaMemcpyDeviceToHost, st));
            NSS_CUDA_TRY(c, cudaStreamSynchronize(st));
            double a[16], q[16], lam[4];
            for (int i = 0; i < k; ++i)
                for (int j = 0; j < k; ++j) a[i * k + j] = 0.5 * (g[i * k + j] + g[j * k + i]);
            sym_eig_small(k, a, lam, q);
            for (int e = 0; e < k; ++e) rr_lam[e] = lam[e];
            rr_k = k;
            Rot4 R{};
            for (int i = 0; i < k; ++i)
                for (int j = 0; j < k; ++j) R.q[j * 4 + i] = q[j * k + i];
            c.launches += 2;
            k_rot<<<608, 256, 0, st>>>(z.evecs, k, n, R);
            k_rot<<<608, 256, 0, st>>>(z.rrw, k, n, R);   // H U along, for the next check
            NSS_CUDA_TRY(c, cudaGetLastError());
            rr_fresh = true;
            return NSS_OK;
        };
        // k: the cluster (wanted vectors and partners); the passes
        int k = kcl;
        if (!rc) rc = ensure_rrw(c, n);
        bool done = false, rr_due = k > ne, rerun = false;
        double prev[4] = {0, 0, 0, 0};
        int passes = 0;
        for (; passes < MAX_PASSES && !rc && !done; ++passes) {
            if (rr_due && (rc = rayleigh_ritz(k))) break;
            const bool rr_now = rr_due;
            rr_due = false;
            bool all = true, redo = false;
            for (int e = 0; e < ne && !rc; ++e) {
                double beta0 = 0.0;
                if ((rc = check(e, &beta0))) break;
                if (res[e] <= tol * std::fabs(th[e])) continue;
                all = false;
                // a correction that gained less than 20x: the vector is mixed
                // with a near-degenerate state the cluster lacks or resolves
                // no longer
                const bool stalled = passes > 0 && !rr_now && res[e] > 0.05 * prev[e];
                if (stalled && k > ne) {
                    rr_due = redo = true;
                    break;
                }
                if (stalled && ne == 1 && !rerun) {
                    // the FP32 phase stopped before it resolved the pair: a
                    // short FP32 Lanczos run from the vector, which lies
                    // almost inside the pair's plane, finds both states
                    rerun = true;
                    int it3 = 0, m3 = 0, k3 = 2;
                    const int rc3 = run_lanczos<float>(c, z.V32, z.w32, 2, std::min(mmax, 160), std::max(tol, mixed_tol()),
                                                       seed, &it3, &m3, nullptr, 4, &k3, z.evecs);
                    numop_ += it3;
                    if (rc3 == NSS_ERR_NOCONV) break;   // left to the passes' limit
                    if ((rc = rc3)) break;
                    k = std::max(k3, 2);
                    rr_due = redo = true;
                    break;
                }
                if (!(beta0 > 0.0)) continue;
                if ((rc = refine(e, beta0))) break;
            }
            if (rc) break;
            if (all) done = true;
            else if (!redo)
                for (int e = 0; e < ne; ++e) prev[e] = res[e];
        }
        c.refine_passes = passes;
        c.refine_cluster = k;
        c.last_pair = rr_k > ne && rr_lam[ne] - rr_lam[ne - 1] <= CLUSTER_GAP * std::fabs(rr_lam[0]);
        if (!rc && done) {
            for (int e = 0; e < ne; ++e) z.last_resid[e] = res[e];
            NSS_CUDA_TRY(c, cudaMemcpyAsync(z.theta, th, ne * sizeof(double), cudaMemcpyHostToDevice, st));
            NSS_CUDA_TRY(c, cudaStreamSynchronize(st));
        } else if (!rc) {
            // the FP32 corrections did not reach tol: the plain FP64 method
            ++c.mixed_fallbacks;
            if ((rc = ensure_lanczos(c, n, mmax + 1, false)) == NSS_OK) {
                int it64 = 0;
                rc = run_lanczos<double>(c, c.lz.V, c.lz.w, neigen, mmax, tol, seed, &it64, &m_done);
                numop_ += it64;
            }
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
    if (mixed) tune_record(c, ms, numop_);
    z.last_iters = m_done;
    z.neigen_done = ne;
    if (numop) *numop = numop_;
    return NSS_OK;
}


// ---------------------------------------------------------------------------
// Batch engine (mixed precision): every solve keeps its own context
// (superblock, Krylov basis, host mirrors); one cooperative launch of
// k_batch32 per round runs CHECK iterations of every solve in flight, then
// the host checks each solve (tridiagonal or anchored problem) and moves it
// through FP32 Lanczos -> anchored refinement -> FP64 energy, as
// lanczos_eigh does for one context.  Solves can join between rounds
// (continuous batching: nss_batch_add) and leave when done (nss_batch_step
// reports them).  The per-round follow-up work of all solves (Ritz vectors,
// FP64 products, restarts) is queued back to back with one synchronisation.

namespace {

struct BatchState {
    Ctx *c = nullptr;
    int id = 0;
    int64_t n = 0;
    int mmax = 0, phase = 1, j0 = 0, m_done = 0, numop = 0, rc = 0;
    bool from_v = true, have_upper = false;
    double tol = 0.0, tol_final = 0.0, theta0 = 0.0, result = 0.0;
    uint64_t seed = 0, restarts = 0;
    std::vector<double> theta, resid, upper, svec, work, cvec;
    AnchorSpec as{};
};

}  // namespace

struct BatchEngine {
    Ctx *c0 = nullptr;           // owns the stream, the barrier and the argument buffers
    std::vector<BatchState> solves;
    int next_id = 1;
    BatchSolve *d_solves = nullptr, *h_solves = nullptr;
    int2 *d_gitems = nullptr, *h_gitems = nullptr;
    int cap_items = 0;
    float *d_st = nullptr;
    unsigned *d_q = nullptr;     // item queue heads of a launch
    double *h_res = nullptr;     // [BATCH_MAX][8] pinned refinement results
    size_t smem_set = 0;         // dynamic shared memory of its launches (the most any round needed)
    ~BatchEngine() {
        if (!c0) return;
        cudaStreamSynchronize(c0->stream);
        ctx_free(*c0, d_solves);
        ctx_free(*c0, d_gitems);
        ctx_free(*c0, d_st);
        ctx_free(*c0, d_q);
        if (h_solves) cudaFreeHost(h_solves);
        if (h_gitems) cudaFreeHost(h_gitems);
        if (h_res) cudaFreeHost(h_res);
    }
};

namespace {

int engine_init(BatchEngine &E, Ctx &c0) {
    E.c0 = &c0;
    // the barrier, error word and refinement scratch live in c0's Lanczos state
    if (!c0.lz.flags) {
        int rc = ensure_lanczos(c0, std::max<int64_t>(c0.sb.valid ? c0.sb.n : 1, 1), 8, true);
        if (rc) return rc;
    }
    NSS_CUDA_TRY(c0, ctx_alloc(c0, &E.d_solves, (size_t)BATCH_MAX));
    NSS_CUDA_TRY(c0, ctx_alloc(c0, &E.d_st, (size_t)4 * BATCH_MAX));
    NSS_CUDA_TRY(c0, ctx_alloc(c0, &E.d_q, (size_t)CHUNK_MAXIT));
    NSS_CUDA_TRY(c0, cudaMallocHost((void **)&E.h_solves, sizeof(BatchSolve) * BATCH_MAX));
    NSS_CUDA_TRY(c0, cudaMallocHost((void **)&E.h_res, sizeof(double) * 8 * BATCH_MAX));
    NSS_CUDA_TRY(c0, cudaMemsetAsync(c0.lz.counter, 0, 4 * sizeof(unsigned), c0.stream));
    NSS_CUDA_TRY(c0, cudaMemsetAsync(c0.lz.flags, 0, F_NFLAGS * sizeof(int), c0.stream));
    return NSS_OK;
}

int engine_start_run(BatchEngine &E, BatchState &B) {
    Ctx &c0 = *E.c0;
    DevLanczos &z = B.c->lz;
    volatile int *hf = z.h_flags;
    for (int i = 0; i < F_NFLAGS + 8; ++i) hf[i] = 0;
    for (int i = 0; i < 3 * (z.cap + 1); ++i) z.h_ab[i] = 0.0;
    cudaStream_t st = c0.stream;
    NSS_CUDA_TRY(c0, cudaMemsetAsync(z.flags, 0, F_NFLAGS * sizeof(int), st));
    NSS_CUDA_TRY(c0, cudaMemsetAsync(z.beta, 0, (z.cap + 1) * sizeof(double), st));
    NSS_CUDA_TRY(c0, cudaMemsetAsync(z.slot32 + B.n, 0, (size_t)2 * B.n * sizeof(float), st));
    B.j0 = 0;
    B.from_v = true;
    B.have_upper = false;
    return NSS_OK;
}

int engine_add(BatchEngine &E, Ctx &c, uint64_t seed, int nitermax, double tol, int *id) {
    Ctx &c0 = *E.c0;
    if ((int)E.solves.size() >= std::min(BATCH_MAX, c0.lz.orth_grid)) {
        c0.err = "nss_batch_add: the batch is full";
        return NSS_ERR_INVALID;
    }
    if (c.device != c0.device) { c0.err = "nss_batch_add: the context is on another device"; return NSS_ERR_INVALID; }
    if (!c.sb.valid) { c0.err = "nss_batch_add: the context has no superblock"; return NSS_ERR_STATE; }
    for (auto &S : E.solves)
        if (S.c == &c) { c0.err = "nss_batch_add: the context is already in the batch"; return NSS_ERR_INVALID; }
    if (tol <= 0.0) tol = 1e-15;
    if (nitermax <= 0) nitermax = 512;
    BatchState B;
    B.c = &c;
    B.id = E.next_id++;
    B.n = c.sb.n;
    B.mmax = (int)std::min<int64_t>(B.n, nitermax);
    B.tol = std::max(tol, mixed_tol());
    B.tol_final = tol;
    B.seed = seed;
    B.theta.assign(4, 0.0);
    B.resid.assign(4, 0.0);
    B.upper.assign(4, 0.0);
    int rc = ensure_lanczos(c, B.n, B.mmax + 1, true);
    if (rc) { c0.err = c.err; return rc; }
    DevLanczos &z = c.lz;
    if (!z.chunk_ok) { c0.err = "nss_batch_add: the persistent kernel does not fit this Krylov basis"; return NSS_ERR_INVALID; }
    if (!z.pitem || z.cap_pitem < c.sb.nitems32) {
        ctx_free(c, z.pitem);
        z.pitem = nullptr;
        NSS_CUDA_TRY(c0, ctx_alloc(c, &z.pitem, (size_t)std::max(c.sb.nitems32, 1)));
        z.cap_pitem = c.sb.nitems32;
    }
    if ((rc = engine_start_run(E, B))) return rc;
    cudaStream_t st = c0.stream;
    c0.launches += 2;
    k_random<float><<<608, 256, 0, st>>>(z.V32, B.n, B.seed, 0);
    normalize_dev<float>(z, z.V32, B.n, st, c0.launches);
    NSS_CUDA_TRY(c0, cudaGetLastError());
    if (id) *id = B.id;
    E.solves.push_back(std::move(B));
    return NSS_OK;
}

// One round: a launch over every solve in flight, the host checks, the
// follow-up work.  Finished solves are removed and reported.
int engine_step(BatchEngine &E, int max_done, int *ndone, int *ids, double *energies, int *numops) {
    Ctx &c0 = *E.c0;
    cudaStream_t st = c0.stream;
    if (ndone) *ndone = 0;
    const int G = c0.lz.orth_grid;
    std::vector<int> act;
    for (int b = 0; b < (int)E.solves.size(); ++b)
        if ((E.solves[b].phase == 1 || E.solves[b].phase == 2) && E.solves[b].rc == 0) act.push_back(b);
    const int na = (int)act.size();
    if (na > 0) {
        double ntot = 0.0;
        for (int b : act) ntot += (double)E.solves[b].n;
        // CTAs per solve for its rows: one each, the rest in proportion to
        // the orthogonalisation's work, rows x basis columns (largest
        // remainders take the leftovers)
        std::vector<int> ncta(na, 1);
        {
            std::vector<double> wgt(na);
            double wtot = 0.0;
            for (int q = 0; q < na; ++q) {
                const BatchState &B = E.solves[act[q]];
                wgt[q] = (double)B.n * (double)(B.j0 + CHECK + 16);
                wtot += wgt[q];
            }
            int left = G - na;
            std::vector<std::pair<double, int>> rem;
            const int pool = left;
            for (int q = 0; q < na && pool > 0; ++q) {
                const double share = pool * wgt[q] / wtot;
                const int whole = std::min(left, (int)share);
                ncta[q] += whole;
                left -= whole;
                rem.push_back({share - whole, q});
            }
            std::stable_sort(rem.begin(), rem.end(), [](const auto &x, const auto &y) { return x.first > y.first; });
            for (size_t r = 0; r < rem.size() && left > 0; ++r, --left) ++ncta[rem[r].second];
        }
        int tot_items = 0;
        for (int b : act) tot_items += E.solves[b].c->sb.nitems32;
        if (tot_items > E.cap_items) {
            ctx_free(c0, E.d_gitems);
            E.d_gitems = nullptr;
            if (E.h_gitems) cudaFreeHost(E.h_gitems);
            E.h_gitems = nullptr;
            NSS_CUDA_TRY(c0, ctx_alloc(c0, &E.d_gitems, (size_t)tot_items));
            NSS_CUDA_TRY(c0, cudaMallocHost((void **)&E.h_gitems, sizeof(int2) * tot_items));
            E.cap_items = tot_items;
        }
        int cta = 0, ng = 0;
        size_t smem_max = 0;
        std::vector<std::pair<int, int2>> order;
        order.reserve(tot_items);
        for (int q = 0; q < na; ++q) {
            BatchState &B = E.solves[act[q]];
            Ctx &c = *B.c;
            DevLanczos &z = c.lz;
            smem_max = std::max(smem_max, z.chunk_smem);
            BatchSolve bs{};
            ChunkArgs &ca = bs.c;
            OrthArgs &oa = ca.o;
            oa.V = z.V32;
            oa.w = z.w32;
            oa.n = B.n;
            oa.j = B.j0;
            oa.mmax = B.mmax;
            oa.pstride = z.cap + 8;
            oa.alpha = z.alpha;
            oa.beta = z.beta;
            oa.part = z.part;
            oa.bar = nullptr;
            oa.flags = z.flags;
            oa.h_alpha = z.d_h_ab;
            oa.h_beta = z.d_h_ab + (z.cap + 1);
            oa.h_flags = z.d_h_flags;
            oa.h_m = z.d_h_ab + 2 * (z.cap + 1);
            oa.spin = wait_limit();
            const bool anc = B.phase == 2;
            oa.anc_u = anc ? (const void *)B.as.u32 : nullptr;
            oa.anc_r = anc ? (const void *)B.as.r32 : nullptr;
            oa.defl = anc ? (const void *)B.as.defl32 : nullptr;
            oa.ndefl = 0;
            ca.buf[0] = z.wbuf32;
            ca.buf[1] = z.wbuf32 + B.n;
            ca.slot[0] = z.slot32;
            ca.slot[1] = z.slot32 + B.n;
            ca.slot[2] = z.slot32 + 2 * B.n;
            ca.j0 = B.j0;
            ca.jend = std::min(B.mmax, B.j0 + CHECK);
            ca.first_from_v = B.from_v ? 1 : 0;
            ca.items = c.sb.d_items32;
            ca.nitems = c.sb.nitems32;
            ca.op = hv32_ops(c.sb);
            bs.pitem = z.pitem;
            bs.cta0 = cta;
            bs.ncta = ncta[q];
            bs.active = 1;
            cta += ncta[q];
            E.h_solves[q] = bs;
            for (int li = 0; li < c.sb.nitems32; ++li) order.push_back({c.sb.item_cost[li], make_int2(q, li)});
            B.from_v = false;
        }
        std::stable_sort(order.begin(), order.end(),
                         [](const std::pair<int, int2> &x, const std::pair<int, int2> &y) { return x.first > y.first; });
        for (auto &o : order) E.h_gitems[ng++] = o.second;
        NSS_CUDA_TRY(c0, cudaMemcpyAsync(E.d_solves, E.h_solves, sizeof(BatchSolve) * na, cudaMemcpyHostToDevice, st));
        NSS_CUDA_TRY(c0, cudaMemcpyAsync(E.d_gitems, E.h_gitems, sizeof(int2) * std::max(ng, 1), cudaMemcpyHostToDevice,
                                         st));
        NSS_CUDA_TRY(c0, allow_smem((const void *)k_batch32, smem_max));
        E.smem_set = std::max(E.smem_set, smem_max);
        NSS_CUDA_TRY(c0, cudaMemsetAsync(E.d_q, 0, CHUNK_MAXIT * sizeof(unsigned), st));
        BatchArgs ba;
        ba.qcnt = E.d_q;
        ba.s = E.d_solves;
        ba.ns = na;
        ba.nitems = ng;
        ba.gitems = E.d_gitems;
        ba.st = E.d_st;
        ba.bar = c0.lz.counter + 2;
        ba.err = c0.lz.flags + F_ERR;
        ba.steps = CHECK;
        ba.spin = wait_limit();
        void *args[] = {&ba};
        cudaError_t e = cudaLaunchCooperativeKernel((const void *)k_batch32, dim3(G), dim3(ORTH_THREADS), args,
                                                    E.smem_set, st);
        ++c0.launches;
        if (e != cudaSuccess) {
            c0.err = std::string("nss_batch: cooperative launch failed: ") + cudaGetErrorString(e);
            return NSS_ERR_CUDA;
        }
        cudaError_t ce = cudaStreamSynchronize(st);
        if (ce != cudaSuccess) { c0.err = cudaGetErrorString(ce); return NSS_ERR_CUDA; }
        int err_flag = 0;
        NSS_CUDA_TRY(c0, cudaMemcpy(&err_flag, c0.lz.flags + F_ERR, sizeof(int), cudaMemcpyDeviceToHost));
        if (err_flag) {
            c0.err = "nss_batch: a grid barrier timed out (results discarded)";
            return NSS_ERR_CUDA;
        }
    }
    // host checks
    std::vector<int> p1, p2, p3;
    for (int b : act) {
        BatchState &B = E.solves[b];
        Ctx &c = *B.c;
        DevLanczos &z = c.lz;
        volatile int *hf = z.h_flags;
        const double *ha = z.h_ab, *hb = z.h_ab + (z.cap + 1), *hm = z.h_ab + 2 * (z.cap + 1);
        const int jend = std::min(B.mmax, B.j0 + CHECK);
        int m = jend;
        const bool brk = hf[F_STOP] == 2 && hf[F_BREAK] <= jend;
        if (brk) m = hf[F_BREAK];
        bool conv = false;
        if (B.phase == 1) {
            B.svec.resize((size_t)m);
            tridiag_lowest(ha, hb, m, 1, hb[m - 1], B.theta.data(), B.svec.data(), B.resid.data(),
                           B.have_upper ? B.upper.data() : nullptr, B.work);
            B.upper[0] = B.theta[0];
            B.have_upper = true;
            conv = B.resid[0] <= B.tol * std::max(std::fabs(B.theta[0]), 1e-300) || (int64_t)m >= B.n;
        } else {
            B.cvec.resize((size_t)m + 1);
            double lam = 0.0, res = 0.0;
            if (arrow_lowest(B.theta0, hm, ha, hb, m, hb[m - 1], &lam, B.cvec.data(), &res, B.work))
                conv = res <= B.tol_final * std::max(std::fabs(lam), 1e-300) || brk;
            else
                B.cvec.clear();
        }
        B.m_done = m;
        if (!conv) {
            if (brk && B.phase == 1) {
                // invariant subspace without convergence: restart from a random
                // vector orthogonal to the basis
                ++B.restarts;
                float *vn = z.V32 + (int64_t)m * B.n;
                const size_t dots_smem = (size_t)(z.cap + 2) * sizeof(double) + SUB * sizeof(float);
                const size_t upd_smem = (size_t)(z.cap + 2) * sizeof(double);
                allow_smem((const void *)k_dots<float>, dots_smem);
                allow_smem((const void *)k_update<float>, upd_smem);
                double *h1 = z.scal + S_NSCAL;
                double *rs_alpha = h1 + 2 * (z.cap + 2), *rs_beta = rs_alpha + (z.cap + 2);
                c0.launches += 6;
                k_random<float><<<608, 256, 0, st>>>(vn, B.n, B.seed, B.restarts);
                NSS_CUDA_TRY(c0, cudaMemsetAsync(z.flags, 0, F_NFLAGS * sizeof(int), st));
                for (int pass = 0; pass < 2; ++pass) {
                    NSS_CUDA_TRY(c0, cudaMemsetAsync(z.scal + S_ALPHA, 0, sizeof(double), st));
                    k_dots<float><<<NBLK, 256, dots_smem, st>>>(z.V32, m, vn, B.n, z.part, h1, z.scal, z.counter,
                                                                z.flags, 0, 0, z.beta);
                    k_update<float><<<NBLK, 256, upd_smem, st>>>(z.V32, m, vn, B.n, h1, z.part, z.scal, z.counter,
                                                                 z.flags, rs_alpha, rs_beta, 0);
                }
                normalize_dev<float>(z, vn, B.n, st, c0.launches);
                NSS_CUDA_TRY(c0, cudaMemsetAsync(z.beta + (m - 1), 0, sizeof(double), st));
                NSS_CUDA_TRY(c0, cudaMemsetAsync(z.flags, 0, F_NFLAGS * sizeof(int), st));
                z.h_ab[(z.cap + 1) + m - 1] = 0.0;
                hf[F_STOP] = 0;
                hf[F_BREAK] = 0;
                B.j0 = m;
                B.from_v = true;
            } else if (m >= B.mmax) {
                c.err = "nss_eigh: no convergence within nitermax=" + std::to_string(B.mmax) + " iterations";
                B.rc = NSS_ERR_NOCONV;
            } else {
                B.j0 = jend;
            }
            continue;
        }
        B.numop += m;
        (B.phase == 1 ? p1 : p2).push_back(b);
    }
    for (int b = 0; b < (int)E.solves.size(); ++b)
        if (E.solves[b].phase == 3) p3.push_back(b);
    // follow-up work, queued back to back: refinement results land in h_res
    double *r = c0.lz.scal + S_NSCAL + 4 * (c0.lz.cap + 2);
    auto fp64_energy = [&](BatchState &B, int slot, bool anchor) -> int {
        Ctx &c = *B.c;
        DevLanczos &z = c.lz;
        const cudaStream_t keep = c.stream;
        c.stream = st;
        int r2 = hv_device(c, z.evecs, z.w);
        c.stream = keep;
        if (r2) { c0.err = c.err; return r2; }
        ++B.numop;
        c0.launches += 2;
        k_rq<<<NBLK, 256, 0, st>>>(z.evecs, z.w, B.n, z.part, r, c0.lz.counter);
        if (anchor) k_anchor_r<<<NBLK, 256, 0, st>>>(z.evecs, z.w, B.n, z.part, r, c0.lz.counter);
        else k_resid<<<NBLK, 256, 0, st>>>(z.evecs, z.w, B.n, z.part, r, c0.lz.counter);
        NSS_CUDA_TRY(c0, cudaMemcpyAsync(E.h_res + 8 * slot, r, 8 * sizeof(double), cudaMemcpyDeviceToHost, st));
        return NSS_OK;
    };
    int rc = NSS_OK;
    for (int b : p1) {
        BatchState &B = E.solves[b];
        DevLanczos &z = B.c->lz;
        const int m = B.m_done;
        NSS_CUDA_TRY(c0, cudaMemcpyAsync(z.svec, B.svec.data(), (size_t)m * sizeof(double), cudaMemcpyHostToDevice, st));
        c0.launches += 2;
        k_ritz<float><<<NBLK, 256, (size_t)m * sizeof(double), st>>>(z.V32, m, B.n, z.svec, m, 1, z.evecs);
        normalize_dev<double>(z, z.evecs, B.n, st, c0.launches);
        if ((rc = fp64_energy(B, b, true))) return rc;
    }
    for (int b : p2) {
        BatchState &B = E.solves[b];
        DevLanczos &z = B.c->lz;
        NSS_CUDA_TRY(c0, cudaMemcpyAsync(z.svec, B.cvec.data(), B.cvec.size() * sizeof(double), cudaMemcpyHostToDevice,
                                         st));
        c0.launches += 2;
        k_ritz_anchor<float><<<NBLK, 256, B.cvec.size() * sizeof(double), st>>>(z.V32, B.m_done, B.n, z.svec, z.evecs,
                                                                                z.evecs);
        normalize_dev<double>(z, z.evecs, B.n, st, c0.launches);
        if ((rc = fp64_energy(B, b, false))) return rc;
    }
    for (int b : p3)
        if ((rc = fp64_energy(E.solves[b], b, false))) return rc;
    NSS_CUDA_TRY(c0, cudaStreamSynchronize(st));
    auto finish = [&](BatchState &B, int slot) -> int {
        const double *hr = E.h_res + 8 * slot;
        B.result = hr[0] / hr[2];
        DevLanczos &z = B.c->lz;
        z.last_resid[0] = std::sqrt(std::max(hr[3], 0.0));
        NSS_CUDA_TRY(c0, cudaMemcpyAsync(z.theta, &B.result, sizeof(double), cudaMemcpyHostToDevice, st));
        z.last_iters = B.m_done;
        z.neigen_done = 1;
        B.c->last_numop = B.numop;
        B.phase = 4;
        return NSS_OK;
    };
    for (int b : p1) {
        BatchState &B = E.solves[b];
        DevLanczos &z = B.c->lz;
        const double *hr = E.h_res + 8 * b;
        B.theta0 = hr[0] / hr[2];
        const double beta0 = std::sqrt(std::max(hr[4], 0.0));
        if (!(beta0 > B.tol_final * std::fabs(B.theta0))) {
            B.phase = 3;   // the FP32 vector is converged already: its FP64 energy next round
            continue;
        }
        float *u32 = z.anc32, *r32 = z.anc32 + B.n;
        c0.launches += 3;
        k_to32<<<608, 256, 0, st>>>(z.V32, z.w, 1.0 / beta0, B.n);
        k_to32<<<608, 256, 0, st>>>(u32, z.evecs, 1.0, B.n);
        k_to32<<<608, 256, 0, st>>>(r32, z.w, 1.0, B.n);
        B.as = AnchorSpec{z.evecs, u32, r32, z.anc32 + 2 * B.n, 0, B.theta0, z.evecs};
        if ((rc = engine_start_run(E, B))) return rc;
        B.phase = 2;
    }
    for (int b : p2)
        if ((rc = finish(E.solves[b], b))) return rc;
    for (int b : p3)
        if ((rc = finish(E.solves[b], b))) return rc;
    // report and remove the finished solves
    int nd = 0;
    std::vector<BatchState> keep;
    for (auto &B : E.solves) {
        if ((B.phase == 4 || B.rc) && nd < max_done) {
            if (ids) ids[nd] = B.rc ? -B.id : B.id;
            if (energies) energies[nd] = B.result;
            if (numops) numops[nd] = B.numop;
            ++nd;
        } else {
            keep.push_back(std::move(B));
        }
    }
    E.solves = std::move(keep);
    if (ndone) *ndone = nd;
    return NSS_OK;
}

}  // namespace

BatchEngine *batch_create(Ctx &c0) {
    BatchEngine *E = new BatchEngine();
    if (engine_init(*E, c0)) {
        delete E;
        return nullptr;
    }
    return E;
}

void batch_destroy(BatchEngine *E) { delete E; }

int batch_add(BatchEngine *E, Ctx &c, uint64_t seed, int nitermax, double tol, int *id) {
    return engine_add(*E, c, seed, nitermax, tol, id);
}

int batch_step(BatchEngine *E, int max_done, int *ndone, int *ids, double *energies, int *numops) {
    const int rc = engine_step(*E, max_done, ndone, ids, energies, numops);
    if (rc) {
        // a failed round drops every solve in flight, so that the engine
        // holds no context its caller may now solve alone or release; the
        // shared barrier and error word start the next round cleared
        E->solves.clear();
        if (ndone) *ndone = 0;
        Ctx &c0 = *E->c0;
        cudaMemsetAsync(c0.lz.counter, 0, 4 * sizeof(unsigned), c0.stream);
        cudaMemsetAsync(c0.lz.flags, 0, F_NFLAGS * sizeof(int), c0.stream);
    }
    return rc;
}

int batch_inflight(const BatchEngine *E) { return (int)E->solves.size(); }

int lanczos_eigh_batch(Ctx *const *cs, int nb, int nitermax, double tol, const uint64_t *seeds,
                       double *evals_host, int *numops) {
    if (nb < 1 || nb > BATCH_MAX) {
        cs[0]->err = "nss_eigh_batch: between 1 and " + std::to_string(BATCH_MAX) + " solves per batch";
        return NSS_ERR_INVALID;
    }
    BatchEngine E;
    int rc = engine_init(E, *cs[0]);
    if (rc) return rc;
    std::vector<int> ids(nb);
    for (int b = 0; b < nb; ++b)
        if ((rc = engine_add(E, *cs[b], seeds ? seeds[b] : 1234, nitermax, tol, &ids[b]))) return rc;
    std::vector<int> did(nb), nop(nb);
    std::vector<double> en(nb);
    int first_rc = NSS_OK;
    for (int round = 0; round < 1000000 && !E.solves.empty(); ++round) {
        int nd = 0;
        if ((rc = engine_step(E, nb, &nd, did.data(), en.data(), nop.data()))) return rc;
        for (int q = 0; q < nd; ++q) {
            const int id = did[q] < 0 ? -did[q] : did[q];
            const int b = (int)(std::find(ids.begin(), ids.end(), id) - ids.begin());
            if (b >= nb) continue;
            if (evals_host) evals_host[b] = en[q];
            if (numops) numops[b] = nop[q];
            if (did[q] < 0 && !first_rc) {
                first_rc = NSS_ERR_NOCONV;
                cs[0]->err = cs[b]->err;
            }
        }
    }
    return first_rc;
}

}  // namespace nss
