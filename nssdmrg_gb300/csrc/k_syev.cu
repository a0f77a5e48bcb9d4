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

#include <cooperative_groups.h>

#include <algorithm>
#include <cfloat>
#include <cmath>

namespace nss {

namespace {

constexpr int TRD_THREADS = 512;
constexpr int BIS_EPC = 8;          // eigenvalues per CTA
constexpr int BIS_THREADS = 160;    // 4 warps x 2 eigenvalues x 16 shifts, 1 warp for L D L^T
constexpr int VEC_WARPS = 4;
constexpr double RELGAP_MIN = 1e-2;
constexpr int VEC_MAXCL = 16;       // kept members of one relative cluster
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
        // p = t A v over the trailing block (symmetric reads of the lower
        // triangle): four threads per row, each with two accumulators, so the
        // whole CTA streams FMAs instead of one warp reduction per row
        for (int i0 = 0; i0 < m; i0 += TRD_THREADS / 4) {
            const int i = i0 + (tid >> 2), qd = tid & 3;
            double a0 = 0.0, a1 = 0.0;
            if (i < m) {
                const int r = k + 1 + i;
                int j = qd;
                for (; j + 4 < m; j += 8) {
                    const int c0 = k + 1 + j, c1 = c0 + 4;
                    a0 = fma(A[j <= i ? r * ld + c0 : c0 * ld + r], v[j], a0);
                    a1 = fma(A[j + 4 <= i ? r * ld + c1 : c1 * ld + r], v[j + 4], a1);
                }
                if (j < m) {
                    const int c0 = k + 1 + j;
                    a0 = fma(A[j <= i ? r * ld + c0 : c0 * ld + r], v[j], a0);
                }
            }
            double acc = a0 + a1;
            acc += __shfl_xor_sync(0xffffffffu, acc, 1);
            acc += __shfl_xor_sync(0xffffffffu, acc, 2);
            if (i < m && qd == 0) w[i] = t * acc;
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
                A[r * ld + c] = fma(-vi, w[j], fma(-wi, v[j], A[r * ld + c]));   // two FMAs
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

// The same Householder reduction for mid-size blocks on a thread-block
// cluster of C CTAs (C = 8 or 16, one cluster per block).  CTA r holds the
// full columns j = r + C jj of the symmetric block in shared memory.  Step
// k: the owner of column k forms the reflector and publishes v and tau in
// its shared memory; cluster barrier; every CTA copies v through
// distributed shared memory and forms p_j = tau A_j . v for its active
// columns and its share of p . v; cluster barrier; every CTA gathers p and
// the shares, w = p - (tau/2)(p.v) v, and applies the rank-2 update to its
// columns.  Two cluster barriers a step, the FP64 work spread over C SMs.
// The buffers that cross CTAs alternate with the parity of k, so a
// barrier always separates a buffer's writes from the previous step's reads.
// GLOBAL: the block's columns live in a global (L2-resident) copy instead
// of the cluster's shared memory, for blocks too large for it; gA + goff[b]
// is block b's n x n column-major scratch.
template <bool GLOBAL>
__global__ void __launch_bounds__(TRD_THREADS, 1)
    k_trd_cl(const double *__restrict__ rho, const int64_t *__restrict__ rho_off, const int *__restrict__ dims,
             const int *__restrict__ ev_off, const int *__restrict__ blocks, double *__restrict__ refl,
             double *__restrict__ td, double *__restrict__ te, double *__restrict__ tau, int *__restrict__ perm,
             double *__restrict__ gA, const int64_t *__restrict__ goff) {
    namespace cg = cooperative_groups;
    cg::cluster_group cl = cg::this_cluster();
    constexpr int NW = TRD_THREADS / 32;
    const int C = (int)cl.num_blocks(), r = (int)cl.block_rank();
    const int bq = blockIdx.x / C;
    const int q = blocks[bq];
    const int n = dims[q], eo = ev_off[q];
    const int ncmax = (n + C - 1) / C, ncol = r < n ? (n - r + C - 1) / C : 0;
    extern __shared__ double trc_smem[];
    double *const G = GLOBAL ? gA + goff[bq] : nullptr;
    double *const As = trc_smem;
    // local column jj = global column r + C jj
    auto colp = [&](int jj) -> double * { return GLOBAL ? G + (int64_t)(r + C * jj) * n : As + (size_t)jj * n; };
    double *v = GLOBAL ? trc_smem : As + (size_t)ncmax * n;
    double *w = v + n, *pbuf = w + n, *vbuf = pbuf + 2 * ncmax, *sbuf = vbuf + 2 * n;
    __shared__ double red[NW];
    __shared__ double kk;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const double *R = rho + rho_off[q];
    double *Vq = refl + rho_off[q];
    for (int e = tid; e < ncol * n; e += TRD_THREADS) {
        const int jj = e / n, i = e - jj * n;
        colp(jj)[i] = R[(int64_t)(r + C * jj) * n + i];     // column j = row j (symmetric)
    }
    if (GLOBAL) __threadfence_block();
    if (r == 0)
        for (int i = tid; i < n; i += TRD_THREADS) perm[eo + i] = i;
    cl.sync();
    for (int k = 0; k + 2 < n; ++k) {
        const int m = n - k - 1, par = k & 1, o = k % C;
        double *vb = vbuf + par * n, *pb = pbuf + par * ncmax, *sb = sbuf + par * 4;
        if (r == o) {
            const double *colk = colp(k / C);
            if (warp == 0) {
                double ss = 0.0;
                for (int i = k + 2 + lane; i < n; i += 32) ss = fma(colk[i], colk[i], ss);
                ss = wsum(ss);
                if (lane == 0) {
                    const double alpha = colk[k + 1];
                    double t = 0.0, beta = alpha, scal = 0.0;
                    if (ss > 0.0) {
                        beta = -copysign(sqrt(fma(alpha, alpha, ss)), alpha);
                        t = (beta - alpha) / beta;
                        scal = 1.0 / (alpha - beta);
                    }
                    sb[0] = t;
                    sb[1] = scal;
                    td[eo + k] = colk[k];
                    te[eo + k] = beta;
                    tau[eo + k] = t;
                }
            }
            __syncthreads();
            const double scal = sb[1];
            for (int i = tid; i < m; i += TRD_THREADS) {
                const double x = (i == 0) ? 1.0 : colk[k + 1 + i] * scal;
                vb[i] = x;
                Vq[(int64_t)k * n + k + 1 + i] = x;
            }
        }
        cl.sync();                                   // v and tau of step k published
        const double t = cl.map_shared_rank(sb, o)[0];
        const double *rv = cl.map_shared_rank(vb, o);
        for (int i = tid; i < m; i += TRD_THREADS) v[i] = rv[i];
        __syncthreads();
        const int jj0 = k + 1 > r ? (k + 1 - r + C - 1) / C : 0;   // first column j = r + C jj > k
        double sp = 0.0;
        if (t != 0.0)
            for (int jj = jj0 + warp; jj < ncol; jj += NW) {
                const double *a = colp(jj) + k + 1;
                double a0 = 0.0, a1 = 0.0;
                int i = lane;
                if (GLOBAL)   // columns in L2: eight rounds' loads out before the first FMA
                    for (; i + 32 + 448 < m; i += 512) {
                        double x[16];
#pragma unroll
                        for (int u = 0; u < 16; ++u) x[u] = a[i + 32 * u];
#pragma unroll
                        for (int u = 0; u < 8; ++u) {
                            a0 = fma(x[2 * u], v[i + 64 * u], a0);
                            a1 = fma(x[2 * u + 1], v[i + 64 * u + 32], a1);
                        }
                    }
                for (; i + 32 < m; i += 64) {
                    a0 = fma(a[i], v[i], a0);
                    a1 = fma(a[i + 32], v[i + 32], a1);
                }
                if (i < m) a0 = fma(a[i], v[i], a0);
                const double pj = t * wsum(a0 + a1);
                if (lane == 0) pb[jj] = pj;
                sp = fma(pj, v[r + C * jj - k - 1], sp);
            }
        if (lane == 0) red[warp] = sp;
        __syncthreads();
        if (tid == 0) {
            double x = 0.0;
            for (int u = 0; u < NW; ++u) x += red[u];
            sb[2] = x;
        }
        cl.sync();                                   // p and the p.v shares published
        if (warp == 0) {
            double x = lane < C ? cl.map_shared_rank(sb, lane)[2] : 0.0;
            x = wsum(x);
            if (lane == 0) kk = -0.5 * t * x;
        }
        __syncthreads();
        const double K = kk;
        if (t != 0.0)
            for (int i = tid; i < m; i += TRD_THREADS) {
                const int g = k + 1 + i;
                w[i] = fma(K, v[i], cl.map_shared_rank(pb, g % C)[g / C]);
            }
        __syncthreads();
        if (t != 0.0)
            for (int jj = jj0 + warp; jj < ncol; jj += NW) {
                const int jc = r + C * jj - k - 1;
                const double vj = v[jc], wj = w[jc];
                double *a = colp(jj) + k + 1;
                const double nvj = -vj, nwj = -wj;
                if (GLOBAL) {   // two FMAs an element, eight loads in flight
                    for (int i0 = lane; i0 < m; i0 += 256) {
                        double x[8];
#pragma unroll
                        for (int u = 0; u < 8; ++u) {
                            const int i = i0 + 32 * u;
                            x[u] = i < m ? a[i] : 0.0;
                        }
#pragma unroll
                        for (int u = 0; u < 8; ++u) {
                            const int i = i0 + 32 * u;
                            if (i < m) a[i] = fma(v[i], nwj, fma(w[i], nvj, x[u]));
                        }
                    }
                } else {
                    for (int i = lane; i < m; i += 32) a[i] = fma(v[i], nwj, fma(w[i], nvj, a[i]));   // two FMAs
                }
            }
        __syncthreads();
    }
    if (n >= 2 && r == (n - 2) % C && tid == 0) {
        const double *c2 = colp((n - 2) / C);
        td[eo + n - 2] = c2[n - 2];
        te[eo + n - 2] = c2[n - 1];
        tau[eo + n - 2] = 0.0;
    }
    if (r == (n - 1) % C && tid == 0) {
        td[eo + n - 1] = colp((n - 1) / C)[n - 1];
        te[eo + n - 1] = 0.0;
        tau[eo + n - 1] = 0.0;
    }
    cl.sync();                                       // no CTA leaves while its memory may be read
}

// Bounded barrier of one CTA group of k_trd_grid (cooperative launch, all
// CTAs resident): barrier e of a launch waits for e * G arrivals on *bar, G
// the group's CTAs; a wait that runs past `spin` polls sets *err, and every
// later barrier (of any group) returns false at once, so the kernel always
// ends.  The counters and *err are zero at launch.
__device__ __forceinline__ bool tg_sync(unsigned *bar, unsigned G, unsigned &epoch, int *err, uint32_t spin) {
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        int good = 1;
        epoch += G;
        __threadfence();
        atomicAdd(bar, 1u);
        uint32_t it = 0;
        while (true) {
            unsigned v;
            asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(bar) : "memory");
            if (v >= epoch) break;
            if (++it > spin) { atomicExch(err, 1); good = 0; break; }
            if ((it & 255u) == 0 && *(volatile int *)err) { good = 0; break; }
        }
        ok = good;
    }
    __syncthreads();
    return ok != 0;
}

// Blocks of one k_trd_grid launch: group g (CTAs c0[g] .. c0[g+1]-1)
// reduces block q[g], whose copy is gA + goff[g] and whose exchange buffers
// are comm + coff[g]; its barrier counter is bars[g].
constexpr int TG_MAXG = 8;
struct TgGroups {
    int ng;
    int q[TG_MAXG];
    int c0[TG_MAXG + 1];
    int64_t goff[TG_MAXG], coff[TG_MAXG];
    uint32_t spin;               // poll limit of the group barriers (wait_limit)
};

// The Householder reduction of very large blocks by the whole GPU (a
// cooperative launch of one CTA per SM, split into one CTA group per block
// in proportion to the blocks' n^3): k_trd_cl's step with a group's CTAs in
// place of a cluster's, so the FP64 FMAs spread over every SM instead of 16
// per block.  CTA r of a group holds columns j = r + G jj of its block's
// global (L2-resident) copy; the reflector, the p_j and the partial sums p.v
// cross CTAs through global buffers (v [2][n], p [2][n], t [2], partials
// [2][G]) that alternate with the parity of k, between two group barriers a
// step.
__global__ void __launch_bounds__(TRD_THREADS, 1)
    k_trd_grid(const double *__restrict__ rho, const int64_t *__restrict__ rho_off, const int *__restrict__ dims,
               const int *__restrict__ ev_off, TgGroups grp, double *__restrict__ refl, double *__restrict__ td,
               double *__restrict__ te, double *__restrict__ tau, int *__restrict__ perm, double *__restrict__ gA0,
               double *__restrict__ comm0, unsigned *bars, int *err) {
    constexpr int NW = TRD_THREADS / 32;
    int g = 0;
    while (g + 1 < grp.ng && (int)blockIdx.x >= grp.c0[g + 1]) ++g;
    const int G = grp.c0[g + 1] - grp.c0[g], r = (int)blockIdx.x - grp.c0[g];
    const int q = grp.q[g];
    double *const gA = gA0 + grp.goff[g];
    double *const comm = comm0 + grp.coff[g];
    unsigned *const bar = bars + g;
    const int n = dims[q], eo = ev_off[q];
    const int ncol = r < n ? (n - r + G - 1) / G : 0;
    extern __shared__ double tg_smem[];
    double *v = tg_smem, *w = v + n;
    __shared__ double red[NW];
    __shared__ double hs[2];
    __shared__ double kk;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const double *R = rho + rho_off[q];
    double *Vq = refl + rho_off[q];
    double *gv = comm, *gp = comm + 2 * (int64_t)n, *gt = comm + 4 * (int64_t)n, *gs = gt + 2;
    auto colp = [&](int jj) -> double * { return gA + (int64_t)(r + G * jj) * n; };
    for (int e = tid; e < ncol * n; e += TRD_THREADS) {
        const int jj = e / n, i = e - jj * n;
        colp(jj)[i] = R[(int64_t)(r + G * jj) * n + i];   // column j = row j (symmetric)
    }
    if (r == 0)
        for (int i = tid; i < n; i += TRD_THREADS) perm[eo + i] = i;
    unsigned epoch = 0;
    bool alive = tg_sync(bar, G, epoch, err, grp.spin);
    for (int k = 0; alive && k + 2 < n; ++k) {
        const int m = n - k - 1, par = k & 1, o = k % G;
        double *vb = gv + par * (int64_t)n, *pb = gp + par * (int64_t)n, *sb = gs + par * G;
        if (r == o) {
            const double *colk = colp(k / G);
            double ss = 0.0;                         // sum of squares below the subdiagonal, all warps
            for (int i0 = k + 2 + tid; i0 < n; i0 += 8 * TRD_THREADS) {   // eight loads in flight
                double x[8];
#pragma unroll
                for (int u = 0; u < 8; ++u) {
                    const int i = i0 + u * TRD_THREADS;
                    x[u] = i < n ? colk[i] : 0.0;
                }
#pragma unroll
                for (int u = 0; u < 8; ++u) ss = fma(x[u], x[u], ss);
            }
            ss = wsum(ss);
            if (lane == 0) red[warp] = ss;
            __syncthreads();
            if (tid == 0) {
                double x = 0.0;
                for (int u = 0; u < NW; ++u) x += red[u];
                const double alpha = colk[k + 1];
                double t = 0.0, beta = alpha, scal = 0.0;
                if (x > 0.0) {
                    beta = -copysign(sqrt(fma(alpha, alpha, x)), alpha);
                    t = (beta - alpha) / beta;
                    scal = 1.0 / (alpha - beta);
                }
                hs[0] = t;
                hs[1] = scal;
                gt[par] = t;
                td[eo + k] = colk[k];
                te[eo + k] = beta;
                tau[eo + k] = t;
            }
            __syncthreads();
            const double scal = hs[1];
            for (int i = tid; i < m; i += TRD_THREADS) {
                const double x = (i == 0) ? 1.0 : colk[k + 1 + i] * scal;
                vb[i] = x;
                Vq[(int64_t)k * n + k + 1 + i] = x;
            }
        }
        if (!(alive = tg_sync(bar, G, epoch, err, grp.spin))) break;   // v and t of step k published
        const double t = *(volatile double *)(gt + par);
        for (int i0 = tid; i0 < m; i0 += 4 * TRD_THREADS) {   // written by another CTA: past L1
            double x[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int i = i0 + u * TRD_THREADS;
                x[u] = i < m ? __ldcg(vb + i) : 0.0;
            }
#pragma unroll
            for (int u = 0; u < 4; ++u)
                if (i0 + u * TRD_THREADS < m) v[i0 + u * TRD_THREADS] = x[u];
        }
        __syncthreads();
        const int jj0 = k + 1 > r ? (k + 1 - r + G - 1) / G : 0;   // first own column j > k
        double sp = 0.0;
        if (t != 0.0)
            for (int jj = jj0 + warp; jj < ncol; jj += NW) {
                const double *a = colp(jj) + k + 1;
                double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
                int i = lane;
                // four rounds of the four accumulators per batch: their sixteen
                // loads go out before the first FMA
                for (; i + 96 + 384 < m; i += 512) {
                    double x[16];
#pragma unroll
                    for (int u = 0; u < 16; ++u) x[u] = a[i + 32 * u];
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        a0 = fma(x[4 * u], v[i + 128 * u], a0);
                        a1 = fma(x[4 * u + 1], v[i + 128 * u + 32], a1);
                        a2 = fma(x[4 * u + 2], v[i + 128 * u + 64], a2);
                        a3 = fma(x[4 * u + 3], v[i + 128 * u + 96], a3);
                    }
                }
                for (; i + 96 < m; i += 128) {
                    a0 = fma(a[i], v[i], a0);
                    a1 = fma(a[i + 32], v[i + 32], a1);
                    a2 = fma(a[i + 64], v[i + 64], a2);
                    a3 = fma(a[i + 96], v[i + 96], a3);
                }
                for (; i < m; i += 32) a0 = fma(a[i], v[i], a0);
                const int jc = r + G * jj - k - 1;
                const double pj = t * wsum((a0 + a1) + (a2 + a3));
                if (lane == 0) pb[jc] = pj;
                sp = fma(pj, v[jc], sp);
            }
        if (lane == 0) red[warp] = sp;
        __syncthreads();
        if (tid == 0) {
            double x = 0.0;
            for (int u = 0; u < NW; ++u) x += red[u];
            sb[r] = x;
        }
        if (!(alive = tg_sync(bar, G, epoch, err, grp.spin))) break;   // p and the p.v shares published
        if (warp == 0) {
            double x = 0.0;
            for (int u = lane; u < G; u += 32) x += ((volatile double *)sb)[u];
            x = wsum(x);
            if (lane == 0) kk = -0.5 * t * x;
        }
        __syncthreads();
        const double K = kk;
        if (t != 0.0) {
            for (int i0 = tid; i0 < m; i0 += 4 * TRD_THREADS) {
                double x[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int i = i0 + u * TRD_THREADS;
                    x[u] = i < m ? __ldcg(pb + i) : 0.0;
                }
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int i = i0 + u * TRD_THREADS;
                    if (i < m) w[i] = fma(K, v[i], x[u]);
                }
            }
            __syncthreads();
            for (int jj = jj0 + warp; jj < ncol; jj += NW) {
                const int jc = r + G * jj - k - 1;
                const double vj = v[jc], wj = w[jc];
                double *a = colp(jj) + k + 1;
                const double nvj = -vj, nwj = -wj;
                for (int i0 = lane; i0 < m; i0 += 256) {   // two FMAs an element, eight loads in flight
                    double x[8];
#pragma unroll
                    for (int u = 0; u < 8; ++u) {
                        const int i = i0 + 32 * u;
                        x[u] = i < m ? a[i] : 0.0;
                    }
#pragma unroll
                    for (int u = 0; u < 8; ++u) {
                        const int i = i0 + 32 * u;
                        if (i < m) a[i] = fma(v[i], nwj, fma(w[i], nvj, x[u]));
                    }
                }
            }
        }
        __syncthreads();
    }
    if (alive && n >= 2 && r == (n - 2) % G && tid == 0) {
        const double *c2 = colp((n - 2) / G);
        td[eo + n - 2] = c2[n - 2];
        te[eo + n - 2] = c2[n - 1];
        tau[eo + n - 2] = 0.0;
    }
    if (alive && r == (n - 1) % G && tid == 0) {
        td[eo + n - 1] = colp((n - 1) / G)[n - 1];
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

// The same count in FP32 (rescaled every 4 steps), for bracketing.
__device__ __forceinline__ int sturm_count32(const float *a, const float *bb, int n, float s) {
    float pm = 0.0f, pc = 1.0f;
    int cnt = 0;
    for (int i = 0; i < n; ++i) {
        const float t = bb[i] * pm;
        float pn = fmaf(a[i] - s, pc, -t);
        int bn = __float_as_int(pn);
        if ((bn << 1) == 0) {
            pn = -pc * 0x1p-50f;
            bn = __float_as_int(pn);
        }
        cnt += (int)((unsigned)(bn ^ __float_as_int(pc)) >> 31);
        pm = pc;
        pc = pn;
        if ((i & 3) == 3) {
            const int eb = max((__float_as_int(pm) >> 23) & 0xff, (__float_as_int(pc) >> 23) & 0xff);
            if (eb > 0) {
                const float f = __int_as_float((254 - eb) << 23);
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
             double *__restrict__ bsig, int *__restrict__ flags, int *__restrict__ sub, int nmax) {
    extern __shared__ double bis_smem[];
    double *sa = bis_smem, *sbb = sa + nmax, *sb = sbb + nmax;
    float *fa = (float *)(sb + nmax), *fbb = fa + nmax;
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
        // phase A, FP32: 16 shifts per eigenvalue, 5 rounds (~20 bits); two
        // eigenvalues per warp.  Only brackets the eigenvalue: an FP32 count
        // is exact for a matrix within ~2^-21 of the scaled T, so the bracket
        // is widened by 2^-16 and checked with FP64 counts in phase B.
        __shared__ double blo[BIS_EPC], bhi[BIS_EPC];
        __shared__ int bk[BIS_EPC][3];               // r0, r1, exact (1 x 1 block)
        for (int i = tid; i < n; i += 128) {
            fa[i] = (float)sa[i];
            fbb[i] = (float)sbb[i];
        }
        asm volatile("bar.sync 1, 128;" ::: "memory");
        {
            const int g = lane >> 4, j = lane & 15, e = warp * 2 + g;
            const int k = k0 + e;
            const bool active = k < n && e < BIS_EPC;
            int r0 = 0, r1 = 0;
            if (active) {                            // unreduced block [r0, r1) holding row k
                r0 = k;
                while (r0 > 0 && sb[r0 - 1] != 0.0) --r0;
                r1 = k + 1;
                while (r1 < n && sb[r1 - 1] != 0.0) ++r1;
            }
            const int kl = k - r0;
            float lo = -1.0f, hi = 1.0f;
            bool done = !active || r1 - r0 <= 1;
            for (int round = 0; round < 5 && __any_sync(0xffffffffu, !done); ++round) {
                const float h = (hi - lo) * (1.0f / 17.0f);
                const int c = sturm_count32(fa + r0, fbb + r0, r1 - r0, lo + (float)(j + 1) * h);
                const unsigned gm = (__ballot_sync(0xffffffffu, c > kl) >> (16 * g)) & 0xffffu;
                if (!done) {
                    if (gm == 0) {
                        lo = lo + 16.0f * h;
                    } else {
                        const int jj = __ffs(gm) - 1;
                        const float nh = lo + (float)(jj + 1) * h;
                        if (jj > 0) lo = lo + (float)jj * h;
                        hi = nh;
                    }
                }
            }
            if (active && j == 0) {
                bk[e][0] = r0;
                bk[e][1] = r1;
                bk[e][2] = r1 - r0 == 1;
                blo[e] = r1 - r0 == 1 ? sa[k] : fmax(-1.0, (double)lo - 0x1p-16);
                bhi[e] = r1 - r0 == 1 ? sa[k] : fmin(1.0, (double)hi + 0x1p-16);
            }
        }
        asm volatile("bar.sync 1, 128;" ::: "memory");
        if (warp >= 2) return;
        // phase B, FP64: 8 shifts per eigenvalue (~3.2 bits a round), four
        // eigenvalues per warp; the first round checks the FP32 bracket
        const int g = lane >> 3, j = lane & 7, e = warp * 4 + g;
        const int k = k0 + e;
        const bool active = k < n && e < BIS_EPC;
        int r0 = 0, r1 = 0;
        double lo = -1.0, hi = 1.0;
        bool done = !active;
        if (active) {
            r0 = bk[e][0];
            r1 = bk[e][1];
            lo = blo[e];
            hi = bhi[e];
            done = bk[e][2] != 0;
        }
        const int kl = k - r0;
        {
            const int c = sturm_count(sa + r0, sbb + r0, r1 - r0, j == 0 ? lo : hi);
            const unsigned m8 = (__ballot_sync(0xffffffffu, c > kl) >> (8 * g)) & 0xffu;
            // lane 0 of the group holds count(lo) > kl (bad), lane 1 count(hi) > kl (good)
            if (!done && ((m8 & 1u) || !(m8 & 2u))) {
                lo = -1.0;
                hi = 1.0;
            }
        }
        for (int round = 0; round < 64 && __any_sync(0xffffffffu, !done); ++round) {
            const double h = (hi - lo) * (1.0 / 9.0);
            const int c = sturm_count(sa + r0, sbb + r0, r1 - r0, lo + (double)(j + 1) * h);
            const unsigned gm = (__ballot_sync(0xffffffffu, c > kl) >> (8 * g)) & 0xffu;
            if (!done) {
                const double wold = hi - lo;
                if (gm == 0) {
                    lo = lo + 8.0 * h;
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

// 1/x from the hardware approximation (rcp.approx.ftz.f64) refined by two
// Newton-Raphson steps r <- r + r (1 - x r) (each squares the relative
// error): ~1 ulp, in ~5 dependent FP64 operations where a correctly rounded
// division costs ~650 cycles on this GPU.  Used in the dependent chains of
// the qd transforms, whose error analysis needs only a small relative error
// per operation.  x is normal and nonzero there (|x| >= PIVMIN).
__device__ __forceinline__ double rcp_nr(double x) {
    double r;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
    double e = fma(-x, r, 1.0);
    r = fma(r, e, r);
    e = fma(-x, r, 1.0);
    return fma(r, e, r);
}

// Where a kept eigenvalue of one side lives: j < ms of side s maps to
// position order[j] + ev_base of the block-concatenated eigenvalue list;
// the side's block tables start at block o.
struct VecSide {
    const int *order;
    int ev_base, ms, o;
};

struct VecArgs {
    VecSide side[2];
    int nsb;
    const int *rank;             // rank within its side of every position
    const int *ev_off, *dims, *bmode, *sub, *perm;
    const int64_t *rho_off;
    const double *evals, *ldd, *ldl, *bscale, *bsig, *tau, *refl;
    int *flags;
    double *vec;
};

// (q, col) of kept eigenvalue j of the concatenated left + right list
__device__ __forceinline__ bool vec_locate(const VecArgs &a, int j, int &side, int &q, int &col) {
    side = j < a.side[0].ms ? 0 : 1;
    const int jj = side == 0 ? j : j - a.side[0].ms;
    if (jj >= a.side[side].ms) return false;
    const VecSide &sd = a.side[side];
    const int pos = sd.order[jj] + sd.ev_base;
    int k = 0;
    while (k + 1 < a.nsb && a.ev_off[sd.o + k + 1] <= pos) ++k;
    q = sd.o + k;
    col = pos - a.ev_off[q];
    return true;
}

// relative cluster [c0, c1] of column col within its unreduced block
struct VecCluster {
    int r0, r1, c0, c1;
};

__device__ __forceinline__ VecCluster vec_cluster(const VecArgs &a, int q, int col) {
    const int eo = a.ev_off[q];
    const double scale = a.bscale[q], sig0 = a.bsig[q];
    const int sr = a.sub[eo + col];
    VecCluster c{sr & 0xffff, sr >> 16, col, col};
    auto lamS = [&](int x) { return a.evals[eo + x] * scale - sig0; };
    auto linked = [&](int x) {
        if (x + 1 >= c.r1) return false;
        const double u = lamS(x), w = lamS(x + 1);
        return w - u < RELGAP_MIN * fmax(u, w);
    };
    while (c.c0 > c.r0 && linked(c.c0 - 1)) --c.c0;
    while (linked(c.c1)) ++c.c1;
    return c;
}

// Per-warp scratch of the vector kernels: seven arrays of n_max doubles.
struct VecScratch {
    double *dD, *dL, *lp, *um, *ss, *pp, *z;
};

__device__ __forceinline__ VecScratch vec_scratch(double *sw, int nmax) {
    return VecScratch{sw, sw + nmax, sw + 2 * nmax, sw + 3 * nmax, sw + 4 * nmax, sw + 5 * nmax, sw + 6 * nmax};
}

// Stationary transform L+ D+ L+^T = L D L^T - lam over rows [r0, r1) on
// lane 0: lp = L+, ss = the s_i of the differential form; dplus (may be
// null) receives the pivots D+.
__device__ __forceinline__ void dstqds_lane0(const VecScratch &w, int r0, int r1, double lam, double *dplus) {
    double s = -lam;
    for (int i = r0; i + 1 < r1; ++i) {
        w.ss[i] = s;
        double dp = w.dD[i] + s;
        if (fabs(dp) < PIVMIN) dp = -PIVMIN;
        if (dplus) dplus[i] = dp;
        const double l = w.dD[i] * w.dL[i] * rcp_nr(dp);
        w.lp[i] = l;
        s = l * w.dL[i] * s - lam;
    }
    w.ss[r1 - 1] = s;
    if (dplus) {
        double dp = w.dD[r1 - 1] + s;
        if (fabs(dp) < PIVMIN) dp = -PIVMIN;
        dplus[r1 - 1] = dp;
    }
}

// Twisted-factorisation eigenvector of L D L^T (rows [r0, r1) of the block,
// zero elsewhere in z[0, n)) for the eigenvalue near lam0, with Rayleigh
// corrections that stay within gap / 4; z comes out normalised.
__device__ bool twisted_vector(const VecScratch &w, int lane, int n, int r0, int r1, double lam0, double gap) {
    double lam = lam0, ztz = 1.0;
    bool conv = false;
    for (int itr = 0; itr < 8; ++itr) {
        if (lane == 0) {
            dstqds_lane0(w, r0, r1, lam, nullptr);
        } else if (lane == 1) {                      // progressive: U- D- U-^T = L D L^T - lam
            double p = w.dD[r1 - 1] - lam;
            for (int i = r1 - 2; i >= r0; --i) {
                w.pp[i + 1] = p;
                double dm = w.dD[i] * w.dL[i] * w.dL[i] + p;
                if (fabs(dm) < PIVMIN) dm = -PIVMIN;
                const double t = w.dD[i] * rcp_nr(dm);
                w.um[i] = w.dL[i] * t;
                p = p * t - lam;
            }
            w.pp[r0] = p;
        }
        __syncwarp();
        double best = INFINITY;
        int bi = r1;
        for (int k = r0 + lane; k < r1; k += 32) {
            const double gk = fabs(w.ss[k] + w.pp[k] + lam);
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
        if (bi >= r1) break;                         // every gamma NaN
        const int r = bi;
        const double gam = w.ss[r] + w.pp[r] + lam;
        __syncwarp();
        for (int i = lane; i < n; i += 32) w.z[i] = 0.0;
        __syncwarp();
        if (lane == 0) {
            double zz = 1.0;
            w.z[r] = 1.0;
            for (int i = r - 1; i >= r0; --i) {
                zz = -w.lp[i] * zz;
                w.z[i] = zz;
            }
        } else if (lane == 1) {
            double zz = 1.0;
            for (int i = r; i + 1 < r1; ++i) {
                zz = -w.um[i] * zz;
                w.z[i + 1] = zz;
            }
        }
        __syncwarp();
        double t2 = 0.0;
        for (int k = r0 + lane; k < r1; k += 32) t2 = fma(w.z[k], w.z[k], t2);
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
    if (conv) {
        const double inv = 1.0 / sqrt(ztz);
        for (int k = lane; k < n; k += 32) w.z[k] *= inv;
    }
    __syncwarp();
    return conv;
}

// z <- z - sum_y (y . z) y over the vectors ys[0..ny) (length n, global),
// then normalised; returns the norm after the projection.
__device__ double project_out(double *z, int n, const double *const *ys, int ny, int lane) {
    for (int t = 0; t < ny; ++t) {
        const double *y = ys[t];
        double d = 0.0;
        for (int i = lane; i < n; i += 32) d = fma(y[i], z[i], d);
        d = wsum(d);
        for (int i = lane; i < n; i += 32) z[i] = fma(-d, y[i], z[i]);
        __syncwarp();
    }
    double nz = 0.0;
    for (int i = lane; i < n; i += 32) nz = fma(z[i], z[i], nz);
    nz = sqrt(wsum(nz));
    if (nz > 0.0) {
        const double inv = 1.0 / nz;
        for (int i = lane; i < n; i += 32) z[i] *= inv;
    }
    __syncwarp();
    return nz;
}

// x = H_0 H_1 ... H_{n-3} z (z in shared memory, overwritten), then written
// to column X in the block's own row order.
__device__ void back_transform_store(const VecArgs &a, int q, int n, int eo, double *z, double *Xc, int lane) {
    const double *Vq = a.refl + a.rho_off[q];
    for (int k = n - 3; k >= 0; --k) {
        const double t = a.tau[eo + k];
        if (t == 0.0) continue;
        const double *vk = Vq + (int64_t)k * n;
        double d = 0.0;
        for (int i = k + 1 + lane; i < n; i += 32) d = fma(vk[i], z[i], d);
        d = t * wsum(d);
        for (int i = k + 1 + lane; i < n; i += 32) z[i] = fma(-d, vk[i], z[i]);
        __syncwarp();
    }
    for (int i = lane; i < n; i += 32) Xc[a.perm[eo + i]] = z[i];
    __syncwarp();
}

// relative cluster with a pair closer than 32 eps (tight), counting the
// neighbours just outside it in the unreduced block: those clusters are
// done by k_vec_cl
__device__ __forceinline__ bool cluster_tight(const VecArgs &a, int q, const VecCluster &cl) {
    const int eo = a.ev_off[q];
    const double scale = a.bscale[q];
    for (int c = max(cl.c0 - 1, cl.r0); c <= min(cl.c1, cl.r1 - 2); ++c)
        if (!(a.evals[eo + c + 1] * scale - a.evals[eo + c] * scale > 32.0 * 0x1p-52)) return true;
    return false;
}

// One warp per kept eigenvalue (both sides in one launch).  Blocks of the
// library path (bmode != 0) already hold their vectors; kept eigenvalues of
// tight clusters are left to k_vec_cl.  The vector is written to column col
// of the block's column-major slot in vec, rows in the block's own order.
// Failure sets bit 1 of flags[q] and a reason bit:
// 4 = factorisation not positive definite, 8 = gap below 32 eps,
// 16 = Rayleigh iteration not settled, 32 = Gram-Schmidt remainder < 1/2,
// 64 = cluster larger than VEC_MAXCL.
__global__ void __launch_bounds__(VEC_WARPS * 32) k_vec(VecArgs a, int nmax) {
    extern __shared__ double vec_smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int j = blockIdx.x * nw + warp;
    int side, q, col;
    if (!vec_locate(a, j, side, q, col)) return;
    if (a.bmode[q] != 0) return;
    const int n = a.dims[q], eo = a.ev_off[q];
    double *X = a.vec + a.rho_off[q];
    if (n == 1) {
        if (lane == 0) X[0] = 1.0;
        return;
    }
    if (cluster_tight(a, q, vec_cluster(a, q, col))) return;
    const VecScratch w = vec_scratch(vec_smem + (size_t)warp * 7 * nmax, nmax);
    const double scale = a.bscale[q], sig0 = a.bsig[q];
    const int sr = a.sub[eo + col], r0 = sr & 0xffff, r1 = sr >> 16;
    auto lamS = [&](int c) { return a.evals[eo + c] * scale - sig0; };
    const double lam0 = lamS(col);
    const double gap = fmin(col > r0 ? lam0 - lamS(col - 1) : INFINITY, col + 1 < r1 ? lamS(col + 1) - lam0 : INFINITY);
    int why = (a.flags[q] & 1) ? 4 : 0;
    if (!why) {
        for (int i = lane; i < n; i += 32) {
            w.dD[i] = a.ldd[eo + i];
            w.dL[i] = a.ldl[eo + i];
        }
        __syncwarp();
        if (twisted_vector(w, lane, n, r0, r1, lam0, gap))
            back_transform_store(a, q, n, eo, w.z, X + (int64_t)col * n, lane);
        else
            why |= 16;
    }
    if (why && lane == 0) atomicOr(&a.flags[q], 2 | why);
}

// Tight clusters (a pair of kept or neighbouring eigenvalues closer than
// 32 eps within one unreduced block): one warp, the cluster's first kept
// member, computes all kept members in the tridiagonal basis: the twisted
// vector where the member's own gap allows it, otherwise inverse iteration
// with the stationary factorisation L+ D+ L+^T = L D L^T - lam from a
// pseudo-random start, Gram-Schmidt against the members before it inside
// every iteration (the classical remedy for clustered inverse iteration);
// the orthonormal set is then back-transformed.
__global__ void __launch_bounds__(VEC_WARPS * 32) k_vec_cl(VecArgs a, int nmax) {
    extern __shared__ double vec_smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int j = blockIdx.x * nw + warp;
    int side, q, col;
    if (!vec_locate(a, j, side, q, col)) return;
    if (a.bmode[q] != 0) return;
    const int n = a.dims[q], eo = a.ev_off[q];
    if (n == 1) return;
    const VecCluster cl = vec_cluster(a, q, col);
    if (!cluster_tight(a, q, cl)) return;
    const int ms = a.side[side].ms;
    auto kept = [&](int c) { return a.rank[eo + c] < ms; };
    for (int c = cl.c0; c < col; ++c)
        if (kept(c)) return;                         // an earlier kept member leads
    const VecScratch w = vec_scratch(vec_smem + (size_t)warp * 7 * nmax, nmax);
    double *X = a.vec + a.rho_off[q];
    const double scale = a.bscale[q], sig0 = a.bsig[q];
    auto lamS = [&](int c) { return a.evals[eo + c] * scale - sig0; };
    int why = (a.flags[q] & 1) ? 4 : 0;
    int nm = 0;
    for (int c = col; c <= cl.c1; ++c) nm += kept(c);
    if (nm > VEC_MAXCL) why |= 64;
    if (!why) {
        for (int i = lane; i < n; i += 32) {
            w.dD[i] = a.ldd[eo + i];
            w.dL[i] = a.ldl[eo + i];
        }
        __syncwarp();
    }
    const double *prev[VEC_MAXCL];
    int np = 0;
    for (int c = col; !why && c <= cl.c1; ++c) {
        if (!kept(c)) continue;
        const int sr = a.sub[eo + c], r0 = sr & 0xffff, r1 = sr >> 16;
        const double lam0 = lamS(c);
        const double gap =
            fmin(c > r0 ? lam0 - lamS(c - 1) : INFINITY, c + 1 < r1 ? lamS(c + 1) - lam0 : INFINITY);
        bool done = gap > 32.0 * 0x1p-52 && twisted_vector(w, lane, n, r0, r1, lam0, gap);
        if (done) {
            if (!(project_out(w.z, n, prev, np, lane) >= 0.5)) why |= 32;
        } else {
            // inverse iteration at lam0 with in-loop Gram-Schmidt
            if (lane == 0) dstqds_lane0(w, r0, r1, lam0, w.pp);
            __syncwarp();
            for (int i = lane; i < n; i += 32) {
                unsigned hsh = (unsigned)(i + 1) * 2654435761u ^ (unsigned)(c + 7) * 40503u;
                hsh ^= hsh >> 15;
                hsh *= 2246822519u;
                hsh ^= hsh >> 13;
                w.z[i] = (i >= r0 && i < r1) ? ((double)(hsh & 0xffffu) / 32768.0 - 1.0) : 0.0;
            }
            __syncwarp();
            project_out(w.z, n, prev, np, lane);
            double nz = 0.0;
            for (int it = 0; it < 3; ++it) {
                if (lane == 0) {                     // L+ w = x
                    for (int i = r0; i + 1 < r1; ++i) w.z[i + 1] -= w.lp[i] * w.z[i];
                }
                __syncwarp();
                for (int i = r0 + lane; i < r1; i += 32) w.z[i] *= rcp_nr(w.pp[i]);   // D+^-1
                __syncwarp();
                if (lane == 0) {                     // L+^T y = w
                    for (int i = r1 - 2; i >= r0; --i) w.z[i] -= w.lp[i] * w.z[i + 1];
                }
                __syncwarp();
                double t2 = 0.0;
                for (int i = lane; i < n; i += 32) t2 = fma(w.z[i], w.z[i], t2);
                const double gz = sqrt(wsum(t2));
                if (!(gz > 0.0) || !isfinite(gz)) break;
                for (int i = lane; i < n; i += 32) w.z[i] *= 1.0 / gz;
                __syncwarp();
                nz = project_out(w.z, n, prev, np, lane);
            }
            if (!(nz >= 0.5)) why |= 32;
        }
        if (why) break;
        // the tridiagonal-basis vector waits in its own column until the set is complete
        double *Xc = X + (int64_t)c * n;
        for (int i = lane; i < n; i += 32) Xc[i] = w.z[i];
        __syncwarp();
        prev[np++] = Xc;
    }
    for (int t = 0; !why && t < np; ++t) {
        double *Xc = const_cast<double *>(prev[t]);
        for (int i = lane; i < n; i += 32) w.z[i] = Xc[i];
        __syncwarp();
        back_transform_store(a, q, n, eo, w.z, Xc, lane);
    }
    if (why && lane == 0) atomicOr(&a.flags[q], 2 | why);
}

// Gram-Schmidt within relative clusters of kept eigenvalues: each member's
// twisted vector lies in the cluster's invariant subspace up to
// eps / (gap to the rest), so orthogonalising the cluster's kept vectors in
// ascending order gives an orthonormal basis of it.  One warp per kept
// eigenvalue; the warp of the first kept member does the cluster.
__global__ void __launch_bounds__(VEC_WARPS * 32) k_vec_gs(VecArgs a) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int j = blockIdx.x * VEC_WARPS + warp;
    int side, q, col;
    if (!vec_locate(a, j, side, q, col)) return;
    if (a.bmode[q] != 0 || (a.flags[q] & 2)) return;
    const int n = a.dims[q], eo = a.ev_off[q];
    if (n == 1) return;
    const int ms = a.side[side].ms;
    auto kept = [&](int c) { return a.rank[eo + c] < ms; };
    const VecCluster cl = vec_cluster(a, q, col);
    if (cluster_tight(a, q, cl)) return;             // done by k_vec_cl
    for (int c = cl.c0; c < col; ++c)
        if (kept(c)) return;                         // an earlier kept member leads
    int nm = 0;
    for (int c = col; c <= cl.c1; ++c) nm += kept(c);
    if (nm < 2) return;
    bool ok = nm <= VEC_MAXCL;
    int why = ok ? 0 : 64;
    double *X = a.vec + a.rho_off[q];
    for (int c = col + 1; ok && c <= cl.c1; ++c) {
        if (!kept(c)) continue;
        double *Z = X + (int64_t)c * n;
        for (int cp = col; cp < c; ++cp) {
            if (!kept(cp)) continue;
            const double *Y = X + (int64_t)cp * n;
            double d = 0.0;
            for (int i = lane; i < n; i += 32) d = fma(Y[i], Z[i], d);
            d = wsum(d);
            for (int i = lane; i < n; i += 32) Z[i] = fma(-d, Y[i], Z[i]);
            __syncwarp();
        }
        double nz = 0.0;
        for (int i = lane; i < n; i += 32) nz = fma(Z[i], Z[i], nz);
        nz = sqrt(wsum(nz));
        if (!(nz >= 0.5)) {
            ok = false;
            why |= 32;
            break;
        }
        const double inv = 1.0 / nz;
        for (int i = lane; i < n; i += 32) Z[i] *= inv;
        __syncwarp();
    }
    if (!ok && lane == 0) atomicOr(&a.flags[q], 2 | why);
}

// Flagged blocks (k_vec / k_vec_cl / k_vec_gs could not certify their kept
// vectors, e.g. a relative cluster whose twisted vectors came out nearly
// dependent): one warp per block recomputes every kept vector of the block
// by inverse iteration with the stationary factorisation at its eigenvalue
// from a pseudo-random start, with Gram-Schmidt inside every iteration
// against the kept vectors before it in the same unreduced block whose
// eigenvalues lie within FB_ORTOL of it (scaled units; the
// reorthogonalisation rule of LAPACK's inverse-iteration routine), then
// back-transforms the set.  Members of a cluster tighter than the
// eigenvalues' own accuracy have no individual vectors: inverse iteration
// from a random start then returns some vector of the cluster's subspace,
// and Gram-Schmidt against the members before it leaves a remainder of
// about sqrt(left / size) of it.  So a remainder down to FB_KEEP is kept:
// two projections make it orthogonal to the others to eps whatever its
// size, and a residual test on L D L^T then decides whether it is an
// eigenvector; a smaller remainder is retried from another start.  A block
// whose L D L^T is not positive definite, or whose vectors fail, keeps bit 1
// of flags[q] for the library eigensolver.
constexpr double FB_ORTOL = 1e-3;
constexpr double FB_KEEP = 1e-3;
__global__ void __launch_bounds__(VEC_WARPS * 32) k_vec_fb(VecArgs a, const int *__restrict__ blocks, int nb,
                                                            int nmax) {
    extern __shared__ double vec_smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int b = blockIdx.x * nw + warp;
    if (b >= nb) return;
    const int q = blocks[b];
    const int side = q < a.side[1].o ? 0 : 1;
    const int ms = a.side[side].ms;
    const int n = a.dims[q], eo = a.ev_off[q];
    if (n < 2) return;
    double *X = a.vec + a.rho_off[q];
    auto kept = [&](int c) { return a.rank[eo + c] < ms; };
    if (a.flags[q] & 1) {                            // no positive definite root representation
        if (lane == 0) atomicOr(&a.flags[q], 2);
        return;
    }
    const VecScratch w = vec_scratch(vec_smem + (size_t)warp * 7 * nmax, nmax);
    const double scale = a.bscale[q], sig0 = a.bsig[q];
    auto lamS = [&](int c) { return a.evals[eo + c] * scale - sig0; };
    for (int i = lane; i < n; i += 32) {
        w.dD[i] = a.ldd[eo + i];
        w.dL[i] = a.ldl[eo + i];
    }
    __syncwarp();
    // z -= sum over earlier kept columns of the same unreduced block within
    // FB_ORTOL of lam0 (tridiagonal basis), then normalised; returns |z|
    auto reorth = [&](int c, int r0, double lam0) -> double {
        for (int cp = c - 1; cp >= r0; --cp) {
            if (!(lam0 - lamS(cp) < FB_ORTOL)) break;
            if (!kept(cp)) continue;
            const double *Y = X + (int64_t)cp * n;
            double d = 0.0;
            for (int i = lane; i < n; i += 32) d = fma(Y[i], w.z[i], d);
            d = wsum(d);
            for (int i = lane; i < n; i += 32) w.z[i] = fma(-d, Y[i], w.z[i]);
            __syncwarp();
        }
        double nz = 0.0;
        for (int i = lane; i < n; i += 32) nz = fma(w.z[i], w.z[i], nz);
        nz = sqrt(wsum(nz));
        if (nz > 0.0) {
            const double inv = 1.0 / nz;
            for (int i = lane; i < n; i += 32) w.z[i] *= inv;
        }
        __syncwarp();
        return nz;
    };
    // number of eigenvalues of L D L^T (rows [r0, r1)) below sig: negative
    // pivots of the stationary transform L D L^T - sig = L+ D+ L+^T, whose
    // relative accuracy carries over to small eigenvalues (the bisection
    // that found the eigenvalues counted on T, with absolute accuracy only)
    auto ldl_count = [&](int r0, int r1, double sig) -> int {
        double sv = -sig;
        int cnt = 0;
        for (int i = r0; i + 1 < r1; ++i) {
            double dp = w.dD[i] + sv;
            if (fabs(dp) < PIVMIN) dp = -PIVMIN;
            cnt += dp < 0.0;
            sv = w.dD[i] * w.dL[i] * rcp_nr(dp) * w.dL[i] * sv - sig;
        }
        double dp = w.dD[r1 - 1] + sv;
        if (fabs(dp) < PIVMIN) dp = -PIVMIN;
        return cnt + (dp < 0.0);
    };
    bool ok = true;
    for (int c = 0; ok && c < n; ++c) {
        if (!kept(c)) continue;
        const int sr = a.sub[eo + c], r0 = sr & 0xffff, r1 = sr >> 16;
        // the eigenvalue's index inside its unreduced block, refined to the
        // relative accuracy of L D L^T by 32-way multisection on the counts
        int idx = 0;
        for (int cp = 0; cp < c; ++cp) idx += a.sub[eo + cp] == sr;
        double lam0 = lamS(c);
        {
            double w0 = fmax(fabs(lam0) * 1e-6, 1e-30), lo = lam0 - w0, hi = lam0 + w0;
            for (int grow = 0; grow < 100; ++grow) {     // bracket: count(lo) <= idx < count(hi)
                const int cl = ldl_count(r0, r1, lo), ch = ldl_count(r0, r1, hi);
                if (cl <= idx && ch > idx) break;
                w0 *= 4.0;
                if (cl > idx) lo = lam0 - w0;
                if (ch <= idx) hi = lam0 + w0;
            }
            for (int round = 0; round < 12 && hi - lo > 4e-16 * fmax(fabs(lo), fabs(hi)); ++round) {
                const double x = lo + (hi - lo) * (lane + 1) / 33.0;
                const int below = ldl_count(r0, r1, x) > idx ? 1 : 0;
                const unsigned m = __ballot_sync(0xffffffffu, below);
                const int first = m ? __ffs(m) - 1 : 32;   // first lane whose shift lies above
                const double nlo = first > 0 ? lo + (hi - lo) * first / 33.0 : lo;
                const double nhi = first < 32 ? lo + (hi - lo) * (first + 1) / 33.0 : hi;
                lo = nlo;
                hi = nhi;
            }
            lam0 = 0.5 * (lo + hi);
        }
        if (lane == 0) dstqds_lane0(w, r0, r1, lam0, w.pp);
        __syncwarp();
        double nz = 0.0;
        for (int attempt = 0; attempt < 3 && !(nz >= FB_KEEP); ++attempt) {
        for (int i = lane; i < n; i += 32) {
            unsigned hsh = (unsigned)(i + 1) * 2654435761u ^ (unsigned)(c + 7 + 7919 * attempt) * 40503u;
            hsh ^= hsh >> 15;
            hsh *= 2246822519u;
            hsh ^= hsh >> 13;
            w.z[i] = (i >= r0 && i < r1) ? ((double)(hsh & 0xffffu) / 32768.0 - 1.0) : 0.0;
        }
        __syncwarp();
        reorth(c, r0, lam0);
        nz = 0.0;
        for (int it = 0; it < 3; ++it) {
            if (lane == 0) {                         // L+ w = x
                for (int i = r0; i + 1 < r1; ++i) w.z[i + 1] -= w.lp[i] * w.z[i];
            }
            __syncwarp();
            for (int i = r0 + lane; i < r1; i += 32) w.z[i] *= rcp_nr(w.pp[i]);   // D+^-1
            __syncwarp();
            if (lane == 0) {                         // L+^T y = w
                for (int i = r1 - 2; i >= r0; --i) w.z[i] -= w.lp[i] * w.z[i + 1];
            }
            __syncwarp();
            double t2 = 0.0;
            for (int i = lane; i < n; i += 32) t2 = fma(w.z[i], w.z[i], t2);
            const double gz = sqrt(wsum(t2));
            if (!(gz > 0.0) || !isfinite(gz)) break;
            for (int i = lane; i < n; i += 32) w.z[i] *= 1.0 / gz;
            __syncwarp();
            nz = reorth(c, r0, lam0);
        }
        }
        if (!(nz >= FB_KEEP)) ok = false;
        else if (nz < 0.5) nz = reorth(c, r0, lam0);   // a second projection for a small remainder
        if (ok) {
            // residual ||L D L^T z - lam0 z|| (scaled units, ~1 the norm of
            // the block): a vector that did not settle goes to the library
            for (int i = r0 + lane; i < r1; i += 32)
                w.um[i] = w.dD[i] * (w.z[i] + (i + 1 < r1 ? w.dL[i] * w.z[i + 1] : 0.0));
            __syncwarp();
            double rr = 0.0;
            for (int i = r0 + lane; i < r1; i += 32) {
                const double y = w.um[i] + (i > r0 ? w.dL[i - 1] * w.um[i - 1] : 0.0) - lam0 * w.z[i];
                rr = fma(y, y, rr);
            }
            rr = wsum(rr);
            __syncwarp();
            if (!(sqrt(rr) <= 1e-11)) ok = false;
        }
        double *Xc = X + (int64_t)c * n;             // tridiagonal basis until the set is complete
        for (int i = lane; i < n; i += 32) Xc[i] = w.z[i];
        __syncwarp();
    }
    for (int c = 0; ok && c < n; ++c) {
        if (!kept(c)) continue;
        double *Xc = X + (int64_t)c * n;
        for (int i = lane; i < n; i += 32) w.z[i] = Xc[i];
        __syncwarp();
        back_transform_store(a, q, n, eo, w.z, Xc, lane);
    }
    if (!ok && lane == 0) atomicOr(&a.flags[q], 2 | 32);
}

// Kept columns of the blocks in `blocks`, already in their tridiagonal
// basis in vec (the host QL fallback puts them there): back-transformed in
// place, one warp per column.
__global__ void __launch_bounds__(VEC_WARPS * 32) k_backtr(VecArgs a, const int2 *__restrict__ cols, int ncols,
                                                            int nmax) {
    extern __shared__ double vec_smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int t = blockIdx.x * nw + warp;
    if (t >= ncols) return;
    const int q = cols[t].x, c = cols[t].y;
    const int n = a.dims[q], eo = a.ev_off[q];
    double *z = vec_smem + (size_t)warp * nmax;
    double *Xc = a.vec + a.rho_off[q] + (int64_t)c * n;
    for (int i = lane; i < n; i += 32) z[i] = Xc[i];
    __syncwarp();
    back_transform_store(a, q, n, eo, z, Xc, lane);
}

}  // namespace

int syev_backtr(const int *dims, const int *ev_off, const int64_t *rho_off, const double *tau, const double *refl,
                const int *perm, double *vec, const int2 *cols, int ncols, int nmax, cudaStream_t st) {
    if (ncols <= 0) return 0;
    VecArgs a{};
    a.dims = dims;
    a.ev_off = ev_off;
    a.rho_off = rho_off;
    a.tau = tau;
    a.refl = refl;
    a.perm = perm;
    a.vec = vec;
    const int nw = VEC_WARPS;
    const size_t smem = (size_t)nw * nmax * sizeof(double);
    cudaError_t e = cudaFuncSetAttribute(k_backtr, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return (int)e;
    k_backtr<<<(ncols + nw - 1) / nw, nw * 32, smem, st>>>(a, cols, ncols, nmax);
    return (int)cudaGetLastError();
}

int syev_trd(const double *rho, const int64_t *rho_off, const int *dims, const int *ev_off, const int *blocks,
             int nblocks, int maxn, double *refl, double *td, double *te, double *tau, int *perm, cudaStream_t st) {
    if (nblocks <= 0) return 0;
    const int smem = (int)(((size_t)maxn * (maxn + 1) + 2 * (size_t)maxn) * sizeof(double));
    cudaError_t e = cudaFuncSetAttribute(k_trd, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return (int)e;
    k_trd<<<nblocks, TRD_THREADS, smem, st>>>(rho, rho_off, dims, ev_off, blocks, refl, td, te, tau, perm);
    return (int)cudaGetLastError();
}

// cluster size for k_trd_cl (16 where the device allows non-portable
// clusters of that size with this shared memory, else 8) and the largest
// block it takes
int syev_trd_cl_size(int *nmax_out) {
    struct Limits {
        int csize, nmax;
    };
    // found once per process (thread-safe initialisation)
    static const Limits lim = [] {
        int csize = 0, nmax = 0;
        cudaFuncSetAttribute(k_trd_cl<false>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        cudaFuncSetAttribute(k_trd_cl<true>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        const int smem = 200 * 1024;
        cudaFuncSetAttribute(k_trd_cl<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        cudaLaunchConfig_t cfg = {};
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = 16;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.gridDim = dim3(16);
        cfg.blockDim = dim3(TRD_THREADS);
        cfg.dynamicSmemBytes = smem;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        int nc = 0;
        csize = (cudaOccupancyMaxActiveClusters(&nc, k_trd_cl<false>, &cfg) == cudaSuccess && nc > 0) ? 16 : 8;
        cudaGetLastError();
        // (ncmax + 4) n doubles within 200 KB
        nmax = 64;
        while (true) {
            const int nn = nmax + 1, nc2 = (nn + csize - 1) / csize;
            if ((size_t)((nc2 + 4) * (size_t)nn + 2 * nc2 + 8) * sizeof(double) > 200u * 1024u) break;
            nmax = nn;
        }
        return Limits{csize, nmax};
    }();
    if (nmax_out) *nmax_out = lim.nmax;
    return lim.csize;
}

int syev_trd_cl(const double *rho, const int64_t *rho_off, const int *dims, const int *ev_off, const int *blocks,
                int nblocks, int maxn, double *refl, double *td, double *te, double *tau, int *perm, double *gA,
                const int64_t *goff, cudaStream_t st) {
    if (nblocks <= 0) return 0;
    int nmax = 0;
    const int C = syev_trd_cl_size(&nmax);
    const bool glob = gA != nullptr;
    if (!glob && maxn > nmax) return (int)cudaErrorInvalidValue;
    const int ncmax = (maxn + C - 1) / C;
    const size_t smem = ((size_t)(glob ? 4 : ncmax + 4) * maxn + 2 * ncmax + 8) * sizeof(double);
    auto kern = glob ? k_trd_cl<true> : k_trd_cl<false>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return (int)e;
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = C;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(nblocks * C);
    cfg.blockDim = dim3(TRD_THREADS);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    e = cudaLaunchKernelEx(&cfg, kern, rho, rho_off, dims, ev_off, blocks, refl, td, te, tau, perm, gA, goff);
    return (int)e;
}

// k_trd_grid launches for the blocks of `blocks` (host list, sizes nb): up
// to TG_MAXG blocks a launch, the SMs split among them in proportion to n^3
// (at least 8 each).  gA + goff_h[b] is block b's n x n scratch; comm holds
// 4 n + 2 + 2 nsm doubles per block of a launch (syev_trd_grid_comm), bar
// TG_MAXG unsigned and err one int of device memory (zeroed here).
int64_t syev_trd_grid_comm(const std::vector<int> &nb, int nsm) {
    int64_t tot = 0;
    for (int x : nb) tot += 4 * (int64_t)x + 2 + 2 * (int64_t)nsm;
    return tot;
}

int syev_trd_grid(const double *rho, const int64_t *rho_off, const int *dims, const int *ev_off,
                  const std::vector<int> &blocks, const std::vector<int> &nb, double *refl, double *td, double *te,
                  double *tau, int *perm, double *gA, const std::vector<int64_t> &goff_h, double *comm,
                  unsigned *bar, int *err, cudaStream_t st) {
    if (blocks.empty()) return 0;
    int dev = 0, nsm = 0, maxn = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    for (int x : nb) maxn = std::max(maxn, x);
    const size_t smem = 2 * (size_t)maxn * sizeof(double);
    cudaError_t e = cudaFuncSetAttribute(k_trd_grid, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return (int)e;
    int occ = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_trd_grid, TRD_THREADS, smem);
    if (e != cudaSuccess) return (int)e;
    if (occ < 1) return (int)cudaErrorCooperativeLaunchTooLarge;
    e = cudaMemsetAsync(err, 0, sizeof(int), st);
    if (e != cudaSuccess) return (int)e;
    const int per = std::max(1, std::min(TG_MAXG, nsm / 8));
    for (size_t b0 = 0; b0 < blocks.size(); b0 += per) {
        const int ng = (int)std::min<size_t>(per, blocks.size() - b0);
        TgGroups grp{};
        grp.ng = ng;
        grp.spin = wait_limit();
        double w3[TG_MAXG], wsum3 = 0.0;
        for (int g = 0; g < ng; ++g) {
            const double x = nb[b0 + g];
            w3[g] = x * x * x;
            wsum3 += w3[g];
        }
        // CTAs in proportion to n^3, at least 8 a group, all nsm used
        int cnt[TG_MAXG], left = nsm - 8 * ng;
        for (int g = 0; g < ng; ++g) cnt[g] = 8 + (int)std::floor(left * (w3[g] / wsum3));
        int used = 0;
        for (int g = 0; g < ng; ++g) used += cnt[g];
        for (int g = 0; used < nsm; g = (g + 1) % ng, ++used) ++cnt[g];
        int64_t coff = 0;
        grp.c0[0] = 0;
        for (int g = 0; g < ng; ++g) {
            grp.q[g] = blocks[b0 + g];
            grp.c0[g + 1] = grp.c0[g] + cnt[g];
            grp.goff[g] = goff_h[b0 + g];
            grp.coff[g] = coff;
            coff += 4 * (int64_t)nb[b0 + g] + 2 + 2 * (int64_t)nsm;
        }
        e = cudaMemsetAsync(bar, 0, TG_MAXG * sizeof(unsigned), st);
        if (e != cudaSuccess) return (int)e;
        void *args[] = {(void *)&rho, (void *)&rho_off, (void *)&dims, (void *)&ev_off, (void *)&grp, (void *)&refl,
                        (void *)&td, (void *)&te, (void *)&tau, (void *)&perm, (void *)&gA, (void *)&comm,
                        (void *)&bar, (void *)&err};
        e = cudaLaunchCooperativeKernel((const void *)k_trd_grid, dim3(nsm), dim3(TRD_THREADS), args, smem, st);
        if (e != cudaSuccess) return (int)e;
    }
    return 0;
}

int syev_bisect(const int *dims, const int *ev_off, const int2 *items, int nitems, const double *td,
                const double *te, double *evals, double *ldd, double *ldl, double *bscale, double *bsig,
                int *flags, int *sub, int nmax, cudaStream_t st) {
    if (nitems <= 0) return 0;
    const int smem = nmax * (3 * (int)sizeof(double) + 2 * (int)sizeof(float));
    cudaError_t e = cudaFuncSetAttribute(k_bisect, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return (int)e;
    k_bisect<<<nitems, BIS_THREADS, smem, st>>>(dims, ev_off, items, td, te, evals, ldd, ldl, bscale, bsig, flags,
                                                sub, nmax);
    return (int)cudaGetLastError();
}


int syev_vec(const int *order, const int *rank, const int ms[2], int nl, int nsb, const int *ev_off,
             const int *dims, const int64_t *rho_off, const int *bmode, const int *sub, const double *evals,
             const double *ldd, const double *ldl, const double *bscale, const double *bsig, const double *tau,
             const double *refl, const int *perm, int *flags, double *vec, int nmax, cudaStream_t st) {
    VecArgs a;
    a.side[0] = VecSide{order, 0, ms[0], 0};
    a.side[1] = VecSide{order + nl, nl, ms[1], nsb};
    a.nsb = nsb;
    a.rank = rank;
    a.ev_off = ev_off;
    a.dims = dims;
    a.bmode = bmode;
    a.sub = sub;
    a.perm = perm;
    a.rho_off = rho_off;
    a.evals = evals;
    a.ldd = ldd;
    a.ldl = ldl;
    a.bscale = bscale;
    a.bsig = bsig;
    a.tau = tau;
    a.refl = refl;
    a.flags = flags;
    a.vec = vec;
    const int tot = ms[0] + ms[1];
    if (tot <= 0) return 0;
    // per warp 7 n_max doubles of shared memory: up to 4 warps a CTA within 200 KB
    const int per_warp = 7 * nmax * (int)sizeof(double);
    const int nw = std::max(1, std::min(VEC_WARPS, (200 * 1024) / per_warp));
    cudaError_t e = cudaFuncSetAttribute(k_vec, cudaFuncAttributeMaxDynamicSharedMemorySize, nw * per_warp);
    if (e != cudaSuccess) return (int)e;
    k_vec<<<(tot + nw - 1) / nw, nw * 32, nw * per_warp, st>>>(a, nmax);
    e = cudaFuncSetAttribute(k_vec_cl, cudaFuncAttributeMaxDynamicSharedMemorySize, nw * per_warp);
    if (e != cudaSuccess) return (int)e;
    k_vec_cl<<<(tot + nw - 1) / nw, nw * 32, nw * per_warp, st>>>(a, nmax);
    k_vec_gs<<<(tot + VEC_WARPS - 1) / VEC_WARPS, VEC_WARPS * 32, 0, st>>>(a);
    return (int)cudaGetLastError();
}

int syev_vec_fallback(const int *order, const int *rank, const int ms[2], int nl, int nsb, const int *ev_off,
                      const int *dims, const int64_t *rho_off, const int *sub, const double *evals, const double *ldd,
                      const double *ldl, const double *bscale, const double *bsig, const double *tau,
                      const double *refl, const int *perm, int *flags, double *vec, const int *blocks, int nb,
                      int nmax, cudaStream_t st) {
    if (nb <= 0) return 0;
    VecArgs a{};
    a.side[0] = VecSide{order, 0, ms[0], 0};
    a.side[1] = VecSide{order + nl, nl, ms[1], nsb};
    a.nsb = nsb;
    a.rank = rank;
    a.ev_off = ev_off;
    a.dims = dims;
    a.sub = sub;
    a.perm = perm;
    a.rho_off = rho_off;
    a.evals = evals;
    a.ldd = ldd;
    a.ldl = ldl;
    a.bscale = bscale;
    a.bsig = bsig;
    a.tau = tau;
    a.refl = refl;
    a.flags = flags;
    a.vec = vec;
    const int per_warp = 7 * nmax * (int)sizeof(double);
    const int nw = std::max(1, std::min(VEC_WARPS, (200 * 1024) / per_warp));
    cudaError_t e = cudaFuncSetAttribute(k_vec_fb, cudaFuncAttributeMaxDynamicSharedMemorySize, nw * per_warp);
    if (e != cudaSuccess) return (int)e;
    k_vec_fb<<<(nb + nw - 1) / nw, nw * 32, nw * per_warp, st>>>(a, blocks, nb, nmax);
    return (int)cudaGetLastError();
}

int syev_eigs_per_cta() { return BIS_EPC; }

}  // namespace nss
