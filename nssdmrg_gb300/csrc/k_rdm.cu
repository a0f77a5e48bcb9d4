// Reduced density matrices, their block eigendecomposition and the
// truncation choice, on the GPU.
//
// sb_get_rdm / build_density_matrix (src/DMRG_RDM.f90:18-162): for every
// superblock sector k, Psi = W_k [Dl x Dr]; rho_L(k) = Psi Psi^T and
// rho_R(k) = Psi^T Psi, appended in sector order (left block QN q, right
// block QN target - q).  eigh_blocks_matrix (src/MATRIX/MATRIX_BLOCKS.f90:
// 589-657): per-block symmetric eigensolve, negative eigenvalues set to
// tiny(1d0), then one descending order over all blocks (ascending sort then
// reversal: among exactly equal eigenvalues the later block position comes
// first).  renormalize_block (src/DMRG_RDM.f90:204-221): m_s =
// min(Mstates, m_block, #lambda), extended by every later eigenvalue within
// deg_evals_threshold (relative) of lambda(m_s); trunc = 1 - sum lambda(1:m_s);
// U = rho%sparse(m_block, m_s) (src/MATRIX/MATRIX_BLOCKS.f90:556-576).
// Entropy -sum lambda log(lambda + 1e-32) (src/DMRG_MAIN.f90:511-518).
//
// The block eigensolve is cuSOLVER dsyevd, one call per block on the
// context stream (a library call; the sector blocks are small, < 600).
#include "device.cuh"
#include "host_tridiag.hpp"

#include <cstdlib>
#include <cstring>

#include <cusolverDn.h>

#include <algorithm>
#include <cstdio>
#include <functional>
#include <map>
#include <cfloat>
#include <cmath>

namespace nss {

namespace {

constexpr int RT = 16;

__device__ __forceinline__ double warp_sum_d(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

struct RhoItem {     // one 16x16 tile of one rho block
    int side, k, r0, c0;
};

// rho_L[a][b] = sum_r W[a][r] W[b][r] ; rho_R[a][b] = sum_l W[l][a] W[l][b]
__global__ void __launch_bounds__(256) k_rho(const double *__restrict__ psi, const RhoItem *__restrict__ items,
                                             const int *__restrict__ dls, const int *__restrict__ drs,
                                             const int64_t *__restrict__ off, const int64_t *__restrict__ rho_off,
                                             int nsb, double *__restrict__ rho) {
    __shared__ double sa[RT][33];
    __shared__ double sb[RT][33];
    const RhoItem it = items[blockIdx.x];
    const int dl = dls[it.k], dr = drs[it.k];
    const double *W = psi + off[it.k];
    const int dim = it.side == 0 ? dl : dr;       // rho is dim x dim
    const int kk = it.side == 0 ? dr : dl;        // contraction length
    double *R = rho + rho_off[it.side * nsb + it.k];
    const int tid = threadIdx.x, ty = tid / RT, tx = tid % RT;
    double acc = 0.0;
    for (int j0 = 0; j0 < kk; j0 += 32) {
        for (int e = tid; e < RT * 32; e += 256) {
            const int r = e / 32, cc = e % 32;
            const int ga = it.r0 + r, gb = it.c0 + r, gj = j0 + cc;
            double va = 0.0, vb = 0.0;
            if (gj < kk) {
                if (it.side == 0) {
                    if (ga < dim) va = W[(int64_t)ga * dr + gj];
                    if (gb < dim) vb = W[(int64_t)gb * dr + gj];
                } else {
                    if (ga < dim) va = W[(int64_t)gj * dr + ga];
                    if (gb < dim) vb = W[(int64_t)gj * dr + gb];
                }
            }
            sa[r][cc] = va;
            sb[r][cc] = vb;
        }
        __syncthreads();
#pragma unroll 8
        for (int j = 0; j < 32; ++j) acc = fma(sa[ty][j], sb[tx][j], acc);
        __syncthreads();
    }
    const int a = it.r0 + ty, b = it.c0 + tx;
    if (a < dim && b < dim) R[(int64_t)a * dim + b] = acc;
}

// |rho - rho^T| > 1e-12 -> error flag (build_density_matrix, :159-160)
__global__ void k_symcheck(const double *rho, int64_t total_dummy, const int64_t *rho_off, const int *dims,
                           int nblk, int *err) {
    for (int q = blockIdx.x; q < nblk; q += gridDim.x) {
        const int d = dims[q];
        const double *R = rho + rho_off[q];
        for (int e = threadIdx.x; e < d * d; e += blockDim.x) {
            const int a = e / d, b = e % d;
            if (fabs(R[(int64_t)a * d + b] - R[(int64_t)b * d + a]) > 1e-12) atomicExch(err, 1);
        }
    }
    (void)total_dummy;
}

// negative eigenvalues -> tiny(1d0) (MATRIX_BLOCKS.f90:629)
__global__ void k_clamp(double *ev, int n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        if (ev[i] < 0.0) ev[i] = DBL_MIN;
}

// Descending rank of every eigenvalue; ties: larger position first (the
// reversal of a stable ascending order).  After k_clamp the values are >= 0,
// whose IEEE bit patterns order like the values, so the n^2 comparisons are
// integer compares (an FP64 compare costs a 64-cycle slot of GB300's FP64
// pipe); -0.0 is read as +0.0.  Keys are staged through shared memory.
__device__ __forceinline__ long long rank_key(double x) { return x == 0.0 ? 0ll : __double_as_longlong(x); }

__global__ void __launch_bounds__(256) k_rank(const double *ev, int n, double *sorted, int *order,
                                              int *rank_of /* may be null */) {
    __shared__ long long ks[1024];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const long long xi = i < n ? rank_key(ev[i]) : 0ll;
    int r = 0;
    for (int j0 = 0; j0 < n; j0 += 1024) {
        const int jn = min(1024, n - j0);
        __syncthreads();
        for (int t = threadIdx.x; t < jn; t += blockDim.x) ks[t] = rank_key(ev[j0 + t]);
        __syncthreads();
        if (i < n)
            for (int t = 0; t < jn; ++t) {
                const long long y = ks[t];
                r += (y > xi) || (y == xi && j0 + t > i);
            }
    }
    if (i < n) {
        sorted[r] = ev[i];
        order[r] = i;
        if (rank_of) rank_of[i] = r;
    }
}

// Truncation choice, truncation error and entropy of one side, one CTA of
// 1024 threads: the degeneracy extension is a count over the tail, the sums
// are block reductions (the reference sums sequentially; the orders differ by
// rounding only).
// Truncation choice of renormalize_block (src/DMRG_RDM.f90:204-221, right
// side :277-294) on the descending eigenvalues (negatives read as 0):
//   Mstates != 0 : m_s = min(Mstates, m_block, n)
//   else         : m_s = the first minimum over i of |1 - sum(lambda(1:i)) - Estates|
//                  (minloc of abs(1-cumulate(lambda)-Estates))
// then extended over every later eigenvalue within deg_evals_threshold
// (relative) of lambda(m_s); truncation error 1 - sum(lambda(1:m_s)) and the
// entropy S = -sum lambda log(lambda + 1e-32) (src/DMRG_MAIN.f90:501-518).
// The prefix sums of the Estates rule: each thread sums a contiguous chunk,
// the chunk totals are scanned over the block, then every thread walks its
// chunk again with its offset; ties keep the lowest index.
__global__ void __launch_bounds__(1024) k_truncate(const double *sorted, int n, int mstates, double estates,
                                                   int mblock, double thr,
                                                   double *out_d /*trunc, entropy*/, int *out_i /*m_s*/) {
    __shared__ double red_s[32], red_e[32];
    __shared__ int red_c[32];
    __shared__ int ms_s;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    int ms = min(mstates, min(mblock, n));
    if (mstates == 0) {
        __shared__ double wsum[32];
        __shared__ double best_v[32];
        __shared__ int best_i[32];
        const int per = (n + (int)blockDim.x - 1) / (int)blockDim.x;
        const int c0 = min(n, tid * per), c1 = min(n, c0 + per);
        double loc = 0.0;
        for (int i = c0; i < c1; ++i) loc += sorted[i] < 0.0 ? 0.0 : sorted[i];
        // inclusive scan of the chunk totals: warps, then the warp totals
        double inc = loc;
        for (int o = 1; o < 32; o <<= 1) {
            const double y = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += y;
        }
        if (lane == 31) wsum[warp] = inc;
        __syncthreads();
        if (warp == 0) {
            double t = lane < (int)(blockDim.x >> 5) ? wsum[lane] : 0.0;
            for (int o = 1; o < 32; o <<= 1) {
                const double y = __shfl_up_sync(0xffffffffu, t, o);
                if (lane >= o) t += y;
            }
            wsum[lane] = t;
        }
        __syncthreads();
        double run = (warp > 0 ? wsum[warp - 1] : 0.0) + inc - loc;   // sum of all earlier chunks
        double bv = 1e300;
        int bi = n;
        for (int i = c0; i < c1; ++i) {
            run += sorted[i] < 0.0 ? 0.0 : sorted[i];
            const double dv = fabs(1.0 - run - estates);
            if (dv < bv) { bv = dv; bi = i; }
        }
        for (int o = 16; o > 0; o >>= 1) {
            const double v2 = __shfl_xor_sync(0xffffffffu, bv, o);
            const int i2 = __shfl_xor_sync(0xffffffffu, bi, o);
            if (v2 < bv || (v2 == bv && i2 < bi)) { bv = v2; bi = i2; }
        }
        if (lane == 0) { best_v[warp] = bv; best_i[warp] = bi; }
        __syncthreads();
        if (tid == 0) {
            double v = best_v[0];
            int b = best_i[0];
            for (int q = 1; q < (int)(blockDim.x >> 5); ++q)
                if (best_v[q] < v || (best_v[q] == v && best_i[q] < b)) { v = best_v[q]; b = best_i[q]; }
            ms_s = b + 1;
        }
        __syncthreads();
        ms = ms_s;
        __syncthreads();
    }
    if (ms < 1) ms = 1;
    const double e_ = sorted[ms - 1] < 0.0 ? 0.0 : sorted[ms - 1];
    int cnt = 0;
    for (int i = ms + tid; i < n; i += blockDim.x) {
        const double li = sorted[i] < 0.0 ? 0.0 : sorted[i];
        if (fabs(e_ - li) / e_ <= thr) ++cnt;
    }
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    if (lane == 0) red_c[warp] = cnt;
    __syncthreads();
    if (tid == 0) {
        int t = 0;
        for (int q = 0; q < (int)(blockDim.x >> 5); ++q) t += red_c[q];
        ms_s = ms + t;
    }
    __syncthreads();
    const int msf = ms_s;
    double sk = 0.0, ent = 0.0;
    for (int i = tid; i < n; i += blockDim.x) {
        const double li = sorted[i] < 0.0 ? 0.0 : sorted[i];
        if (i < msf) sk += li;
        ent -= li * log(li + 1e-32);
    }
    for (int o = 16; o > 0; o >>= 1) {
        sk += __shfl_xor_sync(0xffffffffu, sk, o);
        ent += __shfl_xor_sync(0xffffffffu, ent, o);
    }
    if (lane == 0) { red_s[warp] = sk; red_e[warp] = ent; }
    __syncthreads();
    if (tid == 0) {
        double a = 0.0, b = 0.0;
        for (int q = 0; q < (int)(blockDim.x >> 5); ++q) { a += red_s[q]; b += red_e[q]; }
        out_d[0] = 1.0 - a;
        out_d[1] = b;
        out_i[0] = msf;
    }
}

// write_entanglement's S_N and S_c (src/DMRG_MAIN.f90:523-561), one CTA per
// side over its rho blocks (the tiny-clamped eigenvalues of each block):
// P_q = sum lambda, S_q = sum (lambda/P_q) log(lambda/P_q + 1e-32),
// S_N = -sum_q P_q log(P_q + 1e-32), S_c = -sum_q P_q S_q.  out[2 side] =
// S_N, out[2 side + 1] = S_c.
__global__ void __launch_bounds__(256) k_qn_entropy(const double *__restrict__ evals, const int *__restrict__ ev_off,
                                                    int nsb, double *__restrict__ out) {
    __shared__ double red[2][8];
    const int side = blockIdx.x, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    double sn = 0.0, sc = 0.0;
    for (int k = warp; k < nsb; k += 8) {
        const int b0 = ev_off[side * nsb + k], b1 = ev_off[side * nsb + k + 1];
        double p = 0.0;
        for (int i = b0 + lane; i < b1; i += 32) p += evals[i];
        p = warp_sum_d(p);
        double sq = 0.0;
        for (int i = b0 + lane; i < b1; i += 32) {
            const double o = evals[i] / p;
            sq += o * log(o + 1e-32);
        }
        sq = warp_sum_d(sq);
        sn -= p * log(p + 1e-32);
        sc -= p * sq;
    }
    if (lane == 0) {
        red[0][warp] = sn;
        red[1][warp] = sc;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, b = 0.0;
        for (int w = 0; w < 8; ++w) {
            a += red[0][w];
            b += red[1][w];
        }
        out[2 * side] = a;
        out[2 * side + 1] = b;
    }
}

// Compact form of the kept columns of one side (U without its zero rows):
// kept[j] = block of column j (side-local), uoff[j] = start of its n_q
// values in ucomp, ucomp[uoff[j] + p] = row p of the eigenvector.  One CTA:
// an exclusive scan of n_q over j, then the copies.
__global__ void __launch_bounds__(1024) k_ucompact(const double *__restrict__ vec, const int64_t *__restrict__ rho_off,
                                                  const int *__restrict__ dims, const int *__restrict__ ev_off,
                                                  int ev_base, int nblk, const int *__restrict__ order, int ms,
                                                  int *__restrict__ kept, int *__restrict__ uoff,
                                                  double *__restrict__ ucomp) {
    __shared__ int wsum_s[32];
    __shared__ int carry_s;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) carry_s = 0;
    __syncthreads();
    for (int j0 = 0; j0 < ms; j0 += 1024) {
        const int j = j0 + tid;
        int nq = 0;
        if (j < ms) {
            const int pos = order[j] + ev_base;
            int q = 0;
            while (q + 1 < nblk && ev_off[q + 1] <= pos) ++q;
            nq = dims[q];
            kept[j] = q;
        }
        int x = nq;                                  // inclusive warp scan
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) wsum_s[warp] = x;
        __syncthreads();
        if (warp == 0) {
            int t = wsum_s[lane];
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, t, o);
                if (lane >= o) t += y;
            }
            wsum_s[lane] = t;                        // inclusive over warps
        }
        __syncthreads();
        const int base = carry_s + (warp > 0 ? wsum_s[warp - 1] : 0);
        if (j < ms) uoff[j] = base + x - nq;
        __syncthreads();
        if (tid == 0) carry_s += wsum_s[31];
        __syncthreads();
    }
    for (int j = warp; j < ms; j += 32) {
        const int q = kept[j];
        const int pos = order[j] + ev_base, col = pos - ev_off[q], nq = dims[q];
        const double *E = vec + rho_off[q] + (int64_t)col * nq;
        double *D = ucomp + uoff[j];
        for (int p = lane; p < nq; p += 32) D[p] = E[p];
    }
}

// Batched cyclic Jacobi eigensolver for the small rho blocks (n <= JAC_MAX):
// one CTA per block, the block and its eigenvectors in shared memory.  Each
// sweep visits all n(n-1)/2 pairs in n-1 rounds of n/2 disjoint rotations
// (round-robin tournament), so a round's rotations are applied in parallel:
// rows of A, then columns of A and of V.  Sweeps stop when the off-diagonal
// Frobenius norm is below 1e-15 of the whole norm (quadratic convergence, a
// handful of sweeps), at most JAC_SWEEPS.  Output as cuSOLVER's: eigenvalues
// ascending, eigenvectors as the columns of a column-major block.
constexpr int JAC_MAX = 64, JAC_SWEEPS = 24;
constexpr int JAC_DEFAULT = 32;

// blocks up to this size take k_jacobi (env NSS_JACOBI_MAX, 0..JAC_MAX, default
// 32; 0 sends every block to the batched library eigensolver)
// padded size classes from this size on go one matrix at a time through the
// library's blocked solver (all SMs) instead of its batched one (one CTA
// per matrix, seconds at these sizes)
constexpr int LIB_WHOLE_GPU_N = 1024;
constexpr int LIB_FALLBACK_WHOLE_N = 128;   // the same for the own path's flagged blocks
constexpr int QL_HOST_MAX = 800;             // flagged blocks up to this size: host QL on their tridiagonal matrix

int jacobi_max() {
    static const int v = [] {
        const char *e = std::getenv("NSS_JACOBI_MAX");
        if (!e) return JAC_DEFAULT;
        const int x = std::atoi(e);
        return x < 0 ? 0 : (x > JAC_MAX ? JAC_MAX : x);
    }();
    return v;
}

__global__ void __launch_bounds__(256) k_jacobi(const double *rho, const int64_t *__restrict__ rho_off,
                                                const int *__restrict__ dims, const int *__restrict__ ev_off,
                                                const int *__restrict__ blocks, double *vec_out,
                                                double *evals /* may be null: vectors only */) {
    extern __shared__ double jac_smem[];            // A and V: 2 x JAC_MAX x (JAC_MAX+1)
    double(*A)[JAC_MAX + 1] = reinterpret_cast<double(*)[JAC_MAX + 1]>(jac_smem);
    double(*V)[JAC_MAX + 1] = reinterpret_cast<double(*)[JAC_MAX + 1]>(jac_smem + JAC_MAX * (JAC_MAX + 1));
    __shared__ double cs[JAC_MAX / 2][2];
    __shared__ int pr[JAC_MAX / 2][2];
    __shared__ double red[8][2];
    __shared__ int perm[JAC_MAX];
    const int q = blocks[blockIdx.x];
    const int n = dims[q];
    const double *R = rho + rho_off[q];
    double *Vout = vec_out + rho_off[q];
    const int tid = threadIdx.x;
    for (int e = tid; e < n * n; e += blockDim.x) {
        const int i = e / n, j = e % n;
        A[i][j] = R[e];
        V[i][j] = (i == j) ? 1.0 : 0.0;
    }
    __syncthreads();
    const int ne = n + (n & 1);          // even number of players (one dummy if n is odd)
    for (int sweep = 0; sweep < JAC_SWEEPS && n > 1; ++sweep) {
        // off-diagonal and total squared norms
        double off = 0.0, tot = 0.0;
        for (int e = tid; e < n * n; e += blockDim.x) {
            const int i = e / n, j = e % n;
            const double x = A[i][j] * A[i][j];
            tot += x;
            if (i != j) off += x;
        }
        for (int o = 16; o > 0; o >>= 1) {
            off += __shfl_xor_sync(0xffffffffu, off, o);
            tot += __shfl_xor_sync(0xffffffffu, tot, o);
        }
        if ((tid & 31) == 0) { red[tid >> 5][0] = off; red[tid >> 5][1] = tot; }
        __syncthreads();
        double offs = 0.0, tots = 0.0;
        for (int w = 0; w < 8; ++w) { offs += red[w][0]; tots += red[w][1]; }
        __syncthreads();
        if (!(offs > 1e-30 * tots)) break;
        for (int round = 0; round < ne - 1; ++round) {
            // round-robin pairing: player 0 fixed, the others rotate
            if (tid < ne / 2) {
                const int a0 = (tid == 0) ? 0 : 1 + (tid - 1 + round) % (ne - 1);
                const int b0 = 1 + (ne - 2 - tid + round) % (ne - 1);
                int p = min(a0, b0), r = max(a0, b0);
                double c = 1.0, sn = 0.0;
                if (r < n && p != r) {
                    const double apq = A[p][r];
                    if (apq != 0.0) {
                        const double th = (A[r][r] - A[p][p]) / (2.0 * apq);
                        // t = tan of the rotation angle; 1/(2 th) where th*th would overflow
                        const double t = fabs(th) > 1e150 ? 0.5 / th
                                                          : (th >= 0.0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1.0));
                        c = 1.0 / sqrt(t * t + 1.0);
                        sn = t * c;
                    }
                } else {
                    p = r = -1;
                }
                pr[tid][0] = p;
                pr[tid][1] = r;
                cs[tid][0] = c;
                cs[tid][1] = sn;
            }
            __syncthreads();
            // rows: A <- J^T A
            for (int e = tid; e < (ne / 2) * n; e += blockDim.x) {
                const int k = e / n, col = e % n;
                const int p = pr[k][0], r = pr[k][1];
                if (p < 0) continue;
                const double c = cs[k][0], sn = cs[k][1];
                const double ap = A[p][col], ar = A[r][col];
                A[p][col] = c * ap - sn * ar;
                A[r][col] = sn * ap + c * ar;
            }
            __syncthreads();
            // columns: A <- A J and V <- V J
            for (int e = tid; e < (ne / 2) * n; e += blockDim.x) {
                const int k = e / n, row = e % n;
                const int p = pr[k][0], r = pr[k][1];
                if (p < 0) continue;
                const double c = cs[k][0], sn = cs[k][1];
                const double ap = A[row][p], ar = A[row][r];
                A[row][p] = c * ap - sn * ar;
                A[row][r] = sn * ap + c * ar;
                const double vp = V[row][p], vr = V[row][r];
                V[row][p] = c * vp - sn * vr;
                V[row][r] = sn * vp + c * vr;
            }
            __syncthreads();
        }
    }
    // ascending order of the eigenvalues (ties: lower index first)
    for (int i = tid; i < n; i += blockDim.x) {
        const double x = A[i][i];
        int rnk = 0;
        for (int j = 0; j < n; ++j) rnk += (A[j][j] < x) || (A[j][j] == x && j < i);
        perm[rnk] = i;
    }
    __syncthreads();
    for (int e = tid; e < n * n; e += blockDim.x) {
        const int col = e / n, row = e % n;         // column-major output
        Vout[e] = V[row][perm[col]];
        if (row == 0 && evals) evals[ev_off[q] + col] = A[perm[col]][perm[col]];
    }
}

// Embed block q = list[b] (d x d) in the N x N column-major matrix A_b of a
// batched eigensolve: the extra diagonal entries are -(1 + i/N) * tr(rho_q)
// (tr >= every eigenvalue of the positive semidefinite block), so the
// padding eigenvalues come first in ascending order and the block's
// eigenvectors have no component outside its d rows.
__global__ void __launch_bounds__(256) k_pack(const double *__restrict__ rho, const int64_t *__restrict__ rho_off,
                                              const int *__restrict__ dims, const int *__restrict__ list, int N,
                                              double *__restrict__ A) {
    const int b = blockIdx.x, q = list[b], d = dims[q];
    const double *R = rho + rho_off[q];
    double *Ab = A + (int64_t)b * N * N;
    __shared__ double tr;
    if (threadIdx.x < 32) {
        double t = 0.0;
        for (int i = threadIdx.x; i < d; i += 32) t += fabs(R[(int64_t)i * d + i]);
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if (threadIdx.x == 0) tr = fmax(t, 1e-200);
    }
    __syncthreads();
    for (int e = threadIdx.x; e < N * N; e += blockDim.x) {
        const int col = e / N, row = e % N;
        double x = 0.0;
        if (row < d && col < d) x = R[(int64_t)col * d + row];
        else if (row == col) x = -(1.0 + (double)(row - d) * (1.0 / 64.0)) * tr;
        Ab[e] = x;
    }
}

// Back from the batched layout: the last d eigenpairs of A_b are the block's
// (ascending), eigenvector rows 0..d-1, column-major d x d into the block slot.
__global__ void __launch_bounds__(256) k_unpack(const double *__restrict__ A, const double *__restrict__ Wb, int N,
                                                const int *__restrict__ list, const int *__restrict__ dims,
                                                const int64_t *__restrict__ rho_off, const int *__restrict__ ev_off,
                                                double *__restrict__ vec_out, double *__restrict__ evals) {
    const int b = blockIdx.x, q = list[b], d = dims[q], sh = N - d;
    const double *Ab = A + (int64_t)b * N * N;
    double *R = vec_out + rho_off[q];
    for (int e = threadIdx.x; e < d * d; e += blockDim.x) {
        const int col = e / d, row = e % d;
        R[e] = Ab[(int64_t)(sh + col) * N + row];
    }
    if (evals)
        for (int i = threadIdx.x; i < d; i += blockDim.x) evals[ev_off[q] + i] = Wb[(int64_t)b * N + sh + i];
}

// Library vectors of the blocks whose own-path vectors were rejected: the
// library orders a block's eigenpairs ascending over the whole block, the
// own path ascending within each unreduced part of its tridiagonal form, so
// column col of the output takes the library column whose rank matches the
// rank of evals[col] in the block (ties by position).
__global__ void __launch_bounds__(256) k_fbperm(const int *__restrict__ list, const int *__restrict__ dims,
                                              const int *__restrict__ ev_off, const int64_t *__restrict__ rho_off,
                                              const double *__restrict__ evals, const double *__restrict__ src,
                                              double *__restrict__ dst) {
    extern __shared__ int perm[];
    const int q = list[blockIdx.x], n = dims[q];
    const double *ev = evals + ev_off[q];
    for (int col = threadIdx.x; col < n; col += blockDim.x) {
        const double x = ev[col];
        int rk = 0;
        for (int i = 0; i < n; ++i) rk += (ev[i] < x) || (ev[i] == x && i < col);
        perm[col] = rk;
    }
    __syncthreads();
    const double *S = src + rho_off[q];
    double *D = dst + rho_off[q];
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
        const int col = e / n, row = e - col * n;
        D[e] = S[(int64_t)perm[col] * n + row];
    }
}

// rho-block eigensolver: blocks up to SYEV_MAX take the eigensolver of
// k_syev.cu, larger ones k_jacobi / the batched library eigensolve (which
// also recomputes the vectors of blocks the former marks).  Env
// NSS_RDM_EIG=library sends every block to the library path.
bool rdm_own_eigensolver() {
    const char *e = std::getenv("NSS_RDM_EIG");
    return !(e && std::string(e) == "library");
}

// blocks from this many states on are reduced by the whole GPU (env
// NSS_TRD_GRID_MIN; 0 keeps every big block on one cluster).  Alone, a
// 1000-state block is faster on the whole GPU (17.5 against 39.5 ms); in a
// sweep the cluster tier runs several such blocks side by side, and the
// spin-1 L=64 M=512 finite sweep took 6.59-6.67 s with 1400 (three runs)
// against 6.73-6.81 s with 900 and 6.77 s with 600.
int trd_grid_min() {
    const char *e = std::getenv("NSS_TRD_GRID_MIN");
    return e ? std::atoi(e) : 1400;
}

template <class T>
int ensure_n(Ctx &c, T **p, int64_t &cap, int64_t need) {
    if (*p && cap >= need) return NSS_OK;
    ctx_free(c, *p);
    *p = nullptr;
    NSS_CUDA_TRY(c, ctx_alloc(c, p, (size_t)std::max<int64_t>(need, 1)));
    cap = need;
    return NSS_OK;
}

}  // namespace

void rdm_release(Ctx &c) {
    DevRdm &r = c.rdm;
    void *ptrs[] = {r.rho, r.evals, r.sorted, r.order, r.u, r.work, r.info, r.scal, r.iscal, r.bat, r.bat_info,
                    r.vec, r.syd, r.syi, r.tab, r.big, r.tg};
    for (void *p : ptrs) ctx_free(c, p);
    if (r.htab) cudaFreeHost(r.htab);
    if (r.hu) cudaFreeHost(r.hu);
    for (int i = 0; i < DevRdm::NSIDE; ++i) {
        if (r.side[i]) cudaStreamDestroy(r.side[i]);
        if (r.ev_join[i]) cudaEventDestroy(r.ev_join[i]);
    }
    if (r.ev_fork) cudaEventDestroy(r.ev_fork);
    for (int i = 0; i < DevRdm::NPH; ++i)
        if (r.ph[i]) cudaEventDestroy(r.ph[i]);
    if (r.params) cusolverDnDestroyParams((cusolverDnParams_t)r.params);
    r = DevRdm{};
}

int rdm_run(Ctx &c, const double *d_psi, int mstates, double estates, double deg_thr, nss_rdm_side out[2], double *lam_l,
            double *lam_r, int32_t *kept_l, int32_t *kept_r, double *u_l, double *u_r, KeptLayout *kl, int vec_sides) {
    DevSb &s = c.sb;
    if (!s.valid) { c.err = "nss_rdm: no superblock uploaded"; return NSS_ERR_STATE; }
    if (s.ai.empty() || s.bi.empty()) { c.err = "nss_rdm: descriptor had no ai/bi state maps"; return NSS_ERR_INVALID; }
    if (mstates < 0) { c.err = "nss_rdm: Mstates must not be negative"; return NSS_ERR_INVALID; }
    if (mstates == 0 && !(estates != 0.0)) {
        c.err = "Mdmrg=Edmrg=0 can not fix a threshold for the RDM";
        return NSS_ERR_INVALID;
    }
    cudaStream_t st = c.stream;
    DevRdm &r = c.rdm;
    const int nsb = s.nsb, nblk = 2 * nsb;
    // block layout: left blocks 0..nsb-1 then right blocks
    std::vector<int64_t> rho_off(nblk + 1);
    std::vector<int> dims(nblk), ev_off(nblk + 2);
    int64_t acc = 0;
    int eacc = 0;
    for (int side = 0; side < 2; ++side)
        for (int k = 0; k < nsb; ++k) {
            const int d = side == 0 ? s.dls[k] : s.drs[k];
            const int q = side * nsb + k;
            rho_off[q] = acc;
            dims[q] = d;
            ev_off[q] = eacc;
            acc += (int64_t)d * d;
            eacc += d;
        }
    rho_off[nblk] = acc;
    ev_off[nblk] = eacc;
    const int nl = ev_off[nsb], nr = eacc - nl;
    std::vector<RhoItem> items;
    for (int side = 0; side < 2; ++side)
        for (int k = 0; k < nsb; ++k) {
            const int d = side == 0 ? s.dls[k] : s.drs[k];
            for (int r0 = 0; r0 < d; r0 += RT)
                for (int c0 = 0; c0 < d; c0 += RT) items.push_back({side, k, r0, c0});
        }
    // eigensolver path of each block
    const bool own_path = rdm_own_eigensolver();
    const int jmax = jacobi_max();
    // own: reduced in one CTA (k_trd); big: by the library's blocked
    // tridiagonal reduction; both then share bisection and vectors (the
    // "own path"); small / large: the library eigensolvers throughout
    // own: one CTA per block up to SYEV_MAX states (k_trd, with the
    // component reordering; measured faster than a cluster at 120 states),
    // clu: a thread-block cluster per block up to the size its shared memory
    // holds (k_trd_cl; env NSS_TRD_CLUSTER=0 disables it), big: the same
    // cluster kernel on a global (L2-resident) copy of the block, up to
    // SYEV_BIG_MAX; larger blocks take the library eigensolver
    int cl_nmax = 0;
    syev_trd_cl_size(&cl_nmax);
    if (const char *sm = std::getenv("NSS_TRD_CL_SHARED_MAX")) cl_nmax = std::min(cl_nmax, std::atoi(sm));
    const char *tce = std::getenv("NSS_TRD_CLUSTER");
    const bool use_cl = !(tce && std::string(tce) == "0");
    const int cta_max = SYEV_MAX;
    std::vector<int> own, clu, big, small, large;
    int maxn_own = 1, maxn_clu = 1, maxn_path = 1;
    for (int q = 0; q < nblk; ++q) {
        if (own_path && dims[q] <= cta_max) {
            own.push_back(q);
            maxn_own = std::max(maxn_own, dims[q]);
        } else if (own_path && use_cl && dims[q] <= cl_nmax) {
            clu.push_back(q);
            maxn_clu = std::max(maxn_clu, dims[q]);
        } else if (own_path && use_cl && dims[q] <= SYEV_BIG_MAX) {
            big.push_back(q);                        // the cluster kernel on a global copy
        } else if (dims[q] <= jmax) {
            small.push_back(q);
        } else {
            large.push_back(q);
        }
    }
    // big blocks of at least trd_grid_min() states are reduced by the whole
    // GPU (k_trd_grid; a 16-SM cluster is bound by n^3/16 FP64 FMAs per SM,
    // 0.45 s at 2645 states): the cluster ones first, then those
    const int gmin = trd_grid_min();
    std::stable_partition(big.begin(), big.end(), [&](int q) { return gmin <= 0 || dims[q] < gmin; });
    int nbig_cl = 0;
    for (int q : big) nbig_cl += (gmin <= 0 || dims[q] < gmin) ? 1 : 0;
    std::vector<int> path(own);
    path.insert(path.end(), clu.begin(), clu.end());
    path.insert(path.end(), big.begin(), big.end());
    for (int q : path) maxn_path = std::max(maxn_path, dims[q]);
    std::vector<int2> bis;
    const int epc = syev_eigs_per_cta();
    for (int q : path)
        for (int k0 = 0; k0 < dims[q]; k0 += epc) bis.push_back(make_int2(q, k0));
    std::vector<int> bmode(nblk, 1);
    for (int q : path) bmode[q] = 0;
    std::vector<int> maps(s.ai), map_off(s.ai_off);
    for (int k = 1; k <= nsb; ++k) map_off.push_back((int)s.ai.size() + s.bi_off[k]);
    maps.insert(maps.end(), s.bi.begin(), s.bi.end());
    const int mblk[2] = {s.m_left, s.m_right};
    const int kmax = std::max(1, std::max(s.m_left, s.m_right));
    // device scratch (grow-only)
    int rc;
    int64_t cap_sorted = r.cap_evals;
    if ((rc = ensure_n(c, &r.rho, r.cap_rho, acc))) return rc;
    if ((rc = ensure_n(c, &r.vec, r.cap_vec, acc))) return rc;
    if ((rc = ensure_n(c, &r.evals, r.cap_evals, eacc))) return rc;
    if (!r.sorted || cap_sorted < eacc || !r.order) {
        ctx_free(c, r.sorted);
        ctx_free(c, r.order);
        NSS_CUDA_TRY(c, ctx_alloc(c, &r.sorted, (size_t)eacc));
        NSS_CUDA_TRY(c, ctx_alloc(c, &r.order, (size_t)eacc));
    }
    int maxd = 1;
    for (int d : dims) maxd = std::max(maxd, d);
    const int64_t ucap = 2 * (int64_t)kmax * maxd;   // compact kept columns of both sides
    if ((rc = ensure_n(c, &r.u, r.cap_u, ucap))) return rc;
    if (!r.scal) {
        NSS_CUDA_TRY(c, ctx_alloc(c, &r.scal, 8));
        NSS_CUDA_TRY(c, ctx_alloc(c, &r.iscal, 8));
        NSS_CUDA_TRY(c, ctx_alloc(c, &r.info, DevRdm::NSIDE));
    }
    // own eigensolver: reflectors (rho layout), T, tau, L D L^T (eigenvalue
    // layout), per-block scale and shift; per-block flags
    const int64_t syd_need = path.empty() ? 1 : acc + 5 * (int64_t)eacc + 2 * nblk;
    if ((rc = ensure_n(c, &r.syd, r.cap_syd, syd_need))) return rc;
    if ((rc = ensure_n(c, &r.syi, r.cap_syi, nblk + 3 * (int64_t)eacc))) return rc;
    double *refl = r.syd, *td = refl + acc, *te = td + eacc, *tau = te + eacc, *ldd = tau + eacc,
           *ldl = ldd + eacc, *bscale = ldl + eacc, *bsig = bscale + nblk;
    int *flags = r.syi, *sub = flags + nblk, *rnk = sub + eacc, *perm = rnk + eacc;
    // the call's tables: packed into one pinned staging buffer, one copy
    size_t tot = 0;
    auto slot = [&](size_t bytes) {
        const size_t o = (tot + 15) & ~size_t(15);
        tot = o + bytes;
        return o;
    };
    const size_t o_items = slot(items.size() * sizeof(RhoItem)), o_rho_off = slot(rho_off.size() * sizeof(int64_t)),
                 o_dims = slot(dims.size() * sizeof(int)), o_ev_off = slot(ev_off.size() * sizeof(int)),
                 o_own = slot(own.size() * sizeof(int)), o_clu = slot(clu.size() * sizeof(int)),
                 o_big = slot(big.size() * sizeof(int)), o_goff = slot(big.size() * sizeof(int64_t)),
                 o_bis = slot(bis.size() * sizeof(int2)),
                 o_bmode = slot(bmode.size() * sizeof(int)), o_kept = slot(4 * (size_t)kmax * sizeof(int));
    if (!r.htab || r.cap_htab < (int64_t)tot) {
        if (r.htab) cudaFreeHost(r.htab);
        r.htab = nullptr;
        NSS_CUDA_TRY(c, cudaHostAlloc((void **)&r.htab, tot, cudaHostAllocDefault));
        r.cap_htab = (int64_t)tot;
    }
    if ((rc = ensure_n(c, &r.tab, r.cap_tab, (int64_t)tot))) return rc;
    auto put = [&](size_t o, const auto &v) {
        if (!v.empty()) std::memcpy(r.htab + o, v.data(), v.size() * sizeof(v[0]));
    };
    put(o_items, items);
    put(o_rho_off, rho_off);
    put(o_dims, dims);
    put(o_ev_off, ev_off);
    put(o_own, own);
    put(o_clu, clu);
    put(o_big, big);
    std::vector<int64_t> goff(big.size());
    int64_t gneed = 0;
    for (size_t b = 0; b < big.size(); ++b) {
        goff[b] = gneed;
        gneed += (int64_t)dims[big[b]] * dims[big[b]];
    }
    put(o_goff, goff);
    put(o_bis, bis);
    put(o_bmode, bmode);
    NSS_CUDA_TRY(c, cudaMemcpyAsync(r.tab, r.htab, o_kept, cudaMemcpyHostToDevice, st));
    const RhoItem *d_items = (const RhoItem *)(r.tab + o_items);
    const int64_t *d_rho_off = (const int64_t *)(r.tab + o_rho_off);
    const int *d_dims = (const int *)(r.tab + o_dims), *d_ev_off = (const int *)(r.tab + o_ev_off),
              *d_own = (const int *)(r.tab + o_own), *d_bmode = (const int *)(r.tab + o_bmode),
              *d_clu = (const int *)(r.tab + o_clu), *d_big = (const int *)(r.tab + o_big);
    const int64_t *d_goff = (const int64_t *)(r.tab + o_goff);
    const int2 *d_bis = (const int2 *)(r.tab + o_bis);
    int *d_kept = (int *)(r.tab + o_kept);
    std::vector<void *> temps;
    auto cleanup = [&]() {
        cudaStreamSynchronize(st);
        for (void *p : temps) ctx_free(c, p);
    };
    if (!r.ph[0])
        for (int i = 0; i < DevRdm::NPH; ++i) NSS_CUDA_TRY(c, cudaEventCreate(&r.ph[i]));
    NSS_CUDA_TRY(c, cudaEventRecord(r.ph[0], st));
    ++c.launches;
    k_rho<<<(int)items.size(), 256, 0, st>>>(d_psi, d_items, s.d_dls, s.d_drs, s.d_off, d_rho_off, nsb, r.rho);
    NSS_CUDA_TRY(c, cudaMemsetAsync(r.iscal, 0, 8 * sizeof(int), st));
    ++c.launches;
    k_symcheck<<<std::min(nblk, 304), 256, 0, st>>>(r.rho, acc, d_rho_off, d_dims, nblk, r.iscal + 7);
    NSS_CUDA_TRY(c, cudaEventRecord(r.ph[1], st));
    cusolverDnHandle_t h = (cusolverDnHandle_t)c.solver;
    auto make_side_streams = [&]() -> int {
        if (!r.ev_fork) {
            NSS_CUDA_TRY(c, cudaEventCreateWithFlags(&r.ev_fork, cudaEventDisableTiming));
            for (int i = 0; i < DevRdm::NSIDE; ++i) {
                NSS_CUDA_TRY(c, cudaStreamCreateWithFlags(&r.side[i], cudaStreamNonBlocking));
                NSS_CUDA_TRY(c, cudaEventCreateWithFlags(&r.ev_join[i], cudaEventDisableTiming));
            }
        }
        return NSS_OK;
    };
    if (!path.empty()) NSS_CUDA_TRY(c, cudaMemsetAsync(flags, 0, nblk * sizeof(int), st));
    if (!big.empty())
        if ((rc = ensure_n(c, &r.big, r.cap_big, gneed))) { cleanup(); return rc; }
    if (!path.empty()) {
        int e = 0;
        if (!own.empty()) {
            ++c.launches;
            e = syev_trd(r.rho, d_rho_off, d_dims, d_ev_off, d_own, (int)own.size(), maxn_own, refl, td, te, tau,
                         perm, st);
        }
        if (!e && !clu.empty()) {
            ++c.launches;
            e = syev_trd_cl(r.rho, d_rho_off, d_dims, d_ev_off, d_clu, (int)clu.size(), maxn_clu, refl, td, te, tau,
                            perm, nullptr, nullptr, st);
        }
        if (!e && nbig_cl > 0) {
            int maxn_big = 1;
            for (int b = 0; b < nbig_cl; ++b) maxn_big = std::max(maxn_big, dims[big[b]]);
            ++c.launches;
            e = syev_trd_cl(r.rho, d_rho_off, d_dims, d_ev_off, d_big, nbig_cl, maxn_big, refl, td, te, tau,
                            perm, r.big, d_goff, st);
        }
        if (!e && (int)big.size() > nbig_cl) {
            std::vector<int> gb(big.begin() + nbig_cl, big.end()), gn;
            std::vector<int64_t> gofs(goff.begin() + nbig_cl, goff.end());
            int maxn_g = 1, nsm = 0, dev = 0;
            for (int q : gb) {
                gn.push_back(dims[q]);
                maxn_g = std::max(maxn_g, dims[q]);
            }
            cudaGetDevice(&dev);
            cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
            const int64_t ncomm = syev_trd_grid_comm(gn, nsm);
            if ((rc = ensure_n(c, &r.tg, r.cap_tg, ncomm + 8))) { cleanup(); return rc; }
            unsigned *bar = (unsigned *)(r.tg + ncomm);          // 8 counters
            int *gerr = (int *)(r.tg + ncomm + 4);
            c.launches += (int64_t)(gb.size() + 7) / 8;
            e = syev_trd_grid(r.rho, d_rho_off, d_dims, d_ev_off, gb, gn, refl, td, te, tau, perm, r.big, gofs,
                              r.tg, bar, gerr, st);
            if (!e) {
                int herr = 0;
                e = (int)cudaMemcpyAsync(&herr, gerr, sizeof(int), cudaMemcpyDeviceToHost, st);
                if (!e) e = (int)cudaStreamSynchronize(st);
                if (!e && herr) {
                    cleanup();
                    c.err = "nss_rdm: a grid barrier of the whole-GPU tridiagonalisation timed out";
                    return NSS_ERR_CUDA;
                }
            }
        }
        if (!e) e = (int)cudaEventRecord(r.ph[2], st);
        ++c.launches;
        if (!e) e = syev_bisect(d_dims, d_ev_off, d_bis, (int)bis.size(), td, te, r.evals, ldd, ldl, bscale, bsig,
                                flags, sub, maxn_path, st);
        if (e) {
            cleanup();
            c.err = std::string("nss_rdm: eigensolver launch failed: ") + cudaGetErrorString((cudaError_t)e);
            return NSS_ERR_CUDA;
        }
    }
    // Library eigensolves of a list of blocks, vectors into r.vec (and the
    // eigenvalues when write_evals): blocks up to the Jacobi size in one
    // k_jacobi launch on the main stream, the others one batched library
    // eigensolve per padded size class N = 32*ceil(d/32) (each block embedded
    // in an N x N matrix whose extra diagonal lies below its spectrum), the
    // classes on side streams.
    auto lib_eigh = [&](const std::vector<int> &sm, const std::vector<int> &lg, bool write_evals,
                        double *vec_out, int whole_min) -> int {
        if (sm.empty() && lg.empty()) return NSS_OK;
        if ((rc = make_side_streams())) return rc;
        if (!r.params) {
            cusolverDnParams_t prm = nullptr;
            if (cusolverDnCreateParams(&prm) != CUSOLVER_STATUS_SUCCESS) {
                c.err = "nss_rdm: cusolverDnCreateParams failed";
                return NSS_ERR_CUDA;
            }
            r.params = prm;
        }
        std::map<int, std::vector<int>, std::greater<int>> classes;
        for (int q : lg) classes[32 * ((dims[q] + 31) / 32)].push_back(q);
        struct Cls {
            int N, batch;
            int64_t a_off, w_off, ws_off, list_off;
            size_t ws;
            std::vector<char> hws;
        };
        std::vector<Cls> cls;
        std::vector<int> lists(sm);
        int64_t pool = 0;
        for (auto &kv : classes) {
            Cls cl;
            cl.N = kv.first;
            cl.batch = (int)kv.second.size();
            cl.list_off = (int64_t)lists.size();
            lists.insert(lists.end(), kv.second.begin(), kv.second.end());
            size_t wd = 0, wh = 0;
            if (cl.N >= whole_min) {
                // one matrix at a time through the blocked whole-GPU solver
                int lw = 0;
                if (cusolverDnDsyevd_bufferSize(h, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, cl.N, r.rho,
                                                cl.N, r.evals, &lw) != CUSOLVER_STATUS_SUCCESS) {
                    c.err = "nss_rdm: cusolverDnDsyevd_bufferSize failed";
                    return NSS_ERR_CUDA;
                }
                wd = (size_t)lw * sizeof(double);
            } else if (cusolverDnXsyevBatched_bufferSize(h, (cusolverDnParams_t)r.params, CUSOLVER_EIG_MODE_VECTOR,
                                                         CUBLAS_FILL_MODE_LOWER, cl.N, CUDA_R_64F, r.rho, cl.N,
                                                         CUDA_R_64F, r.evals, CUDA_R_64F, &wd, &wh, cl.batch) !=
                       CUSOLVER_STATUS_SUCCESS) {
                c.err = "nss_rdm: cusolverDnXsyevBatched_bufferSize failed";
                return NSS_ERR_CUDA;
            }
            cl.ws = wd;
            cl.hws.resize(wh + 16);
            cl.a_off = pool;
            pool += (int64_t)cl.batch * cl.N * cl.N;
            cl.w_off = pool;
            pool += (int64_t)cl.batch * cl.N;
            cl.ws_off = pool;
            pool += (int64_t)(wd + 7) / 8 + 32;
            cls.push_back(std::move(cl));
        }
        if ((rc = ensure_n(c, &r.bat, r.cap_bat, std::max<int64_t>(pool, 1)))) return rc;
        if ((rc = ensure_n(c, &r.bat_info, r.cap_bat_info, (int64_t)lg.size() + 1))) return rc;
        int *d_list = nullptr;
        NSS_CUDA_TRY(c, ctx_alloc(c, &d_list, lists.size()));
        temps.push_back(d_list);
        NSS_CUDA_TRY(c, cudaMemcpyAsync(d_list, lists.data(), lists.size() * sizeof(int), cudaMemcpyHostToDevice, st));
        NSS_CUDA_TRY(c, cudaEventRecord(r.ev_fork, st));
        for (int i = 0; i < DevRdm::NSIDE; ++i) NSS_CUDA_TRY(c, cudaStreamWaitEvent(r.side[i], r.ev_fork, 0));
        double *ev_out = write_evals ? r.evals : nullptr;
        int info_off = 0;
        for (size_t ci = 0; ci < cls.size(); ++ci) {
            Cls &cl = cls[ci];
            cudaStream_t ss = r.side[ci % DevRdm::NSIDE];
            double *A = r.bat + cl.a_off, *W = r.bat + cl.w_off, *ws = r.bat + cl.ws_off;
            c.launches += 2;
            k_pack<<<cl.batch, 256, 0, ss>>>(r.rho, d_rho_off, d_dims, d_list + cl.list_off, cl.N, A);
            cusolverDnSetStream(h, ss);
            cusolverStatus_t cs = CUSOLVER_STATUS_SUCCESS;
            if (cl.N >= whole_min) {
                for (int b = 0; b < cl.batch && cs == CUSOLVER_STATUS_SUCCESS; ++b)
                    cs = cusolverDnDsyevd(h, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, cl.N,
                                          A + (int64_t)b * cl.N * cl.N, cl.N, W + (int64_t)b * cl.N, ws,
                                          (int)(cl.ws / sizeof(double)), r.bat_info + info_off + b);
            } else {
                cs = cusolverDnXsyevBatched(h, (cusolverDnParams_t)r.params, CUSOLVER_EIG_MODE_VECTOR,
                                            CUBLAS_FILL_MODE_LOWER, cl.N, CUDA_R_64F, A, cl.N, CUDA_R_64F, W,
                                            CUDA_R_64F, ws, cl.ws, cl.hws.data(), cl.hws.size() - 16,
                                            r.bat_info + info_off, cl.batch);
            }
            cusolverDnSetStream(h, st);
            if (cs != CUSOLVER_STATUS_SUCCESS) {
                c.err = "nss_rdm: cusolverDnXsyevBatched failed";
                return NSS_ERR_CUDA;
            }
            k_unpack<<<cl.batch, 256, 0, ss>>>(A, W, cl.N, d_list + cl.list_off, d_dims, d_rho_off, d_ev_off,
                                               vec_out, ev_out);
            NSS_CUDA_TRY(c, cudaGetLastError());
            info_off += cl.batch;
        }
        if (!sm.empty()) {
            constexpr int jac_smem = 2 * JAC_MAX * (JAC_MAX + 1) * (int)sizeof(double);
            NSS_CUDA_TRY(c, cudaFuncSetAttribute(k_jacobi, cudaFuncAttributeMaxDynamicSharedMemorySize, jac_smem));
            ++c.launches;
            k_jacobi<<<(int)sm.size(), 256, jac_smem, st>>>(r.rho, d_rho_off, d_dims, d_ev_off, d_list, vec_out,
                                                            ev_out);
            NSS_CUDA_TRY(c, cudaGetLastError());
        }
        for (int i = 0; i < DevRdm::NSIDE; ++i) {
            NSS_CUDA_TRY(c, cudaEventRecord(r.ev_join[i], r.side[i]));
            NSS_CUDA_TRY(c, cudaStreamWaitEvent(st, r.ev_join[i], 0));
        }
        return NSS_OK;
    };
    if (path.empty()) NSS_CUDA_TRY(c, cudaEventRecord(r.ph[2], st));
    if ((rc = lib_eigh(small, large, true, r.vec, LIB_WHOLE_GPU_N))) {
        cleanup();
        return rc;
    }
    NSS_CUDA_TRY(c, cudaEventRecord(r.ph[3], st));
    c.rdm_own_blocks = (int)path.size();
    c.rdm_path_blocks[0] = (int)own.size();
    c.rdm_path_blocks[1] = (int)clu.size();
    c.rdm_path_blocks[2] = (int)big.size();
    c.rdm_path_blocks[3] = (int)(small.size() + large.size());
    c.rdm_max_block = 0;
    for (int d : dims) c.rdm_max_block = std::max(c.rdm_max_block, d);
    c.rdm_lib_blocks = (int)(small.size() + large.size());
    c.rdm_fallback_blocks = 0;
    c.rdm_refined_blocks = 0;
    ++c.launches;
    k_clamp<<<8, 256, 0, st>>>(r.evals, eacc);
    ++c.launches;
    k_qn_entropy<<<2, 256, 0, st>>>(r.evals, d_ev_off, nsb, r.scal + 4);
    // per side: rank, truncation, U
    const int nside[2] = {nl, nr};
    for (int side = 0; side < 2; ++side) {
        const int n = nside[side], base = side == 0 ? 0 : nl;
        ++c.launches;
        k_rank<<<(n + 255) / 256, 256, 0, st>>>(r.evals + base, n, r.sorted + base, r.order + base,
                                                path.empty() ? nullptr : rnk + base);
        ++c.launches;
        k_truncate<<<1, 1024, 0, st>>>(r.sorted + base, n, mstates, estates, mblk[side], deg_thr, r.scal + 2 * side,
                                     r.iscal + side);
    }
    NSS_CUDA_TRY(c, cudaGetLastError());
    NSS_CUDA_TRY(c, cudaEventRecord(r.ph[4], st));
    double hs[8];
    int hi[8];
    NSS_CUDA_TRY(c, cudaMemcpyAsync(hs, r.scal, 8 * sizeof(double), cudaMemcpyDeviceToHost, st));
    NSS_CUDA_TRY(c, cudaMemcpyAsync(hi, r.iscal, 8 * sizeof(int), cudaMemcpyDeviceToHost, st));
    NSS_CUDA_TRY(c, cudaStreamSynchronize(st));
    if (hi[7]) {
        cleanup();
        c.err = "build_density_matrix error: rho not Symmetric";
        return NSS_ERR_ASYMMETRIC;
    }
    double *lam_out[2] = {lam_l, lam_r};
    int32_t *kept_out[2] = {kept_l, kept_r};
    double *u_out[2] = {u_l, u_r};
    for (int side = 0; side < 2; ++side) {
        const int n = nside[side], base = side == 0 ? 0 : nl;
        out[side].nevals = n;
        out[side].m_s = hi[side];
        out[side].trunc_err = hs[2 * side];
        out[side].entropy = hs[2 * side + 1];
        out[side].s_number = hs[4 + 2 * side];
        out[side].s_config = hs[4 + 2 * side + 1];
        if (lam_out[side]) {
            // lambda clipped at 0 (DMRG_RDM.f90:88,97): tiny stays as is, as the
            // reference clips only negative values after the tiny substitution
            NSS_CUDA_TRY(c, cudaMemcpyAsync(lam_out[side], r.sorted + base, n * sizeof(double),
                                            cudaMemcpyDeviceToHost, st));
        }
    }
    // kept eigenvectors of the own path's blocks; marked blocks again
    // through the library
    if (!path.empty() && (u_l || u_r || kl)) {
        const int msv[2] = {((vec_sides & 1) && (u_l || kl)) ? hi[0] : 0,
                            ((vec_sides & 2) && (u_r || kl)) ? hi[1] : 0};
        c.launches += 3;
        const int e = syev_vec(r.order, rnk, msv, nl, nsb, d_ev_off, d_dims, d_rho_off, d_bmode, sub, r.evals, ldd,
                               ldl, bscale, bsig, tau, refl, perm, flags, r.vec, maxn_path, st);
        if (e) {
            cleanup();
            c.err = std::string("nss_rdm: eigenvector launch failed: ") + cudaGetErrorString((cudaError_t)e);
            return NSS_ERR_CUDA;
        }
        std::vector<int> hflags(nblk);
        NSS_CUDA_TRY(c, cudaMemcpyAsync(hflags.data(), flags, nblk * sizeof(int), cudaMemcpyDeviceToHost, st));
        NSS_CUDA_TRY(c, cudaStreamSynchronize(st));
        // flagged blocks: first inverse iteration with Gram-Schmidt in near
        // clusters (k_vec_fb), then the library for what that cannot do
        std::vector<int> fb_own;
        // env NSS_RDM_REDO_ALL=1 sends every own-path block through k_vec_fb
        // (to check that path against the others)
        const char *redo = std::getenv("NSS_RDM_REDO_ALL");
        if (redo && std::string(redo) == "1")
            for (int q : path) hflags[q] |= 2;
        for (int q : path)
            if (hflags[q] & 2) {
                fb_own.push_back(q);
                for (int b = 0; b < 5; ++b)
                    if (hflags[q] & (4 << b)) ++c.rdm_fail_why[b];
                hflags[q] &= 1;                      // keep only "no positive definite L D L^T"
            }
        c.rdm_refined_blocks = (int)fb_own.size();
        if (!fb_own.empty()) {
            int *d_fo = nullptr;
            NSS_CUDA_TRY(c, ctx_alloc(c, &d_fo, fb_own.size()));
            temps.push_back(d_fo);
            NSS_CUDA_TRY(c, cudaMemcpyAsync(d_fo, fb_own.data(), fb_own.size() * sizeof(int), cudaMemcpyHostToDevice, st));
            NSS_CUDA_TRY(c, cudaMemcpyAsync(flags, hflags.data(), nblk * sizeof(int), cudaMemcpyHostToDevice, st));
            ++c.launches;
            const int e2 = syev_vec_fallback(r.order, rnk, msv, nl, nsb, d_ev_off, d_dims, d_rho_off, sub, r.evals, ldd,
                                             ldl, bscale, bsig, tau, refl, perm, flags, r.vec, d_fo,
                                             (int)fb_own.size(), maxn_path, st);
            if (e2) {
                cleanup();
                c.err = std::string("nss_rdm: eigenvector launch failed: ") + cudaGetErrorString((cudaError_t)e2);
                return NSS_ERR_CUDA;
            }
            NSS_CUDA_TRY(c, cudaMemcpyAsync(hflags.data(), flags, nblk * sizeof(int), cudaMemcpyDeviceToHost, st));
            NSS_CUDA_TRY(c, cudaStreamSynchronize(st));
        }
        // still flagged: blocks of up to QL_HOST_MAX states get all
        // eigenvectors of their tridiagonal matrix from implicit QL on the
        // host, written into their vec slot and back-transformed on the
        // device (cuSOLVER measured 0.9 s for a lone 305-state block); larger
        // ones go to the library
        std::vector<int> fs, fl, fq;
        // env NSS_RDM_QL_ALL=1 sends every flagged block to host QL (to check
        // that path; with NSS_RDM_REDO_ALL=1, every block)
        const char *qla = std::getenv("NSS_RDM_QL_ALL");
        const bool ql_all = qla && std::string(qla) == "1";
        for (int q : fb_own)
            if ((hflags[q] & 2) || ql_all) (dims[q] <= QL_HOST_MAX ? fq : (dims[q] <= jmax ? fs : fl)).push_back(q);
        if (!fq.empty()) {
            std::vector<int2> cols;
            int qmax = 1;
            for (int q : fq) {
                const int nq = dims[q];
                qmax = std::max(qmax, nq);
                std::vector<double> d(nq), e(nq), Z((size_t)nq * nq, 0.0);
                std::vector<int> sr(nq);
                NSS_CUDA_TRY(c, cudaMemcpyAsync(d.data(), td + ev_off[q], nq * sizeof(double), cudaMemcpyDeviceToHost, st));
                NSS_CUDA_TRY(c, cudaMemcpyAsync(e.data(), te + ev_off[q], nq * sizeof(double), cudaMemcpyDeviceToHost, st));
                NSS_CUDA_TRY(c, cudaMemcpyAsync(sr.data(), sub + ev_off[q], nq * sizeof(int), cudaMemcpyDeviceToHost, st));
                NSS_CUDA_TRY(c, cudaStreamSynchronize(st));
                // the own path's columns: the eigenvalues of each unreduced
                // block [r0, r1) of T ascending in columns r0 .. r1-1, so QL
                // runs on each of those blocks
                bool ql_ok = true;
                for (int r0 = 0; r0 < nq && ql_ok;) {
                    const int r1 = sr[r0] >> 16, nb = r1 - r0;
                    if ((sr[r0] & 0xffff) != r0 || r1 <= r0 || r1 > nq) { ql_ok = false; break; }
                    std::vector<double> db(d.begin() + r0, d.begin() + r1), eb(nb, 0.0), Zb((size_t)nb * nb);
                    for (int i = 0; i + 1 < nb; ++i) eb[i] = e[r0 + i];
                    if (!tridiag_ql(nb, db.data(), eb.data(), Zb.data())) { ql_ok = false; break; }
                    for (int j = 0; j < nb; ++j)
                        std::copy(Zb.begin() + (size_t)j * nb, Zb.begin() + (size_t)(j + 1) * nb,
                                  Z.begin() + (size_t)(r0 + j) * nq + r0);
                    r0 = r1;
                }
                if (!ql_ok) {
                    (nq <= jmax ? fs : fl).push_back(q);
                    continue;
                }
                NSS_CUDA_TRY(c, cudaMemcpy(r.vec + rho_off[q], Z.data(), Z.size() * sizeof(double),
                                           cudaMemcpyHostToDevice));
                for (int col = 0; col < nq; ++col) cols.push_back(make_int2(q, col));
            }
            c.rdm_ql_blocks += (int)(fq.size());
            if (!cols.empty()) {
                int2 *d_cols = nullptr;
                NSS_CUDA_TRY(c, ctx_alloc(c, &d_cols, cols.size()));
                temps.push_back(d_cols);
                NSS_CUDA_TRY(c, cudaMemcpyAsync(d_cols, cols.data(), cols.size() * sizeof(int2), cudaMemcpyHostToDevice,
                                                st));
                ++c.launches;
                const int e3 = syev_backtr(d_dims, d_ev_off, d_rho_off, tau, refl, perm, r.vec, d_cols, (int)cols.size(),
                                           qmax, st);
                if (e3) {
                    cleanup();
                    c.err = std::string("nss_rdm: back-transformation launch failed: ") +
                            cudaGetErrorString((cudaError_t)e3);
                    return NSS_ERR_CUDA;
                }
            }
        }
        c.rdm_fallback_blocks = (int)(fs.size() + fl.size());
        if (c.rdm_fallback_blocks) {
            // library vectors into the blocks' rho slots (consumed by then),
            // then matched to the own path's eigenvalue order in r.vec
            // a handful of blocks: the whole-GPU solver from 128 states on
            // (the batched one measured 3.1 s for a lone 356-state block)
            if ((rc = lib_eigh(fs, fl, false, r.rho, LIB_FALLBACK_WHOLE_N))) {
                cleanup();
                return rc;
            }
            std::vector<int> fb(fs);
            fb.insert(fb.end(), fl.begin(), fl.end());
            int *d_fb = nullptr;
            NSS_CUDA_TRY(c, ctx_alloc(c, &d_fb, fb.size()));
            temps.push_back(d_fb);
            NSS_CUDA_TRY(c, cudaMemcpyAsync(d_fb, fb.data(), fb.size() * sizeof(int), cudaMemcpyHostToDevice, st));
            ++c.launches;
            int fbmax = 1;
            for (int q : fb) fbmax = std::max(fbmax, dims[q]);
            k_fbperm<<<(int)fb.size(), 256, fbmax * sizeof(int), st>>>(d_fb, d_dims, d_ev_off, d_rho_off, r.evals,
                                                                        r.rho, r.vec);
            NSS_CUDA_TRY(c, cudaGetLastError());
        }
    }
    NSS_CUDA_TRY(c, cudaEventRecord(r.ph[5], st));
    // kept columns, compact (no zero rows) -> pinned staging -> the dense
    // m_block x m_s host matrices (zero rows outside each column's block)
    NSS_CUDA_TRY(c, cudaGetLastError());
    int64_t hneed = 0;
    for (int side = 0; side < 2; ++side) hneed += (int64_t)hi[side] * (maxd + 2);
    if (!r.hu || r.cap_hu < hneed) {
        if (r.hu) NSS_CUDA_TRY(c, cudaFreeHost(r.hu));
        r.hu = nullptr;
        NSS_CUDA_TRY(c, cudaHostAlloc((void **)&r.hu, (size_t)std::max<int64_t>(hneed, 1) * sizeof(double),
                                      cudaHostAllocDefault));
        r.cap_hu = hneed;
    }
    double *hval[2];
    int *hkept[2], *hoff[2];
    {
        double *hp = r.hu;
        for (int side = 0; side < 2; ++side) {
            hval[side] = hp;
            hp += (int64_t)hi[side] * maxd;
        }
        int *ip = (int *)hp;
        for (int side = 0; side < 2; ++side) {
            hkept[side] = ip;
            hoff[side] = ip + hi[side];
            ip += 2 * (int64_t)hi[side];
        }
    }
    bool any = false;
    for (int side = 0; side < 2; ++side) {
        const int base = side == 0 ? 0 : nl;
        const int ms = hi[side];
        if (!(u_out[side] || kept_out[side] || kl) || !(vec_sides & (1 << side))) continue;
        any = true;
        int *dk = d_kept + side * 2 * kmax, *doff = dk + kmax;
        double *du = r.u + (int64_t)side * kmax * maxd;
        ++c.launches;
        k_ucompact<<<1, 1024, 0, st>>>(r.vec, d_rho_off + side * nsb, d_dims + side * nsb, d_ev_off + side * nsb,
                                       base, nsb, r.order + base, ms, dk, doff, du);
        NSS_CUDA_TRY(c, cudaGetLastError());
        NSS_CUDA_TRY(c, cudaMemcpyAsync(hkept[side], dk, ms * sizeof(int), cudaMemcpyDeviceToHost, st));
        NSS_CUDA_TRY(c, cudaMemcpyAsync(hoff[side], doff, ms * sizeof(int), cudaMemcpyDeviceToHost, st));
        if (u_out[side])
            NSS_CUDA_TRY(c, cudaMemcpyAsync(hval[side], du, (size_t)ms * maxd * sizeof(double),
                                            cudaMemcpyDeviceToHost, st));
    }
    if (any) NSS_CUDA_TRY(c, cudaStreamSynchronize(st));
    if (kl)
        for (int side = 0; side < 2; ++side) {
            KeptLayout &L = kl[side];
            if (!(vec_sides & (1 << side))) {   // no kept vectors computed for this side
                L = KeptLayout{};
                continue;
            }
            const int ms = hi[side], o = side * nsb;
            L.ms = ms;
            L.q.assign(hkept[side], hkept[side] + ms);
            L.off.assign(hoff[side], hoff[side] + ms);
            L.dims.assign(dims.begin() + o, dims.begin() + o + nsb);
            L.map_off.assign(nsb, 0);
            L.maps.clear();
            for (int k = 0; k < nsb; ++k) {
                L.map_off[k] = (int)L.maps.size();
                L.maps.insert(L.maps.end(), maps.begin() + map_off[o + k], maps.begin() + map_off[o + k] + dims[o + k]);
            }
            L.dcomp = r.u + (int64_t)side * kmax * maxd;
        }
    for (int side = 0; side < 2; ++side) {
        const int ms = hi[side];
        if (!(vec_sides & (1 << side))) continue;
        if (kept_out[side])
            for (int j = 0; j < ms; ++j) kept_out[side][j] = hkept[side][j];
        if (!u_out[side]) continue;
        double *U = u_out[side];
        std::memset(U, 0, (size_t)mblk[side] * ms * sizeof(double));
        for (int j = 0; j < ms; ++j) {
            const int q = side * nsb + hkept[side][j], nq = dims[q];
            const int *mp = maps.data() + map_off[q];
            const double *src = hval[side] + hoff[side][j];
            double *dst = U + (int64_t)j * mblk[side];
            for (int p = 0; p < nq; ++p) dst[mp[p]] = src[p];
        }
    }
    NSS_CUDA_TRY(c, cudaEventRecord(r.ph[6], st));
    cleanup();
    for (int i = 0; i + 1 < DevRdm::NPH; ++i) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, r.ph[i], r.ph[i + 1]);
        c.rdm_phase_ms[i] = ms;
    }
    return NSS_OK;
}

}  // namespace nss
