// Tile bodies of the sector product H_sb psi shared by the stand-alone
// kernels (k_matvec.cu) and the persistent Lanczos kernel (k_lanczos.cu).
//
// One output tile is rows [row0, row0+TR) x columns [col0, col0+TC) of
// sector k, W_k[il][ir] (ir fastest).  The dense part is
//     H_L(k) W_k + W_k H_R(k)^T           (src/DMRG_SUPERBLOCK_SETUP.f90:767-796)
// and the A x B terms of the sector add A W_q B^T (:808-857), regrouped by
// the sector they write.  A tile is computed by a group of 256 threads that
// synchronise through a `Sync` functor: the whole CTA (__syncthreads) in the
// stand-alone kernels, a named barrier of 256 threads when two tiles share a
// CTA of the persistent kernel.
#pragma once

#include "device.cuh"

namespace nss {

struct CtaSync {
    __device__ __forceinline__ void operator()() const { __syncthreads(); }
};

// bar.sync id, 256: one of the two 256-thread groups of a 512-thread CTA
struct GroupSync {
    int id;
    __device__ __forceinline__ void operator()() const {
        asm volatile("bar.sync %0, 256;" ::"r"(id) : "memory");
    }
};

// A x B terms of one output tile, staged.  The block operators of the two
// sites at the centre bond have at most one stored element per row (the
// enlarged blocks are block (x) site), so for each term of the output sector
// the tile's rows of A and columns of B are staged in shared memory as
// (column, value) pairs, and each output then needs only independent
// gathers W_q[aj][bj], in flight together.  A row with more than one element
// sends that batch of terms to the general CSR loop.
constexpr int AB_MAXT = 16;

template <class V, int TR, int TC>
struct AbStage {
    int ac[AB_MAXT][TR], bc[AB_MAXT][TC];
    V av[AB_MAXT][TR], bv[AB_MAXT][TC];
    const V *wq[AB_MAXT];
    int drq[AB_MAXT];
    int multi;
};

// stage terms [tb, tb+nt) for rows row0.. and columns col0..; `lt` is the
// thread's index in its group of `nthr`; ends with a group barrier
template <class V, int TR, int TC, class Sync>
__device__ __forceinline__ void ab_stage(AbStage<V, TR, TC> &S, const V *__restrict__ v, int tb, int nt, int row0,
                                         int col0, int dl, int dr, const int *__restrict__ drs,
                                         const int64_t *__restrict__ off, const DevTerm *__restrict__ terms,
                                         const int *__restrict__ ab_rp, const int *__restrict__ ab_col,
                                         const V *__restrict__ ab_val, int lt, int nthr, Sync sync) {
    if (lt == 0) S.multi = 0;
    sync();
    for (int e = lt; e < nt * (TR + TC); e += nthr) {
        const int tt = e / (TR + TC), r = e % (TR + TC);
        const DevTerm tm = terms[tb + tt];
        int c = -1;
        V x = (V)0;
        if (r < TR) {
            const int il = row0 + r;
            if (il < dl) {
                const int p0 = ab_rp[tm.a_rp + il], p1 = ab_rp[tm.a_rp + il + 1];
                if (p1 > p0) { c = ab_col[p0]; x = ab_val[p0]; }
                if (p1 - p0 > 1) S.multi = 1;
            }
            S.ac[tt][r] = c;
            S.av[tt][r] = x;
        } else {
            const int ir = col0 + (r - TR);
            if (ir < dr) {
                const int p0 = ab_rp[tm.b_rp + ir], p1 = ab_rp[tm.b_rp + ir + 1];
                if (p1 > p0) { c = ab_col[p0]; x = ab_val[p0]; }
                if (p1 - p0 > 1) S.multi = 1;
            }
            S.bc[tt][r - TR] = c;
            S.bv[tt][r - TR] = x;
            if (r == TR) {
                S.wq[tt] = v + off[tm.in_sec];
                S.drq[tt] = drs[tm.in_sec];
            }
        }
    }
    sync();
}

// general loop for output (il, ir) over terms [tb, tb+nt): the reference's
// sum over the stored elements of A and B
template <class V>
__device__ __forceinline__ V ab_csr(V acc, const V *__restrict__ v, int tb, int nt, int il, int ir,
                                    const int *__restrict__ drs, const int64_t *__restrict__ off,
                                    const DevTerm *__restrict__ terms, const int *__restrict__ ab_rp,
                                    const int *__restrict__ ab_col, const V *__restrict__ ab_val) {
    for (int ti = tb; ti < tb + nt; ++ti) {
        const DevTerm tm = terms[ti];
        const V *Wq = v + off[tm.in_sec];
        const int drq = drs[tm.in_sec];
        const int *arp = ab_rp + tm.a_rp, *brp = ab_rp + tm.b_rp;
        for (int ja = arp[il]; ja < arp[il + 1]; ++ja) {
            const int aj = ab_col[ja];
            V cb = (V)0;
            for (int jb = brp[ir]; jb < brp[ir + 1]; ++jb) cb = fma(ab_val[jb], Wq[(int64_t)aj * drq + ab_col[jb]], cb);
            acc = fma(ab_val[ja], cb, acc);
        }
    }
    return acc;
}

// Shared memory of one FP32 tile group.
struct Tile32Smem {
    float sa[32][33];
    float sb[32][33];
    AbStage<float, 32, 32> S;
};

// Operands of the FP32 sector product (device pointers of DevSb).
struct Hv32Ops {
    const int *dls, *drs;
    const int64_t *off;
    const float *hl;
    const int64_t *hl_off;
    const float *hr;
    const int64_t *hr_off;
    const int *term_ptr;
    const DevTerm *terms;
    const int *ab_rp, *ab_col;
    const float *ab_val;
};

// One 32x32 FP32 output tile t = (sector, row0, col0, flags) by 256 threads
// (lt = thread index in the group), each owning rows {ty, ty+16} x columns
// {tx, tx+16}.  A "terms only" tile (t.w & 1) skips the two dense products.
// The outputs, multiplied by `scale`, go to hv; returns this thread's share
// of sum_i v[i] * out[i] * scale^2 over its outputs (the Lanczos alpha of a
// unit vector v * scale), meaningful for whole tiles (t.w == 0).
template <class Sync>
__device__ __forceinline__ float hv32_tile(int4 t, const float *__restrict__ v, float *__restrict__ hv,
                                           const Hv32Ops &op, Tile32Smem &sm, int lt, Sync sync, float scale) {
    const int k = t.x, row0 = t.y, col0 = t.z;
    const int dl = op.dls[k], dr = op.drs[k];
    const int64_t o = op.off[k];
    const float *W = v + o;
    const float *HL = op.hl + op.hl_off[k];
    const float *HR = op.hr + op.hr_off[k];
    const int ty = lt / 16, tx = lt % 16;
    float acc[2][2] = {{0.f, 0.f}, {0.f, 0.f}};
    const int kdl = (t.w & 1) ? 0 : dl, kdr = (t.w & 1) ? 0 : dr;
    // H_L W
    for (int j0 = 0; j0 < kdl; j0 += 32) {
        for (int e = lt; e < 32 * 32; e += 256) {
            const int r = e / 32, cc = e % 32;
            const int gi = row0 + r, gj = j0 + cc;
            sm.sa[r][cc] = (gi < dl && gj < dl) ? HL[(int64_t)gi * dl + gj] : 0.f;
            const int gj2 = j0 + r, gc = col0 + cc;
            sm.sb[r][cc] = (gj2 < dl && gc < dr) ? W[(int64_t)gj2 * dr + gc] : 0.f;
        }
        sync();
#pragma unroll 8
        for (int j = 0; j < 32; ++j) {
            const float a0 = sm.sa[ty][j], a1 = sm.sa[ty + 16][j], b0 = sm.sb[j][tx], b1 = sm.sb[j][tx + 16];
            acc[0][0] = fmaf(a0, b0, acc[0][0]);
            acc[0][1] = fmaf(a0, b1, acc[0][1]);
            acc[1][0] = fmaf(a1, b0, acc[1][0]);
            acc[1][1] = fmaf(a1, b1, acc[1][1]);
        }
        sync();
    }
    // W H_R^T
    for (int j0 = 0; j0 < kdr; j0 += 32) {
        for (int e = lt; e < 32 * 32; e += 256) {
            const int r = e / 32, cc = e % 32;
            const int gi = row0 + r, gj = j0 + cc;
            sm.sa[r][cc] = (gi < dl && gj < dr) ? W[(int64_t)gi * dr + gj] : 0.f;
            const int gr = col0 + r;                 // sb[j][x] = HR[col0+x][j0+j]
            sm.sb[cc][r] = (gr < dr && gj < dr) ? HR[(int64_t)gr * dr + gj] : 0.f;
        }
        sync();
#pragma unroll 8
        for (int j = 0; j < 32; ++j) {
            const float a0 = sm.sa[ty][j], a1 = sm.sa[ty + 16][j], b0 = sm.sb[j][tx], b1 = sm.sb[j][tx + 16];
            acc[0][0] = fmaf(a0, b0, acc[0][0]);
            acc[0][1] = fmaf(a0, b1, acc[0][1]);
            acc[1][0] = fmaf(a1, b0, acc[1][0]);
            acc[1][1] = fmaf(a1, b1, acc[1][1]);
        }
        sync();
    }
    // A x B terms, staged per batch of terms (see ab_stage)
    AbStage<float, 32, 32> &S = sm.S;
    for (int tb = op.term_ptr[k]; tb < op.term_ptr[k + 1]; tb += AB_MAXT) {
        const int nt = min(AB_MAXT, op.term_ptr[k + 1] - tb);
        ab_stage<float, 32, 32>(S, v, tb, nt, row0, col0, dl, dr, op.drs, op.off, op.terms, op.ab_rp, op.ab_col,
                                op.ab_val, lt, 256, sync);
        if (!S.multi) {
            for (int tt = 0; tt < nt; ++tt) {
                const float *Wq = S.wq[tt];
                const int drq = S.drq[tt];
#pragma unroll
                for (int rr = 0; rr < 2; ++rr)
#pragma unroll
                    for (int cc = 0; cc < 2; ++cc) {
                        const int aj = S.ac[tt][ty + 16 * rr], bj = S.bc[tt][tx + 16 * cc];
                        if (aj >= 0 && bj >= 0)
                            acc[rr][cc] = fmaf(S.av[tt][ty + 16 * rr] * S.bv[tt][tx + 16 * cc],
                                               Wq[(int64_t)aj * drq + bj], acc[rr][cc]);
                    }
            }
        } else {
            for (int rr = 0; rr < 2; ++rr)
                for (int cc = 0; cc < 2; ++cc) {
                    const int il = row0 + ty + 16 * rr, ir = col0 + tx + 16 * cc;
                    if (il < dl && ir < dr)
                        acc[rr][cc] = ab_csr<float>(acc[rr][cc], v, tb, nt, il, ir, op.drs, op.off, op.terms,
                                                    op.ab_rp, op.ab_col, op.ab_val);
                }
        }
        sync();
    }
    float part = 0.f;
    for (int rr = 0; rr < 2; ++rr)
        for (int cc = 0; cc < 2; ++cc) {
            const int il = row0 + ty + 16 * rr, ir = col0 + tx + 16 * cc;
            if (il < dl && ir < dr) {
                const int64_t idx = (int64_t)il * dr + ir;
                const float y = acc[rr][cc] * scale;
                hv[o + idx] = y;
                part = fmaf(W[idx] * scale, y, part);
            }
        }
    return part;
}

}  // namespace nss

namespace nss {

// Work items of the persistent kernel's H*psi phase.  An item is a 32x32
// output tile (x = sector, y = row0, z = col0) and a part (w):
//   HV_FULL   H_L W + W H_R^T + A x B terms       -> slot 0
//   HV_LEFT   H_L W                               -> slot 1
//   HV_RIGHT  W H_R^T + A x B terms               -> slot 0
// Sectors whose tiles have long K loops (Dl or Dr > 64) are split into a
// LEFT and a RIGHT item so the two halves run on different SMs; the result
// is slot 0 + slot 1 (regions of slot 1 that no item writes stay zero).
enum { HV_FULL = 0, HV_LEFT = 1, HV_RIGHT = 2 };
constexpr int HV_KMAX = 128;     // K extent staged at once

struct Item32Smem {
    float sa[32][HV_KMAX + 1];   // A rows x K
    float sb[HV_KMAX][33];       // K x B columns
    AbStage<float, 32, 32> S;
};

// One item by 256 threads (lt = thread index in the group): each thread owns
// rows {ty, ty+16} x columns {tx, tx+16}.  A whole K range (up to HV_KMAX) is
// staged at once, so a phase costs one load latency instead of one per 32 K.
// The outputs times `scale` go to slot[0] or slot[1]; returns this thread's
// share of sum_i (v[i] scale) (out[i] scale) over its outputs.
template <class Sync>
__device__ __forceinline__ float hv32_item(int4 t, const float *__restrict__ v, float *__restrict__ slot0,
                                           float *__restrict__ slot1, const Hv32Ops &op, Item32Smem &sm, int lt,
                                           Sync sync, float scale) {
    const int k = t.x, row0 = t.y, col0 = t.z, part = t.w;
    const int dl = op.dls[k], dr = op.drs[k];
    const int64_t o = op.off[k];
    const float *W = v + o;
    const int ty = lt / 16, tx = lt % 16;
    float acc[2][2] = {{0.f, 0.f}, {0.f, 0.f}};
    for (int ph = 0; ph < 2; ++ph) {
        if ((ph == 0 && part == HV_RIGHT) || (ph == 1 && part == HV_LEFT)) continue;
        const int K = ph == 0 ? dl : dr;
        const float *H = ph == 0 ? op.hl + op.hl_off[k] : op.hr + op.hr_off[k];
        for (int kb = 0; kb < K; kb += HV_KMAX) {
            const int kn = min(HV_KMAX, K - kb);
            for (int e = lt; e < 32 * kn; e += 256) {
                const int r = e / kn, c = e % kn;       // A[r][c], K index kb + c
                const int gi = row0 + r, gj = kb + c;
                float x = 0.f;
                if (gi < dl) x = ph == 0 ? H[(int64_t)gi * dl + gj] : W[(int64_t)gi * dr + gj];
                sm.sa[r][c] = x;
            }
            for (int e = lt; e < 32 * kn; e += 256) {
                float x = 0.f;
                if (ph == 0) {                           // B[c][xx] = W[kb+c][col0+xx]
                    const int c = e / 32, xx = e % 32, gc = col0 + xx;
                    if (gc < dr) x = W[(int64_t)(kb + c) * dr + gc];
                    sm.sb[c][xx] = x;
                } else {                                 // B[c][xx] = HR[col0+xx][kb+c]
                    const int xx = e / kn, c = e % kn, gr = col0 + xx;
                    if (gr < dr) x = H[(int64_t)gr * dr + kb + c];
                    sm.sb[c][xx] = x;
                }
            }
            sync();
#pragma unroll 8
            for (int j = 0; j < kn; ++j) {
                const float a0 = sm.sa[ty][j], a1 = sm.sa[ty + 16][j], b0 = sm.sb[j][tx], b1 = sm.sb[j][tx + 16];
                acc[0][0] = fmaf(a0, b0, acc[0][0]);
                acc[0][1] = fmaf(a0, b1, acc[0][1]);
                acc[1][0] = fmaf(a1, b0, acc[1][0]);
                acc[1][1] = fmaf(a1, b1, acc[1][1]);
            }
            sync();
        }
    }
    if (part != HV_LEFT) {
        AbStage<float, 32, 32> &S = sm.S;
        for (int tb = op.term_ptr[k]; tb < op.term_ptr[k + 1]; tb += AB_MAXT) {
            const int nt = min(AB_MAXT, op.term_ptr[k + 1] - tb);
            ab_stage<float, 32, 32>(S, v, tb, nt, row0, col0, dl, dr, op.drs, op.off, op.terms, op.ab_rp,
                                    op.ab_col, op.ab_val, lt, 256, sync);
            if (!S.multi) {
                for (int tt = 0; tt < nt; ++tt) {
                    const float *Wq = S.wq[tt];
                    const int drq = S.drq[tt];
#pragma unroll
                    for (int rr = 0; rr < 2; ++rr)
#pragma unroll
                        for (int cc = 0; cc < 2; ++cc) {
                            const int aj = S.ac[tt][ty + 16 * rr], bj = S.bc[tt][tx + 16 * cc];
                            if (aj >= 0 && bj >= 0)
                                acc[rr][cc] = fmaf(S.av[tt][ty + 16 * rr] * S.bv[tt][tx + 16 * cc],
                                                   Wq[(int64_t)aj * drq + bj], acc[rr][cc]);
                        }
                }
            } else {
                for (int rr = 0; rr < 2; ++rr)
                    for (int cc = 0; cc < 2; ++cc) {
                        const int il = row0 + ty + 16 * rr, ir = col0 + tx + 16 * cc;
                        if (il < dl && ir < dr)
                            acc[rr][cc] = ab_csr<float>(acc[rr][cc], v, tb, nt, il, ir, op.drs, op.off, op.terms,
                                                        op.ab_rp, op.ab_col, op.ab_val);
                    }
            }
            sync();
        }
    }
    float *out = (part == HV_LEFT ? slot1 : slot0) + o;
    float p = 0.f;
    for (int rr = 0; rr < 2; ++rr)
        for (int cc = 0; cc < 2; ++cc) {
            const int il = row0 + ty + 16 * rr, ir = col0 + tx + 16 * cc;
            if (il < dl && ir < dr) {
                const int64_t idx = (int64_t)il * dr + ir;
                const float y = acc[rr][cc] * scale;
                out[idx] = y;
                p = fmaf(W[idx] * scale, y, p);
            }
        }
    return p;
}

}  // namespace nss
