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
    // per work item of the persistent kernel: offset of its A x B table in
    // `ell` (-1: a row with several elements, use the CSR loop)
    const int *item_ell;
    const int2 *ell;             // (column, value bits) of A rows / B columns
    const int4 *term_hdr;        // per term: offset of its input sector (lo, hi), its Dr
    // output planes of the tensor-core sector GEMM (null when it has no
    // sectors): a "terms only" tile adds them, plane 0 first, to its A x B
    // terms; tcn planes, tcs floats apart
    const float *tc;
    int tcn;
    int64_t tcs;
};

// One 32x32 FP32 output tile t = (sector, row0, col0, flags) by 256 threads
// (lt = thread index in the group), each owning rows {ty, ty+16} x columns
// {tx, tx+16}.  A "terms only" tile (t.w & 1) skips the two dense products
// and adds them from the tensor-core output planes op.tc instead.
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
                float y = acc[rr][cc] * scale;
                if ((t.w & 1) && op.tc) {
                    float d = op.tc[o + idx];
                    for (int p = 1; p < op.tcn; ++p) d += op.tc[(int64_t)p * op.tcs + o + idx];
                    y += d;
                }
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
//   HV_RIGHT  W H_R^T                             -> slot 2
//   HV_TERMS  A x B terms                         -> slot 0
// Sectors whose tiles have long K loops (Dl or Dr > 64) are split into the
// last three so the parts run on different SMs; the result is slot 0 +
// slot 1 + slot 2 (regions of slots 1 and 2 that no item writes stay zero).
enum { HV_FULL = 0, HV_LEFT = 1, HV_RIGHT = 2, HV_TERMS = 3 };
constexpr int HV_KMAX = 128;            // K extent staged at once
constexpr int SA_LD = HV_KMAX + 4;      // A rows: float4 reads along K
constexpr int SB_LD = 34;               // B rows: float2 reads along the columns

// A work item with everything it needs to start its operand loads, so that
// these depend on one load only: (sector, row0, col0, part), (Dl, Dr, first
// term, end term), (sector offset lo/hi, A x B table offset, 0), (H_L and
// H_R offsets lo/hi).
struct ItemRec {
    int4 a, b, c, d;
};

__device__ __forceinline__ int64_t lohi(int lo, int hi) { return (int64_t)(unsigned)lo | ((int64_t)hi << 32); }

struct __align__(16) Item32Smem {
    float sa[32][SA_LD];                // A rows x K
    float sb[HV_KMAX][SB_LD];           // K x B columns
    AbStage<float, 32, 32> S;
};

// K loop over staged operands: sa[r][k0..k0+kn4) x sb[k0..k0+kn4)[cols]
__device__ __forceinline__ void item_mma(const Item32Smem &sm, int k0, int kn4, int ty, int tx, float (&acc)[2][2]) {
#pragma unroll 2
    for (int j = k0; j < k0 + kn4; j += 4) {
        const float4 a0 = *reinterpret_cast<const float4 *>(&sm.sa[ty][j]);
        const float4 a1 = *reinterpret_cast<const float4 *>(&sm.sa[ty + 16][j]);
        const float av0[4] = {a0.x, a0.y, a0.z, a0.w}, av1[4] = {a1.x, a1.y, a1.z, a1.w};
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const float2 b = *reinterpret_cast<const float2 *>(&sm.sb[j + q][2 * tx]);
            acc[0][0] = fmaf(av0[q], b.x, acc[0][0]);
            acc[0][1] = fmaf(av0[q], b.y, acc[0][1]);
            acc[1][0] = fmaf(av1[q], b.x, acc[1][0]);
            acc[1][1] = fmaf(av1[q], b.y, acc[1][1]);
        }
    }
}

// Staged operands of one phase into columns [k0, k0 + ext) of sa / rows of
// sb: A[r][c] and B[c][x] of H_L W (ph 0) or W H_R^T (ph 1), K range
// [kb, kb + kn), zero beyond kn; EXT (64 or 128) is the staged extent, so a
// thread loads EXT/8 elements per operand, all in flight before the stores.
template <int EXT>
__device__ __forceinline__ void item_load(int ph, const float *__restrict__ H, const float *__restrict__ W, int dl,
                                          int dr, int row0, int col0, int kb, int kn, int lt, float *ra, float *rb) {
    constexpr int PER = 32 * EXT / 256;
    constexpr int SH = EXT == 64 ? 6 : 7;
#pragma unroll
    for (int q = 0; q < PER; ++q) {
        const int e = lt + q * 256;
        const int r = e >> SH, c = e & (EXT - 1);
        const int gi = row0 + r;
        float x = 0.f;
        if (gi < dl && c < kn) x = ph == 0 ? H[(int64_t)gi * dl + kb + c] : W[(int64_t)gi * dr + kb + c];
        ra[q] = x;
        float y = 0.f;
        if (ph == 0) {
            const int c2 = e >> 5, xx = e & 31, gc = col0 + xx;
            if (gc < dr && c2 < kn) y = W[(int64_t)(kb + c2) * dr + gc];
        } else {
            const int xx = e >> SH, gr = col0 + xx;
            if (gr < dr && c < kn) y = H[(int64_t)gr * dr + kb + c];
        }
        rb[q] = y;
    }
}

template <int EXT>
__device__ __forceinline__ void item_store(Item32Smem &sm, int ph, int k0, int kn4, int lt, const float *ra,
                                           const float *rb) {
    constexpr int PER = 32 * EXT / 256;
    constexpr int SH = EXT == 64 ? 6 : 7;
#pragma unroll
    for (int q = 0; q < PER; ++q) {
        const int e = lt + q * 256;
        const int r = e >> SH, c = e & (EXT - 1);
        if (c < kn4) sm.sa[r][k0 + c] = ra[q];
        if (ph == 0) {
            const int c2 = e >> 5, xx = e & 31;
            if (c2 < kn4) sm.sb[k0 + c2][xx] = rb[q];
        } else {
            const int xx = e >> SH;
            if (c < kn4) sm.sb[k0 + c][xx] = rb[q];
        }
    }
}

// One item by 256 threads (lt = thread index in the group): each thread owns
// rows {ty, ty+16} x columns {2tx, 2tx+1}, so a K step of four costs two
// float4 and four float2 shared-memory reads for sixteen FMAs.  The staged
// operands are loaded with every load of a thread in flight before its
// stores: a FULL item (both K <= 64) stages both products in one round (H_L
// part in columns 0..63, H_R part in 64..127), a LEFT / RIGHT item its K
// range (<= HV_KMAX) in one round per 128.  The A x B tables (and the
// per-term offsets) are read in the same round.  The outputs times `scale`
// go to the item's slot; returns this thread's share of sum_i (v[i] scale)
// (out[i] scale) over its outputs.
template <class Sync>
__device__ __forceinline__ float hv32_item(const ItemRec &it, const float *__restrict__ v, float *const *slots,
                                           const Hv32Ops &op, Item32Smem &sm, int lt, Sync sync, float scale) {
    const int row0 = it.a.y, col0 = it.a.z, part = it.a.w;
    const int dl = it.b.x, dr = it.b.y, t0 = it.b.z, t1 = it.b.w;
    const int64_t o = lohi(it.c.x, it.c.y);
    const float *W = v + o;
    const float *HLk = op.hl + lohi(it.d.x, it.d.y), *HRk = op.hr + lohi(it.d.z, it.d.w);
    const int ty = lt / 16, tx = lt % 16;
    float acc[2][2] = {{0.f, 0.f}, {0.f, 0.f}};
    const bool terms = part == HV_FULL || part == HV_TERMS;
    const int eo = terms ? it.c.z : -1;
    constexpr int NE = AB_MAXT * 64 / 256;
    int2 ee[NE];
    int4 hd = make_int4(0, 0, 0, 0);
    const int nt0 = min(AB_MAXT, t1 - t0);
    // first batch of the A x B table, issued with the operand loads
    auto ell_load = [&](int tb, int nt) {
        const int2 *src = op.ell + eo + (int64_t)(tb - t0) * 64;
#pragma unroll
        for (int q = 0; q < NE; ++q) {
            const int e = lt + q * 256;
            ee[q] = e < nt * 64 ? src[e] : make_int2(-1, 0);
        }
        if (lt < nt) hd = op.term_hdr[tb + lt];
    };
    if (eo >= 0 && nt0 > 0) ell_load(t0, nt0);
    if (part == HV_FULL) {
        float ra[8], rb[8];
        item_load<64>(0, HLk, W, dl, dr, row0, col0, 0, dl, lt, ra, rb);
        float rc[8], rd[8];
        item_load<64>(1, HRk, W, dl, dr, row0, col0, 0, dr, lt, rc, rd);
        const int kl4 = (dl + 3) & ~3, kr4 = (dr + 3) & ~3;
        item_store<64>(sm, 0, 0, kl4, lt, ra, rb);
        item_store<64>(sm, 1, 64, kr4, lt, rc, rd);
        sync();
        item_mma(sm, 0, kl4, ty, tx, acc);
        item_mma(sm, 64, kr4, ty, tx, acc);
        sync();
    } else if (part == HV_LEFT || part == HV_RIGHT) {
        const int ph = part == HV_LEFT ? 0 : 1;
        const int K = ph == 0 ? dl : dr;
        const float *H = ph == 0 ? HLk : HRk;
        for (int kb = 0; kb < K; kb += HV_KMAX) {
            const int kn = min(HV_KMAX, K - kb), kn4 = (kn + 3) & ~3;
            float ra[16], rb[16];
            item_load<HV_KMAX>(ph, H, W, dl, dr, row0, col0, kb, kn, lt, ra, rb);
            item_store<HV_KMAX>(sm, ph, 0, kn4, lt, ra, rb);
            sync();
            item_mma(sm, 0, kn4, ty, tx, acc);
            sync();
        }
    }
    if (terms) {
        AbStage<float, 32, 32> &S = sm.S;
        for (int tb = t0; tb < t1; tb += AB_MAXT) {
            const int nt = min(AB_MAXT, t1 - tb);
            bool multi = false;
            if (eo >= 0) {
                if (tb != t0) ell_load(tb, nt);
                if (lt < nt) {
                    S.wq[lt] = v + ((int64_t)(unsigned)hd.x | ((int64_t)hd.y << 32));
                    S.drq[lt] = hd.z;
                }
#pragma unroll
                for (int q = 0; q < NE; ++q) {
                    const int e = lt + q * 256;
                    if (e < nt * 64) {
                        const int tt = e >> 6, r = e & 63;
                        if (r < 32) {
                            S.ac[tt][r] = ee[q].x;
                            S.av[tt][r] = __int_as_float(ee[q].y);
                        } else {
                            S.bc[tt][r - 32] = ee[q].x;
                            S.bv[tt][r - 32] = __int_as_float(ee[q].y);
                        }
                    }
                }
                sync();
            } else {
                ab_stage<float, 32, 32>(S, v, tb, nt, row0, col0, dl, dr, op.drs, op.off, op.terms, op.ab_rp,
                                        op.ab_col, op.ab_val, lt, 256, sync);
                multi = S.multi != 0;
            }
            if (!multi) {
                // the gathers of eight terms issued before their FMAs
                for (int t8 = 0; t8 < nt; t8 += 8) {
                    float g[8][2][2], f[8][2][2];
#pragma unroll
                    for (int u = 0; u < 8; ++u) {
                        const int tt = t8 + u;
                        const bool on = tt < nt;
                        const float *Wq = on ? S.wq[tt] : nullptr;
                        const int drq = on ? S.drq[tt] : 0;
#pragma unroll
                        for (int rr = 0; rr < 2; ++rr)
#pragma unroll
                            for (int cc = 0; cc < 2; ++cc) {
                                const int aj = on ? S.ac[tt][ty + 16 * rr] : -1;
                                const int bj = on ? S.bc[tt][2 * tx + cc] : -1;
                                const bool hit = aj >= 0 && bj >= 0;
                                f[u][rr][cc] = hit ? S.av[tt][ty + 16 * rr] * S.bv[tt][2 * tx + cc] : 0.f;
                                g[u][rr][cc] = hit ? Wq[(int64_t)aj * drq + bj] : 0.f;
                            }
                    }
#pragma unroll
                    for (int u = 0; u < 8; ++u)
#pragma unroll
                        for (int rr = 0; rr < 2; ++rr)
#pragma unroll
                            for (int cc = 0; cc < 2; ++cc) acc[rr][cc] = fmaf(f[u][rr][cc], g[u][rr][cc], acc[rr][cc]);
                }
            } else {
                for (int rr = 0; rr < 2; ++rr)
                    for (int cc = 0; cc < 2; ++cc) {
                        const int il = row0 + ty + 16 * rr, ir = col0 + 2 * tx + cc;
                        if (il < dl && ir < dr)
                            acc[rr][cc] = ab_csr<float>(acc[rr][cc], v, tb, nt, il, ir, op.drs, op.off, op.terms,
                                                        op.ab_rp, op.ab_col, op.ab_val);
                    }
            }
            sync();
        }
    }
    float *out = slots[part == HV_LEFT ? 1 : (part == HV_RIGHT ? 2 : 0)] + o;
    float p = 0.f;
    for (int rr = 0; rr < 2; ++rr)
        for (int cc = 0; cc < 2; ++cc) {
            const int il = row0 + ty + 16 * rr, ir = col0 + 2 * tx + cc;
            if (il < dl && ir < dr) {
                const int64_t idx2 = (int64_t)il * dr + ir;
                const float y = acc[rr][cc] * scale;
                out[idx2] = y;
                p = fmaf(W[idx2] * scale, y, p);
            }
        }
    return p;
}

}  // namespace nss
