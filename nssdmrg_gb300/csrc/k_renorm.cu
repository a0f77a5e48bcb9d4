// Operator renormalisation O' = U^T O U of the two blocks on the GPU
// (operators_renormalization, src/DMRG_RDM.f90:355-404).
//
// U is block-sparse by construction: kept column j is the eigenvector of
// rho block q_j, scattered onto that block's states (sparse_blocks_matrix,
// src/MATRIX/MATRIX_BLOCKS.f90:556-576).  So
//     O'[j, j'] = (U_q^T  O_{q q'}  U_q')[loc(j), loc(j')],
// q = q_j, q' = q_j', with U_q the n_q x k_q matrix of block q's kept
// columns and O_{q q'} the dense n_q x n_q' block of O between the two
// blocks' states.  Every nonzero block pair of every operator of both blocks
// becomes two FP64 products (T = O_{q q'} U_q', O'_{q q'} = U_q^T T), all of
// one kind in one launch of a batched tile kernel: the pairs are a few
// hundred states wide, so one library GEMM per pair would occupy a dozen
// SMs at a time.  The operators stay sparse on the host between steps as in
// the reference, and only their nonzero blocks travel; the two blocks'
// host-side scan, extraction and CSR assembly run on two threads.  The kept
// columns come from the RDM step in compact form (no zero rows) and stay on
// the device.
#include "device.cuh"
#include "host_sparse.hpp"

#include <algorithm>
#include <chrono>
#include <cstring>
#include <exception>
#include <thread>

namespace nss {

namespace {

// U_q blocks: column j of the compact buffer (length n_q) -> column loc of
// the n_q x k_q column-major matrix at dst_off[j] in ublk.
__global__ void __launch_bounds__(128) k_gather_u(const double *__restrict__ comp, const int *__restrict__ src_off,
                                                 const int64_t *__restrict__ dst_off, const int *__restrict__ len,
                                                 double *__restrict__ ublk) {
    const int j = blockIdx.x;
    const double *s = comp + src_off[j];
    double *d = ublk + dst_off[j];
    for (int p = threadIdx.x; p < len[j]; p += blockDim.x) d[p] = s[p];
}

// The operators' nonzero entries into their zeroed dense block pairs:
// (position in the O buffer, value) pairs from the host.
struct RnEntry {
    int64_t at;
    double val;
};
__global__ void __launch_bounds__(256) k_rn_scatter(const RnEntry *__restrict__ e, int64_t n, double *__restrict__ o) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        o[e[i].at] = e[i].val;
}

// One product C (m x n, column-major, ldc) = op(A) B, B column-major k x n
// (ldb); op(A) = A (m x k, lda) or A^T (A stored k x m, lda).  Its 64 x 64
// output tiles are blocks tile0 .. tile0 + tiles_m * ceil(n/64) - 1.
struct RnJob {
    const double *a;
    const double *b;
    double *c;
    int m, n, k, lda, ldb, ldc, transa, tiles_m, tile0, pad;
};

constexpr int RN_TILE = 64, RN_K = 16;

// Batched FP64 tile product: one CTA per 64 x 64 output tile of any job,
// 256 threads with 4 x 4 outputs each (rows tm + 16 i, columns tn + 16 j),
// K in steps of 16 through shared memory, zero-filled at the edges.
__global__ void __launch_bounds__(256) k_rn_gemm(const RnJob *__restrict__ jobs, const int *__restrict__ tile_job) {
    __shared__ double As[RN_K][RN_TILE + 1];
    __shared__ double Bs[RN_K][RN_TILE + 1];
    const RnJob jb = jobs[tile_job[blockIdx.x]];
    const int local = blockIdx.x - jb.tile0;
    const int m0 = (local % jb.tiles_m) * RN_TILE, n0 = (local / jb.tiles_m) * RN_TILE;
    const int tid = threadIdx.x, tm = tid & 15, tn = tid >> 4;
    double acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = 0.0;
    for (int k0 = 0; k0 < jb.k; k0 += RN_K) {
        if (!jb.transa) {
            const int m = tid & 63, gm = m0 + m;
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                const int kk = (tid >> 6) + 4 * r, gk = k0 + kk;
                As[kk][m] = (gm < jb.m && gk < jb.k) ? jb.a[(int64_t)gk * jb.lda + gm] : 0.0;
            }
        } else {
            const int kk = tid & 15, gk = k0 + kk;
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                const int m = (tid >> 4) + 16 * r, gm = m0 + m;
                As[kk][m] = (gm < jb.m && gk < jb.k) ? jb.a[(int64_t)gm * jb.lda + gk] : 0.0;
            }
        }
        {
            const int kk = tid & 15, gk = k0 + kk;
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                const int n = (tid >> 4) + 16 * r, gn = n0 + n;
                Bs[kk][n] = (gn < jb.n && gk < jb.k) ? jb.b[(int64_t)gn * jb.ldb + gk] : 0.0;
            }
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < RN_K; ++kk) {
            double a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) a[i] = As[kk][tm + 16 * i];
#pragma unroll
            for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tn + 16 * j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int gn = n0 + tn + 16 * j;
        if (gn >= jb.n) continue;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int gm = m0 + tm + 16 * i;
            if (gm < jb.m) jb.c[(int64_t)gn * jb.ldc + gm] = acc[i][j];
        }
    }
}

template <class T>
int grow_dev(Ctx &c, T **p, int64_t &cap, int64_t need) {
    if (*p && cap >= need) return NSS_OK;
    ctx_free(c, *p);
    *p = nullptr;
    NSS_CUDA_TRY(c, ctx_alloc(c, p, (size_t)std::max<int64_t>(need, 1)));
    cap = need;
    return NSS_OK;
}

template <class T>
int grow_host(Ctx &c, T **p, int64_t &cap, int64_t need) {
    if (*p && cap >= need) return NSS_OK;
    if (*p) cudaFreeHost(*p);
    *p = nullptr;
    NSS_CUDA_TRY(c, cudaHostAlloc((void **)p, (size_t)std::max<int64_t>(need, 1) * sizeof(T), cudaHostAllocDefault));
    cap = need;
    return NSS_OK;
}

struct Pair {
    int op, qr, qc;
    int64_t o_off, t_off, r_off;   // offsets into the side's O, T and R shares
};

// One block's share of the work.
struct Side {
    const KeptLayout *kl = nullptr;
    Block *blk = nullptr;
    const std::vector<Qn> *kept_qn = nullptr;
    int nb = 0, ms = 0;
    std::vector<int> kq, loc;
    std::vector<int64_t> uoff;            // U_q blocks, offsets into the side's U share
    std::vector<int> bof, lof;            // enlarged-block state -> (block, local row)
    std::vector<Pair> pairs;
    std::vector<std::vector<int>> pidx;   // [op][qr * nb + qc] -> pair or -1
    int64_t o_tot = 0, t_tot = 0, r_tot = 0, u_tot = 0;
    int64_t nent = 0;                     // operator entries inside kept block pairs
    std::vector<int64_t> ent_first;       // per operator: its first entry (extract order)
};

// kept columns per block, state maps and the nonzero block pairs of every
// operator (both blocks with kept columns)
void scan_side(Side &s) {
    if (!s.blk) return;   // a side not renormalised: no columns, no pairs
    const KeptLayout &kl = *s.kl;
    const Block &blk = *s.blk;
    s.ms = kl.ms;
    s.nb = (int)kl.dims.size();
    const int nb = s.nb;
    s.kq.assign(nb, 0);
    s.loc.resize(s.ms);
    for (int j = 0; j < s.ms; ++j) s.loc[j] = s.kq[kl.q[j]]++;
    s.uoff.assign(nb + 1, 0);
    for (int q = 0; q < nb; ++q) s.uoff[q + 1] = s.uoff[q] + (int64_t)kl.dims[q] * s.kq[q];
    s.u_tot = s.uoff[nb];
    const int mblock = blk.dim;
    s.bof.assign(mblock, -1);
    s.lof.assign(mblock, -1);
    for (int q = 0; q < nb; ++q)
        for (int p = 0; p < kl.dims[q]; ++p) {
            const int st = kl.maps[kl.map_off[q] + p];
            if (st >= 0 && st < mblock) {
                s.bof[st] = q;
                s.lof[st] = p;
            }
        }
    s.pidx.assign(blk.ops.size(), std::vector<int>((size_t)nb * nb, -1));
    s.ent_first.assign(blk.ops.size() + 1, 0);
    for (size_t io = 0; io < blk.ops.size(); ++io) {
        s.ent_first[io] = s.nent;
        const Csr &m = blk.ops[io].m;
        for (int r = 0; r < m.nrow; ++r) {
            const int qr = r < mblock ? s.bof[r] : -1;
            if (qr < 0 || !s.kq[qr]) continue;
            for (int e = m.rowptr[r]; e < m.rowptr[r + 1]; ++e) {
                const int cc = m.col[e];
                const int qc = cc < mblock ? s.bof[cc] : -1;
                if (qc < 0 || !s.kq[qc]) continue;
                ++s.nent;
                const int key = qr * nb + qc;
                if (s.pidx[io][key] >= 0) continue;
                s.pidx[io][key] = (int)s.pairs.size();
                s.pairs.push_back({(int)io, qr, qc, s.o_tot, s.t_tot, s.r_tot});
                s.o_tot += (int64_t)kl.dims[qr] * kl.dims[qc];
                s.t_tot += (int64_t)kl.dims[qr] * s.kq[qc];
                s.r_tot += (int64_t)s.kq[qr] * s.kq[qc];
            }
        }
    }
    s.ent_first[blk.ops.size()] = s.nent;
}

// the operators' entries inside kept block pairs as (position in the
// column-major n_qr x n_qc block of their pair, offset by ob, value) into
// ent, the side's share of the staging buffer; the device scatters them
void extract_side(const Side &s, RnEntry *ent, int64_t ob) {
    if (!s.blk) return;
    const KeptLayout &kl = *s.kl;
    const Block &blk = *s.blk;
    const int nb = s.nb, mblock = blk.dim;
    // the operators in parallel, each from its first entry
    parallel_for((int)blk.ops.size(), [&](int io) {
        int64_t at = s.ent_first[io];
        const Csr &m = blk.ops[io].m;
        const std::vector<int> &pi = s.pidx[io];
        for (int r = 0; r < m.nrow; ++r) {
            const int qr = r < mblock ? s.bof[r] : -1;
            if (qr < 0 || !s.kq[qr]) continue;
            const int64_t rowbase = s.lof[r];
            for (int e = m.rowptr[r]; e < m.rowptr[r + 1]; ++e) {
                const int cc = m.col[e];
                const int qc = cc < mblock ? s.bof[cc] : -1;
                if (qc < 0 || !s.kq[qc]) continue;
                const Pair &pr = s.pairs[pi[qr * nb + qc]];
                ent[at++] = RnEntry{ob + pr.o_off + (int64_t)s.lof[cc] * kl.dims[qr] + rowbase, m.val[e]};
            }
        }
    }, s.nent > 50000);
}

// O' in CSR, rows and columns in kept order, exact zeros dropped; hres is
// the side's share of the result staging buffer
void assemble_side(Side &s, const double *hres) {
    if (!s.blk) return;
    const KeptLayout &kl = *s.kl;
    Block &blk = *s.blk;
    const int nb = s.nb, ms = s.ms;
    std::vector<std::vector<int>> jof(nb);
    for (int j = 0; j < ms; ++j) jof[kl.q[j]].push_back(j);
    // the operators in parallel (each writes only its own matrix)
    parallel_for((int)blk.ops.size(), [&](int io) {
        std::vector<std::pair<int, double>> row;
        std::vector<std::vector<int>> prow(nb);   // pairs of this operator by row block
        for (int key = 0; key < nb * nb; ++key)
            if (s.pidx[io][key] >= 0) prow[key / nb].push_back(s.pidx[io][key]);
        Csr out;
        out.init(ms, ms);
        for (int j = 0; j < ms; ++j) {
            const int qr = kl.q[j], a = s.loc[j];
            row.clear();
            for (int pi : prow[qr]) {
                const Pair &pr = s.pairs[pi];
                const int kr = s.kq[qr];
                const double *R = hres + pr.r_off;
                const std::vector<int> &cols = jof[pr.qc];
                for (size_t b = 0; b < cols.size(); ++b) {
                    const double v = R[(int64_t)b * kr + a];
                    if (v != 0.0) row.push_back({cols[b], v});
                }
            }
            std::sort(row.begin(), row.end(), [](const auto &x, const auto &y) { return x.first < y.first; });
            for (const auto &e : row) {
                out.col.push_back(e.first);
                out.val.push_back(e.second);
            }
            out.rowptr[j + 1] = (int)out.col.size();
        }
        blk.ops[io].m = std::move(out);
    }, s.r_tot > 50000);
    blk.dim = ms;
    blk.basis.clear();
    for (const Qn &q : *s.kept_qn) blk.basis.insert(blk.basis.end(), q.begin(), q.end());
}

}  // namespace

void renorm_release(Ctx &c) {
    DevRenorm &w = c.ren;
    void *ptrs[] = {w.ublk, w.dblk, w.tbuf, w.rbuf, w.itab};
    for (void *p : ptrs) ctx_free(c, p);
    if (w.hblk) cudaFreeHost(w.hblk);
    if (w.hres) cudaFreeHost(w.hres);
    if (w.hitab) cudaFreeHost(w.hitab);
    w = DevRenorm{};
}

int renorm_device(Ctx &c, const KeptLayout kl[2], Block *blk[2], const std::vector<Qn> *kept_qn[2]) {
    DevRenorm &w = c.ren;
    cudaStream_t st = c.stream;
    using clk = std::chrono::steady_clock;
    auto ms_since = [](clk::time_point t) { return std::chrono::duration<double, std::milli>(clk::now() - t).count(); };
    const auto t0 = clk::now();
    Side sd[2];
    for (int s = 0; s < 2; ++s) {
        sd[s].kl = &kl[s];
        sd[s].blk = blk[s];
        sd[s].kept_qn = kept_qn[s];
    }
    run_pair([&] { scan_side(sd[0]); }, [&] { scan_side(sd[1]); });
    // shared buffers: side 1's share after side 0's
    const int64_t o_tot = sd[0].o_tot + sd[1].o_tot, t_tot = sd[0].t_tot + sd[1].t_tot,
                  r_tot = sd[0].r_tot + sd[1].r_tot, u_tot = sd[0].u_tot + sd[1].u_tot;
    const int ms_tot = sd[0].ms + sd[1].ms;
    const int npairs = (int)(sd[0].pairs.size() + sd[1].pairs.size());
    int rc;
    const int64_t nent = sd[0].nent + sd[1].nent;
    if ((rc = grow_host(c, &w.hblk, w.cap_hblk, 2 * nent))) return rc;   // RnEntry = two doubles
    if ((rc = grow_host(c, &w.hres, w.cap_hres, r_tot))) return rc;
    if ((rc = grow_dev(c, &w.dblk, w.cap_dblk, o_tot))) return rc;
    if ((rc = grow_dev(c, &w.rbuf, w.cap_rbuf, r_tot))) return rc;
    if ((rc = grow_dev(c, &w.ublk, w.cap_ublk, u_tot))) return rc;
    RnEntry *hent = (RnEntry *)w.hblk;
    run_pair([&] { extract_side(sd[0], hent, 0); }, [&] { extract_side(sd[1], hent + sd[0].nent, sd[0].o_tot); });
    c.renorm_phase_ms[0] += ms_since(t0);
    const auto t1 = clk::now();
    // the entries go to the device as pairs and land in the zeroed blocks
    // there (the T buffer holds them until the first product overwrites it)
    if ((rc = grow_dev(c, &w.tbuf, w.cap_tbuf, std::max<int64_t>(t_tot, 2 * nent)))) return rc;
    NSS_CUDA_TRY(c, cudaMemsetAsync(w.dblk, 0, (size_t)o_tot * sizeof(double), st));
    if (nent > 0) {
        NSS_CUDA_TRY(c, cudaMemcpyAsync(w.tbuf, w.hblk, (size_t)nent * sizeof(RnEntry), cudaMemcpyHostToDevice, st));
        ++c.launches;
        k_rn_scatter<<<(unsigned)std::min<int64_t>((nent + 255) / 256, 4 * 152), 256, 0, st>>>(
            (const RnEntry *)w.tbuf, nent, w.dblk);
        NSS_CUDA_TRY(c, cudaGetLastError());
    }
    // product jobs of both sides: pass 0 T = O U_qc, pass 1 R = U_qr^T T
    int ntiles[2] = {0, 0};
    std::vector<RnJob> jobs[2];
    for (int pass = 0; pass < 2; ++pass) jobs[pass].reserve(npairs);
    for (int s = 0; s < 2; ++s) {
        const Side &S = sd[s];
        const int64_t ob = s ? sd[0].o_tot : 0, tb = s ? sd[0].t_tot : 0, rb = s ? sd[0].r_tot : 0,
                      ub = s ? sd[0].u_tot : 0;
        for (const Pair &pr : S.pairs) {
            const int nr = S.kl->dims[pr.qr], nc = S.kl->dims[pr.qc], kr = S.kq[pr.qr], kc = S.kq[pr.qc];
            double *T = w.tbuf + tb + pr.t_off;
            const int tn = (kc + RN_TILE - 1) / RN_TILE;
            RnJob a{w.dblk + ob + pr.o_off, w.ublk + ub + S.uoff[pr.qc], T, nr, kc, nc, nr, nc, nr, 0,
                    (nr + RN_TILE - 1) / RN_TILE, ntiles[0], 0};
            ntiles[0] += a.tiles_m * tn;
            jobs[0].push_back(a);
            RnJob b{w.ublk + ub + S.uoff[pr.qr], T, w.rbuf + rb + pr.r_off, kr, kc, nr, nr, nr, kr, 1,
                    (kr + RN_TILE - 1) / RN_TILE, ntiles[1], 0};
            ntiles[1] += b.tiles_m * tn;
            jobs[1].push_back(b);
        }
    }
    // index staging, 16-byte aligned sections: kept-column gather tables of
    // both sides (src offsets, lengths, 64-bit dst offsets), the jobs of the
    // two passes, and their tile -> job maps
    auto al16 = [](size_t x) { return (x + 15) / 16 * 16; };
    const size_t b_src = 0, b_len = al16(b_src + sizeof(int) * (size_t)ms_tot);
    const size_t b_dst = al16(b_len + sizeof(int) * (size_t)ms_tot);
    const size_t b_jobs = al16(b_dst + sizeof(int64_t) * (size_t)ms_tot);
    const size_t b_tj = al16(b_jobs + sizeof(RnJob) * (size_t)npairs * 2);
    const size_t b_end = b_tj + sizeof(int) * (size_t)(ntiles[0] + ntiles[1]);
    const int64_t words = (int64_t)((b_end + sizeof(int) - 1) / sizeof(int));
    if ((rc = grow_host(c, &w.hitab, w.cap_hitab, words))) return rc;
    if ((rc = grow_dev(c, &w.itab, w.cap_itab, words))) return rc;
    char *hb = (char *)w.hitab;
    {
        int *src = (int *)(hb + b_src), *len = (int *)(hb + b_len);
        int64_t *dst = (int64_t *)(hb + b_dst);
        int at = 0;
        for (int s = 0; s < 2; ++s) {
            const Side &S = sd[s];
            const int64_t ub = s ? sd[0].u_tot : 0;
            for (int j = 0; j < S.ms; ++j, ++at) {
                const int q = S.kl->q[j];
                src[at] = S.kl->off[j];
                dst[at] = ub + S.uoff[q] + (int64_t)S.loc[j] * S.kl->dims[q];
                len[at] = S.kl->dims[q];
            }
        }
        RnJob *hj = (RnJob *)(hb + b_jobs);
        std::copy(jobs[0].begin(), jobs[0].end(), hj);
        std::copy(jobs[1].begin(), jobs[1].end(), hj + npairs);
        int *tj = (int *)(hb + b_tj);
        for (int pass = 0; pass < 2; ++pass) {
            int *t = tj + (pass ? ntiles[0] : 0);
            for (int i = 0; i < npairs; ++i) {
                const RnJob &jb = jobs[pass][i];
                const int nt = jb.tiles_m * ((jb.n + RN_TILE - 1) / RN_TILE);
                for (int k = 0; k < nt; ++k) t[jb.tile0 + k] = i + (pass ? npairs : 0);
            }
        }
    }
    NSS_CUDA_TRY(c, cudaMemcpyAsync(w.itab, w.hitab, b_end, cudaMemcpyHostToDevice, st));
    const char *db = (const char *)w.itab;
    // U_q from the compact kept columns (each side's columns live in its
    // own compact buffer)
    for (int s = 0, at = 0; s < 2; at += sd[s].ms, ++s) {
        if (sd[s].ms == 0) continue;
        ++c.launches;
        k_gather_u<<<sd[s].ms, 128, 0, st>>>(kl[s].dcomp, (const int *)(db + b_src) + at,
                                             (const int64_t *)(db + b_dst) + at, (const int *)(db + b_len) + at,
                                             w.ublk);
        NSS_CUDA_TRY(c, cudaGetLastError());
    }
    const RnJob *dj = (const RnJob *)(db + b_jobs);
    const int *dtj = (const int *)(db + b_tj);
    for (int pass = 0; pass < 2; ++pass) {
        if (ntiles[pass] == 0) continue;
        ++c.launches;
        k_rn_gemm<<<ntiles[pass], 256, 0, st>>>(dj, dtj + (pass ? ntiles[0] : 0));
        NSS_CUDA_TRY(c, cudaGetLastError());
    }
    NSS_CUDA_TRY(c, cudaMemcpyAsync(w.hres, w.rbuf, (size_t)r_tot * sizeof(double), cudaMemcpyDeviceToHost, st));
    NSS_CUDA_TRY(c, cudaStreamSynchronize(st));
    c.renorm_phase_ms[1] += ms_since(t1);
    const auto t2 = clk::now();
    run_pair([&] { assemble_side(sd[0], w.hres); }, [&] { assemble_side(sd[1], w.hres + sd[0].r_tot); });
    c.renorm_phase_ms[2] += ms_since(t2);
    return NSS_OK;
}

int kept_u_csr(Ctx &c, const KeptLayout &kl, int mblock, Csr &u) {
    int64_t tot = 0;
    for (int j = 0; j < kl.ms; ++j) tot = std::max<int64_t>(tot, (int64_t)kl.off[j] + kl.dims[kl.q[j]]);
    std::vector<double> h((size_t)tot);
    if (tot) NSS_CUDA_TRY(c, cudaMemcpy(h.data(), kl.dcomp, (size_t)tot * sizeof(double), cudaMemcpyDeviceToHost));
    std::vector<std::vector<std::pair<int, double>>> rows(mblock);
    for (int j = 0; j < kl.ms; ++j) {
        const int q = kl.q[j];
        for (int p = 0; p < kl.dims[q]; ++p) {
            const int st = kl.maps[kl.map_off[q] + p];
            const double v = h[(size_t)kl.off[j] + p];
            if (st >= 0 && st < mblock && v != 0.0) rows[st].push_back({j, v});
        }
    }
    u.init(mblock, kl.ms);
    for (int i = 0; i < mblock; ++i) {
        for (const auto &e : rows[i]) {
            u.col.push_back(e.first);
            u.val.push_back(e.second);
        }
        u.rowptr[i + 1] = (int)u.col.size();
    }
    return NSS_OK;
}

}  // namespace nss
