// Operator renormalisation O' = U^T O U of one block on the GPU
// (operators_renormalization, src/DMRG_RDM.f90:355-404).
//
// U is block-sparse by construction: kept column j is the eigenvector of
// rho block q_j, scattered onto that block's states (sparse_blocks_matrix,
// src/MATRIX/MATRIX_BLOCKS.f90:556-576).  So
//     O'[j, j'] = (U_q^T  O_{q q'}  U_q')[loc(j), loc(j')],
// q = q_j, q' = q_j', with U_q the n_q x k_q matrix of block q's kept
// columns and O_{q q'} the dense n_q x n_q' block of O between the two
// blocks' states.  Every nonzero block pair of every operator becomes two
// FP64 GEMMs (cuBLAS DGEMM: T = O_{q q'} U_q', O'_{q q'} = U_q^T T); the
// operators stay sparse on the host between steps as in the reference, and
// only their nonzero blocks travel.  The kept columns come from the RDM
// step in compact form (no zero rows) and stay on the device.
#include "device.cuh"
#include "host_sparse.hpp"

#include <cublas_v2.h>

#include <algorithm>
#include <cstring>

namespace nss {

namespace {

// U_q blocks: column j of the compact buffer (length n_q) -> column loc of
// the n_q x k_q column-major matrix at uoff[j] in ublk.
__global__ void __launch_bounds__(128) k_gather_u(const double *__restrict__ comp, const int *__restrict__ src_off,
                                                 const int *__restrict__ dst_off, const int *__restrict__ len,
                                                 double *__restrict__ ublk) {
    const int j = blockIdx.x;
    const double *s = comp + src_off[j];
    double *d = ublk + dst_off[j];
    for (int p = threadIdx.x; p < len[j]; p += blockDim.x) d[p] = s[p];
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

}  // namespace

void renorm_release(Ctx &c) {
    DevRenorm &w = c.ren;
    void *ptrs[] = {w.ublk, w.dblk, w.tbuf, w.rbuf, w.itab};
    for (void *p : ptrs) ctx_free(c, p);
    if (w.hblk) cudaFreeHost(w.hblk);
    if (w.hres) cudaFreeHost(w.hres);
    if (w.hitab) cudaFreeHost(w.hitab);
    if (w.blas) cublasDestroy((cublasHandle_t)w.blas);
    w = DevRenorm{};
}

int renorm_device(Ctx &c, const KeptLayout &kl, Block &blk, const std::vector<Qn> &kept_qn) {
    DevRenorm &w = c.ren;
    cudaStream_t st = c.stream;
    const int ms = kl.ms, nb = (int)kl.dims.size();
    if (!w.blas) {
        cublasHandle_t h = nullptr;
        if (cublasCreate(&h) != CUBLAS_STATUS_SUCCESS) {
            c.err = "renormalisation: cublasCreate failed";
            return NSS_ERR_CUDA;
        }
        w.blas = h;
    }
    cublasHandle_t h = (cublasHandle_t)w.blas;
    if (cublasSetStream(h, st) != CUBLAS_STATUS_SUCCESS) {
        c.err = "renormalisation: cublasSetStream failed";
        return NSS_ERR_CUDA;
    }
    // kept columns per block, in ascending j
    std::vector<int> kq(nb, 0), loc(ms);
    for (int j = 0; j < ms; ++j) loc[j] = kq[kl.q[j]]++;
    std::vector<int64_t> uoff(nb + 1, 0);
    for (int q = 0; q < nb; ++q) uoff[q + 1] = uoff[q] + (int64_t)kl.dims[q] * kq[q];
    // enlarged-block state -> (block, local row)
    const int mblock = blk.dim;
    std::vector<int> bof(mblock, -1), lof(mblock, -1);
    for (int q = 0; q < nb; ++q)
        for (int p = 0; p < kl.dims[q]; ++p) {
            const int s = kl.maps[kl.map_off[q] + p];
            if (s >= 0 && s < mblock) {
                bof[s] = q;
                lof[s] = p;
            }
        }
    // nonzero block pairs of every operator (both blocks with kept columns)
    struct Pair {
        int op, qr, qc;
        int64_t o_off, t_off, r_off;
    };
    std::vector<Pair> pairs;
    std::vector<std::vector<int>> pidx(blk.ops.size(), std::vector<int>((size_t)nb * nb, -1));
    int64_t o_tot = 0, t_tot = 0, r_tot = 0;
    for (size_t io = 0; io < blk.ops.size(); ++io) {
        const Csr &m = blk.ops[io].m;
        for (int r = 0; r < m.nrow; ++r) {
            const int qr = r < mblock ? bof[r] : -1;
            if (qr < 0 || !kq[qr]) continue;
            for (int e = m.rowptr[r]; e < m.rowptr[r + 1]; ++e) {
                const int cc = m.col[e];
                const int qc = cc < mblock ? bof[cc] : -1;
                if (qc < 0 || !kq[qc]) continue;
                const int key = qr * nb + qc;
                if (pidx[io][key] >= 0) continue;
                Pair pr{(int)io, qr, qc, o_tot, t_tot, r_tot};
                o_tot += (int64_t)kl.dims[qr] * kl.dims[qc];
                t_tot += (int64_t)kl.dims[qr] * kq[qc];
                r_tot += (int64_t)kq[qr] * kq[qc];
                pidx[io][key] = (int)pairs.size();
                pairs.push_back(pr);
            }
        }
    }
    int rc;
    if ((rc = grow_host(c, &w.hblk, w.cap_hblk, o_tot))) return rc;
    if ((rc = grow_host(c, &w.hres, w.cap_hres, r_tot))) return rc;
    if ((rc = grow_dev(c, &w.dblk, w.cap_dblk, o_tot))) return rc;
    if ((rc = grow_dev(c, &w.tbuf, w.cap_tbuf, t_tot))) return rc;
    if ((rc = grow_dev(c, &w.rbuf, w.cap_rbuf, r_tot))) return rc;
    if ((rc = grow_dev(c, &w.ublk, w.cap_ublk, uoff[nb]))) return rc;
    // dense blocks of the operators (column-major n_qr x n_qc)
    std::memset(w.hblk, 0, (size_t)o_tot * sizeof(double));
    for (size_t io = 0; io < blk.ops.size(); ++io) {
        const Csr &m = blk.ops[io].m;
        for (int r = 0; r < m.nrow; ++r) {
            const int qr = r < mblock ? bof[r] : -1;
            if (qr < 0 || !kq[qr]) continue;
            for (int e = m.rowptr[r]; e < m.rowptr[r + 1]; ++e) {
                const int cc = m.col[e];
                const int qc = cc < mblock ? bof[cc] : -1;
                if (qc < 0 || !kq[qc]) continue;
                const Pair &pr = pairs[pidx[io][qr * nb + qc]];
                w.hblk[pr.o_off + (int64_t)lof[cc] * kl.dims[qr] + lof[r]] = m.val[e];
            }
        }
    }
    NSS_CUDA_TRY(c, cudaMemcpyAsync(w.dblk, w.hblk, (size_t)o_tot * sizeof(double), cudaMemcpyHostToDevice, st));
    // U_q from the compact kept columns
    if (ms > 0) {
        if ((rc = grow_host(c, &w.hitab, w.cap_hitab, 3 * (int64_t)ms))) return rc;
        if ((rc = grow_dev(c, &w.itab, w.cap_itab, 3 * (int64_t)ms))) return rc;
        int *src = w.hitab, *dst = src + ms, *len = dst + ms;
        for (int j = 0; j < ms; ++j) {
            const int q = kl.q[j];
            src[j] = kl.off[j];
            dst[j] = (int)(uoff[q] + (int64_t)loc[j] * kl.dims[q]);
            len[j] = kl.dims[q];
        }
        NSS_CUDA_TRY(c, cudaMemcpyAsync(w.itab, w.hitab, 3 * (size_t)ms * sizeof(int), cudaMemcpyHostToDevice, st));
        ++c.launches;
        k_gather_u<<<ms, 128, 0, st>>>(kl.dcomp, w.itab, w.itab + ms, w.itab + 2 * ms, w.ublk);
        NSS_CUDA_TRY(c, cudaGetLastError());
    }
    // two GEMMs per block pair
    const double one = 1.0, zero = 0.0;
    for (const Pair &pr : pairs) {
        const int nr = kl.dims[pr.qr], nc = kl.dims[pr.qc], kr = kq[pr.qr], kc = kq[pr.qc];
        const double *O = w.dblk + pr.o_off, *Ur = w.ublk + uoff[pr.qr], *Uc = w.ublk + uoff[pr.qc];
        double *T = w.tbuf + pr.t_off, *R = w.rbuf + pr.r_off;
        if (cublasDgemm(h, CUBLAS_OP_N, CUBLAS_OP_N, nr, kc, nc, &one, O, nr, Uc, nc, &zero, T, nr) !=
                CUBLAS_STATUS_SUCCESS ||
            cublasDgemm(h, CUBLAS_OP_T, CUBLAS_OP_N, kr, kc, nr, &one, Ur, nr, T, nr, &zero, R, kr) !=
                CUBLAS_STATUS_SUCCESS) {
            c.err = "renormalisation: cublasDgemm failed";
            return NSS_ERR_CUDA;
        }
        c.launches += 2;
    }
    NSS_CUDA_TRY(c, cudaMemcpyAsync(w.hres, w.rbuf, (size_t)r_tot * sizeof(double), cudaMemcpyDeviceToHost, st));
    NSS_CUDA_TRY(c, cudaStreamSynchronize(st));
    // O' in CSR, rows and columns in kept order, exact zeros dropped
    std::vector<std::vector<int>> jof(nb);
    for (int j = 0; j < ms; ++j) jof[kl.q[j]].push_back(j);
    for (size_t io = 0; io < blk.ops.size(); ++io) {
        std::vector<std::vector<int>> prow(nb);       // pairs of this operator by row block
        for (int key = 0; key < nb * nb; ++key)
            if (pidx[io][key] >= 0) prow[key / nb].push_back(pidx[io][key]);
        Csr out;
        out.init(ms, ms);
        std::vector<std::pair<int, double>> row;
        for (int j = 0; j < ms; ++j) {
            const int qr = kl.q[j], a = loc[j];
            row.clear();
            for (int pi : prow[qr]) {
                const Pair &pr = pairs[pi];
                const int kr = kq[qr];
                const double *R = w.hres + pr.r_off;
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
    }
    blk.dim = ms;
    blk.basis.clear();
    for (const Qn &q : kept_qn) blk.basis.insert(blk.basis.end(), q.begin(), q.end());
    return NSS_OK;
}

}  // namespace nss
