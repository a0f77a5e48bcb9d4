// Superblock upload and the direct H_sb * psi product (plain FP64 path).
//
// Restates spMatVec_direct_main (src/DMRG_SUPERBLOCK_SETUP.f90:740-865) as one
// kernel over output tiles.  For output sector k, with W_k the row-major
// [Dl x Dr] view of the sector (i = ir + il*Dr + Offset, :770),
//     Out_k = H_L(k) W_k + W_k H_R(k)^T + sum_t A_t W_q(t) B_t^T,
// where the last sum runs over the terms whose RowOffset is sector k
// (:808-857, regrouped by output sector so each tile has one writer).
#include "device.cuh"
#include "hv_tile.cuh"
#include "host_sparse.hpp"
#include "sector_mma.cuh"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>

namespace nss {

int tc_min_dl_default() {
    const char *e = std::getenv("NSS_TC_MIN_DL");
    if (!e) return 1024;
    const int x = std::atoi(e);
    return x < 0 ? 0 : x;
}

void mma_tile_default(int *bn, bool *split) {
    const char *b = std::getenv("NSS_TC_BN");
    *bn = (b && std::atoi(b) == 128) ? 128 : 64;
    const char *sp = std::getenv("NSS_TC_SPLIT");
    *split = !(sp && std::atoi(sp) == 0);
}

int mma_kps_default() {
    const char *e = std::getenv("NSS_TC_KPS");
    return (e && std::atoi(e) == 2) ? 2 : 1;
}

bool mma_lolo_default() {
    const char *e = std::getenv("NSS_TC_LOLO");
    return e && std::atoi(e) != 0;
}

uint32_t wait_limit() {
    const char *e = std::getenv("NSS_WAIT_LIMIT");
    if (!e) return 1u << 22;
    const long x = std::atol(e);
    return x < 0 ? 0u : (uint32_t)std::min<long>(x, 1l << 30);
}

void ctx_free(Ctx &c, void *p) {
    if (!p) return;
    auto it = c.sizes.find(p);
    if (it != c.sizes.end()) {
        c.used -= it->second;
        c.sizes.erase(it);
    }
    cudaFree(p);
}

// The pool's device arrays are sections of one device arena, filled from
// one pinned staging buffer by one copy; both grow only and are kept from
// one upload to the next (a DMRG run uploads a new pool every step).
void sb_release(Ctx &c, bool free_arena) {
    c.sb = DevSb{};
    if (free_arena) {
        ctx_free(c, c.sb_arena);
        if (c.sb_stage) cudaFreeHost(c.sb_stage);
        c.sb_arena = nullptr;
        c.sb_stage = nullptr;
        c.sb_arena_cap = c.sb_stage_cap = 0;
    }
}

namespace {

constexpr int TILE = 16;
constexpr int TILE32 = 32;

// Sections of the pool's arena: each array at a 256-byte boundary (at least
// 16 bytes, so that every pointer is distinct and valid).
struct Stager {
    struct Item {
        void **dst;
        const void *src;
        size_t bytes, off;
    };
    std::vector<Item> items;
    size_t total = 0;
    template <class T>
    void add(T **dst, const std::vector<T> &v) {
        const size_t bytes = v.size() * sizeof(T);
        items.push_back({(void **)dst, (const void *)v.data(), bytes, total});
        total += (std::max<size_t>(bytes, 16) + 255) / 256 * 256;
    }
    // a section the device fills (no host source, not copied)
    template <class T>
    void add_dev(T **dst, size_t count) {
        const size_t bytes = count * sizeof(T);
        items.push_back({(void **)dst, nullptr, bytes, total});
        total += (std::max<size_t>(bytes, 16) + 255) / 256 * 256;
    }
};

// Dense sector operators from their CSR rows: one thread per row of one
// sector's H_L or H_R (rows of both sides in one launch), duplicates summed
// as the host build did; the blocks are zeroed beforehand.  FP32 copies
// follow in k_dense32.
struct DenseRows {
    const int *rowptr;      // per side: all sectors' rows, global entry offsets
    const int *col;
    const double *val;
    const int *row_sec;     // sector of each row (global row index)
    const int64_t *row_first;   // first global row of each sector
};
__global__ void __launch_bounds__(256) k_densify(DenseRows L, DenseRows R, int nrow_l, int nrow_r,
                                                  const int *__restrict__ dls, const int *__restrict__ drs,
                                                  const int64_t *__restrict__ hl_off, const int64_t *__restrict__ hr_off,
                                                  double *__restrict__ hl, double *__restrict__ hr) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= (int64_t)nrow_l + nrow_r) return;
    const bool right = t >= nrow_l;
    const DenseRows &D = right ? R : L;
    const int g = (int)(right ? t - nrow_l : t);
    const int k = D.row_sec[g];
    const int d = right ? drs[k] : dls[k];
    const int i = (int)(g - D.row_first[k]);
    double *row = (right ? hr + hr_off[k] : hl + hl_off[k]) + (int64_t)i * d;
    for (int p = D.rowptr[g]; p < D.rowptr[g + 1]; ++p) row[D.col[p]] += D.val[p];
}

__global__ void __launch_bounds__(256) k_dense32(const double *__restrict__ x, float *__restrict__ y, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        y[i] = (float)x[i];
}

int stage_commit(Ctx &c, Stager &sg) {
    // the previous upload's copy out of the staging buffer may still be in
    // flight on the stream (two uploads with no solve between them)
    NSS_CUDA_TRY(c, cudaStreamSynchronize(c.stream));
    if (c.sb_arena_cap < sg.total) {
        ctx_free(c, c.sb_arena);
        c.sb_arena = nullptr;
        c.sb_arena_cap = 0;
        const size_t cap = sg.total + sg.total / 4;   // headroom: the pool size varies from step to step
        NSS_CUDA_TRY(c, ctx_alloc(c, &c.sb_arena, cap));
        c.sb_arena_cap = cap;
    }
    if (c.sb_stage_cap < sg.total) {
        if (c.sb_stage) cudaFreeHost(c.sb_stage);
        c.sb_stage = nullptr;
        c.sb_stage_cap = 0;
        const size_t cap = sg.total + sg.total / 4;
        NSS_CUDA_TRY(c, cudaHostAlloc((void **)&c.sb_stage, cap, cudaHostAllocDefault));
        c.sb_stage_cap = cap;
    }
    // the staging copy in pieces of at most 1 MiB, spread over host threads
    struct Piece {
        char *dst;
        const char *src;
        size_t bytes;
    };
    std::vector<Piece> pieces;
    constexpr size_t PIECE = (size_t)1 << 20;
    for (const auto &it : sg.items)
        if (it.bytes && it.src)
            for (size_t o = 0; o < it.bytes; o += PIECE)
                pieces.push_back({c.sb_stage + it.off + o, (const char *)it.src + o, std::min(PIECE, it.bytes - o)});
    parallel_for((int)pieces.size(), [&](int i) { std::memcpy(pieces[i].dst, pieces[i].src, pieces[i].bytes); },
                 sg.total > ((size_t)4 << 20));
    NSS_CUDA_TRY(c, cudaMemcpyAsync(c.sb_arena, c.sb_stage, sg.total, cudaMemcpyHostToDevice, c.stream));
    for (const auto &it : sg.items) {
        *it.dst = (void *)(c.sb_arena + it.off);
        if (it.src) c.sb.h2d_bytes += (int64_t)it.bytes;
    }
    return NSS_OK;
}

// shape and row pointers always; the column of every entry unless the
// caller built the matrices itself (cols_known)
bool csr_ok(const nss_csr &m, int nrow, int ncol, bool cols_known = false) {
    if (m.nrow != nrow || m.ncol != ncol) return false;
    if (nrow == 0) return true;
    if (!m.rowptr || m.rowptr[0] != 0) return false;
    int nnz = m.rowptr[nrow];
    if (nnz < 0 || (nnz > 0 && (!m.colidx || !m.vals))) return false;
    for (int i = 0; i < nrow; ++i)
        if (m.rowptr[i + 1] < m.rowptr[i]) return false;
    if (cols_known) return true;
    for (int j = 0; j < nnz; ++j)
        if (m.colidx[j] < 0 || m.colidx[j] >= ncol) return false;
    return true;
}

// every stored value finite (a NaN or Inf operator entry would poison every
// H*psi and the Lanczos scalars without any other sign)
bool csr_finite(const nss_csr &m) {
    const int nnz = m.nrow > 0 ? m.rowptr[m.nrow] : 0;
    for (int j = 0; j < nnz; ++j)
        if (!std::isfinite(m.vals[j])) return false;
    return true;
}

}  // namespace

// Validate and copy the operator pool.  Errors mirror the reference's stop
// conditions (wrong sizes, vecDim != m_sb) as NSS_ERR_INVALID.
int sb_upload(Ctx &c, const nss_sb_desc *d, bool trusted) {
    if (!d || d->nsb <= 0 || d->tnso < 0 || !d->dls || !d->drs || !d->offset || !d->hleft ||
        !d->hright) {
        c.err = "nss_sb_upload: incomplete descriptor";
        return NSS_ERR_INVALID;
    }
    // kernels of the previous pool may still be reading the arena (a
    // batch runs several contexts' solves on one stream)
    NSS_CUDA_TRY(c, cudaDeviceSynchronize());
    sb_release(c, false);
    DevSb &s = c.sb;
    s.nsb = d->nsb;
    s.tnso = d->tnso;
    s.m_left = d->m_left;
    s.m_right = d->m_right;
    s.dls.assign(d->dls, d->dls + s.nsb);
    s.drs.assign(d->drs, d->drs + s.nsb);
    s.off.assign(d->offset, d->offset + s.nsb);
    int64_t pos = 0;
    std::map<int64_t, int> sec_at;
    for (int k = 0; k < s.nsb; ++k) {
        if (s.dls[k] <= 0 || s.drs[k] <= 0 || s.off[k] != pos) {
            c.err = "nss_sb_upload: sector dims/offsets inconsistent at sector " + std::to_string(k);
            return NSS_ERR_INVALID;
        }
        sec_at[pos] = k;
        pos += (int64_t)s.dls[k] * s.drs[k];
    }
    s.n = pos;
    // sector block maps (for the RDM)
    if (d->ai && d->bi) {
        int la = 0, lb = 0;
        for (int k = 0; k < s.nsb; ++k) {
            s.ai_off.push_back(la);
            s.bi_off.push_back(lb);
            la += s.dls[k];
            lb += s.drs[k];
        }
        s.ai_off.push_back(la);
        s.bi_off.push_back(lb);
        s.ai.assign(d->ai, d->ai + la);
        s.bi.assign(d->bi, d->bi + lb);
        for (int x : s.ai)
            if (x < 0 || x >= d->m_left) { c.err = "nss_sb_upload: ai out of range"; return NSS_ERR_INVALID; }
        for (int x : s.bi)
            if (x < 0 || x >= d->m_right) { c.err = "nss_sb_upload: bi out of range"; return NSS_ERR_INVALID; }
    }

    // dense sector operators: their CSR rows travel and the device scatters
    // them into zeroed row-major blocks (k_densify), FP32 copies after
    int64_t hl_tot = 0, hr_tot = 0, nnz_l = 0, nnz_r = 0, nrow_l = 0, nrow_r = 0;
    for (int k = 0; k < s.nsb; ++k) {
        const int dl = s.dls[k], dr = s.drs[k];
        if (!csr_ok(d->hleft[k], dl, dl, trusted) || !csr_ok(d->hright[k], dr, dr, trusted)) {
            c.err = "nss_sb_upload: Hleft/Hright shape or index error at sector " + std::to_string(k);
            return NSS_ERR_INVALID;
        }
        if (!trusted && (!csr_finite(d->hleft[k]) || !csr_finite(d->hright[k]))) {
            c.err = "nss_sb_upload: non-finite value in Hleft/Hright at sector " + std::to_string(k);
            return NSS_ERR_INVALID;
        }
        s.hl_off.push_back(hl_tot);
        s.hr_off.push_back(hr_tot);
        hl_tot += (int64_t)dl * dl;
        hr_tot += (int64_t)dr * dr;
        nnz_l += d->hleft[k].rowptr[dl];
        nnz_r += d->hright[k].rowptr[dr];
        nrow_l += dl;
        nrow_r += dr;
        s.flops_dense += 2.0 * dl * dr * ((double)dl + dr);
    }
    s.hl_off.push_back(hl_tot);
    s.hr_off.push_back(hr_tot);
    if (nnz_l > INT32_MAX || nnz_r > INT32_MAX) {
        c.err = "nss_sb_upload: more than 2^31 entries in the sector operators";
        return NSS_ERR_INVALID;
    }
    struct PackedRows {
        std::vector<int> rowptr, col, row_sec;
        std::vector<double> val;
        std::vector<int64_t> row_first;
    } pk[2];
    const bool big_pool = nnz_l + nnz_r > 100000;
    run_pair(
        [&] {
            for (int side = 0; side < 2; ++side) {
                PackedRows &P = pk[side];
                P.rowptr.reserve((size_t)(side ? nrow_r : nrow_l) + 1);
                P.rowptr.push_back(0);
                P.row_first.reserve(s.nsb);
                P.row_sec.reserve((size_t)(side ? nrow_r : nrow_l));
                int64_t rows = 0;
                for (int k = 0; k < s.nsb; ++k) {
                    const nss_csr &M = side ? d->hright[k] : d->hleft[k];
                    const int base = P.rowptr.back();
                    P.row_first.push_back(rows);
                    for (int i = 0; i < M.nrow; ++i) {
                        P.rowptr.push_back(base + M.rowptr[i + 1]);
                        P.row_sec.push_back(k);
                    }
                    rows += M.nrow;
                }
            }
        },
        [&] {
            std::vector<int64_t> at(2 * (size_t)s.nsb);
            for (int side = 0; side < 2; ++side) {
                PackedRows &P = pk[side];
                P.col.resize((size_t)(side ? nnz_r : nnz_l));
                P.val.resize((size_t)(side ? nnz_r : nnz_l));
                int64_t a = 0;
                for (int k = 0; k < s.nsb; ++k) {
                    at[(size_t)side * s.nsb + k] = a;
                    const nss_csr &M = side ? d->hright[k] : d->hleft[k];
                    a += M.rowptr[M.nrow];
                }
            }
            // the sectors' entries copied in parallel
            parallel_for(2 * s.nsb, [&](int t) {
                const int side = t / s.nsb, k = t % s.nsb;
                PackedRows &P = pk[side];
                const nss_csr &M = side ? d->hright[k] : d->hleft[k];
                const int nz = M.rowptr[M.nrow];
                const int64_t o = at[(size_t)t];
                if (nz) {
                    std::memcpy(P.col.data() + o, M.colidx, sizeof(int) * (size_t)nz);
                    std::memcpy(P.val.data() + o, M.vals, sizeof(double) * (size_t)nz);
                }
            }, big_pool, 6);
        },
        big_pool);

    // A x B terms, regrouped by output sector
    std::vector<std::vector<DevTerm>> by_out(s.nsb);
    std::vector<int> rowptr;
    std::vector<int> col;
    std::vector<double> val;
    auto push_csr = [&](const nss_csr &m) {
        int64_t at = (int64_t)rowptr.size();
        int base = (int)col.size();
        for (int i = 0; i <= m.nrow; ++i) rowptr.push_back(base + m.rowptr[i]);
        int nnz = m.rowptr[m.nrow];
        col.insert(col.end(), m.colidx, m.colidx + nnz);
        val.insert(val.end(), m.vals, m.vals + nnz);
        return at;
    };
    const int nt = s.tnso * s.nsb;
    for (int idx = 0; idx < nt; ++idx) {
        const nss_csr &A = d->a[idx], &B = d->b[idx];
        if (A.nrow == 0 || B.nrow == 0) continue;   // status=.false. -> skipped (:810)
        auto ro = sec_at.find(d->row_offset[idx]);
        auto co = sec_at.find(d->col_offset[idx]);
        if (ro == sec_at.end() || co == sec_at.end()) {
            c.err = "nss_sb_upload: Row/ColOffset not at a sector start (term " + std::to_string(idx) + ")";
            return NSS_ERR_INVALID;
        }
        int o = ro->second, q = co->second;
        if (!csr_ok(A, s.dls[o], s.dls[q], trusted) || !csr_ok(B, s.drs[o], s.drs[q], trusted)) {
            c.err = "nss_sb_upload: A/B shape or index error (term " + std::to_string(idx) + ")";
            return NSS_ERR_INVALID;
        }
        if (!trusted && (!csr_finite(A) || !csr_finite(B))) {
            c.err = "nss_sb_upload: non-finite value in A/B (term " + std::to_string(idx) + ")";
            return NSS_ERR_INVALID;
        }
        DevTerm t;
        t.out_sec = o;
        t.in_sec = q;
        t.a_nrow = A.nrow; t.a_ncol = A.ncol;
        t.b_nrow = B.nrow; t.b_ncol = B.ncol;
        t.a_rp = push_csr(A);
        t.b_rp = push_csr(B);
        by_out[o].push_back(t);
        // the reference's loop count, src/DMRG_SUPERBLOCK_SETUP.f90:819-853
        s.flops_ab += 2.0 * ((double)B.rowptr[B.nrow] * A.ncol + (double)A.rowptr[A.nrow] * B.nrow);
    }
    s.term_ptr.push_back(0);
    for (int k = 0; k < s.nsb; ++k) {
        for (auto &t : by_out[k]) s.terms.push_back(t);
        s.term_ptr.push_back((int)s.terms.size());
    }
    // tiles
    std::vector<int4> tiles;
    for (int k = 0; k < s.nsb; ++k)
        for (int r = 0; r < s.dls[k]; r += TILE)
            for (int cc = 0; cc < s.drs[k]; cc += TILE) tiles.push_back(make_int4(k, r, cc, 0));
    s.ntiles = (int)tiles.size();

    // FP32 copies for the mixed path, and its 32x32 tiles.  The FP32 A/B
    // pool drops entries below 1e-12 of the largest entry of their matrix:
    // the renormalised sign operator P carries rounding-level off-diagonal
    // entries (up to 33 per row at m=256) whose contribution (~1e-17 of the
    // result) is far below FP32 rounding, while each of them costs a gather.
    // The FP64 pool keeps every entry, as the reference does.
    std::vector<int> rowptr32, col32;
    std::vector<float> val32;
    std::vector<DevTerm> terms32 = s.terms;
    for (DevTerm &t : terms32) {
        for (int which = 0; which < 2; ++which) {
            const int64_t rp = which == 0 ? t.a_rp : t.b_rp;
            const int nrow = which == 0 ? t.a_nrow : t.b_nrow;
            double mx = 0.0;
            for (int jj = rowptr[rp]; jj < rowptr[rp + nrow]; ++jj) mx = std::max(mx, std::fabs(val[jj]));
            const int64_t at = (int64_t)rowptr32.size();
            rowptr32.push_back((int)col32.size());
            for (int i = 0; i < nrow; ++i) {
                for (int jj = rowptr[rp + i]; jj < rowptr[rp + i + 1]; ++jj)
                    if (std::fabs(val[jj]) > 1e-12 * mx) {
                        col32.push_back(col[jj]);
                        val32.push_back((float)val[jj]);
                    }
                rowptr32.push_back((int)col32.size());
            }
            if (which == 0) t.a_rp = at;
            else t.b_rp = at;
        }
    }
    // Sectors on the tensor-core GEMM (k_sector_mma.cu) get their A x B
    // terms from "terms only" CUDA-core tiles (w = 1), listed first, which
    // k_hv_fp32 runs after the GEMM and which add its two output planes.
    MmaPlan plan;
    int tc_thr = c.tc_min_dl, tc_bn = c.mma_bn;
    c.tune_cand = -1;
    if (c.tc_auto) tune_choose(c, s, &tc_thr, &tc_bn);
    int nsm = 0;
    NSS_CUDA_TRY(c, cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c.device));
    mma_layout(s, tc_thr, tc_bn, c.mma_split, nsm, plan);
    std::vector<char> on_tc(s.nsb, 0);
    for (int k : plan.sectors) on_tc[k] = 1;
    std::vector<int4> tiles32;
    for (int k = 0; k < s.nsb; ++k)
        if (on_tc[k])
            for (int r = 0; r < s.dls[k]; r += TILE32)
                for (int cc = 0; cc < s.drs[k]; cc += TILE32) tiles32.push_back(make_int4(k, r, cc, 1));
    for (int k = 0; k < s.nsb; ++k)
        if (!on_tc[k])
            for (int r = 0; r < s.dls[k]; r += TILE32)
                for (int cc = 0; cc < s.drs[k]; cc += TILE32) tiles32.push_back(make_int4(k, r, cc, 0));
    // work items of the persistent kernel: 32x32 tiles of every sector,
    // split into H_L, H_R and A x B parts when a K loop is long
    std::vector<int4> items32;
    for (int k = 0; k < s.nsb; ++k) {
        const bool split = std::max(s.dls[k], s.drs[k]) > 64;
        for (int r = 0; r < s.dls[k]; r += TILE32)
            for (int cc = 0; cc < s.drs[k]; cc += TILE32) {
                if (split) {
                    items32.push_back(make_int4(k, r, cc, HV_LEFT));
                    items32.push_back(make_int4(k, r, cc, HV_RIGHT));
                    if (s.term_ptr[k + 1] > s.term_ptr[k]) items32.push_back(make_int4(k, r, cc, HV_TERMS));
                } else {
                    items32.push_back(make_int4(k, r, cc, HV_FULL));
                }
            }
    }
    // longest first, so the split halves start at once
    std::stable_sort(items32.begin(), items32.end(), [&](const int4 &x, const int4 &y) {
        auto cost = [&](const int4 &t) {
            const int dl = s.dls[t.x], dr = s.drs[t.x];
            return t.w == HV_LEFT ? dl : (t.w == HV_RIGHT ? dr : (t.w == HV_TERMS ? 48 : dl + dr + 48));
        };
        return cost(x) > cost(y);
    });
    // A x B tables of the items that carry terms: for each term of the
    // sector, the (column, value) of the tile's 32 rows of A and 32 columns
    // of B in the FP32 pool (-1: empty row); items with a row of several
    // elements keep -1 and use the CSR loop
    std::vector<int> item_ell(items32.size(), -1);
    std::vector<int2> ell;
    for (size_t ii = 0; ii < items32.size(); ++ii) {
        const int4 it = items32[ii];
        if (it.w != HV_FULL && it.w != HV_TERMS) continue;
        const int k = it.x, dl = s.dls[k], dr = s.drs[k];
        const size_t base = ell.size();
        bool ok = true;
        for (int ti = s.term_ptr[k]; ti < s.term_ptr[k + 1] && ok; ++ti) {
            const DevTerm &tm = terms32[ti];
            for (int side = 0; side < 2 && ok; ++side) {
                const int64_t rp = side == 0 ? tm.a_rp : tm.b_rp;
                const int lim = side == 0 ? dl : dr, first = side == 0 ? it.y : it.z;
                for (int r = 0; r < 32; ++r) {
                    const int g = first + r;
                    int2 e = make_int2(-1, 0);
                    if (g < lim) {
                        const int p0 = rowptr32[rp + g], p1 = rowptr32[rp + g + 1];
                        if (p1 - p0 > 1) { ok = false; break; }
                        if (p1 > p0) {
                            float fv = val32[p0];
                            int bits;
                            std::memcpy(&bits, &fv, sizeof(bits));
                            e = make_int2(col32[p0], bits);
                        }
                    }
                    ell.push_back(e);
                }
            }
        }
        if (ok) item_ell[ii] = (int)base;
        else ell.resize(base);
    }
    if (ell.empty()) ell.push_back(make_int2(-1, 0));
    std::vector<int4> term_hdr(std::max<size_t>(terms32.size(), 1), make_int4(0, 0, 0, 0));
    for (size_t ti = 0; ti < terms32.size(); ++ti) {
        const int64_t of = s.off[terms32[ti].in_sec];
        term_hdr[ti] = make_int4((int)(uint32_t)(of & 0xffffffff), (int)(of >> 32), s.drs[terms32[ti].in_sec], 0);
    }
    std::vector<ItemRec> recs(items32.size());
    for (size_t ii = 0; ii < items32.size(); ++ii) {
        const int4 it = items32[ii];
        const int k = it.x;
        const int64_t of = s.off[k], hlo = s.hl_off[k], hro = s.hr_off[k];
        auto lo = [](int64_t x) { return (int)(uint32_t)(x & 0xffffffff); };
        auto hi = [](int64_t x) { return (int)(x >> 32); };
        recs[ii].a = it;
        recs[ii].b = make_int4(s.dls[k], s.drs[k], s.term_ptr[k], s.term_ptr[k + 1]);
        recs[ii].c = make_int4(lo(of), hi(of), item_ell[ii], 0);
        recs[ii].d = make_int4(lo(hlo), hi(hlo), lo(hro), hi(hro));
    }
    s.nitems32 = (int)items32.size();
    s.item_cost.resize(items32.size());
    for (size_t ii = 0; ii < items32.size(); ++ii) {
        const int4 t = items32[ii];
        const int dl = s.dls[t.x], dr = s.drs[t.x];
        s.item_cost[ii] = t.w == HV_LEFT ? dl : (t.w == HV_RIGHT ? dr : (t.w == HV_TERMS ? 48 : dl + dr + 48));
    }
    s.ntiles32 = (int)tiles32.size();
    std::vector<int> tc_err(1, 0);

    Stager sg;
    sg.add_dev(&s.d_hl32, (size_t)hl_tot);
    sg.add_dev(&s.d_hr32, (size_t)hr_tot);
    sg.add(&s.d_ab_val32, val32);
    sg.add(&s.d_ab_rowptr32, rowptr32);
    sg.add(&s.d_ab_col32, col32);
    sg.add(&s.d_terms32, terms32);
    sg.add(&s.d_tiles32, tiles32);
    sg.add(&s.d_items32, recs);
    sg.add(&s.d_item_ell, item_ell);
    sg.add(&s.d_ell, ell);
    sg.add(&s.d_term_hdr, term_hdr);
    sg.add(&s.d_tc_err, tc_err);
    sg.add_dev(&s.d_mma_pool, (size_t)(plan.items.empty() ? 0 : plan.plane_rows * MM_KC));
    sg.add_dev(&s.d_mma_out, (size_t)(plan.items.empty() ? 0 : plan.nplanes * s.n));
    sg.add(&s.d_mma_items, plan.items);
    sg.add(&s.d_mma_rng, plan.rng);
    sg.add(&s.d_mma_wt, plan.wt);
    sg.add(&s.d_mma_sec, plan.ps);
    sg.add(&s.d_dls, s.dls);
    sg.add(&s.d_drs, s.drs);
    sg.add(&s.d_off, s.off);
    sg.add(&s.d_hl_off, s.hl_off);
    sg.add(&s.d_hr_off, s.hr_off);
    sg.add_dev(&s.d_hl, (size_t)hl_tot);
    sg.add_dev(&s.d_hr, (size_t)hr_tot);
    DenseRows dr_dev[2];
    for (int side = 0; side < 2; ++side) {
        sg.add((int **)&dr_dev[side].rowptr, pk[side].rowptr);
        sg.add((int **)&dr_dev[side].col, pk[side].col);
        sg.add((double **)&dr_dev[side].val, pk[side].val);
        sg.add((int **)&dr_dev[side].row_sec, pk[side].row_sec);
        sg.add((int64_t **)&dr_dev[side].row_first, pk[side].row_first);
    }
    sg.add(&s.d_term_ptr, s.term_ptr);
    sg.add(&s.d_terms, s.terms);
    sg.add(&s.d_ab_rowptr, rowptr);
    sg.add(&s.d_ab_col, col);
    sg.add(&s.d_ab_val, val);
    sg.add(&s.d_tiles, tiles);
    int rc;
    if ((rc = stage_commit(c, sg))) return rc;
    NSS_CUDA_TRY(c, cudaMemsetAsync(s.d_hl, 0, (size_t)hl_tot * sizeof(double), c.stream));
    NSS_CUDA_TRY(c, cudaMemsetAsync(s.d_hr, 0, (size_t)hr_tot * sizeof(double), c.stream));
    {
        const int64_t nr = nrow_l + nrow_r;
        c.launches += 3;
        k_densify<<<(unsigned)((nr + 255) / 256), 256, 0, c.stream>>>(dr_dev[0], dr_dev[1], (int)nrow_l, (int)nrow_r,
                                                                      s.d_dls, s.d_drs, s.d_hl_off, s.d_hr_off,
                                                                      s.d_hl, s.d_hr);
        k_dense32<<<608, 256, 0, c.stream>>>(s.d_hl, s.d_hl32, hl_tot);
        k_dense32<<<608, 256, 0, c.stream>>>(s.d_hr, s.d_hr32, hr_tot);
        NSS_CUDA_TRY(c, cudaGetLastError());
    }
    if ((rc = mma_finish(c, plan))) return rc;
    NSS_CUDA_TRY(c, cudaStreamSynchronize(c.stream));
    static std::atomic<uint64_t> g_gen{0};
    s.gen = ++g_gen;
    s.valid = true;
    return NSS_OK;
}

// One CTA per 16x16 output tile; thread (ty,tx) owns W_k[row0+ty][col0+tx].
// GB300 issues FP64 at about 1/64 of its FP32 rate, so this kernel is bound
// by the FP64 pipe; the operand tiles are staged in shared memory only to
// keep the loads coalesced.
__global__ void __launch_bounds__(256) k_hv_fp64(
    const double *__restrict__ v, double *__restrict__ hv, const int4 *__restrict__ tiles,
    const int *__restrict__ dls, const int *__restrict__ drs, const int64_t *__restrict__ off,
    const double *__restrict__ hlp, const int64_t *__restrict__ hl_off,
    const double *__restrict__ hrp, const int64_t *__restrict__ hr_off,
    const int *__restrict__ term_ptr, const DevTerm *__restrict__ terms,
    const int *__restrict__ ab_rp, const int *__restrict__ ab_col, const double *__restrict__ ab_val,
    const int *stop) {
    if (stop && *stop) return;   // the Lanczos loop has already finished
    __shared__ double sa[TILE][33];
    __shared__ double sb[32][TILE + 1];
    const int4 t = tiles[blockIdx.x];
    const int k = t.x, row0 = t.y, col0 = t.z;
    const int dl = dls[k], dr = drs[k];
    const int64_t o = off[k];
    const double *W = v + o;
    const double *HL = hlp + hl_off[k];
    const double *HR = hrp + hr_off[k];
    const int tid = threadIdx.x, ty = tid / TILE, tx = tid % TILE;
    const int il = row0 + ty, ir = col0 + tx;
    double acc = 0.0;

    // H_L W : sum_j HL[il][j] W[j][ir]   (the H^L x 1^R loop, :784-796)
    for (int j0 = 0; j0 < dl; j0 += 32) {
        for (int e = tid; e < TILE * 32; e += 256) {
            int r = e / 32, cc = e % 32;
            int gi = row0 + r, gj = j0 + cc;
            sa[r][cc] = (gi < dl && gj < dl) ? HL[(int64_t)gi * dl + gj] : 0.0;
        }
        for (int e = tid; e < 32 * TILE; e += 256) {
            int r = e / TILE, cc = e % TILE;
            int gj = j0 + r, gc = col0 + cc;
            sb[r][cc] = (gj < dl && gc < dr) ? W[(int64_t)gj * dr + gc] : 0.0;
        }
        __syncthreads();
#pragma unroll 8
        for (int j = 0; j < 32; ++j) acc = fma(sa[ty][j], sb[j][tx], acc);
        __syncthreads();
    }
    // W H_R^T : sum_j W[il][j] HR[ir][j]   (the 1^L x H^R loop, :767-779)
    for (int j0 = 0; j0 < dr; j0 += 32) {
        for (int e = tid; e < TILE * 32; e += 256) {
            int r = e / 32, cc = e % 32;
            int gi = row0 + r, gj = j0 + cc;
            sa[r][cc] = (gi < dl && gj < dr) ? W[(int64_t)gi * dr + gj] : 0.0;
        }
        for (int e = tid; e < 32 * TILE; e += 256) {
            int r = e / TILE, cc = e % TILE;   // sb[j][x] = HR[col0+x][j0+j]
            int gr = col0 + cc, gj = j0 + r;
            sb[r][cc] = (gr < dr && gj < dr) ? HR[(int64_t)gr * dr + gj] : 0.0;
        }
        __syncthreads();
#pragma unroll 8
        for (int j = 0; j < 32; ++j) acc = fma(sa[ty][j], sb[j][tx], acc);
        __syncthreads();
    }
    // sum_t A W_q B^T : Out[ai][bi] += A[ai][aj] B[bi][bj] W_q[aj][bj] (:808-857)
    __shared__ AbStage<double, TILE, TILE> S;
    const bool in = il < dl && ir < dr;
    for (int tb = term_ptr[k]; tb < term_ptr[k + 1]; tb += AB_MAXT) {
        const int nt = min(AB_MAXT, term_ptr[k + 1] - tb);
        ab_stage<double, TILE, TILE>(S, v, tb, nt, row0, col0, dl, dr, drs, off, terms, ab_rp, ab_col, ab_val,
                                     threadIdx.x, blockDim.x, CtaSync{});
        if (in) {
            if (!S.multi) {
                for (int tt = 0; tt < nt; ++tt) {
                    const int aj = S.ac[tt][ty], bj = S.bc[tt][tx];
                    if (aj >= 0 && bj >= 0)
                        acc = fma(S.av[tt][ty] * S.bv[tt][tx], S.wq[tt][(int64_t)aj * S.drq[tt] + bj], acc);
                }
            } else {
                acc = ab_csr<double>(acc, v, tb, nt, il, ir, drs, off, terms, ab_rp, ab_col, ab_val);
            }
        }
        __syncthreads();
    }
    if (in) hv[o + (int64_t)il * dr + ir] = acc;
}

// FP32 variant for the mixed-precision Lanczos phase: 32x32 output tiles,
// each thread owns rows {ty, ty+16} x cols {tx, tx+16}; FP32 operands and
// accumulation (GB300 issues FP32 FMAs 64x faster than FP64 ones).
__global__ void __launch_bounds__(256) k_hv_fp32(const float *__restrict__ v, float *__restrict__ hv,
                                                 const int4 *__restrict__ tiles, Hv32Ops op, const int *stop) {
    if (stop && *stop) return;   // the Lanczos loop has already finished
    __shared__ Tile32Smem sm;
    hv32_tile(tiles[blockIdx.x], v, hv, op, sm, threadIdx.x, CtaSync{}, 1.0f);
}

Hv32Ops hv32_ops(const DevSb &s) {
    Hv32Ops op;
    op.dls = s.d_dls;
    op.drs = s.d_drs;
    op.off = s.d_off;
    op.hl = s.d_hl32;
    op.hl_off = s.d_hl_off;
    op.hr = s.d_hr32;
    op.hr_off = s.d_hr_off;
    op.term_ptr = s.d_term_ptr;
    op.terms = s.d_terms32;
    op.ab_rp = s.d_ab_rowptr32;
    op.ab_col = s.d_ab_col32;
    op.ab_val = s.d_ab_val32;
    op.item_ell = s.d_item_ell;
    op.ell = s.d_ell;
    op.term_hdr = s.d_term_hdr;
    op.tc = s.mma_nitems ? s.d_mma_out : nullptr;
    op.tcn = s.mma_nitems ? s.mma_nplanes : 0;
    op.tcs = s.n;
    return op;
}

// hv[i] += the tensor-core planes' sum at i (plane 0 first; zero outside the
// tensor-core sectors)
__global__ void __launch_bounds__(256) k_add_planes(float *__restrict__ hv, const float *__restrict__ planes,
                                                    int64_t n, int np, const int *stop) {
    if (stop && *stop) return;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        float d = planes[i];
        for (int p = 1; p < np; ++p) d += planes[(int64_t)p * n + i];
        hv[i] += d;
    }
}

int hv_device_fp32(Ctx &c, const float *d_v, float *d_hv, const int *stop) {
    DevSb &s = c.sb;
    if (!s.valid) {
        c.err = "nss_hv: no superblock uploaded";
        return NSS_ERR_STATE;
    }
    if (s.mma_nitems == 0) {
        if (s.ntiles32 > 0) {
            k_hv_fp32<<<s.ntiles32, 256, 0, c.stream>>>(d_v, d_hv, s.d_tiles32, hv32_ops(s), stop);
            c.launches += 1;
            NSS_CUDA_TRY(c, cudaGetLastError());
        }
        return NSS_OK;
    }
    // tensor-core sectors: the CUDA-core tiles (their A x B terms, and the
    // small sectors) run on a side stream beside the W packing and the GEMM;
    // the GEMM's planes are added when both are done
    if (!c.hv_side) {
        NSS_CUDA_TRY(c, cudaStreamCreateWithFlags(&c.hv_side, cudaStreamNonBlocking));
        NSS_CUDA_TRY(c, cudaEventCreateWithFlags(&c.hv_fork, cudaEventDisableTiming));
        NSS_CUDA_TRY(c, cudaEventCreateWithFlags(&c.hv_join, cudaEventDisableTiming));
    }
    NSS_CUDA_TRY(c, cudaEventRecord(c.hv_fork, c.stream));
    NSS_CUDA_TRY(c, cudaStreamWaitEvent(c.hv_side, c.hv_fork, 0));
    if (s.ntiles32 > 0) {
        Hv32Ops op = hv32_ops(s);
        op.tc = nullptr;   // the planes come afterwards
        k_hv_fp32<<<s.ntiles32, 256, 0, c.hv_side>>>(d_v, d_hv, s.d_tiles32, op, stop);
        c.launches += 1;
    }
    NSS_CUDA_TRY(c, cudaEventRecord(c.hv_join, c.hv_side));
    if (int rc = hv_device_mma(c, d_v, stop)) return rc;
    NSS_CUDA_TRY(c, cudaStreamWaitEvent(c.stream, c.hv_join, 0));
    int nsm = 0;
    NSS_CUDA_TRY(c, cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c.device));
    k_add_planes<<<(unsigned)std::min<int64_t>(4 * nsm, (s.n + 255) / 256), 256, 0, c.stream>>>(
        d_hv, s.d_mma_out, s.n, s.mma_nplanes, stop);
    c.launches += 1;
    NSS_CUDA_TRY(c, cudaGetLastError());
    return NSS_OK;
}

int hv_device(Ctx &c, const double *d_v, double *d_hv, const int *stop) {
    DevSb &s = c.sb;
    if (!s.valid) {
        c.err = "nss_hv: no superblock uploaded";
        return NSS_ERR_STATE;
    }
    k_hv_fp64<<<s.ntiles, 256, 0, c.stream>>>(d_v, d_hv, s.d_tiles, s.d_dls, s.d_drs, s.d_off, s.d_hl,
                                              s.d_hl_off, s.d_hr, s.d_hr_off, s.d_term_ptr, s.d_terms,
                                              s.d_ab_rowptr, s.d_ab_col, s.d_ab_val, stop);
    c.launches += 1;
    NSS_CUDA_TRY(c, cudaGetLastError());
    return NSS_OK;
}

}  // namespace nss
