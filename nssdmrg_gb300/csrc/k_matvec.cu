// Superblock upload and the direct H_sb * psi product (plain FP64 path).
//
// Restates spMatVec_direct_main (src/DMRG_SUPERBLOCK_SETUP.f90:740-865) as one
// kernel over output tiles.  For output sector k, with W_k the row-major
// [Dl x Dr] view of the sector (i = ir + il*Dr + Offset, :770),
//     Out_k = H_L(k) W_k + W_k H_R(k)^T + sum_t A_t W_q(t) B_t^T,
// where the last sum runs over the terms whose RowOffset is sector k
// (:808-857, regrouped by output sector so each tile has one writer).
#include "device.cuh"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>

namespace nss {

int g_tc_min_dl = [] {
    const char *e = std::getenv("NSS_TC");
    return (e && e[0] == '0') ? 0 : 64;
}();

void ctx_free(Ctx &c, void *p) {
    if (!p) return;
    auto it = c.sizes.find(p);
    if (it != c.sizes.end()) {
        c.used -= it->second;
        c.sizes.erase(it);
    }
    cudaFree(p);
}

void sb_release(Ctx &c) {
    DevSb &s = c.sb;
    void *ptrs[] = {s.d_dls, s.d_drs, s.d_off, s.d_hl_off, s.d_hr_off, s.d_hl, s.d_hr,
                    s.d_term_ptr, s.d_terms, s.d_ab_rowptr, s.d_ab_col, s.d_ab_val,
                    s.d_tiles, s.d_hl32, s.d_hr32, s.d_ab_val32, s.d_tiles32, s.d_tiles_tc, s.d_tc_err,
                    s.d_ab_rowptr32, s.d_ab_col32, s.d_terms32};
    for (void *p : ptrs) ctx_free(c, p);
    s = DevSb{};
}

namespace {

constexpr int TILE = 16;
constexpr int TILE32 = 32;
constexpr int TC_ROWS = 128, TC_COLS = 64;   // k_hv_tc tile

template <class T>
int upload_vec(Ctx &c, T **dst, const std::vector<T> &src) {
    NSS_CUDA_TRY(c, ctx_alloc(c, dst, src.size()));
    c.sb.h2d_bytes += (int64_t)(src.size() * sizeof(T));
    if (!src.empty())
        NSS_CUDA_TRY(c, cudaMemcpyAsync(*dst, src.data(), src.size() * sizeof(T),
                                        cudaMemcpyHostToDevice, c.stream));
    return NSS_OK;
}

bool csr_ok(const nss_csr &m, int nrow, int ncol) {
    if (m.nrow != nrow || m.ncol != ncol) return false;
    if (nrow == 0) return true;
    if (!m.rowptr || m.rowptr[0] != 0) return false;
    int nnz = m.rowptr[nrow];
    if (nnz < 0 || (nnz > 0 && (!m.colidx || !m.vals))) return false;
    for (int i = 0; i < nrow; ++i)
        if (m.rowptr[i + 1] < m.rowptr[i]) return false;
    for (int j = 0; j < nnz; ++j)
        if (m.colidx[j] < 0 || m.colidx[j] >= ncol) return false;
    return true;
}

}  // namespace

// Validate and copy the operator pool.  Errors mirror the reference's stop
// conditions (wrong sizes, vecDim != m_sb) as NSS_ERR_INVALID.
int sb_upload(Ctx &c, const nss_sb_desc *d) {
    if (!d || d->nsb <= 0 || d->tnso < 0 || !d->dls || !d->drs || !d->offset || !d->hleft ||
        !d->hright) {
        c.err = "nss_sb_upload: incomplete descriptor";
        return NSS_ERR_INVALID;
    }
    sb_release(c);
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

    // dense sector operators
    std::vector<double> hl, hr;
    for (int k = 0; k < s.nsb; ++k) {
        const int dl = s.dls[k], dr = s.drs[k];
        if (!csr_ok(d->hleft[k], dl, dl) || !csr_ok(d->hright[k], dr, dr)) {
            c.err = "nss_sb_upload: Hleft/Hright shape or index error at sector " + std::to_string(k);
            return NSS_ERR_INVALID;
        }
        s.hl_off.push_back((int64_t)hl.size());
        s.hr_off.push_back((int64_t)hr.size());
        size_t bl = hl.size(), br = hr.size();
        hl.resize(bl + (size_t)dl * dl, 0.0);
        hr.resize(br + (size_t)dr * dr, 0.0);
        const nss_csr &L = d->hleft[k], &R = d->hright[k];
        for (int i = 0; i < dl; ++i)
            for (int jj = L.rowptr[i]; jj < L.rowptr[i + 1]; ++jj) hl[bl + (size_t)i * dl + L.colidx[jj]] += L.vals[jj];
        for (int i = 0; i < dr; ++i)
            for (int jj = R.rowptr[i]; jj < R.rowptr[i + 1]; ++jj) hr[br + (size_t)i * dr + R.colidx[jj]] += R.vals[jj];
        s.flops_dense += 2.0 * dl * dr * ((double)dl + dr);
    }
    s.hl_off.push_back((int64_t)hl.size());
    s.hr_off.push_back((int64_t)hr.size());

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
        if (!csr_ok(A, s.dls[o], s.dls[q]) || !csr_ok(B, s.drs[o], s.drs[q])) {
            c.err = "nss_sb_upload: A/B shape or index error (term " + std::to_string(idx) + ")";
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
    std::vector<float> hl32(hl.begin(), hl.end()), hr32(hr.begin(), hr.end());
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
    // Sectors on the tensor-core kernel get their A x B terms from "terms
    // only" CUDA-core tiles (w = 1), listed first: k_hv_fp32 writes those
    // terms to H psi and k_hv_tc, launched after it, adds its dense products.
    std::vector<int4> tiles32, tiles_tc;
    for (int k = 0; k < s.nsb; ++k) {
        if (g_tc_min_dl > 0 && s.dls[k] >= g_tc_min_dl) {
            for (int r = 0; r < s.dls[k]; r += TC_ROWS)
                for (int cc = 0; cc < s.drs[k]; cc += TC_COLS) tiles_tc.push_back(make_int4(k, r, cc, 0));
            for (int r = 0; r < s.dls[k]; r += TILE32)
                for (int cc = 0; cc < s.drs[k]; cc += TILE32) tiles32.push_back(make_int4(k, r, cc, 1));
        }
    }
    for (int k = 0; k < s.nsb; ++k) {
        if (g_tc_min_dl > 0 && s.dls[k] >= g_tc_min_dl) {
            continue;
        } else {
            for (int r = 0; r < s.dls[k]; r += TILE32)
                for (int cc = 0; cc < s.drs[k]; cc += TILE32) tiles32.push_back(make_int4(k, r, cc, 0));
        }
    }
    s.ntiles32 = (int)tiles32.size();
    s.ntiles_tc = (int)tiles_tc.size();
    std::vector<int> tc_err(1, 0);

    int rc;
    if ((rc = upload_vec(c, &s.d_hl32, hl32)) || (rc = upload_vec(c, &s.d_hr32, hr32)) ||
        (rc = upload_vec(c, &s.d_ab_val32, val32)) || (rc = upload_vec(c, &s.d_ab_rowptr32, rowptr32)) ||
        (rc = upload_vec(c, &s.d_ab_col32, col32)) || (rc = upload_vec(c, &s.d_terms32, terms32)) ||
        (rc = upload_vec(c, &s.d_tiles32, tiles32)) ||
        (rc = upload_vec(c, &s.d_tiles_tc, tiles_tc)) || (rc = upload_vec(c, &s.d_tc_err, tc_err)))
        return rc;
    if ((rc = upload_vec(c, &s.d_dls, s.dls)) || (rc = upload_vec(c, &s.d_drs, s.drs)) ||
        (rc = upload_vec(c, &s.d_off, s.off)) || (rc = upload_vec(c, &s.d_hl_off, s.hl_off)) ||
        (rc = upload_vec(c, &s.d_hr_off, s.hr_off)) || (rc = upload_vec(c, &s.d_hl, hl)) ||
        (rc = upload_vec(c, &s.d_hr, hr)) || (rc = upload_vec(c, &s.d_term_ptr, s.term_ptr)) ||
        (rc = upload_vec(c, &s.d_terms, s.terms)) || (rc = upload_vec(c, &s.d_ab_rowptr, rowptr)) ||
        (rc = upload_vec(c, &s.d_ab_col, col)) || (rc = upload_vec(c, &s.d_ab_val, val)) ||
        (rc = upload_vec(c, &s.d_tiles, tiles)))
        return rc;
    NSS_CUDA_TRY(c, cudaStreamSynchronize(c.stream));
    s.valid = true;
    return NSS_OK;
}

// One CTA per 16x16 output tile; thread (ty,tx) owns W_k[row0+ty][col0+tx].
// GB300 issues FP64 at about 1/64 of its FP32 rate, so this kernel is bound
// by the FP64 pipe; the operand tiles are staged in shared memory only to
// keep the loads coalesced.
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

// stage terms [tb, tb+nt) for rows row0.. and columns col0..; ends with a barrier
template <class V, int TR, int TC>
__device__ __forceinline__ void ab_stage(AbStage<V, TR, TC> &S, const V *__restrict__ v, int tb, int nt, int row0,
                                         int col0, int dl, int dr, const int *__restrict__ drs,
                                         const int64_t *__restrict__ off, const DevTerm *__restrict__ terms,
                                         const int *__restrict__ ab_rp, const int *__restrict__ ab_col,
                                         const V *__restrict__ ab_val) {
    if (threadIdx.x == 0) S.multi = 0;
    __syncthreads();
    for (int e = threadIdx.x; e < nt * (TR + TC); e += blockDim.x) {
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
    __syncthreads();
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
        ab_stage<double, TILE, TILE>(S, v, tb, nt, row0, col0, dl, dr, drs, off, terms, ab_rp, ab_col, ab_val);
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
__global__ void __launch_bounds__(256) k_hv_fp32(
    const float *__restrict__ v, float *__restrict__ hv, const int4 *__restrict__ tiles,
    const int *__restrict__ dls, const int *__restrict__ drs, const int64_t *__restrict__ off,
    const float *__restrict__ hlp, const int64_t *__restrict__ hl_off,
    const float *__restrict__ hrp, const int64_t *__restrict__ hr_off,
    const int *__restrict__ term_ptr, const DevTerm *__restrict__ terms,
    const int *__restrict__ ab_rp, const int *__restrict__ ab_col, const float *__restrict__ ab_val,
    const int *stop) {
    if (stop && *stop) return;   // the Lanczos loop has already finished
    __shared__ float sa[TILE32][33];
    __shared__ float sb[32][TILE32 + 1];
    const int4 t = tiles[blockIdx.x];
    const int k = t.x, row0 = t.y, col0 = t.z;
    const int dl = dls[k], dr = drs[k];
    const int64_t o = off[k];
    const float *W = v + o;
    const float *HL = hlp + hl_off[k];
    const float *HR = hrp + hr_off[k];
    const int tid = threadIdx.x, ty = tid / 16, tx = tid % 16;
    float acc[2][2] = {{0.f, 0.f}, {0.f, 0.f}};
    // a "terms only" tile (t.w = 1) skips the two dense products
    const int kdl = (t.w & 1) ? 0 : dl, kdr = (t.w & 1) ? 0 : dr;
    // H_L W
    for (int j0 = 0; j0 < kdl; j0 += 32) {
        for (int e = tid; e < TILE32 * 32; e += 256) {
            const int r = e / 32, cc = e % 32;
            const int gi = row0 + r, gj = j0 + cc;
            sa[r][cc] = (gi < dl && gj < dl) ? HL[(int64_t)gi * dl + gj] : 0.f;
            const int gj2 = j0 + r, gc = col0 + cc;
            sb[r][cc] = (gj2 < dl && gc < dr) ? W[(int64_t)gj2 * dr + gc] : 0.f;
        }
        __syncthreads();
#pragma unroll 8
        for (int j = 0; j < 32; ++j) {
            const float a0 = sa[ty][j], a1 = sa[ty + 16][j], b0 = sb[j][tx], b1 = sb[j][tx + 16];
            acc[0][0] = fmaf(a0, b0, acc[0][0]);
            acc[0][1] = fmaf(a0, b1, acc[0][1]);
            acc[1][0] = fmaf(a1, b0, acc[1][0]);
            acc[1][1] = fmaf(a1, b1, acc[1][1]);
        }
        __syncthreads();
    }
    // W H_R^T
    for (int j0 = 0; j0 < kdr; j0 += 32) {
        for (int e = tid; e < TILE32 * 32; e += 256) {
            const int r = e / 32, cc = e % 32;
            const int gi = row0 + r, gj = j0 + cc;
            sa[r][cc] = (gi < dl && gj < dr) ? W[(int64_t)gi * dr + gj] : 0.f;
            const int gr = col0 + r;                 // sb[j][x] = HR[col0+x][j0+j]
            sb[cc][r] = (gr < dr && gj < dr) ? HR[(int64_t)gr * dr + gj] : 0.f;
        }
        __syncthreads();
#pragma unroll 8
        for (int j = 0; j < 32; ++j) {
            const float a0 = sa[ty][j], a1 = sa[ty + 16][j], b0 = sb[j][tx], b1 = sb[j][tx + 16];
            acc[0][0] = fmaf(a0, b0, acc[0][0]);
            acc[0][1] = fmaf(a0, b1, acc[0][1]);
            acc[1][0] = fmaf(a1, b0, acc[1][0]);
            acc[1][1] = fmaf(a1, b1, acc[1][1]);
        }
        __syncthreads();
    }
    // A x B terms, staged per batch of terms (see ab_stage)
    __shared__ AbStage<float, TILE32, TILE32> S;
    for (int tb = term_ptr[k]; tb < term_ptr[k + 1]; tb += AB_MAXT) {
        const int nt = min(AB_MAXT, term_ptr[k + 1] - tb);
        ab_stage<float, TILE32, TILE32>(S, v, tb, nt, row0, col0, dl, dr, drs, off, terms, ab_rp, ab_col, ab_val);
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
                        acc[rr][cc] = ab_csr<float>(acc[rr][cc], v, tb, nt, il, ir, drs, off, terms, ab_rp, ab_col,
                                                    ab_val);
                }
        }
        __syncthreads();
    }
    for (int rr = 0; rr < 2; ++rr)
        for (int cc = 0; cc < 2; ++cc) {
            const int il = row0 + ty + 16 * rr, ir = col0 + tx + 16 * cc;
            if (il < dl && ir < dr) hv[o + (int64_t)il * dr + ir] = acc[rr][cc];
        }
}

int hv_device_fp32(Ctx &c, const float *d_v, float *d_hv, const int *stop) {
    DevSb &s = c.sb;
    if (!s.valid) {
        c.err = "nss_hv: no superblock uploaded";
        return NSS_ERR_STATE;
    }
    if (s.ntiles32 > 0) {
        k_hv_fp32<<<s.ntiles32, 256, 0, c.stream>>>(d_v, d_hv, s.d_tiles32, s.d_dls, s.d_drs, s.d_off, s.d_hl32,
                                                    s.d_hl_off, s.d_hr32, s.d_hr_off, s.d_term_ptr, s.d_terms32,
                                                    s.d_ab_rowptr32, s.d_ab_col32, s.d_ab_val32, stop);
        c.launches += 1;
        NSS_CUDA_TRY(c, cudaGetLastError());
    }
    return hv_device_tc(c, d_v, d_hv, stop);
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
