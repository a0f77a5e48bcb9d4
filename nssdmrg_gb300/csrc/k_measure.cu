// Block-operator expectation values on the superblock: OdotV_direct and
// Average_Op_dmrg (src/DMRG_MEASURE.f90:595-705).
//
// O acts on one side of the superblock, given per sector as O_k, the block
// operator filtered to the sector's left (label 'l') or right ('r') states
// (sp_filter with LI/RI, :619-624).  With Psi_k the row-major Dl x Dr
// view of sector k at Offset(k) (left state slow, as in H*psi):
//     'l':  (O v)(il, ir) = sum_jl O_k(il, jl) Psi_k(jl, ir)    (:672-683)
//     'r':  (O v)(il, ir) = sum_jr O_k(ir, jr) Psi_k(il, jr)    (:685-697)
// and <O> = v . (O v) (:635-641).  One thread per superblock element over
// chunks of 256 elements of one sector: on the left side a warp reads
// consecutive ir of the same rows jl (coalesced), on the right side it
// gathers within one row il of Psi.  The dot product is reduced per CTA and
// the CTA sums are added in a fixed order by one more CTA, so the value does
// not depend on scheduling.
#include "device.cuh"

#include <algorithm>
#include <cstring>

namespace nss {

namespace {

constexpr int MS_THREADS = 256;

// items: (sector, first element of the chunk); rp_off[k]: sector k's row
// pointers in rowptr (already offset into col/val)
__global__ void __launch_bounds__(MS_THREADS) k_odotv(const double *__restrict__ v, double *__restrict__ ov,
                                                       const int2 *__restrict__ items, const int *__restrict__ dls,
                                                       const int *__restrict__ drs, const int64_t *__restrict__ off,
                                                       const int64_t *__restrict__ rp_off,
                                                       const int *__restrict__ rowptr, const int *__restrict__ col,
                                                       const double *__restrict__ val, int right,
                                                       double *__restrict__ part) {
    __shared__ double red[MS_THREADS / 32];
    const int2 it = items[blockIdx.x];
    const int k = it.x, dl = dls[k], dr = drs[k];
    const int64_t e = (int64_t)it.y + threadIdx.x;
    const double *W = v + off[k];
    double dotp = 0.0;
    if (e < (int64_t)dl * dr) {
        const int il = (int)(e / dr), ir = (int)(e % dr);
        const int *rp = rowptr + rp_off[k];
        const int row = right ? ir : il;
        double acc = 0.0;
        for (int p = rp[row]; p < rp[row + 1]; ++p) {
            const int j = col[p];
            acc = fma(val[p], right ? W[(int64_t)il * dr + j] : W[(int64_t)j * dr + ir], acc);
        }
        if (ov) ov[off[k] + e] = acc;
        dotp = acc * W[e];
    }
    for (int o = 16; o > 0; o >>= 1) dotp += __shfl_down_sync(0xffffffffu, dotp, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = dotp;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < MS_THREADS / 32; ++w) s += red[w];
        part[blockIdx.x] = s;
    }
}

__global__ void __launch_bounds__(MS_THREADS) k_sum_fixed(const double *__restrict__ part, int n,
                                                           double *__restrict__ out) {
    __shared__ double red[MS_THREADS / 32];
    double s = 0.0;
    for (int i = threadIdx.x; i < n; i += MS_THREADS) s += part[i];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < MS_THREADS / 32; ++w) t += red[w];
        *out = t;
    }
}

bool csr_shape_ok(const nss_csr &m, int nrow, int ncol) {
    if (m.nrow != nrow || m.ncol != ncol) return false;
    if (!m.rowptr || m.rowptr[0] != 0) return false;
    const int nnz = m.rowptr[nrow];
    if (nnz < 0 || (nnz > 0 && (!m.colidx || !m.vals))) return false;
    for (int i = 0; i < nrow; ++i)
        if (m.rowptr[i + 1] < m.rowptr[i]) return false;
    for (int p = 0; p < nnz; ++p)
        if (m.colidx[p] < 0 || m.colidx[p] >= ncol) return false;
    return true;
}

}  // namespace

void measure_release(Ctx &c) {
    ctx_free(c, c.ms_dev);
    if (c.ms_host) cudaFreeHost(c.ms_host);
    c.ms_dev = nullptr;
    c.ms_host = nullptr;
    c.ms_cap = 0;
}

int odotv_device(Ctx &c, int label, const nss_csr *ops, const double *d_v, double *d_ov, double *val) {
    const DevSb &s = c.sb;
    if (!s.valid) {
        c.err = "OdotV: no superblock uploaded";
        return NSS_ERR_INVALID;
    }
    if ((label != 0 && label != 1) || !ops) {
        c.err = "OdotV: label must be 'l' (0) or 'r' (1) and the operator list non-null";
        return NSS_ERR_INVALID;
    }
    // the per-sector operators, packed: row pointers (offset into col/val),
    // columns, values; validated as the reference's filter would produce them
    std::vector<int64_t> rp_off(s.nsb);
    int64_t nrp = 0, nnz = 0;
    for (int k = 0; k < s.nsb; ++k) {
        const int d = label ? s.drs[k] : s.dls[k];
        if (!csr_shape_ok(ops[k], d, d)) {
            c.err = "OdotV: operator of sector " + std::to_string(k) + " has the wrong shape or a bad index";
            return NSS_ERR_INVALID;
        }
        rp_off[k] = nrp;
        nrp += d + 1;
        nnz += ops[k].rowptr[d];
    }
    if (nnz > INT32_MAX) {
        c.err = "OdotV: more than 2^31 operator entries";
        return NSS_ERR_INVALID;
    }
    std::vector<int2> items;
    for (int k = 0; k < s.nsb; ++k) {
        const int64_t ne = (int64_t)s.dls[k] * s.drs[k];
        if (ne > INT32_MAX) {
            c.err = "OdotV: sector " + std::to_string(k) + " has more than 2^31 states";
            return NSS_ERR_INVALID;
        }
        for (int64_t e = 0; e < ne; e += MS_THREADS) items.push_back(make_int2(k, (int)e));
    }
    const int nit = (int)items.size();
    auto al16 = [](size_t x) { return (x + 15) / 16 * 16; };
    const size_t b_items = 0, b_rpo = al16(b_items + sizeof(int2) * (size_t)nit);
    const size_t b_rp = al16(b_rpo + sizeof(int64_t) * (size_t)s.nsb);
    const size_t b_col = al16(b_rp + sizeof(int) * (size_t)nrp);
    const size_t b_val = al16(b_col + sizeof(int) * (size_t)nnz);
    const size_t b_part = al16(b_val + sizeof(double) * (size_t)nnz);
    const size_t b_out = al16(b_part + sizeof(double) * (size_t)nit);
    const size_t b_end = b_out + sizeof(double);
    if (c.ms_cap < b_end) {
        measure_release(c);
        NSS_CUDA_TRY(c, ctx_alloc(c, &c.ms_dev, b_end));
        NSS_CUDA_TRY(c, cudaHostAlloc((void **)&c.ms_host, b_end, cudaHostAllocDefault));
        c.ms_cap = b_end;
    }
    char *h = c.ms_host;
    std::memcpy(h + b_items, items.data(), sizeof(int2) * (size_t)nit);
    std::memcpy(h + b_rpo, rp_off.data(), sizeof(int64_t) * (size_t)s.nsb);
    {
        int *rp = (int *)(h + b_rp), *cl = (int *)(h + b_col);
        double *vl = (double *)(h + b_val);
        int64_t at = 0;
        for (int k = 0; k < s.nsb; ++k) {
            const int d = label ? s.drs[k] : s.dls[k];
            const nss_csr &m = ops[k];
            for (int i = 0; i <= d; ++i) rp[rp_off[k] + i] = (int)(at + m.rowptr[i]);
            const int nz = m.rowptr[d];
            if (nz) {
                std::memcpy(cl + at, m.colidx, sizeof(int) * (size_t)nz);
                std::memcpy(vl + at, m.vals, sizeof(double) * (size_t)nz);
            }
            at += nz;
        }
    }
    cudaStream_t st = c.stream;
    NSS_CUDA_TRY(c, cudaMemcpyAsync(c.ms_dev, h, b_part, cudaMemcpyHostToDevice, st));
    char *d = c.ms_dev;
    c.launches += 2;
    k_odotv<<<nit, MS_THREADS, 0, st>>>(d_v, d_ov, (const int2 *)(d + b_items), s.d_dls, s.d_drs, s.d_off,
                                        (const int64_t *)(d + b_rpo), (const int *)(d + b_rp),
                                        (const int *)(d + b_col), (const double *)(d + b_val), label,
                                        (double *)(d + b_part));
    NSS_CUDA_TRY(c, cudaGetLastError());
    k_sum_fixed<<<1, MS_THREADS, 0, st>>>((const double *)(d + b_part), nit, (double *)(d + b_out));
    NSS_CUDA_TRY(c, cudaGetLastError());
    double *hv = (double *)(h + b_out);
    NSS_CUDA_TRY(c, cudaMemcpyAsync(hv, d + b_out, sizeof(double), cudaMemcpyDeviceToHost, st));
    NSS_CUDA_TRY(c, cudaStreamSynchronize(st));
    if (val) *val = *hv;
    return NSS_OK;
}

}  // namespace nss
