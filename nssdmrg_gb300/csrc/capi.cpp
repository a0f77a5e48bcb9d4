// C ABI (include/nssdmrg.h).  Every entry point catches C++ exceptions and
// turns them into status codes; nothing here aborts the caller.
#include <cuda_runtime.h>
#include <cusolverDn.h>

#include <algorithm>
#include <climits>
#include <cstdlib>
#include <memory>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "device.cuh"
#include "host_dmrg.hpp"
#include "host_restart.hpp"
#include "host_tridiag.hpp"

struct nss_ctx {
    nss::Ctx c;
    // host tables of the superblock built here: by nss_sb_setup, or the
    // driver's superblock after nss_dmrg_prepare_last
    std::shared_ptr<const nss::SbHost> sbhost;
    double *d_v = nullptr, *d_hv = nullptr, *d_psi = nullptr;
    int64_t tmp_n = 0;
};

struct nss_dmrg {
    nss_ctx *ctx = nullptr;
    nss::Driver drv;
    nss::SbView view;   // last exported superblock
    std::unique_ptr<nss::SbHost> last;
};

namespace {

thread_local std::string g_err;

int fail(nss_ctx *ctx, int code, const std::string &msg) {
    if (ctx) ctx->c.err = msg;
    else g_err = msg;
    return code;
}

template <class F>
int guarded(nss_ctx *ctx, F &&f) {
    try {
        return f();
    } catch (const std::bad_alloc &) {
        return fail(ctx, NSS_ERR_NOMEM, "host allocation failed");
    } catch (const std::exception &e) {
        return fail(ctx, NSS_ERR_INVALID, e.what());
    }
}

// Makes the context's device current for the duration of one entry point
// and gives the caller back the device that was current before, so that a
// host code with its own device binding keeps it.
struct DeviceScope {
    int prev = -1;
    explicit DeviceScope(int dev) {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DeviceScope() {
        int cur = -1;
        if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
    }
    DeviceScope(const DeviceScope &) = delete;
    DeviceScope &operator=(const DeviceScope &) = delete;
};

int ensure_tmp(nss_ctx *ctx, int64_t n) {
    if (ctx->tmp_n >= n && ctx->d_v) return NSS_OK;
    nss::ctx_free(ctx->c, ctx->d_v);
    nss::ctx_free(ctx->c, ctx->d_hv);
    ctx->d_v = ctx->d_hv = nullptr;
    NSS_CUDA_TRY(ctx->c, nss::ctx_alloc(ctx->c, &ctx->d_v, (size_t)n));
    NSS_CUDA_TRY(ctx->c, nss::ctx_alloc(ctx->c, &ctx->d_hv, (size_t)n));
    ctx->tmp_n = n;
    return NSS_OK;
}

}  // namespace

nss::Ctx &nss::ctx_of(nss_ctx *ctx) { return ctx->c; }

extern "C" {

nss_ctx *nss_create(int device, size_t hbm_budget) {
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        g_err = "nss_create: no CUDA device";
        return nullptr;
    }
    if (device < 0 || device >= ndev) {
        g_err = "nss_create: device index out of range";
        return nullptr;
    }
    DeviceScope dscope(device);
    int cur = -1;
    if (cudaGetDevice(&cur) != cudaSuccess || cur != device) {
        g_err = "nss_create: cannot make the device current";
        return nullptr;
    }
    auto *ctx = new (std::nothrow) nss_ctx;
    if (!ctx) {
        g_err = "nss_create: host allocation failed";
        return nullptr;
    }
    ctx->c.device = device;
    ctx->c.tc_min_dl = nss::tc_min_dl_default();
    ctx->c.tc_auto = nss::tune_enabled();
    nss::mma_tile_default(&ctx->c.mma_bn, &ctx->c.mma_split);
    ctx->c.mma_lolo = nss::mma_lolo_default();
    ctx->c.mma_kps = nss::mma_kps_default();
    {
        const char *g = std::getenv("NSS_GRAPH");
        ctx->c.use_graphs = !(g && std::atoi(g) == 0);
    }
    ctx->c.budget = hbm_budget;
    if (cudaStreamCreateWithFlags(&ctx->c.stream, cudaStreamNonBlocking) != cudaSuccess) {
        g_err = "nss_create: stream creation failed";
        delete ctx;
        return nullptr;
    }
    cusolverDnHandle_t h = nullptr;
    if (cusolverDnCreate(&h) != CUSOLVER_STATUS_SUCCESS || cusolverDnSetStream(h, ctx->c.stream) != CUSOLVER_STATUS_SUCCESS) {
        g_err = "nss_create: cuSOLVER initialisation failed";
        cudaStreamDestroy(ctx->c.stream);
        delete ctx;
        return nullptr;
    }
    ctx->c.solver = h;
    return ctx;
}

void nss_destroy(nss_ctx *ctx) {
    if (!ctx) return;
    DeviceScope dscope(ctx->c.device);
    cudaStreamSynchronize(ctx->c.stream);
    nss::sb_release(ctx->c, true);
    nss::lanczos_release(ctx->c);
    nss::rdm_release(ctx->c);
    nss::renorm_release(ctx->c);
    nss::measure_release(ctx->c);
    nss::ctx_free(ctx->c, ctx->d_v);
    nss::ctx_free(ctx->c, ctx->d_hv);
    nss::ctx_free(ctx->c, ctx->d_psi);
    if (ctx->c.solver) cusolverDnDestroy((cusolverDnHandle_t)ctx->c.solver);
    if (ctx->c.hv_side) {
        cudaStreamSynchronize(ctx->c.hv_side);
        cudaStreamDestroy(ctx->c.hv_side);
        cudaEventDestroy(ctx->c.hv_fork);
        cudaEventDestroy(ctx->c.hv_join);
    }
    cudaStreamDestroy(ctx->c.stream);
    delete ctx;
}

const char *nss_last_error(const nss_ctx *ctx) { return ctx ? ctx->c.err.c_str() : g_err.c_str(); }

int nss_sb_upload(nss_ctx *ctx, const nss_sb_desc *desc) {
    if (!ctx) return fail(ctx, NSS_ERR_INVALID, "null context");
    return guarded(ctx, [&] {
        DeviceScope dscope(ctx->c.device);
        ctx->sbhost.reset();
        return nss::sb_upload(ctx->c, desc);
    });
}

int nss_sb_free(nss_ctx *ctx) {
    if (!ctx) return fail(ctx, NSS_ERR_INVALID, "null context");
    DeviceScope dscope(ctx->c.device);
    cudaStreamSynchronize(ctx->c.stream);
    nss::sb_release(ctx->c, true);
    ctx->sbhost.reset();
    return NSS_OK;
}

int64_t nss_sb_dim(const nss_ctx *ctx) { return (ctx && ctx->c.sb.valid) ? ctx->c.sb.n : 0; }

int nss_sb_shape(const nss_ctx *ctx, int32_t *nsb, int32_t *m_left, int32_t *m_right, int64_t *n) {
    if (!ctx || !ctx->c.sb.valid) return NSS_ERR_STATE;
    if (nsb) *nsb = ctx->c.sb.nsb;
    if (m_left) *m_left = ctx->c.sb.m_left;
    if (m_right) *m_right = ctx->c.sb.m_right;
    if (n) *n = ctx->c.sb.n;
    return NSS_OK;
}

int nss_sb_flops(const nss_ctx *ctx, double *dense, double *ab) {
    if (!ctx || !ctx->c.sb.valid) return NSS_ERR_STATE;
    if (dense) *dense = ctx->c.sb.flops_dense;
    if (ab) *ab = ctx->c.sb.flops_ab;
    return NSS_OK;
}

int64_t nss_kernel_launches(const nss_ctx *ctx) { return ctx ? ctx->c.launches : 0; }

int64_t nss_sb_upload_bytes(const nss_ctx *ctx) { return (ctx && ctx->c.sb.valid) ? ctx->c.sb.h2d_bytes : 0; }

void *nss_stream(const nss_ctx *ctx) { return ctx ? (void *)ctx->c.stream : nullptr; }

int nss_hv_device(nss_ctx *ctx, int64_t n, const double *d_v, double *d_hv) {
    if (!ctx) return fail(ctx, NSS_ERR_INVALID, "null context");
    if (!ctx->c.sb.valid) return fail(ctx, NSS_ERR_STATE, "nss_hv: no superblock uploaded");
    if (n != ctx->c.sb.n) return fail(ctx, NSS_ERR_INVALID, "nss_hv: Nloc != superblock dimension");
    if (!d_v || !d_hv) return fail(ctx, NSS_ERR_INVALID, "nss_hv: null vector");
    DeviceScope dscope(ctx->c.device);
    return nss::hv_device(ctx->c, d_v, d_hv);
}

int nss_hv_device_f32(nss_ctx *ctx, int64_t n, const float *d_v, float *d_hv) {
    if (!ctx) return fail(ctx, NSS_ERR_INVALID, "null context");
    if (!ctx->c.sb.valid) return fail(ctx, NSS_ERR_STATE, "nss_hv: no superblock uploaded");
    if (n != ctx->c.sb.n) return fail(ctx, NSS_ERR_INVALID, "nss_hv: Nloc != superblock dimension");
    if (!d_v || !d_hv) return fail(ctx, NSS_ERR_INVALID, "nss_hv: null vector");
    DeviceScope dscope(ctx->c.device);
    return nss::hv_device_fp32(ctx->c, d_v, d_hv);
}

int nss_tune_info(const nss_ctx *ctx, int *candidate, double *ms_per_hv, int *solves) {
    if (!ctx || !ctx->c.sb.valid) return NSS_ERR_STATE;
    if (candidate) *candidate = ctx->c.tune_cand;
    double m[3] = {-1.0, -1.0, -1.0};
    int n[3] = {0, 0, 0};
    if (ctx->c.tune_cand >= 0) nss::tune_lookup(ctx->c.device, ctx->c.tune_class, m, n);
    for (int k = 0; k < 3; ++k) {
        if (ms_per_hv) ms_per_hv[k] = m[k];
        if (solves) solves[k] = n[k];
    }
    return NSS_OK;
}

void nss_tune_reset(void) { nss::tune_reset(); }

int nss_sb_energy_noalloc(nss_ctx *ctx, int64_t n, const double *d_psi, double *energy) {
    if (!ctx) return fail(ctx, NSS_ERR_INVALID, "null context");
    DeviceScope dscope(ctx->c.device);
    return nss::sb_energy_noalloc(ctx->c, n, d_psi, energy);
}

int nss_tridiag_lowest(int m, const double *a, const double *b, int ne, double b_last, double *theta, double *s,
                       double *resid) {
    if (m <= 0 || ne <= 0 || ne > m || !a || (m > 1 && !b) || !theta || !s || !resid) {
        g_err = "nss_tridiag_lowest: need 0 < ne <= m and non-NULL arrays";
        return NSS_ERR_INVALID;
    }
    return guarded(nullptr, [&] {
        std::vector<double> work;
        nss::tridiag_lowest(a, b, m, ne, b_last, theta, s, resid, nullptr, work);
        return NSS_OK;
    });
}

int nss_tridiag_eig(int n, const double *d, const double *e, double *evals, double *Z) {
    if (n <= 0 || !d || (n > 1 && !e) || !evals || !Z) {
        g_err = "nss_tridiag_eig: need n > 0 and non-NULL arrays";
        return NSS_ERR_INVALID;
    }
    return guarded(nullptr, [&] {
        std::vector<double> dd(d, d + n), ee(n, 0.0);
        for (int i = 0; i + 1 < n; ++i) ee[i] = e[i];
        if (!nss::tridiag_ql(n, dd.data(), ee.data(), Z)) {
            g_err = "nss_tridiag_eig: an eigenvalue did not converge in 60 QL iterations";
            return NSS_ERR_NOCONV;
        }
        std::copy(dd.begin(), dd.end(), evals);
        return NSS_OK;
    });
}

int nss_kron_sum(int32_t na, int32_t nb, int32_t nterms, const double *coef, const nss_csr *a, const nss_csr *b,
                 int nthreads, int64_t cap, int64_t *nnz, int32_t *rowptr, int32_t *colidx, double *vals) {
    if (na <= 0 || nb <= 0 || nterms < 0 || (nterms > 0 && (!coef || !a || !b)) || !nnz ||
        (int64_t)na * nb > INT32_MAX - 1) {
        g_err = "nss_kron_sum: need na, nb > 0, na*nb < 2^31 and non-NULL arrays";
        return NSS_ERR_INVALID;
    }
    auto load = [](const nss_csr &c, int n, nss::Csr &m) {
        if (c.nrow != n || c.ncol != n || !c.rowptr || c.rowptr[0] != 0) return false;
        m.init(n, n);
        for (int i = 0; i < n; ++i) {
            if (c.rowptr[i + 1] < c.rowptr[i]) return false;
            for (int e = c.rowptr[i]; e < c.rowptr[i + 1]; ++e) {
                if (!c.colidx || !c.vals || c.colidx[e] < 0 || c.colidx[e] >= n) return false;
                m.col.push_back(c.colidx[e]);
                m.val.push_back(c.vals[e]);
            }
            m.rowptr[i + 1] = (int)m.col.size();
        }
        return true;
    };
    std::vector<nss::Csr> ma(nterms), mb(nterms);
    std::vector<nss::KronTerm> terms;
    for (int t = 0; t < nterms; ++t) {
        if (!load(a[t], na, ma[t]) || !load(b[t], nb, mb[t])) {
            g_err = "nss_kron_sum: term " + std::to_string(t) + " has a wrong shape or a malformed CSR";
            return NSS_ERR_INVALID;
        }
        terms.push_back({&ma[t], &mb[t], coef[t]});
    }
    if (nthreads <= 0) nthreads = (int)std::max(1u, std::thread::hardware_concurrency());
    try {
        const nss::Csr c = nss::csr_kron_sum(na, nb, terms, nthreads);
        *nnz = (int64_t)c.col.size();
        if (!colidx || !vals) return NSS_OK;
        if (!rowptr || cap < *nnz) {
            g_err = "nss_kron_sum: rowptr missing or cap below nnz";
            return NSS_ERR_INVALID;
        }
        std::copy(c.rowptr.begin(), c.rowptr.end(), rowptr);
        std::copy(c.col.begin(), c.col.end(), colidx);
        std::copy(c.val.begin(), c.val.end(), vals);
    } catch (const std::exception &ex) {
        g_err = std::string("nss_kron_sum: ") + ex.what();
        return NSS_ERR_INVALID;
    }
    return NSS_OK;
}

int nss_arrow_lowest(int k, double theta0, const double *m, const double *a, const double *b, double b_last,
                     double *lam, double *c, double *resid) {
    if (k < 0 || (k > 0 && (!m || !a || (k > 1 && !b))) || !lam || !c || !resid) {
        g_err = "nss_arrow_lowest: need k >= 0 and non-NULL arrays";
        return NSS_ERR_INVALID;
    }
    return guarded(nullptr, [&] {
        std::vector<double> work;
        if (!nss::arrow_lowest(theta0, m, a, b, k, b_last, lam, c, resid, work)) {
            g_err = "nss_arrow_lowest: no root below the tridiagonal spectrum";
            return NSS_ERR_NOCONV;
        }
        return NSS_OK;
    });
}

int nss_time_chunks(nss_ctx *ctx, int enable) {
    if (!ctx) return NSS_ERR_INVALID;
    ctx->c.time_chunks = enable != 0;
    return NSS_OK;
}

int nss_graph_stats(const nss_ctx *ctx, int *replays, int *captures) {
    if (!ctx) return NSS_ERR_INVALID;
    if (replays) *replays = ctx->c.graph_replays;
    if (captures) *captures = ctx->c.graph_captures;
    return NSS_OK;
}

int nss_chunk_cache(const nss_ctx *ctx, int *vectors, int64_t *rows) {
    if (!ctx) return NSS_ERR_INVALID;
    if (vectors) *vectors = ctx->c.lz.chunk_vc;
    if (rows) *rows = ctx->c.lz.chunk_cs;
    return NSS_OK;
}

int nss_chunk_stats(const nss_ctx *ctx, double *ms, int *launches, int64_t *iters, double *cols) {
    if (!ctx) return NSS_ERR_INVALID;
    if (ms) *ms = ctx->c.chunk_ms;
    if (launches) *launches = ctx->c.chunk_launches;
    if (iters) *iters = ctx->c.chunk_iters;
    if (cols) *cols = ctx->c.chunk_cols;
    return NSS_OK;
}

int nss_refine_stats(const nss_ctx *ctx, int *passes, int *cluster, int64_t *fp64_fallbacks) {
    if (!ctx) return NSS_ERR_INVALID;
    if (passes) *passes = ctx->c.refine_passes;
    if (cluster) *cluster = ctx->c.refine_cluster;
    if (fp64_fallbacks) *fp64_fallbacks = ctx->c.mixed_fallbacks;
    return NSS_OK;
}

int nss_rdm_stats(const nss_ctx *ctx, int *own_blocks, int *library_blocks, int *fallback_blocks) {
    if (!ctx) return NSS_ERR_INVALID;
    if (own_blocks) *own_blocks = ctx->c.rdm_own_blocks;
    if (library_blocks) *library_blocks = ctx->c.rdm_lib_blocks;
    if (fallback_blocks) *fallback_blocks = ctx->c.rdm_fallback_blocks;
    return NSS_OK;
}

int nss_rdm_fallback_reasons(const nss_ctx *ctx, int64_t out[5]) {
    if (!ctx || !out) return NSS_ERR_INVALID;
    for (int b = 0; b < 5; ++b) out[b] = ctx->c.rdm_fail_why[b];
    return NSS_OK;
}

int nss_hv(nss_ctx *ctx, int64_t n, const double *v, double *hv) {
    if (!ctx) return fail(ctx, NSS_ERR_INVALID, "null context");
    if (!ctx->c.sb.valid) return fail(ctx, NSS_ERR_STATE, "nss_hv: no superblock uploaded");
    if (n != ctx->c.sb.n) return fail(ctx, NSS_ERR_INVALID, "nss_hv: Nloc != superblock dimension");
    if (!v || !hv) return fail(ctx, NSS_ERR_INVALID, "nss_hv: null vector");
    DeviceScope dscope(ctx->c.device);
    return guarded(ctx, [&] {
        int rc = ensure_tmp(ctx, n);
        if (rc) return rc;
        nss::Ctx &c = ctx->c;
        NSS_CUDA_TRY(c, cudaMemcpyAsync(ctx->d_v, v, n * sizeof(double), cudaMemcpyHostToDevice, c.stream));
        rc = nss::hv_device(c, ctx->d_v, ctx->d_hv);
        if (rc) return rc;
        NSS_CUDA_TRY(c, cudaMemcpyAsync(hv, ctx->d_hv, n * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
        NSS_CUDA_TRY(c, cudaStreamSynchronize(c.stream));
        return NSS_OK;
    });
}

namespace {

// 'l'/'s' -> 0 (left, system), 'r'/'e' -> 1 (right, environment), else -1
int side_of(char label) {
    switch (label) {
    case 'l': case 'L': case 's': case 'S': return 0;
    case 'r': case 'R': case 'e': case 'E': return 1;
    default: return -1;
    }
}

}  // namespace

int nss_odotv(nss_ctx *ctx, char label, const nss_csr *ops, const double *v, double *ov) {
    if (!ctx) return fail(ctx, NSS_ERR_INVALID, "null context");
    if (!ctx->c.sb.valid) return fail(ctx, NSS_ERR_STATE, "nss_odotv: no superblock uploaded");
    const int side = side_of(label);
    if (side < 0) return fail(ctx, NSS_ERR_INVALID, "nss_odotv: label not [l,r]");
    if (!ops || !v || !ov) return fail(ctx, NSS_ERR_INVALID, "nss_odotv: null argument");
    DeviceScope dscope(ctx->c.device);
    return guarded(ctx, [&] {
        nss::Ctx &c = ctx->c;
        const int64_t n = c.sb.n;
        int rc = ensure_tmp(ctx, n);
        if (rc) return rc;
        NSS_CUDA_TRY(c, cudaMemcpyAsync(ctx->d_v, v, n * sizeof(double), cudaMemcpyHostToDevice, c.stream));
        if ((rc = nss::odotv_device(c, side, ops, ctx->d_v, ctx->d_hv, nullptr))) return rc;
        NSS_CUDA_TRY(c, cudaMemcpyAsync(ov, ctx->d_hv, n * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
        NSS_CUDA_TRY(c, cudaStreamSynchronize(c.stream));
        return NSS_OK;
    });
}

int nss_average_op(nss_ctx *ctx, char label, const nss_csr *op, const double *psi, double *val) {
    if (!ctx) return fail(ctx, NSS_ERR_INVALID, "null context");
    if (!ctx->c.sb.valid) return fail(ctx, NSS_ERR_STATE, "nss_average_op: no superblock uploaded");
    const int side = side_of(label);
    if (side < 0) return fail(ctx, NSS_ERR_INVALID, "Average_op_dmrg error: label not [l,r]");
    if (!op || !val) return fail(ctx, NSS_ERR_INVALID, "nss_average_op: null argument");
    DeviceScope dscope(ctx->c.device);
    return guarded(ctx, [&] {
        nss::Ctx &c = ctx->c;
        const nss::DevSb &s = c.sb;
        const std::vector<int> &maps = side ? s.bi : s.ai;
        const std::vector<int> &moff = side ? s.bi_off : s.ai_off;
        if (maps.empty()) return fail(ctx, NSS_ERR_STATE, "nss_average_op: the descriptor carried no sector maps (ai/bi)");
        const int mb = side ? s.m_right : s.m_left;
        if (op->nrow != mb || op->ncol != mb || !op->rowptr || (op->rowptr[mb] > 0 && (!op->colidx || !op->vals)))
            return fail(ctx, NSS_ERR_INVALID, "nss_average_op: operator is not m_block x m_block");
        for (int i = 0; i < mb; ++i)
            if (op->rowptr[i + 1] < op->rowptr[i]) return fail(ctx, NSS_ERR_INVALID, "nss_average_op: bad row pointers");
        // sp_filter(Oi, LI(isb)%states) per sector (:617-625)
        std::vector<int> local(mb, -1);
        std::vector<std::vector<int>> rp(s.nsb), cl(s.nsb);
        std::vector<std::vector<double>> vl(s.nsb);
        std::vector<nss_csr> ops(s.nsb);
        for (int k = 0; k < s.nsb; ++k) {
            const int a = moff[k], b = moff[k + 1];
            for (int p = a; p < b; ++p) local[maps[p]] = p - a;
            rp[k].assign(1, 0);
            for (int p = a; p < b; ++p) {
                const int i = maps[p];
                for (int e = op->rowptr[i]; e < op->rowptr[i + 1]; ++e) {
                    const int j = op->colidx[e];
                    if (j < 0 || j >= mb) return fail(ctx, NSS_ERR_INVALID, "nss_average_op: column out of range");
                    if (local[j] < 0) continue;
                    cl[k].push_back(local[j]);
                    vl[k].push_back(op->vals[e]);
                }
                rp[k].push_back((int)cl[k].size());
            }
            for (int p = a; p < b; ++p) local[maps[p]] = -1;
            ops[k] = nss_csr{b - a, b - a, rp[k].data(), cl[k].data(), vl[k].data()};
        }
        const double *d_psi = nullptr;
        if (psi) {
            int rc = ensure_tmp(ctx, s.n);
            if (rc) return rc;
            NSS_CUDA_TRY(c, cudaMemcpyAsync(ctx->d_v, psi, s.n * sizeof(double), cudaMemcpyHostToDevice, c.stream));
            d_psi = ctx->d_v;
        } else {
            if (c.lz.neigen_done < 1 || c.lz.n != s.n)
                return fail(ctx, NSS_ERR_STATE, "nss_average_op: no ground state (call nss_eigh or pass psi)");
            d_psi = c.lz.evecs;
        }
        return nss::odotv_device(c, side, ops.data(), d_psi, nullptr, val);
    });
}

int nss_eigh(nss_ctx *ctx, int neigen, int nitermax, int ncv, double tol, uint64_t seed, int precision,
             double *evals, double *evecs, int *numop) {
    (void)ncv;
    if (!ctx) return fail(ctx, NSS_ERR_INVALID, "null context");
    if (!evals) return fail(ctx, NSS_ERR_INVALID, "nss_eigh: evals is NULL");
    if (precision != NSS_PREC_FP64 && precision != NSS_PREC_MIXED)
        return fail(ctx, NSS_ERR_INVALID, "nss_eigh: unknown precision mode");
    DeviceScope dscope(ctx->c.device);
    return guarded(ctx, [&] {
        int rc = nss::lanczos_eigh(ctx->c, neigen, nitermax, tol, seed, precision, evals, numop);
        if (rc) return rc;
        if (evecs) {
            nss::Ctx &c = ctx->c;
            const int64_t n = c.sb.n;
            NSS_CUDA_TRY(c, cudaMemcpyAsync(evecs, c.lz.evecs, (size_t)c.lz.neigen_done * n * sizeof(double),
                                            cudaMemcpyDeviceToHost, c.stream));
            NSS_CUDA_TRY(c, cudaStreamSynchronize(c.stream));
        }
        return NSS_OK;
    });
}

int nss_eigh_batch(nss_ctx *const *ctxs, int nb, int nitermax, double tol, const uint64_t *seeds, double *evals,
                   int *numops) {
    if (!ctxs || nb < 1 || !ctxs[0]) {
        g_err = "nss_eigh_batch: need at least one context";
        return NSS_ERR_INVALID;
    }
    for (int b = 0; b < nb; ++b)
        if (!ctxs[b]) {
            g_err = "nss_eigh_batch: NULL context";
            return NSS_ERR_INVALID;
        }
    nss_ctx *c0 = ctxs[0];
    return guarded(c0, [&] {
        DeviceScope dscope(c0->c.device);
        std::vector<nss::Ctx *> cs((size_t)nb);
        for (int b = 0; b < nb; ++b) cs[b] = &ctxs[b]->c;
        return nss::lanczos_eigh_batch(cs.data(), nb, nitermax, tol, seeds, evals, numops);
    });
}

struct nss_batch {
    nss_ctx *host = nullptr;
    nss::BatchEngine *eng = nullptr;
};

nss_batch *nss_batch_create(nss_ctx *host) {
    if (!host) {
        g_err = "nss_batch_create: NULL host context";
        return nullptr;
    }
    try {
        DeviceScope dscope(host->c.device);
        nss::BatchEngine *e = nss::batch_create(host->c);
        if (!e) return nullptr;
        nss_batch *b = new nss_batch();
        b->host = host;
        b->eng = e;
        return b;
    } catch (const std::exception &ex) {
        host->c.err = std::string("nss_batch_create: ") + ex.what();
        return nullptr;
    }
}

int nss_batch_add(nss_batch *b, nss_ctx *ctx, uint64_t seed, int nitermax, double tol, int *id) {
    if (!b || !ctx) {
        g_err = "nss_batch_add: NULL argument";
        return NSS_ERR_INVALID;
    }
    return guarded(b->host, [&] {
        DeviceScope dscope(b->host->c.device);
        return nss::batch_add(b->eng, ctx->c, seed, nitermax, tol, id);
    });
}

int nss_batch_step(nss_batch *b, int max_done, int *ndone, int *ids, double *energies, int *numops) {
    if (!b) {
        g_err = "nss_batch_step: NULL batch";
        return NSS_ERR_INVALID;
    }
    return guarded(b->host, [&] {
        DeviceScope dscope(b->host->c.device);
        return nss::batch_step(b->eng, max_done, ndone, ids, energies, numops);
    });
}

int nss_batch_inflight(const nss_batch *b) { return b ? nss::batch_inflight(b->eng) : 0; }

void nss_batch_destroy(nss_batch *b) {
    if (!b) return;
    DeviceScope dscope(b->host->c.device);
    nss::batch_destroy(b->eng);
    delete b;
}

int nss_rdm(nss_ctx *ctx, const double *psi, int mstates, double deg_thr, nss_rdm_side out[2],
            double *lambda_left, double *lambda_right, int32_t *kept_left, int32_t *kept_right, double *u_left,
            double *u_right) {
    return nss_rdm_estates(ctx, psi, mstates, 0.0, deg_thr, out, lambda_left, lambda_right, kept_left, kept_right,
                           u_left, u_right);
}

int nss_rdm_estates(nss_ctx *ctx, const double *psi, int mstates, double estates, double deg_thr,
                    nss_rdm_side out[2], double *lambda_left, double *lambda_right, int32_t *kept_left,
                    int32_t *kept_right, double *u_left, double *u_right) {
    if (!ctx) return fail(ctx, NSS_ERR_INVALID, "null context");
    if (!out) return fail(ctx, NSS_ERR_INVALID, "nss_rdm: out is NULL");
    DeviceScope dscope(ctx->c.device);
    return guarded(ctx, [&] {
        nss::Ctx &c = ctx->c;
        if (!c.sb.valid) return fail(ctx, NSS_ERR_STATE, "nss_rdm: no superblock uploaded");
        const double *d_psi = nullptr;
        if (psi) {
            if (!ctx->d_psi || ctx->tmp_n < c.sb.n) {
                int rc = ensure_tmp(ctx, c.sb.n);
                if (rc) return rc;
            }
            NSS_CUDA_TRY(c, cudaMemcpyAsync(ctx->d_v, psi, c.sb.n * sizeof(double), cudaMemcpyHostToDevice, c.stream));
            d_psi = ctx->d_v;
        } else {
            if (c.lz.neigen_done < 1 || c.lz.n != c.sb.n)
                return fail(ctx, NSS_ERR_STATE, "nss_rdm: no ground state (call nss_eigh or pass psi)");
            d_psi = c.lz.evecs;
        }
        return nss::rdm_run(c, d_psi, mstates, estates, deg_thr, out, lambda_left, lambda_right, kept_left, kept_right,
                            u_left, u_right);
    });
}

int nss_sb_setup(nss_ctx *ctx, int site_type, const nss_block_desc *left, const nss_block_desc *right,
                 const double *target, const double *hij) {
    if (!ctx) return fail(ctx, NSS_ERR_INVALID, "null context");
    if (!left || !right || !target || !hij) return fail(ctx, NSS_ERR_INVALID, "nss_sb_setup: null argument");
    if (site_type != NSS_SITE_SPIN && site_type != NSS_SITE_FERMION)
        return fail(ctx, NSS_ERR_INVALID, "nss_sb_setup: unknown site type");
    DeviceScope dscope(ctx->c.device);
    return guarded(ctx, [&] {
        const bool f = site_type == NSS_SITE_FERMION;
        nss::Block l = nss::block_from_desc(*left, f), r = nss::block_from_desc(*right, f);
        nss::Qn t(target, target + left->qdim);
        auto sb = std::make_unique<nss::SbHost>(nss::sb_build(l, r, t, hij));
        nss::SbView v;
        nss::sb_view(*sb, v);
        int rc = nss::sb_upload(ctx->c, &v.desc, true);
        if (rc) return rc;
        ctx->sbhost = std::move(sb);
        return NSS_OK;
    });
}

int nss_sb_counts(const nss_ctx *ctx, int32_t *nsb, int32_t *qdim, int64_t *n) {
    if (!ctx || !ctx->sbhost) return NSS_ERR_STATE;
    if (nsb) *nsb = ctx->sbhost->nsb();
    if (qdim) *qdim = ctx->sbhost->qdim;
    if (n) *n = ctx->sbhost->n();
    return NSS_OK;
}

int nss_sb_tables(const nss_ctx *ctx, double *qns, int32_t *dls, int32_t *drs, int64_t *offset, int64_t *sb_states) {
    if (!ctx || !ctx->sbhost) return NSS_ERR_STATE;
    const nss::SbHost &s = *ctx->sbhost;
    for (int k = 0; k < s.nsb(); ++k) {
        if (qns)
            for (int t = 0; t < s.qdim; ++t) qns[k * s.qdim + t] = s.qns[k][t];
        if (dls) dls[k] = s.dls[k];
        if (drs) drs[k] = s.drs[k];
        if (offset) offset[k] = s.offset[k];
    }
    if (sb_states)
        for (int64_t i = 0; i < s.n(); ++i) sb_states[i] = s.sb_states[i];
    return NSS_OK;
}

nss_dmrg *nss_dmrg_create(nss_ctx *ctx, const nss_dmrg_params *p) {
    if (!ctx || !p) {
        g_err = "nss_dmrg_create: null argument";
        return nullptr;
    }
    auto *d = new (std::nothrow) nss_dmrg;
    if (!d) return nullptr;
    d->ctx = ctx;
    int rc = guarded(ctx, [&] { return d->drv.init(&ctx->c, *p); });
    if (rc) {
        delete d;
        return nullptr;
    }
    return d;
}

void nss_dmrg_destroy(nss_dmrg *d) { delete d; }

int nss_dmrg_infinite(nss_dmrg *d) {
    if (!d) return NSS_ERR_INVALID;
    DeviceScope dscope(d->ctx->c.device);
    return guarded(d->ctx, [&] { return d->drv.infinite(); });
}

int nss_dmrg_finite(nss_dmrg *d) {
    if (!d) return NSS_ERR_INVALID;
    DeviceScope dscope(d->ctx->c.device);
    return guarded(d->ctx, [&] { return d->drv.finite(); });
}

int nss_restart_rewrite(const char *in_path, const char *out_path) {
    if (!in_path || !out_path) {
        g_err = "nss_restart_rewrite: null path";
        return NSS_ERR_INVALID;
    }
    try {
        nss::save_block_file(out_path, nss::load_block_file(in_path));
    } catch (const std::exception &ex) {
        g_err = ex.what();
        return NSS_ERR_INVALID;
    }
    return NSS_OK;
}

int nss_dmrg_save_blocks(nss_dmrg *d, const char *left_path, const char *right_path) {
    if (!d) return NSS_ERR_INVALID;
    return guarded(d->ctx, [&] {
        if (left_path) nss::save_block_file(left_path, d->drv.left);
        if (right_path) nss::save_block_file(right_path, d->drv.right);
        return NSS_OK;
    });
}

int nss_dmrg_load_blocks(nss_dmrg *d, const char *left_path, const char *right_path) {
    if (!d) return NSS_ERR_INVALID;
    return guarded(d->ctx, [&] {
        const nss::Block &dot = d->drv.dot;
        auto check = [&](const nss::Block &b, const char *path) -> int {
            if (b.fermion != dot.fermion || b.qdim != dot.qdim)
                return fail(d->ctx, NSS_ERR_INVALID, std::string("load_block: ") + path + " is not a block of this model");
            for (const nss::Op &o : dot.ops)
                if (b.find_op(o.key) < 0)
                    return fail(d->ctx, NSS_ERR_INVALID, std::string("load_block: ") + path + " lacks operator " + o.key);
            return NSS_OK;
        };
        nss::Block l = d->drv.left, r = d->drv.right;
        if (left_path) {
            l = nss::load_block_file(left_path);
            if (int rc = check(l, left_path)) return rc;
        }
        if (right_path) {
            r = nss::load_block_file(right_path);
            if (int rc = check(r, right_path)) return rc;
        }
        d->drv.left = std::move(l);
        d->drv.right = std::move(r);
        return NSS_OK;
    });
}

int nss_dmrg_measure(nss_dmrg *d, const nss_csr *op, const int32_t *pos, int npos, double *out) {
    if (!d) return NSS_ERR_INVALID;
    if (!op || (npos > 0 && (!pos || !out)) || npos < 0) return fail(d->ctx, NSS_ERR_INVALID, "nss_dmrg_measure: bad arguments");
    DeviceScope dscope(d->ctx->c.device);
    return guarded(d->ctx, [&] {
        const int dd = d->drv.dot.dim;
        if (op->nrow != dd || op->ncol != dd || !op->rowptr)
            return fail(d->ctx, NSS_ERR_INVALID, "nss_dmrg_measure: operator is not d x d");
        nss::Csr o;
        o.init(dd, dd);
        for (int i = 0; i < dd; ++i) {
            for (int e = op->rowptr[i]; e < op->rowptr[i + 1]; ++e) {
                if (op->colidx[e] < 0 || op->colidx[e] >= dd)
                    return fail(d->ctx, NSS_ERR_INVALID, "nss_dmrg_measure: column out of range");
                o.col.push_back(op->colidx[e]);
                o.val.push_back(op->vals[e]);
            }
            o.rowptr[i + 1] = (int)o.col.size();
        }
        for (int k = 0; k < npos; ++k) {
            int side = 0;
            const nss::Csr oi = d->drv.site_op_on_block(o, pos[k], &side);
            const nss_csr view{oi.nrow, oi.ncol, oi.rowptr.data(), oi.col.data(), oi.val.data()};
            int rc = nss_average_op(d->ctx, side ? 'r' : 'l', &view, nullptr, &out[k]);
            if (rc) return rc;
        }
        return NSS_OK;
    });
}

int nss_dmrg_prepare_last(nss_dmrg *d) {
    if (!d) return NSS_ERR_INVALID;
    DeviceScope dscope(d->ctx->c.device);
    return guarded(d->ctx, [&] {
        d->drv.stop_before_last_solve = true;
        int rc = d->drv.infinite();
        d->drv.stop_before_last_solve = false;
        if (rc) return rc;
        if (!d->drv.stopped) return fail(d->ctx, NSS_ERR_STATE, "nss_dmrg_prepare_last: infinite run already done");
        d->ctx->sbhost = d->drv.last_sb;
        return NSS_OK;
    });
}

int nss_dmrg_nrecords(const nss_dmrg *d) { return d ? (int)d->drv.records.size() : 0; }

int nss_dmrg_records(const nss_dmrg *d, nss_step_record *out, int max) {
    if (!d || !out) return NSS_ERR_INVALID;
    int n = std::min<int>(max, (int)d->drv.records.size());
    for (int i = 0; i < n; ++i) out[i] = d->drv.records[i];
    return n;
}

int nss_dmrg_export_superblock(nss_dmrg *d, nss_sb_desc *out) {
    if (!d || !out) return NSS_ERR_INVALID;
    if (!d->drv.last_sb) return fail(d->ctx, NSS_ERR_STATE, "nss_dmrg_export_superblock: no superblock built yet");
    return guarded(d->ctx, [&] {
        d->last = std::make_unique<nss::SbHost>(*d->drv.last_sb);
        nss::sb_view(*d->last, d->view);
        *out = d->view.desc;
        return NSS_OK;
    });
}

}  // extern "C"
