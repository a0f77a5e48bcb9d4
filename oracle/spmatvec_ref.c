/*
 * CPU restatement of the reference's direct superblock H*v and of a plain
 * Lanczos around it.  Oracle code: test infrastructure and the timed CPU
 * baseline only; the shipped package never links it.
 *
 * ref_hv_serial follows spMatVec_direct_main (src/DMRG_SUPERBLOCK_SETUP.f90:
 * 740-865) loop for loop on row-list (CSR) storage: per sector the 1^L x H^R
 * loop (:767-779), the H^L x 1^R loop with its Drs stride (:784-796), then
 * per stored term a freshly allocated C = B.V (:812-832) and Hv += A.C^T
 * (:839-853).  ref_hv_omp distributes the same arithmetic over output
 * sectors with OpenMP (the terms regrouped by RowOffset, as the reference's
 * MPI version regroups them), so it is race-free on all host cores.
 * ref_lanczos is Lanczos with full reorthogonalisation (the same algorithm
 * family as SciFortran sp_eigh), every vector operation in FP64: the
 * three-term recurrence first, then a classical Gram-Schmidt projection of
 * the residual against the whole basis (a second one when the first removes
 * more than half of it).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/nssdmrg.h"

static void hv_sector(const nss_sb_desc *d, int k, const double *v, double *hv) {
    const int dl = d->dls[k], dr = d->drs[k];
    const int64_t off = d->offset[k];
    const nss_csr *hr = &d->hright[k], *hl = &d->hleft[k];
    /* apply 1^L x H^R */
    for (int il = 0; il < dl; ++il)
        for (int ir = 0; ir < dr; ++ir) {
            const int64_t i = ir + (int64_t)il * dr + off;
            for (int jc = hr->rowptr[ir]; jc < hr->rowptr[ir + 1]; ++jc)
                hv[i] += hr->vals[jc] * v[hr->colidx[jc] + (int64_t)il * dr + off];
        }
    /* apply H^L x 1^R */
    for (int ir = 0; ir < dr; ++ir)
        for (int il = 0; il < dl; ++il) {
            const int64_t i = ir + (int64_t)il * dr + off;
            for (int jc = hl->rowptr[il]; jc < hl->rowptr[il + 1]; ++jc)
                hv[i] += hl->vals[jc] * v[ir + (int64_t)hl->colidx[jc] * dr + off];
        }
}

static void hv_term(const nss_sb_desc *d, int idx, const double *v, double *hv) {
    const nss_csr *A = &d->a[idx], *B = &d->b[idx];
    if (A->nrow == 0 || B->nrow == 0) return;
    double *C = (double *)calloc((size_t)B->nrow * A->ncol, sizeof(double));
    /* C = B.vec(V):  C(bi,aj) = sum_bj B(bi,bj) v(bj + aj*B.Ncol + ColOffset) */
    for (int aj = 0; aj < A->ncol; ++aj)
        for (int bi = 0; bi < B->nrow; ++bi)
            for (int jb = B->rowptr[bi]; jb < B->rowptr[bi + 1]; ++jb)
                C[bi + (int64_t)aj * B->nrow] +=
                    B->vals[jb] * v[B->colidx[jb] + (int64_t)aj * B->ncol + d->col_offset[idx]];
    /* Hv(bi + ai*B.Nrow + RowOffset) += sum_aj A(ai,aj) C(bi,aj) */
    for (int bi = 0; bi < B->nrow; ++bi)
        for (int ai = 0; ai < A->nrow; ++ai) {
            const int64_t i = bi + (int64_t)ai * B->nrow + d->row_offset[idx];
            for (int ja = A->rowptr[ai]; ja < A->rowptr[ai + 1]; ++ja)
                hv[i] += A->vals[ja] * C[bi + (int64_t)A->colidx[ja] * B->nrow];
        }
    free(C);
}

static int64_t sb_n(const nss_sb_desc *d) {
    int64_t n = 0;
    for (int k = 0; k < d->nsb; ++k) n += (int64_t)d->dls[k] * d->drs[k];
    return n;
}

void ref_hv_serial(const nss_sb_desc *d, const double *v, double *hv) {
    memset(hv, 0, sizeof(double) * sb_n(d));
    for (int k = 0; k < d->nsb; ++k) {
        hv_sector(d, k, v, hv);
        for (int it = 0; it < d->tnso; ++it) hv_term(d, it + d->tnso * k, v, hv);
    }
}

/* sector index whose Offset equals off (binary search; offsets ascend) */
static int sector_at(const nss_sb_desc *d, int64_t off) {
    int lo = 0, hi = d->nsb - 1;
    while (lo <= hi) {
        int mid = (lo + hi) / 2;
        if (d->offset[mid] == off) return mid;
        if (d->offset[mid] < off) lo = mid + 1;
        else hi = mid - 1;
    }
    return -1;
}

void ref_hv_omp(const nss_sb_desc *d, const double *v, double *hv, int nthreads) {
    const int64_t n = sb_n(d);
    const int nt = d->tnso * d->nsb;
    int *out_sec = (int *)malloc(sizeof(int) * (nt > 0 ? nt : 1));
    for (int idx = 0; idx < nt; ++idx)
        out_sec[idx] = (d->a[idx].nrow && d->b[idx].nrow) ? sector_at(d, d->row_offset[idx]) : -1;
#pragma omp parallel num_threads(nthreads)
    {
#pragma omp for schedule(static)
        for (int64_t i = 0; i < n; ++i) hv[i] = 0.0;
#pragma omp for schedule(dynamic, 1)
        for (int k = 0; k < d->nsb; ++k) {
            hv_sector(d, k, v, hv);
            for (int idx = 0; idx < nt; ++idx)
                if (out_sec[idx] == k) hv_term(d, idx, v, hv);
        }
    }
    free(out_sec);
}

/* ---- Lanczos ----------------------------------------------------------- */
static uint64_t splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

static int sturm(const double *a, const double *b, int m, double x) {
    double p0 = 1.0, p1 = a[0] - x;
    int cnt = p1 < 0.0;
    for (int i = 1; i < m; ++i) {
        double p2 = (a[i] - x) * p1 - b[i - 1] * b[i - 1] * p0;
        if (p2 == 0.0) p2 = -copysign(1e-300, p1);
        if ((p2 < 0.0) != (p1 < 0.0)) ++cnt;
        p0 = p1;
        p1 = p2;
        double s = fmax(fabs(p0), fabs(p1));
        if (s > 0x1p+600) { p0 *= 0x1p-600; p1 *= 0x1p-600; }
        else if (s < 0x1p-600) { p0 *= 0x1p+600; p1 *= 0x1p+600; }
    }
    return cnt;
}

/* e-th eigenvalue of T by bisection, eigenvector by inverse iteration */
static double tri_eig(const double *a, const double *b, int m, int e, double *s, double *work) {
    double lo = 1e300, hi = -1e300;
    for (int i = 0; i < m; ++i) {
        double r = (i > 0 ? fabs(b[i - 1]) : 0.0) + (i < m - 1 ? fabs(b[i]) : 0.0);
        if (a[i] - r < lo) lo = a[i] - r;
        if (a[i] + r > hi) hi = a[i] + r;
    }
    for (int it = 0; it < 200 && hi - lo > 4e-16 * fmax(fabs(lo), fabs(hi)) + 1e-300; ++it) {
        double mid = 0.5 * (lo + hi);
        if (sturm(a, b, m, mid) > e) hi = mid;
        else lo = mid;
    }
    const double th = 0.5 * (lo + hi), sh = th + 1e-14 * fmax(fabs(th), 1.0);
    double *D = work, *DU = work + m, *DL = work + 2 * m;
    for (int i = 0; i < m; ++i) s[i] = 1.0 + 0.01 * (double)((i * 7 + e * 3) % 11);
    for (int rep = 0; rep < 3; ++rep) {
        for (int i = 0; i < m; ++i) {
            D[i] = a[i] - sh;
            DU[i] = DL[i] = (i < m - 1) ? b[i] : 0.0;
        }
        for (int i = 0; i < m - 1; ++i) {
            if (fabs(D[i]) >= fabs(DL[i])) {
                if (D[i] == 0.0) D[i] = 1e-300;
                double f = DL[i] / D[i];
                D[i + 1] -= f * DU[i];
                s[i + 1] -= f * s[i];
                DL[i] = 0.0;
            } else {
                double f = D[i] / DL[i], t = D[i + 1];
                D[i] = DL[i];
                D[i + 1] = DU[i] - f * t;
                if (i < m - 2) { DL[i] = DU[i + 1]; DU[i + 1] = -f * DL[i]; } else DL[i] = 0.0;
                DU[i] = t;
                double b0 = s[i];
                s[i] = s[i + 1];
                s[i + 1] = b0 - f * s[i + 1];
            }
        }
        if (D[m - 1] == 0.0) D[m - 1] = 1e-300;
        s[m - 1] /= D[m - 1];
        if (m > 1) s[m - 2] = (s[m - 2] - DU[m - 2] * s[m - 1]) / D[m - 2];
        for (int i = m - 3; i >= 0; --i) s[i] = (s[i] - DU[i] * s[i + 1] - DL[i] * s[i + 2]) / D[i];
        double nrm = 0.0;
        for (int i = 0; i < m; ++i) nrm += s[i] * s[i];
        nrm = 1.0 / sqrt(nrm);
        for (int i = 0; i < m; ++i) s[i] *= nrm;
    }
    return th;
}

/* Lowest `neigen` eigenvalues of the superblock H; returns 0 when converged,
 * 1 when nitermax was reached.  The matvec is ref_hv_omp (nthreads > 1) or
 * ref_hv_serial; the numop and the time split are reported to the caller. */
/* ref_lanczos_vec: as ref_lanczos, and when evecs is not NULL it also
 * receives the neigen Ritz vectors (row e = vector e, unit norm). */
int ref_lanczos_vec(const nss_sb_desc *d, int neigen, int nitermax, double tol, uint64_t seed, int nthreads,
                    double *evals, double *evecs, int *numop) {
    const int64_t n = sb_n(d);
    int mmax = nitermax < n ? nitermax : (int)n;
    double *V = (double *)malloc(sizeof(double) * n * (size_t)(mmax + 1));
    double *w = (double *)malloc(sizeof(double) * n);
    double *h = (double *)malloc(sizeof(double) * (mmax + 1));
    double *alpha = (double *)calloc(mmax + 1, sizeof(double));
    double *beta = (double *)calloc(mmax + 1, sizeof(double));
    double *s = (double *)malloc(sizeof(double) * (mmax + 1));
    double *work = (double *)malloc(sizeof(double) * 3 * (mmax + 1));
    if (!V || !w || !h || !alpha || !beta || !s || !work) return -1;
    double nrm = 0.0;
    for (int64_t i = 0; i < n; ++i) {
        uint64_t r = splitmix64(seed ^ splitmix64((uint64_t)i));
        V[i] = 2.0 * ((double)(r >> 11) * (1.0 / 9007199254740992.0)) - 1.0;
        nrm += V[i] * V[i];
    }
    nrm = 1.0 / sqrt(nrm);
    for (int64_t i = 0; i < n; ++i) V[i] *= nrm;
    int m = 0, conv = 0, ops = 0;
    while (m < mmax) {
        const int j = m;
        double *vj = V + (size_t)j * n;
        if (nthreads > 1) ref_hv_omp(d, vj, w, nthreads);
        else ref_hv_serial(d, vj, w);
        ++ops;
        m = j + 1;
        /* three-term recurrence first, then full reorthogonalisation */
        double a = 0.0;
#pragma omp parallel for num_threads(nthreads) reduction(+ : a)
        for (int64_t i = 0; i < n; ++i) a += vj[i] * w[i];
        const double bprev = j > 0 ? beta[j - 1] : 0.0;
        const double *vjm = j > 0 ? V + (size_t)(j - 1) * n : vj;
        double ww = 0.0;
#pragma omp parallel for num_threads(nthreads) reduction(+ : ww)
        for (int64_t i = 0; i < n; ++i) {
            double x = w[i] - a * vj[i];
            if (j > 0) x -= bprev * vjm[i];
            w[i] = x;
            ww += x * x;
        }
        alpha[j] = a;
        double bb = 0.0;
        for (int pass = 0; pass < 2; ++pass) {
            for (int l = 0; l < m; ++l) {
                double acc = 0.0;
                const double *vl = V + (size_t)l * n;
#pragma omp parallel for num_threads(nthreads) reduction(+ : acc)
                for (int64_t i = 0; i < n; ++i) acc += vl[i] * w[i];
                h[l] = acc;
            }
            bb = 0.0;
#pragma omp parallel for num_threads(nthreads) reduction(+ : bb)
            for (int64_t i = 0; i < n; ++i) {
                double x = w[i];
                for (int l = 0; l < m; ++l) x -= V[(size_t)l * n + i] * h[l];
                w[i] = x;
                bb += x * x;
            }
            alpha[j] += h[j];
            if (!(bb < 0.5 * ww)) break;
            ww = bb;
        }
        beta[j] = sqrt(bb);
        if (m % 8 == 0 || m == mmax || m == n) {
            conv = 0;
            for (int e = 0; e < neigen && e < m; ++e) {
                double th = tri_eig(alpha, beta, m, e, s, work);
                evals[e] = th;
                if (fabs(beta[m - 1] * s[m - 1]) <= tol * fmax(fabs(th), 1e-300)) ++conv;
            }
            if (conv >= neigen || m == n) break;
        }
        const double scale = fmax(fabs(alpha[j]), j > 0 ? beta[j - 1] : 0.0);
        if (!(beta[j] > 1e-13 * fmax(scale, 1e-300))) break;
        const double inv = 1.0 / beta[j];
        double *vn = V + (size_t)m * n;
#pragma omp parallel for num_threads(nthreads)
        for (int64_t i = 0; i < n; ++i) vn[i] = w[i] * inv;
    }
    for (int e = 0; e < neigen && e < m; ++e) {
        evals[e] = tri_eig(alpha, beta, m, e, s, work);
        if (!evecs) continue;
        double *x = evecs + (size_t)e * n, nx = 0.0;
#pragma omp parallel for num_threads(nthreads) reduction(+ : nx)
        for (int64_t i = 0; i < n; ++i) {
            double acc = 0.0;
            for (int l = 0; l < m; ++l) acc += s[l] * V[(size_t)l * n + i];
            x[i] = acc;
            nx += acc * acc;
        }
        nx = 1.0 / sqrt(nx);
#pragma omp parallel for num_threads(nthreads)
        for (int64_t i = 0; i < n; ++i) x[i] *= nx;
    }
    if (numop) *numop = ops;
    free(V); free(w); free(h); free(alpha); free(beta); free(s); free(work);
    return conv >= neigen ? 0 : 1;
}

int ref_lanczos(const nss_sb_desc *d, int neigen, int nitermax, double tol, uint64_t seed, int nthreads,
                double *evals, int *numop) {
    return ref_lanczos_vec(d, neigen, nitermax, tol, seed, nthreads, evals, NULL, numop);
}

int ref_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
