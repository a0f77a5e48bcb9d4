/*
 * nssdmrg.h -- C ABI of the GB300 superblock eigensolver for nssDMRG.
 *
 * The reference library (Fortran, aamaricci/nssDMRG) runs its superblock
 * eigensolve through three seams, and this ABI replaces each of them:
 *
 *  1. the H·v callback.  `procedure(sparse_HxV), pointer :: spHtimesV_p`
 *     (src/DMRG_GLOBAL.f90:41-53) is pointed at spMatVec_direct_main
 *     (src/DMRG_SUPERBLOCK_SETUP.f90:740-865), which reads the module-global
 *     operator pool Hleft, Hright, A, B, Dls, Drs, Offset, RowOffset,
 *     ColOffset, isb2jsb, IsHconjg (src/DMRG_GLOBAL.f90:119-124).
 *     nss_sb_upload() takes that pool once per DMRG step; nss_hv() has the
 *     sparse_HxV(Nloc, v, Hv) semantics.
 *  2. the eigensolver.  sb_diag calls SciFortran sp_eigh(spHtimesV_p, ...)
 *     (src/DMRG_SUPERBLOCK.f90:335-474); nss_eigh() replaces that call.
 *  3. the RDM.  sb_get_rdm + blocks_matrix%eigh + the truncation choice of
 *     renormalize_block (src/DMRG_RDM.f90:18-221, :277-294;
 *     src/MATRIX/MATRIX_BLOCKS.f90:589-657) become nss_rdm().
 *
 * Every entry point returns 0 on success or a negative NSS_ERR_* code; none
 * aborts.  nss_last_error() gives the message (the reference `stop`s with a
 * message instead).  A context is single-caller and not re-entrant.
 * Indices in this ABI are 0-based (the reference is 1-based).
 */
#ifndef NSSDMRG_H
#define NSSDMRG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NSS_OK               0
#define NSS_ERR_INVALID     -1   /* bad argument or inconsistent descriptor */
#define NSS_ERR_CUDA        -2   /* CUDA runtime or library error */
#define NSS_ERR_NOMEM       -3   /* allocation failed or over the HBM budget */
#define NSS_ERR_STATE       -4   /* call out of order (e.g. nss_hv before upload) */
#define NSS_ERR_NOCONV      -5   /* eigensolver hit its iteration cap */
#define NSS_ERR_ASYMMETRIC  -6   /* rho not symmetric to 1e-12 (DMRG_RDM.f90:159-160) */
#define NSS_ERR_NOCUDA      -7   /* no CUDA device */

/* Precision modes for nss_eigh. */
#define NSS_PREC_FP64        0   /* plain method: every product in FP64 */
#define NSS_PREC_MIXED       1   /* sector GEMMs on tensor cores, FP64 Lanczos + refinement */

typedef struct nss_ctx nss_ctx;

/* One sparse operator block in row-list (CSR) form, 0-based.  A block with
 * nrow == 0 is "absent" (the reference's status=.false.). */
typedef struct {
    int32_t nrow, ncol;
    const int32_t *rowptr;   /* nrow+1 entries */
    const int32_t *colidx;   /* rowptr[nrow] entries */
    const double  *vals;     /* rowptr[nrow] entries */
} nss_csr;

/* The direct-mode operator pool, flattened.  Arrays of length nsb are per
 * superblock sector k; arrays of length tnso*nsb are indexed it + tnso*k,
 * the column-major order of the reference's A(it,k). */
typedef struct {
    int32_t nsb;              /* size(sb_sector) */
    int32_t tnso;             /* terms per sector (3 spin, 4 Hubbard, OBC) */
    int32_t m_left, m_right;  /* dims of the enlarged left/right blocks */
    const int32_t *dls;       /* [nsb] Dls(k) */
    const int32_t *drs;       /* [nsb] Drs(k) */
    const int64_t *offset;    /* [nsb] Offset(k) */
    const int32_t *ai;        /* [sum dls] left block states of each sector (AI), ascending */
    const int32_t *bi;        /* [sum drs] right block states of each sector (BI), ascending */
    const nss_csr *hleft;     /* [nsb]  Hleft(k)  Dl x Dl */
    const nss_csr *hright;    /* [nsb]  Hright(k) Dr x Dr */
    const nss_csr *a;         /* [tnso*nsb] A(it,k) */
    const nss_csr *b;         /* [tnso*nsb] B(it,k) */
    const int32_t *isb2jsb;   /* [tnso*nsb] isb2jsb(it,k), 0-based (unused when absent) */
    const int32_t *ishconjg;  /* [tnso*nsb] IsHconjg(it,k) */
    const int64_t *row_offset;/* [tnso*nsb] RowOffset(it,k) */
    const int64_t *col_offset;/* [tnso*nsb] ColOffset(it,k) */
} nss_sb_desc;

/* Create a context on CUDA device `device`.  hbm_budget (bytes) caps what
 * the context may allocate; 0 means no cap.  Returns NULL on failure; the
 * reason is then available from nss_last_error(NULL). */
nss_ctx    *nss_create(int device, size_t hbm_budget);
void        nss_destroy(nss_ctx *ctx);
const char *nss_last_error(const nss_ctx *ctx);

/* Upload the superblock operator pool; replaces the Setup_SuperBlock_Direct
 * -> spHtimesV_p assignment (src/DMRG_SUPERBLOCK.f90:553-573,
 * src/DMRG_SUPERBLOCK_SETUP.f90:113-136).  Copies everything: the caller
 * may free its arrays on return.  Replaces any previous superblock.
 * Inconsistent sizes, out-of-range indices and non-finite operator values
 * are refused with NSS_ERR_INVALID; a context over its hbm_budget returns
 * NSS_ERR_NOMEM. */
int nss_sb_upload(nss_ctx *ctx, const nss_sb_desc *desc);
/* Free the device superblock (sb_delete_Hv, src/DMRG_SUPERBLOCK.f90:582-620). */
int nss_sb_free(nss_ctx *ctx);
/* Vector length of the uploaded superblock (sb_vecDim_Hv, :626-646). */
int64_t nss_sb_dim(const nss_ctx *ctx);
/* Shape of the uploaded superblock: sectors, enlarged block dims, N. */
int nss_sb_shape(const nss_ctx *ctx, int32_t *nsb, int32_t *m_left, int32_t *m_right, int64_t *n);

/* Algorithmic work of one H*v on the uploaded superblock: the dense sector
 * products 2 Dl Dr (Dl + Dr) summed over sectors, and the A x B terms counted
 * as the reference's loops count them, 2 (nnz(B) Ncol(A) + nnz(A) Nrow(B))
 * (src/DMRG_SUPERBLOCK_SETUP.f90:819-853).  Either pointer may be NULL. */
int nss_sb_flops(const nss_ctx *ctx, double *dense, double *ab);
/* Number of kernels of this library launched on the context so far (library
 * kernels of cuSOLVER are not counted). */
int64_t nss_kernel_launches(const nss_ctx *ctx);
/* Bytes copied host->device by the last nss_sb_upload / nss_sb_setup. */
int64_t nss_sb_upload_bytes(const nss_ctx *ctx);
/* The CUDA stream (cudaStream_t) all work of the context is ordered on. */
void *nss_stream(const nss_ctx *ctx);

/* sparse_HxV: hv = H_sb v for host vectors of length n (must equal
 * nss_sb_dim).  spMatVec_direct_main semantics: hv is overwritten. */
int nss_hv(nss_ctx *ctx, int64_t n, const double *v, double *hv);
/* Same on device pointers, ordered on the context's stream. */
int nss_hv_device(nss_ctx *ctx, int64_t n, const double *d_v, double *d_hv);
/* The FP32 product of the mixed-precision path, on device pointers. */
int nss_hv_device_f32(nss_ctx *ctx, int64_t n, const float *d_v, float *d_hv);

/* Lowest `neigen` eigenpairs of the uploaded H_sb (replaces sp_eigh at
 * src/DMRG_SUPERBLOCK.f90:394-425).  nitermax caps the Krylov dimension,
 * tol is the relative residual tolerance (lanc_tolerance), seed fixes the
 * random start vector.  evals[neigen] receives the eigenvalues (ascending);
 * evecs, if not NULL, receives the n x neigen eigenvectors (column-major,
 * the reference's gs_vector); they also stay resident on the device for
 * nss_rdm.  numop (may be NULL) receives the number of H·v products.
 * ncv is accepted for interface parity with sp_eigh and ignored (the solver
 * keeps the whole Krylov basis instead of restarting). */
int nss_eigh(nss_ctx *ctx, int neigen, int nitermax, int ncv, double tol,
             uint64_t seed, int precision, double *evals, double *evecs,
             int *numop);

/* Result of nss_rdm for one side of the superblock. */
typedef struct {
    int32_t nevals;        /* number of rho eigenvalues (= sum of block sizes) */
    int32_t m_s;           /* kept states after the degeneracy extension */
    double  trunc_err;     /* 1 - sum(lambda(1:m_s)) */
    double  entropy;       /* -sum lambda log(lambda + 1e-32) */
    double  s_number;      /* S_N = -sum_q P_q log(P_q + 1e-32), P_q = sum of block q's lambda */
    double  s_config;      /* S_c = -sum_q P_q S_q, S_q = sum_i (l_i/P_q) log(l_i/P_q + 1e-32)
                              (write_entanglement, src/DMRG_MAIN.f90:523-561) */
} nss_rdm_side;

/* Batched ground states: nb independent superblocks, one context each (all
 * on one device, each with a superblock uploaded), solved together with the
 * mixed method (precision NSS_PREC_MIXED semantics, one eigenpair) by one
 * persistent cooperative launch per group of iterations, the H*psi work
 * items of all solves shared out over the whole GPU.  evals[b] receives the
 * FP64 energy of solve b, numops[b] its H*psi count; each context keeps its
 * ground state for nss_rdm.  No counterpart in the reference (it solves one
 * superblock at a time); each result equals the one nss_eigh gives for that
 * context alone to within the solver tolerance.  Superblocks with
 * tensor-core sectors (NSS_TC_MIN_DL) are rejected. */
int nss_eigh_batch(nss_ctx *const *ctxs, int nb, int nitermax, double tol, const uint64_t *seeds,
                   double *evals, int *numops);

/* Continuous batching (serving): a batch engine runs rounds of the batched
 * persistent kernel over the solves in flight; solves join between rounds
 * (nss_batch_add: the context must hold an uploaded superblock) and leave
 * when done (nss_batch_step reports up to max_done of them: ids[q] is the id
 * nss_batch_add returned, negative when that solve failed; energies[q] its
 * FP64 energy; the context keeps the ground state for nss_rdm).  `host`
 * provides the device, the stream and the barrier; it may also be one of
 * the solving contexts.  At most one batch per host context.  A round that
 * fails (nss_batch_step returns non-zero) drops every solve in flight: their
 * contexts leave the batch unsolved, may be solved alone or freed, and may
 * join again.  No counterpart in the reference. */
typedef struct nss_batch nss_batch;
nss_batch *nss_batch_create(nss_ctx *host);
int nss_batch_add(nss_batch *b, nss_ctx *ctx, uint64_t seed, int nitermax, double tol, int *id);
int nss_batch_step(nss_batch *b, int max_done, int *ndone, int *ids, double *energies, int *numops);
int nss_batch_inflight(const nss_batch *b);
void nss_batch_destroy(nss_batch *b);

/* Reduced density matrices of the ground state (column 0 of the last
 * nss_eigh, or `psi` when not NULL, length nss_sb_dim), their block
 * eigendecomposition and the truncation choice (src/DMRG_RDM.f90:18-221,
 * :277-294).  mstates is Mstates, deg_thr is deg_evals_threshold.  Per side
 * (index 0 left, 1 right) the optional outputs are
 *   lambda[side]  : nevals eigenvalues, descending, negatives clipped to 0
 *   kept_blk[side]: m_s ints, the rho block (= superblock sector) of each
 *                   kept column, in rank order (its QN is the block's QN)
 *   u[side]       : m_block x m_s column-major rotation matrix (U = trRho)
 * with m_block = m_left / m_right of the descriptor.  Any may be NULL. */
int nss_rdm(nss_ctx *ctx, const double *psi, int mstates, double deg_thr,
            nss_rdm_side out[2], double *lambda_left, double *lambda_right,
            int32_t *kept_left, int32_t *kept_right,
            double *u_left, double *u_right);

/* nss_rdm with the reference's second truncation rule: renormalize_block's
 * (Mstates, Estates) pair (src/DMRG_RDM.f90:204-211, right side :277-284).
 * mstates != 0 keeps min(mstates, m_block, nevals) states as nss_rdm does;
 * mstates == 0 with estates != 0 keeps the m_s that minimises
 * |1 - sum(lambda(1:m_s)) - estates| (the first such m_s), i.e. the
 * discarded weight closest to the threshold Edmrg; both are then extended
 * over degenerate eigenvalues.  mstates == 0 with estates == 0 is refused
 * with NSS_ERR_INVALID, as the reference stops there. */
int nss_rdm_estates(nss_ctx *ctx, const double *psi, int mstates, double estates, double deg_thr,
                    nss_rdm_side out[2], double *lambda_left, double *lambda_right,
                    int32_t *kept_left, int32_t *kept_right,
                    double *u_left, double *u_right);

/* OdotV_direct (src/DMRG_MEASURE.f90:653-705): ov = (O x 1) v for label
 * 'l' (or 's') and ov = (1 x O) v for 'r' (or 'e') on the uploaded
 * superblock, where ops[k] (k < nsb) is the block operator filtered to
 * sector k's left / right states (Dl_k x Dl_k or Dr_k x Dr_k, 0-based CSR)
 * and v, ov are host arrays of length nss_sb_dim. */
int nss_odotv(nss_ctx *ctx, char label, const nss_csr *ops, const double *v, double *ov);

/* Average_Op_dmrg (src/DMRG_MEASURE.f90:595-646): <psi| O |psi> for a whole
 * block operator O (m_left x m_left for label 'l', m_right x m_right for
 * 'r', 0-based CSR).  O is filtered to every sector's states with the sector
 * maps of the uploaded descriptor (ai / bi, the reference's LI / RI) and
 * applied on the device.  psi: host vector of length nss_sb_dim, or NULL
 * for the ground state of the last nss_eigh. */
int nss_average_op(nss_ctx *ctx, char label, const nss_csr *op, const double *psi, double *val);

/* Eigensolver statistics of the last nss_rdm: rho blocks diagonalised by the
 * library's own FP64 eigensolver (Householder tridiagonalisation, bisection,
 * twisted-factorisation vectors of the kept states), blocks sent to the
 * Jacobi / batched cuSOLVER path (larger than 160, or env
 * NSS_RDM_EIG=library), and own blocks whose kept vectors were recomputed by
 * that path (close relative eigenvalue gaps).  No counterpart in the
 * reference (LAPACK dsyev per block, src/MATRIX/MATRIX_BLOCKS.f90:589-657). */
int nss_rdm_stats(const nss_ctx *ctx, int *own_blocks, int *library_blocks, int *fallback_blocks);

/* The mixed method's refinement in the last nss_eigh: the passes it took
 * (each anchors every refined vector in FP64 and corrects it with FP32
 * Lanczos), the size of the refined cluster (the wanted vectors plus
 * near-degenerate partners, resolved by an FP64 Rayleigh-Ritz step before
 * every later pass), and how many mixed solves of the context's life were
 * redone in FP64 because the refinement did not reach the tolerance.  No
 * counterpart in the reference (ARPACK in FP64). */
int nss_refine_stats(const nss_ctx *ctx, int *passes, int *cluster, int64_t *fp64_fallbacks);

/* Why blocks fell back to the library path, counted over the context's life:
 * out[0] L D L^T not positive definite, out[1] a kept eigenvalue within 32 eps
 * of a neighbour, out[2] the Rayleigh iteration did not settle, out[3] a
 * Gram-Schmidt remainder below 1/2, out[4] a relative cluster with more than
 * 16 kept members.  No counterpart in the reference. */
int nss_rdm_fallback_reasons(const nss_ctx *ctx, int64_t out[5]);

/* Timing of the mixed method's persistent Lanczos kernel: with `enable`
 * set, each launch in later nss_eigh calls is bracketed by CUDA events on
 * the context stream; nss_chunk_stats returns, for the last nss_eigh, the
 * summed launch time (ms), the launches and the iterations they completed,
 * and the sum over those iterations of the basis size m (the orthogonalised
 * columns, for the bytes each iteration reads). */
int nss_time_chunks(nss_ctx *ctx, int enable);
int nss_chunk_stats(const nss_ctx *ctx, double *ms, int *launches, int64_t *iters, double *cols);

/* The persistent kernel's shared-memory row cache in the context's Lanczos
 * workspace (set up by the last mixed nss_eigh): how many basis vectors each
 * CTA keeps of its rows, and the rows per CTA (0, 0: no cache; a basis that
 * is too large for it, or NSS_CHUNK_CACHE=0).  No counterpart in the
 * reference. */
int nss_chunk_cache(const nss_ctx *ctx, int *vectors, int64_t *rows);

/* CUDA graphs of the last nss_eigh: Lanczos chunks (four iterations of H*psi
 * and orthogonalisation) that ran as one replayed graph, and graphs captured.
 * They apply where an iteration is several launches (the FP64 method, the
 * mixed method with tensor-core sectors); NSS_GRAPH=0 turns them off.  No
 * counterpart in the reference. */
int nss_graph_stats(const nss_ctx *ctx, int *replays, int *captures);

/* The mixed path's plan for the uploaded superblock, as the tile tuner chose
 * it: candidate 0 puts every sector on CUDA cores (the persistent Lanczos
 * kernel), 1 and 2 the sectors with Dl >= 32 on the tensor-core GEMM with
 * 64- or 128-column tiles (-1: the tuner is off, NSS_TC_MIN_DL or
 * NSS_TC_AUTO=0).  The tuner keys superblocks by N and their largest left
 * sector (quarter-octave bins), plans the first ones of a class with each
 * candidate once, records each converged mixed solve's device time per H*psi
 * product, and then keeps the fastest.  ms_per_hv[3] / solves[3] give the
 * class's measurements so far (-1 / 0: not tried).  nss_tune_reset forgets
 * every class.  No counterpart in the reference. */
int nss_tune_info(const nss_ctx *ctx, int *candidate, double *ms_per_hv, int *solves);
void nss_tune_reset(void);

/* Energy <psi|H|psi> / <psi|psi> of a device vector d_psi (length n =
 * nss_sb_dim) on the uploaded superblock, written to *energy (host), without
 * allocating any memory.  No counterpart in the reference: it is for callers
 * that cannot allocate device memory when they need an energy (a host code
 * whose device heap belongs to another allocator, a context whose HBM budget
 * is spent).  Its scratch is a static device array of 32768 16x16-tile
 * partial sums (512 KiB per GPU that loads the library, held until exit);
 * larger superblocks are rejected with NSS_ERR_INVALID, and so is a psi of
 * zero norm.  The first call on each context looks up that array's device
 * address and should come before any stream capture.  Each call waits for
 * its kernel and copies the energy into host memory before it returns;
 * calls that overlap on the GPU race on the shared array. */
int nss_sb_energy_noalloc(nss_ctx *ctx, int64_t n, const double *d_psi, double *energy);

/* Lowest ne eigenpairs of the symmetric tridiagonal matrix with diagonal
 * a[0..m) and off-diagonal b[0..m-1), computed on the host CPU: the solver
 * nss_eigh runs on the Lanczos matrix T_m while the GPU works on the next
 * iterations (the reference hands T_m to ARPACK on the host,
 * src/DMRG_SUPERBLOCK.f90:412-425).  Outputs theta[ne] ascending, s[ne*m]
 * unit eigenvectors (row e = vector e, largest component positive) and
 * resid[ne] = |b_last * s_e[m-1]|.  Needs no context and no GPU. */
int nss_tridiag_lowest(int m, const double *a, const double *b, int ne, double b_last,
                       double *theta, double *s, double *resid);

/* Lowest eigenpair of the (k+1)x(k+1) matrix [[theta0, m^T], [m, T]] with T
 * tridiagonal (diagonal a[0..k), off-diagonal b[0..k-1)), on the host: the
 * small problem of the FP64-anchored refinement that nss_eigh's mixed
 * precision runs after its FP32 phase (no counterpart in the reference,
 * whose Lanczos is FP64 throughout).  Outputs *lam, c[k+1] (unit norm,
 * c[0] > 0) and *resid = |b_last * c[k]|.  Needs no context and no GPU. */
/* All eigenpairs of the symmetric tridiagonal matrix (diagonal d[n],
 * off-diagonal e[n-1]) by implicit QL with Wilkinson shifts: evals[n]
 * ascending, Z[n*n] column-major with column j the eigenvector of evals[j].
 * The host solver the RDM uses for flagged rho blocks (their tridiagonal
 * matrices after the device reduction); needs no context and no GPU. */
int nss_tridiag_eig(int n, const double *d, const double *e, double *evals, double *Z);
/* The Kronecker sums of enlarge_block, H = Hb + Hd + H2
 * (src/DMRG_CONNECT.f90:75-107 with connect_spin_blocks :437-439 and
 * connect_fermion_blocks :370-371; sp_kron_matrix,
 * src/MATRIX/MATRIX_SPARSE.f90:832-876): out = sum_t coef[t] * (a[t] x b[t]),
 * row i*nb+k, column j*nb+l, each a[t] na x na and b[t] nb x nb.  Host
 * only, no context.  Entries appear in the order of their first term and
 * stay when they cancel, like sp_sum.  With colidx or vals NULL only *nnz is
 * returned; otherwise cap must hold it.  nthreads <= 0 uses every core. */
int nss_kron_sum(int32_t na, int32_t nb, int32_t nterms, const double *coef, const nss_csr *a, const nss_csr *b,
                 int nthreads, int64_t cap, int64_t *nnz, int32_t *rowptr, int32_t *colidx, double *vals);
int nss_arrow_lowest(int k, double theta0, const double *m, const double *a, const double *b, double b_last,
                     double *lam, double *c, double *resid);

/* ---------------------------------------------------------------------------
 * Block-level superblock setup (the enumeration and operator-pool build of
 * sb_get_states / sb_build_dims / Setup_SuperBlock_{Spin,Fermion}_Direct,
 * src/DMRG_SUPERBLOCK.f90:36-283 and src/DMRG_SUPERBLOCK_SETUP.f90:152-693,
 * :1079-1122), for callers that hand over the enlarged blocks instead of a
 * ready pool.  Operators are full block matrices in CSR form.
 * ------------------------------------------------------------------------- */
#define NSS_SITE_SPIN      0   /* operators S_z_n, S_p_n */
#define NSS_SITE_FERMION   1   /* operators C_l1_s1_n, C_l1_s2_n, P_n */

typedef struct {
    int32_t dim;            /* block dimension */
    int32_t qdim;           /* QN tuple length */
    const double *basis;    /* [dim*qdim] QN tuple of every state (row-major) */
    nss_csr h;              /* "H" */
    nss_csr op[3];          /* spin: Sz, S+ ; fermion: C_up, C_dw, P */
} nss_block_desc;

/* Enumerate the superblock of target QN `target` (qdim values) and upload
 * its operator pool.  site_type is NSS_SITE_*; hij is the Nso x Nso coupling
 * matrix (row-major, Nso = 2), the reference's HopH. */
int nss_sb_setup(nss_ctx *ctx, int site_type, const nss_block_desc *left,
                 const nss_block_desc *right, const double *target,
                 const double *hij);
/* Sector tables of the current superblock (built by nss_sb_setup, or by the
 * driver's nss_dmrg_prepare_last on this context): nsb, sector QNs (left QN,
 * qdim each), Dls, Drs, Offset and sb_states (left*m_right + right, 0-based).
 * Pass NULL for anything not wanted; sizes from nss_sb_counts. */
int nss_sb_counts(const nss_ctx *ctx, int32_t *nsb, int32_t *qdim, int64_t *n);
int nss_sb_tables(const nss_ctx *ctx, double *qns, int32_t *dls, int32_t *drs,
                  int64_t *offset, int64_t *sb_states);

/* ---------------------------------------------------------------------------
 * DMRG driver (init_dmrg / run_DMRG / finalize_dmrg, src/DMRG_MAIN.f90:9-14,
 * :22-72, :140-241, :262-433): OBC infinite and finite algorithms with every
 * superblock solve on the GPU.
 * ------------------------------------------------------------------------- */
#define NSS_MODEL_HEISENBERG_HALF 0   /* spin_site(sun=2) */
#define NSS_MODEL_HEISENBERG_ONE  1   /* spin_site(sun=3) */
#define NSS_MODEL_HUBBARD         2   /* electron_site, Norb=1 */

typedef struct {
    int32_t model;          /* NSS_MODEL_* */
    double  jz, jxy;        /* Heisenberg: Hlr = diag(jz, jxy/2) */
    double  t, u;           /* Hubbard: Hlr = diag(-t,-t), Uloc = u */
    int32_t hfmode;         /* Hubbard Hartree shift (HFMODE) */
    double  dmrg_qn[2];     /* target QN in units of L (DMRG_QN, QNtype local) */
    int32_t ldmrg;          /* Ldmrg */
    int32_t mdmrg;          /* Mdmrg */
    int32_t nsweep;         /* number of finite sweeps (0: infinite only) */
    const int32_t *msweep;  /* [nsweep] states per sweep */
    int32_t lanc_neigen;    /* default 2 */
    int32_t lanc_niter;     /* default 512 */
    double  lanc_tolerance; /* default 1e-12 */
    double  deg_evals_threshold; /* default 0.1 */
    uint64_t seed;
    int32_t precision;      /* NSS_PREC_* */
    int32_t save_umat;      /* keep every renormalisation's rotation matrix
                               on the host (SAVE_UMAT with STORE_UMAT='b'),
                               which nss_dmrg_measure needs */
    double  edmrg;          /* Edmrg: truncation threshold used when mdmrg == 0
                               (src/INPUT_VARS.f90:16-19) */
    const double *esweep;   /* [nsweep] Esweep, used where msweep is 0; NULL:
                               edmrg for every sweep */
} nss_dmrg_params;

typedef struct {
    int32_t type;           /* 0 infinite, 1 finite */
    int32_t left_length, right_length, current_l;
    int64_t n;              /* superblock dimension */
    int32_t nsb;
    int32_t numop;
    double  energy[2];      /* gs_energy / current_L / Norb (lanc_neigen <= 2) */
    double  entropy_left, entropy_right;
    double  trunc_left, trunc_right;
    int32_t m_left, m_right;   /* block dims after the step */
    double  ms_solve;       /* device time of nss_eigh + nss_rdm */
    double  ms_eigh;        /* device time of nss_eigh alone */
    double  ms_step;        /* host wall time of the whole step (block build,
                               superblock upload, solve, renormalisation) */
    double  ms_build;       /* host time of the block enlargement and the
                               superblock build */
    double  ms_renorm;      /* host time of the operator renormalisation */
    int64_t nnz_u;          /* nonzeros of the two rotation matrices */
    int64_t nnz_ops;        /* nonzeros of the renormalised block operators */
    int32_t rdm_own_blocks;     /* rho blocks on the own eigensolver ... */
    int32_t rdm_fallback_blocks;/* ... and those whose kept vectors the library recomputed */
    double  sn_left, sc_left, sn_right, sc_right;   /* S_N, S_c per side (SN_ScVSblock.length) */
    double  rdm_phase_ms[6];/* device time of the RDM phases: rho build, tridiagonal
                               reductions, eigenvalues, truncation, kept vectors, U */
    int32_t rdm_path_blocks[4]; /* rho blocks per eigensolver tier: one CTA, cluster,
                                   blocked library reduction, library eigensolver */
    int32_t rdm_max_block;      /* largest rho block */
    double  host_phase_ms[6];   /* host wall time of: the two block enlargements,
                                   the superblock build, the superblock view and
                                   upload, the renormalisation's block scan and
                                   extraction, its wait for the device GEMMs, and
                                   its CSR assembly of the new operators */
} nss_step_record;

typedef struct nss_dmrg nss_dmrg;

nss_dmrg *nss_dmrg_create(nss_ctx *ctx, const nss_dmrg_params *p);
void      nss_dmrg_destroy(nss_dmrg *d);
int       nss_dmrg_infinite(nss_dmrg *d);
int       nss_dmrg_finite(nss_dmrg *d);
/* Run the infinite algorithm up to the last step and stop after building and
 * uploading that step's superblock (no solve), for benchmarking. */
int       nss_dmrg_prepare_last(nss_dmrg *d);
/* The superblock operator pool of the step nss_dmrg_prepare_last stopped at,
 * as the descriptor a Fortran caller would pass to nss_sb_upload (valid until
 * the next call on d). */
int       nss_dmrg_export_superblock(nss_dmrg *d, nss_sb_desc *out);
int       nss_dmrg_nrecords(const nss_dmrg *d);
/* Serving: whole DMRG runs (nss_dmrg_finite with the given parameters, one
 * ground state per step) as requests.  The server admits queued requests,
 * first come first served, while the sum of their estimated HBM footprints
 * (nss_server_footprint: the Krylov basis of the largest superblock of the
 * run, its work vectors, sector operators and rho blocks) stays within
 * hbm_budget (one request always runs).  Each admitted request runs on a
 * worker thread with its own context and its block state resident on the
 * device; the mixed-precision ground-state solves of all running requests
 * share one batch engine (the persistent multi-solve Lanczos kernel), joining
 * it as they arrive; the requests' device phases take turns with the
 * engine's rounds.  nss_server_poll returns finished requests (energy per
 * site of the last step, seconds queued before admission and in service,
 * the footprint estimate and the context's measured peak).
 * nss_server_destroy waits for every submitted request.  No counterpart in
 * the reference. */
typedef struct nss_server nss_server;
typedef struct {
    int32_t id, status;
    double  energy;
    double  wait_s, service_s;
    size_t  footprint_est, peak_bytes;
} nss_served;
nss_server *nss_server_create(int device, size_t hbm_budget);
size_t      nss_server_footprint(const nss_dmrg_params *p);
int         nss_server_submit(nss_server *s, const nss_dmrg_params *p, int *id);
int         nss_server_poll(nss_server *s, int max, nss_served *out);
int         nss_server_stats(nss_server *s, int *queued, int *running, size_t *in_use, size_t *peak_in_use,
                             int64_t *rounds, double *mean_batch);
int64_t     nss_server_solves(nss_server *s);   /* ground-state solves of served requests so far */
void        nss_server_destroy(nss_server *s);

/* Block restart files in the reference's text format (write_block /
 * read_block, src/BLOCKS/BLOCKS.f90:418-537; sector, operator and rotation
 * lists and sparse matrices as src/LIST/LIST_SECTORS.f90:639-705,
 * src/LIST/LIST_OPERATORS.f90:602-667, src/MATRIX/MATRIX_SPARSE.f90:703-770).
 * save writes the driver's current left / right block (either path may be
 * NULL), with its rotation matrices when the run keeps them; load replaces
 * them (load_block), e.g. to continue from the reference's own restart files
 * (older operator names such as "S_z" or "P" are mapped to "S_z_n", "P_n").
 * A loaded block must match the driver's model (site type, QN length and
 * operator keys). */
int       nss_dmrg_save_blocks(nss_dmrg *d, const char *left_path, const char *right_path);
/* Read one restart file and write it back in the current layout (operator
 * names with the link suffix, P typed "psign", 17 significant digits);
 * needs no context and no GPU.  Returns 0 or a negative code
 * (nss_last_error(NULL) has the message). */
int       nss_restart_rewrite(const char *in_path, const char *out_path);
int       nss_dmrg_load_blocks(nss_dmrg *d, const char *left_path, const char *right_path);
/* Measure_DMRG_scalar (src/DMRG_MEASURE.f90:148-220, 288-486, 595-705) after
 * a run with save_umat: for each position pos[i] (1-based along the chain,
 * OBC) the site operator op (dot basis, d x d, 0-based CSR) is placed at
 * that site of the block holding it (Build_Op_dmrg), carried to the last
 * step's block by the stored rotations and enlargements (Advance_Op_dmrg)
 * on the host, and averaged in the last step's ground state on the device
 * (Average_Op_dmrg / OdotV_direct).  out[i] = <gs| O(pos[i]) |gs>. */
int       nss_dmrg_measure(nss_dmrg *d, const nss_csr *op, const int32_t *pos, int npos, double *out);
int       nss_dmrg_records(const nss_dmrg *d, nss_step_record *out, int max);

#ifdef __cplusplus
}
#endif
#endif /* NSSDMRG_H */
