// Device context of the GB300 superblock eigensolver.
//
// HBM layout of one uploaded superblock (all FP64 unless noted):
//   psi-space vectors : N doubles; sector k occupies [Offset(k), Offset(k)+Dl*Dr)
//                       as the row-major W_k[il][ir] (ir fastest), which is the
//                       reference's column-major Psi_k[Dr x Dl]
//                       (src/DMRG_SUPERBLOCK_SETUP.f90:770,787).
//   hl / hr pools     : dense row-major H_L(k) [Dl x Dl] and H_R(k) [Dr x Dr],
//                       one after the other (sector operators are 75-95 %
//                       filled at production bond dimensions, so dense tiles).
//   term tables       : the A(it,k) x B(it,k) terms regrouped by the sector they
//                       write (RowOffset), CSR pools for A and B; regrouping
//                       lets one CTA own an output tile, so no atomics.
//   tiles             : (sector, row0, col0) work items of the matvec kernel.
//   Krylov basis      : nitermax+1 vectors of N doubles, vector-major.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/nssdmrg.h"

namespace nss {

struct DevTerm {          // one A x B term, grouped by output sector
    int out_sec, in_sec;
    int a_nrow, a_ncol, b_nrow, b_ncol;
    int64_t a_rp, b_rp;   // offsets of the rowptr arrays in the pools
};

struct DevSb {
    bool valid = false;
    uint64_t gen = 0;                  // upload generation (process-wide count)
    int nsb = 0, tnso = 0, m_left = 0, m_right = 0;
    int64_t n = 0;
    // host mirrors of the small tables
    std::vector<int> dls, drs;
    std::vector<int64_t> off, hl_off, hr_off;
    std::vector<int> ai, bi, ai_off, bi_off;
    std::vector<int> term_ptr;            // [nsb+1] into terms (by output sector)
    std::vector<DevTerm> terms;
    // F_HV bookkeeping: algorithmic flops of one H*v
    double flops_dense = 0.0, flops_ab = 0.0;
    int64_t h2d_bytes = 0;
    // device arrays
    int *d_dls = nullptr, *d_drs = nullptr;
    int64_t *d_off = nullptr, *d_hl_off = nullptr, *d_hr_off = nullptr;
    double *d_hl = nullptr, *d_hr = nullptr;
    int *d_term_ptr = nullptr;
    DevTerm *d_terms = nullptr;
    int *d_ab_rowptr = nullptr, *d_ab_col = nullptr;
    double *d_ab_val = nullptr;
    int4 *d_tiles = nullptr;
    int ntiles = 0;
    // FP32 copies for the mixed-precision path
    float *d_hl32 = nullptr, *d_hr32 = nullptr, *d_ab_val32 = nullptr;
    int *d_ab_rowptr32 = nullptr, *d_ab_col32 = nullptr;   // pruned FP32 A/B pool
    DevTerm *d_terms32 = nullptr;                            // terms indexing that pool
    int4 *d_tiles32 = nullptr;         // CUDA-core FP32 tiles (small sectors)
    int ntiles32 = 0;
    struct ItemRec *d_items32 = nullptr;   // work items of the persistent mixed kernel
    int nitems32 = 0;
    std::vector<int> item_cost;        // host: relative cost of each item (batch ordering)
    int *d_item_ell = nullptr;         // per item: offset of its A x B table (-1: CSR loop)
    int2 *d_ell = nullptr;             // the tables
    int4 *d_term_hdr = nullptr;        // per FP32 term: input-sector offset (lo, hi), its Dr
    int *d_tc_err = nullptr;           // set when a tensor-core pipeline wait ran out
    // tensor-core sector GEMM (k_sector_mma.cu), sections of the upload arena:
    // operand pool [rows][32] FP32, output planes [nplanes][n], work items
    // with their per-CTA ranges, 32x32 W tiles and their per-sector pack
    // records; the two tensor maps (128-row and BN-row boxes) over the pool
    float *d_mma_pool = nullptr, *d_mma_out = nullptr;
    struct MmaItem *d_mma_items = nullptr;
    int2 *d_mma_rng = nullptr;
    int4 *d_mma_wt = nullptr;
    struct PackSec *d_mma_sec = nullptr;
    int mma_nitems = 0, mma_nwt = 0, mma_plane_rows = 0, mma_bn = 64;
    int mma_nplanes = 0, mma_grid = 0;
    bool mma_split = true;
    alignas(64) unsigned char mma_map_a[128] = {}, mma_map_b[128] = {};
};

// Device-side Lanczos state, kept resident between nss_eigh and nss_rdm.
struct DevLanczos {
    int cap = 0;                 // allocated Krylov vectors
    int64_t n = 0;
    double *V = nullptr;         // [cap+1][n] when full64, else one n-vector of scratch
    bool full64 = false;         // V holds a whole FP64 Krylov basis
    double *w = nullptr;         // [n]
    float *V32 = nullptr;        // [cap][n] mixed-precision basis (lazily)
    float *w32 = nullptr;        // [n]
    float *anc32 = nullptr;      // [6][n] FP32 anchor, residual, deflation vectors (mixed)
    double last_resid[4] = {0, 0, 0, 0};   // FP64 residual norms of the last solve
    int last_iters = 0;
    double *evecs = nullptr;     // [neigen][n] Ritz vectors (last solve)
    double *rrw = nullptr;       // [4][n] H U of the mixed refinement's Rayleigh-Ritz step
    int neigen_done = 0;
    double *scal = nullptr;      // device scalars (see k_lanczos.cu)
    double *part = nullptr;      // per-CTA partial sums
    unsigned *counter = nullptr; // last-block-done counters
    double *alpha = nullptr, *beta = nullptr;   // [cap]
    double *theta = nullptr, *resid = nullptr, *svec = nullptr; // tridiagonal results
    int *flags = nullptr;        // device flags
    int *h_flags = nullptr;      // host-mapped flag mirror + the host's stop request
    double *h_ab = nullptr;      // host-mapped mirror of alpha, beta, anchor couplings ([cap+1] each)
    double last_anchor_theta = 0.0;
    int *d_h_flags = nullptr;    // device addresses of the two mapped buffers
    double *d_h_ab = nullptr;
    int orth_grid = 0;           // CTAs of the cooperative orthogonalisation kernel
    size_t orth_smem = 0;        // its dynamic shared memory
    float *wbuf32 = nullptr;     // [2][n] work vectors of the persistent chunk kernel
    float *slot32 = nullptr;     // [3][n] H*psi parts of the persistent chunk kernel
    size_t chunk_smem = 0;
    bool chunk_ok = false;       // the chunk kernel fits (one CTA per SM)
    int chunk_vc = 0;            // basis vectors in its shared-memory row cache (0: no cache)
    int chunk_cs = 0;            // cached floats per vector (rows of one CTA)
    size_t chunk_smem_vc = 0;    // its dynamic shared memory with the row cache
    float *pitem = nullptr;      // per-item alpha partials of the batched kernel
    int cap_pitem = 0;
    // CUDA-graph replay of the Lanczos chunks that run as separate launches
    // (FP64 method, mixed method with tensor-core sectors): the fixed input
    // vector of H*psi, the device step counter, and the instantiated graph
    // of CHECK iterations with the key it was captured for
    void *vcur = nullptr;        // [n] doubles' room
    int *jdev = nullptr;
    cudaGraphExec_t gx = nullptr;
    uint64_t gx_gen = 0;
    int gx_prec = -1, gx_mmax = 0, gx_ndefl = -1, gx_launches = 0;
    uint32_t gx_spin = 0;        // the wait limit the graph's kernels were captured with
    const void *gx_anc = nullptr;
    bool gx_failed = false;      // capture failed once: this workspace runs without graphs
};

struct DevRdm {
    int64_t cap_rho = 0, cap_evals = 0, cap_u = 0;
    double *rho = nullptr;       // blocks, left then right
    double *evals = nullptr;     // per-block eigenvalues, concatenated
    double *sorted = nullptr;    // descending
    int *order = nullptr;        // block-concatenated position per rank
    double *u = nullptr;         // dense rotation matrix staging
    double *work = nullptr;      // cuSOLVER workspaces, one per side stream
    int64_t lwork = 0;
    int *info = nullptr;         // one per side stream
    static constexpr int NSIDE = 8;
    cudaStream_t side[NSIDE] = {};
    cudaEvent_t ev_fork = nullptr, ev_join[NSIDE] = {};
    double *scal = nullptr;
    int *iscal = nullptr;
    double *bat = nullptr;       // batched eigensolve pool: padded blocks, eigenvalues, workspaces
    int64_t cap_bat = 0;
    int *bat_info = nullptr;
    int64_t cap_bat_info = 0;
    void *params = nullptr;      // cusolverDnParams_t
    double *vec = nullptr;       // eigenvector blocks, column-major, rho layout
    int64_t cap_vec = 0;
    double *syd = nullptr;       // own eigensolver: reflectors, T, tau, L D L^T, scale, shift
    int64_t cap_syd = 0;
    int *syi = nullptr;          // own eigensolver: per-block flags
    int64_t cap_syi = 0;
    unsigned char *tab = nullptr;    // per-call tables (device) ...
    int64_t cap_tab = 0;
    unsigned char *htab = nullptr;   // ... and their pinned host staging
    int64_t cap_htab = 0;
    double *hu = nullptr;            // pinned staging of the compact kept columns
    int64_t cap_hu = 0;
    static constexpr int NPH = 7;    // phase events of the last call (see rdm_phase_ms)
    cudaEvent_t ph[NPH] = {};
    double *big = nullptr;           // global copies of the blocks the cluster kernel reduces in place
    int64_t cap_big = 0;
    double *tg = nullptr;            // k_trd_grid exchange buffers, barrier and error word
    int64_t cap_tg = 0;
};

// Operator renormalisation on the device (k_renorm.cu): grow-only buffers
struct DevRenorm {
    double *ublk = nullptr, *dblk = nullptr, *tbuf = nullptr, *rbuf = nullptr;
    int64_t cap_ublk = 0, cap_dblk = 0, cap_tbuf = 0, cap_rbuf = 0;
    int *itab = nullptr;
    int64_t cap_itab = 0;
    double *hblk = nullptr, *hres = nullptr;     // pinned staging
    int64_t cap_hblk = 0, cap_hres = 0;
    int *hitab = nullptr;
    int64_t cap_hitab = 0;
};

// Kept columns of one side after nss_rdm, for the device renormalisation:
// column j belongs to side-local rho block q[j]; its n_q values (block rows,
// no zero rows) start at off[j] in the device buffer dcomp, valid until the
// next RDM call on the context.  dims/maps/map_off: the side's blocks and
// their enlarged-block states.
struct KeptLayout {
    int ms = 0;
    std::vector<int> q, off, dims, maps, map_off;
    const double *dcomp = nullptr;
};

struct Ctx {
    int device = 0;
    size_t budget = 0, used = 0;
    std::unordered_map<void *, size_t> sizes;   // live allocations
    std::string err;
    cudaStream_t stream = nullptr;
    // the mixed product's side stream (CUDA-core tiles beside the tensor-core
    // GEMM) and its fork / join events, made on first use
    cudaStream_t hv_side = nullptr;
    cudaEvent_t hv_fork = nullptr, hv_join = nullptr;
    void *solver = nullptr;      // cusolverDnHandle_t
    DevSb sb;
    DevLanczos lz;
    DevRdm rdm;
    DevRenorm ren;
    int64_t launches = 0;        // kernels of this library launched
    int tc_min_dl = 1024;        // tensor-core sector threshold (see tc_min_dl_default)
    bool tc_auto = true;         // the tile tuner picks the plan per upload (tile_tune.cpp)
    int tune_class = 0, tune_cand = -1;   // the current superblock's shape class and candidate
    int mma_bn = 64;             // tensor-core tile width (64 or 128) and K-loop split
    bool mma_split = true;
    bool mma_lolo = false;       // fourth product lo.lo in the split-TF32 GEMM
    int mma_kps = 1;             // K slabs (of 32) per tensor-memory accumulation before FP32 promotion
    bool use_graphs = true;      // NSS_GRAPH=0: Lanczos chunks as separate launches, no CUDA graphs
    int graph_replays = 0, graph_captures = 0;   // of the last nss_eigh
    // last nss_eigh statistics
    int last_numop = 0;
    double last_ms_eigh = 0.0;
    // optional CUDA-event timing of the persistent chunk kernel (last solve)
    bool time_chunks = false;
    double chunk_ms = 0.0;       // summed launch durations
    int chunk_launches = 0;
    int64_t chunk_iters = 0;     // iterations those launches completed
    double chunk_cols = 0.0;     // sum over those iterations of the basis size m
    // last nss_rdm: blocks on the own eigensolver, on the library, and own
    // blocks whose vectors were recomputed by the library
    int rdm_own_blocks = 0, rdm_lib_blocks = 0, rdm_fallback_blocks = 0;
    // fallback reasons over the context's life: not positive definite, gap
    // below 32 eps, Rayleigh iteration unsettled, Gram-Schmidt remainder,
    // cluster too large
    int64_t rdm_fail_why[5] = {0, 0, 0, 0, 0};
    // device time of the last nss_rdm's phases: rho build + symmetry check,
    // tridiagonal reductions, eigenvalues (+ library blocks), truncation,
    // kept vectors (+ fallbacks), compact U
    double rdm_phase_ms[6] = {0, 0, 0, 0, 0, 0};
    // blocks per eigensolver tier (one CTA, cluster, blocked library
    // reduction, library eigensolver) and the largest block, last call
    int rdm_path_blocks[4] = {0, 0, 0, 0};
    int rdm_max_block = 0;
    char *sb_arena = nullptr, *sb_stage = nullptr;   // superblock pool: device arena, pinned staging
    size_t sb_arena_cap = 0, sb_stage_cap = 0;
    double renorm_phase_ms[3] = {0, 0, 0};
    int refine_passes = 0, refine_cluster = 0;   // mixed refinement of the last solve
    bool last_pair = false;                      // ... needed a near-degenerate partner
    int rdm_refined_blocks = 0;                  // flagged blocks redone by k_vec_fb in the last nss_rdm
    int rdm_ql_blocks = 0;                       // ... and of those, blocks finished by host QL
    int64_t mixed_fallbacks = 0;                 // mixed solves redone in FP64 (context life)
    char *ms_dev = nullptr, *ms_host = nullptr;   // OdotV tables: device, pinned staging
    size_t ms_cap = 0;   // host: scan+extract, device wait, CSR assembly (summed over calls)
    double *noalloc_scratch = nullptr;   // device address of k_noalloc.cu's static scratch, looked up on first use
    struct Server *serve = nullptr;      // the server running this context's requests (host_serve.cpp)
    size_t peak_used = 0;                // largest `used` so far
};

// Allocation through the context budget.
template <class T>
cudaError_t ctx_alloc(Ctx &c, T **p, size_t count) {
    size_t bytes = count * sizeof(T);
    if (bytes == 0) bytes = 16;
    if (c.budget && c.used + bytes > c.budget) return cudaErrorMemoryAllocation;
    cudaError_t e = cudaMalloc((void **)p, bytes);
    if (e == cudaSuccess) {
        c.used += bytes;
        c.peak_used = c.used > c.peak_used ? c.used : c.peak_used;
        c.sizes[(void *)*p] = bytes;
    }
    return e;
}
void ctx_free(Ctx &c, void *p);

// k_matvec.cu
// trusted: the descriptor comes from this library's own setup (its column
// indices are not re-checked entry by entry)
int sb_upload(Ctx &c, const nss_sb_desc *d, bool trusted = false);
// Drop the pool; free_arena also returns its device arena and pinned
// staging buffer (otherwise kept for the next upload).
void sb_release(Ctx &c, bool free_arena);
// `stop` (may be null): a device flag; the kernels return at once when set
int hv_device(Ctx &c, const double *d_v, double *d_hv, const int *stop = nullptr);
int hv_device_fp32(Ctx &c, const float *d_v, float *d_hv, const int *stop = nullptr);
// k_sector_mma.cu: the dense sector products of the routed sectors into the
// two output planes (the "terms only" tiles of k_hv_fp32 add them)
int hv_device_mma(Ctx &c, const float *d_v, const int *stop = nullptr);
struct Hv32Ops;
Hv32Ops hv32_ops(const DevSb &s);
// sectors with at least this many left states take the tensor-core kernel
// in the mixed path; a context takes env NSS_TC_MIN_DL at creation (default
// 1024: up to a few hundred states the persistent CUDA-core path is faster
// on GB300, 20-25 ms against 29-37 ms per solve of the spin-1 L=64 m=512
// superblock, whose sectors reach 350 states; 0 disables)
int tc_min_dl_default();
// tensor-core tile width and K-loop split of a new context: env NSS_TC_BN
// (64 or 128, default 64) and NSS_TC_SPLIT (0 or 1, default 1)
void mma_tile_default(int *bn, bool *split);
// the split-TF32 GEMM's fourth product lo.lo: env NSS_TC_LOLO (default off)
bool mma_lolo_default();
// NSS_TC_KPS (1 or 2, default 1): K slabs the tensor core accumulates before
// the epilogue promotes the partial sum to FP32 registers
int mma_kps_default();
// Poll limit of every bounded device wait (the grid barriers of the
// cooperative Lanczos and tridiagonalisation kernels): env NSS_WAIT_LIMIT,
// default 2^22 polls (about 2 s).  A wait that runs out makes its kernel
// return and the entry point report NSS_ERR_CUDA; the tests shorten the
// limit to exercise that path.
uint32_t wait_limit();

// host_serve.cpp: a served context's device phases take the server's device
// lock (ServeLock is a no-op for other contexts), and its mixed ground-state
// solves go to the server's batch engine
struct Server;
struct ServeLock {
    Server *s;
    explicit ServeLock(Ctx &c);
    ~ServeLock();
    void unlock();
    ServeLock(const ServeLock &) = delete;
    ServeLock &operator=(const ServeLock &) = delete;
};
int serve_solve(Ctx &c, int nitermax, double tol, uint64_t seed, double *energy, int *numop);
void serve_count(Ctx &c);   // one more ground-state solve of a served request

// tile_tune.cpp: the mixed path's plan per shape class of superblock
bool tune_enabled();
// candidate for the superblock being uploaded (0 CUDA cores, 1 / 2 tensor
// cores with 64 / 128-column tiles): sets *tc_min_dl and *bn for it
int tune_choose(Ctx &c, const DevSb &s, int *tc_min_dl, int *bn);
// a converged mixed solve on the current superblock took ms for numop products
void tune_record(Ctx &c, double ms, int numop);
int tune_lookup(int device, int cls, double *ms_per_hv, int *solves);
void tune_reset();

// k_noalloc.cu
int sb_energy_noalloc(Ctx &c, int64_t n, const double *d_psi, double *energy);

// k_lanczos.cu
int lanczos_eigh(Ctx &c, int neigen, int nitermax, double tol, uint64_t seed,
                 int precision, double *evals_host, int *numop);
// several mixed-precision ground-state solves, one context each, advanced
// together by the batched persistent kernel; cs[0]'s stream runs them
int lanczos_eigh_batch(Ctx *const *cs, int nb, int nitermax, double tol, const uint64_t *seeds,
                       double *evals_host, int *numops);
// continuous batching: solves join with batch_add and leave through
// batch_step (one round per call) when done
struct BatchEngine;
BatchEngine *batch_create(Ctx &c0);
void batch_destroy(BatchEngine *e);
int batch_add(BatchEngine *e, Ctx &c, uint64_t seed, int nitermax, double tol, int *id);
int batch_step(BatchEngine *e, int max_done, int *ndone, int *ids, double *energies, int *numops);
int batch_inflight(const BatchEngine *e);
void lanczos_release(Ctx &c);

// k_syev.cu: FP64 eigensolver of the rho blocks.  Blocks up to SYEV_MAX
// are reduced to tridiagonal form in one CTA (k_trd); larger ones, up to
// SYEV_BIG_MAX, by a thread-block cluster (k_trd_cl, the block in the
// cluster's shared memory or in a global copy); the eigenvalues and kept
// vectors of all come from k_bisect and k_vec.
constexpr int SYEV_MAX = 160;
// k_vec keeps 7 x n doubles per warp in shared memory.  (The cluster's 16
// SMs bound the largest blocks, n^3/16 FP64 FMAs each: 0.5 s at n = 2645,
// the noise-level truncation blocks of the spin-1 m=512 sweep; the
// library's blocked solver measured 0.5-2.2 s there.)
constexpr int SYEV_BIG_MAX = 3500;
int syev_trd(const double *rho, const int64_t *rho_off, const int *dims, const int *ev_off, const int *blocks,
             int nblocks, int maxn, double *refl, double *td, double *te, double *tau, int *perm, cudaStream_t st);
int syev_bisect(const int *dims, const int *ev_off, const int2 *items, int nitems, const double *td,
                const double *te, double *evals, double *ldd, double *ldl, double *bscale, double *bsig,
                int *flags, int *sub, int nmax, cudaStream_t st);
// clusters of 8 or 16 CTAs per block (k_trd_cl); the size and the largest
// block it takes
int syev_trd_cl_size(int *nmax);
// gA (may be null): global column-major scratch for blocks too large for the
// cluster's shared memory, block b at gA + goff[b] (goff on the device)
int syev_trd_cl(const double *rho, const int64_t *rho_off, const int *dims, const int *ev_off, const int *blocks,
                int nblocks, int maxn, double *refl, double *td, double *te, double *tau, int *perm, double *gA,
                const int64_t *goff, cudaStream_t st);
// k_trd_grid: the same reduction of the blocks in `blocks` (dims nb) by the
// whole GPU, up to 8 blocks a cooperative launch on CTA groups sized by
// n^3, for blocks far beyond a cluster's reach; comm needs
// syev_trd_grid_comm(nb, SMs) doubles, bar 8 unsigned; *err (device) is set
// if a barrier timed out.
int64_t syev_trd_grid_comm(const std::vector<int> &nb, int nsm);
int syev_trd_grid(const double *rho, const int64_t *rho_off, const int *dims, const int *ev_off,
                  const std::vector<int> &blocks, const std::vector<int> &nb, double *refl, double *td, double *te,
                  double *tau, int *perm, double *gA, const std::vector<int64_t> &goff_h, double *comm,
                  unsigned *bar, int *err, cudaStream_t st);

// kept eigenvectors of both sides (ms[0] left, ms[1] right; right positions
// start at nl): k_vec + the cluster Gram-Schmidt, two launches
// Back-transformation (Householder reflectors of the tridiagonal reduction,
// then the block's row order) of the columns cols[t] = (block, column) of
// vec, which hold tridiagonal-basis vectors.
int syev_backtr(const int *dims, const int *ev_off, const int64_t *rho_off, const double *tau, const double *refl,
                const int *perm, double *vec, const int2 *cols, int ncols, int nmax, cudaStream_t st);
// Kept vectors of the flagged blocks in `blocks` (device list of nb) again,
// by inverse iteration with Gram-Schmidt inside near clusters (k_vec_fb);
// blocks it cannot do keep bit 1 of their flags.
int syev_vec_fallback(const int *order, const int *rank, const int ms[2], int nl, int nsb, const int *ev_off,
                      const int *dims, const int64_t *rho_off, const int *sub, const double *evals, const double *ldd,
                      const double *ldl, const double *bscale, const double *bsig, const double *tau,
                      const double *refl, const int *perm, int *flags, double *vec, const int *blocks, int nb,
                      int nmax, cudaStream_t st);
int syev_vec(const int *order, const int *rank, const int ms[2], int nl, int nsb, const int *ev_off,
             const int *dims, const int64_t *rho_off, const int *bmode, const int *sub, const double *evals,
             const double *ldd, const double *ldl, const double *bscale, const double *bsig, const double *tau,
             const double *refl, const int *perm, int *flags, double *vec, int nmax, cudaStream_t st);
int syev_eigs_per_cta();

// k_rdm.cu
// kl (may be null): per side, the kept columns left on the device
// mstates = 0 with estates != 0 selects the Edmrg (error threshold) rule
// vec_sides: bit s set = side s gets its kept vectors (U, kept indices, kl);
// the other side only its spectrum, truncation, error and entropies
int rdm_run(Ctx &c, const double *d_psi, int mstates, double estates, double deg_thr, nss_rdm_side out[2],
            double *lam_l, double *lam_r, int32_t *kept_l, int32_t *kept_r,
            double *u_l, double *u_r, KeptLayout *kl = nullptr, int vec_sides = 3);
void rdm_release(Ctx &c);

// k_renorm.cu: blk's operators <- U^T O U for the kept columns kl, blk's
// basis <- kept_qn (one QN tuple per kept column)
struct Block;
struct Csr;
// Both blocks of a step at once: blk[s] is renormalised with the kept
// columns kl[s] and gets the basis kept_qn[s].
int renorm_device(Ctx &c, const KeptLayout kl[2], Block *blk[2], const std::vector<std::vector<double>> *kept_qn[2]);
void renorm_release(Ctx &c);
// The rotation matrix U (m_block x m_s, CSR, exact zeros dropped) of one
// side from its kept columns, for the stored rotations of measurements.
int kept_u_csr(Ctx &c, const KeptLayout &kl, int mblock, Csr &u);

// k_measure.cu: OdotV_direct / Average_Op_dmrg on the uploaded superblock.
// ops[k] (k < nsb): the block operator filtered to sector k's left
// (label 0) or right (label 1) states; d_ov (may be null) receives O v and
// *val (may be null) v . O v.
int odotv_device(Ctx &c, int label, const nss_csr *ops, const double *d_v, double *d_ov, double *val);
void measure_release(Ctx &c);

}  // namespace nss

#define NSS_CUDA_TRY(c, call)                                                   \
    do {                                                                        \
        cudaError_t _e = (call);                                                \
        if (_e != cudaSuccess) {                                                \
            (c).err = std::string(#call) + " (" + __FILE__ + ":" + std::to_string(__LINE__) + "): " + \
                      cudaGetErrorString(_e);                                   \
            return _e == cudaErrorMemoryAllocation ? NSS_ERR_NOMEM : NSS_ERR_CUDA; \
        }                                                                       \
    } while (0)

// the same inside a function that reports failure with its own value `fail`
#define NSS_CUDA_TRY_R(c, call, fail)                                           \
    do {                                                                        \
        cudaError_t _e = (call);                                                \
        if (_e != cudaSuccess) {                                                \
            (c).err = std::string(#call) + " (" + __FILE__ + ":" + std::to_string(__LINE__) + "): " + \
                      cudaGetErrorString(_e);                                   \
            return (fail);                                                      \
        }                                                                       \
    } while (0)
