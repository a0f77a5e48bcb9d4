// Allocation-free energy of a state on the uploaded superblock.
//
// Some callers of this library cannot allocate device memory at the moment
// they need an energy: a Fortran driver whose device heap is owned by
// another pool allocator, or a code that has already given the whole HBM
// budget of its context to the Krylov basis, where one more cudaMalloc would
// fail or fragment a pool that is not this library's.  nss_sb_energy_noalloc
// serves them: it evaluates
//     E = <psi|H|psi> / <psi|psi>
// on the superblock already uploaded with nss_sb_upload / nss_sb_setup,
// without allocating anything.  (The reference computes the same number in a
// commented-out check after sp_eigh, through a freshly allocated copy of H psi.)
//
// How: a variant of the FP64 sector kernel that, instead of writing H psi,
// multiplies each output element by psi and reduces inside the CTA; the
// per-tile partial sums and the last-CTA counter live in the file-scope
// device array g_noalloc_scratch below, NOALLOC_MAX_TILES tiles at most
// (512 KiB + 256 B; every GPU that loads the library keeps it until the
// process exits).  In host code the array's name is only a host-side stand-in,
// so the first call on each context looks up its device address with
// cudaGetSymbolAddress, with the context's device current, and keeps it in
// the context; that first call should come before any stream capture.  Each
// call waits for its kernel and copies E into host memory before it returns.
// All calls on a device share the array and each one clears the counter it
// needs: two calls whose kernels overlap on the GPU race with each other.
#include "device.cuh"

#include <cstdio>

namespace nss {

namespace {

constexpr int NA_TILE = 16;
constexpr int NOALLOC_MAX_TILES = 32768;

// partials: [0, MAX) psi.Hpsi per tile, [MAX, 2 MAX) psi.psi per tile,
// then one 32-double slot for the counter and the results
__device__ __align__(256) double g_noalloc_scratch[2 * NOALLOC_MAX_TILES + 32];

__global__ void __launch_bounds__(256) k_energy_noalloc(
    const double *__restrict__ v, const int4 *__restrict__ tiles, const int *__restrict__ dls,
    const int *__restrict__ drs, const int64_t *__restrict__ off, const double *__restrict__ hlp,
    const int64_t *__restrict__ hl_off, const double *__restrict__ hrp, const int64_t *__restrict__ hr_off,
    const int *__restrict__ term_ptr, const DevTerm *__restrict__ terms, const int *__restrict__ ab_rp,
    const int *__restrict__ ab_col, const double *__restrict__ ab_val, double *scratch) {
    __shared__ double sa[NA_TILE][33];
    __shared__ double sb[32][NA_TILE + 1];
    __shared__ double red[2][8];
    __shared__ unsigned last;
    const int4 t = tiles[blockIdx.x];
    const int k = t.x, row0 = t.y, col0 = t.z;
    const int dl = dls[k], dr = drs[k];
    const int64_t o = off[k];
    const double *W = v + o;
    const double *HL = hlp + hl_off[k];
    const double *HR = hrp + hr_off[k];
    const int tid = threadIdx.x, ty = tid / NA_TILE, tx = tid % NA_TILE;
    const int il = row0 + ty, ir = col0 + tx;
    double acc = 0.0;
    for (int j0 = 0; j0 < dl; j0 += 32) {
        for (int e = tid; e < NA_TILE * 32; e += 256) {
            const int r = e / 32, cc = e % 32, gi = row0 + r, gj = j0 + cc;
            sa[r][cc] = (gi < dl && gj < dl) ? HL[(int64_t)gi * dl + gj] : 0.0;
        }
        for (int e = tid; e < 32 * NA_TILE; e += 256) {
            const int r = e / NA_TILE, cc = e % NA_TILE, gj = j0 + r, gc = col0 + cc;
            sb[r][cc] = (gj < dl && gc < dr) ? W[(int64_t)gj * dr + gc] : 0.0;
        }
        __syncthreads();
        for (int j = 0; j < 32; ++j) acc = fma(sa[ty][j], sb[j][tx], acc);
        __syncthreads();
    }
    for (int j0 = 0; j0 < dr; j0 += 32) {
        for (int e = tid; e < NA_TILE * 32; e += 256) {
            const int r = e / 32, cc = e % 32, gi = row0 + r, gj = j0 + cc;
            sa[r][cc] = (gi < dl && gj < dr) ? W[(int64_t)gi * dr + gj] : 0.0;
        }
        for (int e = tid; e < 32 * NA_TILE; e += 256) {
            const int r = e / NA_TILE, cc = e % NA_TILE, gr = col0 + cc, gj = j0 + r;
            sb[r][cc] = (gr < dr && gj < dr) ? HR[(int64_t)gr * dr + gj] : 0.0;
        }
        __syncthreads();
        for (int j = 0; j < 32; ++j) acc = fma(sa[ty][j], sb[j][tx], acc);
        __syncthreads();
    }
    double p = 0.0, q = 0.0;
    if (il < dl && ir < dr) {
        for (int ti = term_ptr[k]; ti < term_ptr[k + 1]; ++ti) {
            const DevTerm tm = terms[ti];
            const double *Wq = v + off[tm.in_sec];
            const int drq = drs[tm.in_sec];
            const int *arp = ab_rp + tm.a_rp, *brp = ab_rp + tm.b_rp;
            for (int ja = arp[il]; ja < arp[il + 1]; ++ja) {
                const int aj = ab_col[ja];
                double cb = 0.0;
                for (int jb = brp[ir]; jb < brp[ir + 1]; ++jb)
                    cb = fma(ab_val[jb], Wq[(int64_t)aj * drq + ab_col[jb]], cb);
                acc = fma(ab_val[ja], cb, acc);
            }
        }
        const double x = W[(int64_t)il * dr + ir];
        p = x * acc;
        q = x * x;
    }
    for (int s = 16; s > 0; s >>= 1) {
        p += __shfl_xor_sync(0xffffffffu, p, s);
        q += __shfl_xor_sync(0xffffffffu, q, s);
    }
    if ((tid & 31) == 0) {
        red[0][tid >> 5] = p;
        red[1][tid >> 5] = q;
    }
    __syncthreads();
    if (tid == 0) {
        double a = 0.0, b = 0.0;
        for (int w = 0; w < 8; ++w) {
            a += red[0][w];
            b += red[1][w];
        }
        scratch[blockIdx.x] = a;
        scratch[NOALLOC_MAX_TILES + blockIdx.x] = b;
        __threadfence();
        unsigned *counter = (unsigned *)(scratch + 2 * NOALLOC_MAX_TILES);
        last = (atomicAdd(counter, 1u) == gridDim.x - 1);
    }
    __syncthreads();
    if (!last || tid != 0) return;
    __threadfence();
    double a = 0.0, b = 0.0;
    for (int i = 0; i < (int)gridDim.x; ++i) {
        a += scratch[i];
        b += scratch[NOALLOC_MAX_TILES + i];
    }
    double *res = scratch + 2 * NOALLOC_MAX_TILES + 8;
    res[0] = a / b;
    res[1] = a;
    res[2] = b;
}

}  // namespace

int sb_energy_noalloc(Ctx &c, int64_t n, const double *d_psi, double *energy) {
    DevSb &s = c.sb;
    if (!s.valid) {
        c.err = "nss_sb_energy_noalloc: no superblock uploaded";
        return NSS_ERR_STATE;
    }
    if (n != s.n || !d_psi || !energy) {
        c.err = "nss_sb_energy_noalloc: n must equal the superblock dimension and pointers be non-NULL";
        return NSS_ERR_INVALID;
    }
    if (s.ntiles > NOALLOC_MAX_TILES) {
        c.err = "nss_sb_energy_noalloc: superblock has " + std::to_string(s.ntiles) + " 16x16 tiles, more than the " +
                std::to_string(NOALLOC_MAX_TILES) + " its static scratch holds; use nss_hv instead";
        return NSS_ERR_INVALID;
    }
    if (s.ntiles <= 0) {
        c.err = "nss_sb_energy_noalloc: the uploaded superblock has no tiles";
        return NSS_ERR_INVALID;
    }
    double *scratch = c.noalloc_scratch;
    if (!scratch) {
        // once per context, with its device current (the entry point made it so)
        cudaError_t e = cudaGetSymbolAddress((void **)&scratch, g_noalloc_scratch);
        if (e != cudaSuccess || !scratch) {
            c.err = std::string("nss_sb_energy_noalloc: cudaGetSymbolAddress failed: ") + cudaGetErrorString(e);
            return NSS_ERR_CUDA;
        }
        c.noalloc_scratch = scratch;
    }
    // the last-CTA counter must start at zero
    NSS_CUDA_TRY(c, cudaMemsetAsync(scratch + 2 * NOALLOC_MAX_TILES, 0, 8 * sizeof(double), c.stream));
    k_energy_noalloc<<<s.ntiles, 256, 0, c.stream>>>(d_psi, s.d_tiles, s.d_dls, s.d_drs, s.d_off, s.d_hl,
                                                     s.d_hl_off, s.d_hr, s.d_hr_off, s.d_term_ptr, s.d_terms,
                                                     s.d_ab_rowptr, s.d_ab_col, s.d_ab_val, scratch);
    c.launches += 1;
    NSS_CUDA_TRY(c, cudaGetLastError());
    double res[3] = {0.0, 0.0, 0.0};   // E, <psi|H|psi>, <psi|psi>
    NSS_CUDA_TRY(c, cudaMemcpyAsync(res, scratch + 2 * NOALLOC_MAX_TILES + 8, sizeof(res), cudaMemcpyDeviceToHost,
                                    c.stream));
    NSS_CUDA_TRY(c, cudaStreamSynchronize(c.stream));
    if (!(res[2] > 0.0)) {
        c.err = "nss_sb_energy_noalloc: psi has zero norm";
        return NSS_ERR_INVALID;
    }
    *energy = res[0];
    return NSS_OK;
}

}  // namespace nss
