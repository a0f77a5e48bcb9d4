// Tensor-core (tcgen05) sector product for the mixed-precision path.
//
// For one output tile (128 rows il x BN columns ir of sector k) it computes
//     D = H_L(k) W_k + W_k H_R(k)^T
// as two K-loops of UMMA D[128 x BN] += A[128 x 32] . B[BN x 32]^T on the
// 5th-generation tensor cores, kind::tf32, with the 3xTF32 split
// x = hi + lo (hi = x rounded to TF32, lo = x - hi) and three products
// hi.hi + hi.lo + lo.hi per K step, accumulated in FP32 in TMEM: about
// 2^-21 relative accuracy, i.e. FP32-class H*psi.  Operands are staged by the
// CTA's threads into shared memory in the no-swizzle K-major canonical
// layout (8-row x 16-byte core matrices; LBO = next core along K = 128 B,
// SBO = next 8-row group = 8 cores = 1024 B for a 32-wide K chunk), one
// thread issues the MMAs, tcgen05.commit signals an mbarrier, and after the
// K loops the 4 warps read their 32 TMEM lanes each (tcgen05.ld 32x32b) and
// add the dense products to the A x B terms of the sector, which k_hv_fp32
// ("terms only" tiles, launched just before on the same stream) has written
// to H psi.
//
// Two shared-memory stages: the threads stage chunk i+1 while the tensor
// core works on chunk i.  Every mbarrier wait is bounded; a wait that runs
// out sets the context error word, and the CTA still frees its TMEM.
#include "device.cuh"

namespace nss {

namespace {

constexpr int TC_M = 128;
constexpr int TC_BN = 64;
constexpr int TC_K = 32;
constexpr int TC_THREADS = 128;
constexpr uint32_t TC_NCOLS = 64;                     // TMEM columns (>= TC_BN, power of 2)
constexpr int A_FLOATS = TC_M * TC_K;                 // 4096
constexpr int B_FLOATS = TC_BN * TC_K;                // 2048
constexpr int STAGE_FLOATS = 2 * A_FLOATS + 2 * B_FLOATS;   // hi/lo of A and B
constexpr int TC_SMEM = 2 * STAGE_FLOATS * 4;         // two stages: 96 KiB
constexpr uint32_t MAX_SPIN = 1u << 24;

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr) {
    // no swizzle, K-major: LBO = 128 B (core to core along K), SBO = 1024 B
    uint64_t d = (uint64_t)((saddr & 0x3FFFF) >> 4);
    d |= (uint64_t)(128 >> 4) << 16;
    d |= (uint64_t)((TC_K / 4) * 128 >> 4) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

constexpr uint32_t IDESC_TF32 = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(TC_BN >> 3) << 17) |
                                ((uint32_t)(TC_M >> 4) << 24);

__device__ __forceinline__ float tf32_round(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

// byte offset of element (row, k) of a [rows x TC_K] K-major canonical tile
__device__ __forceinline__ int canon(int row, int k) {
    return (row >> 3) * (TC_K / 4) * 32 + (k >> 2) * 32 + (row & 7) * 4 + (k & 3);   // in floats
}

__device__ __forceinline__ void mma_tf32(uint32_t tmem, uint64_t ad, uint64_t bd, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem),
        "l"(ad), "l"(bd), "r"(IDESC_TF32), "r"(acc));
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    uint32_t ok = 0;
    for (uint32_t it = 0; it < MAX_SPIN && !ok; ++it) {
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(ok)
            : "r"(bar), "r"(parity));
    }
    return ok != 0;
}

}  // namespace

// Stage one K chunk: A rows [row0, row0+128) x [j0, j0+32) and B rows (the
// output columns) [col0, col0+BN) x [j0, j0+32), split into TF32 hi/lo.
// phase 0: A = HL[il][j], B[n][j] = W[j][ir];  phase 1: A = W[il][j], B = HR[ir][j]
// All of a thread's global loads are issued before any conversion so that
// they are in flight together.
__device__ __forceinline__ void tc_stage(float *st, int phase, const float *W, const float *H, int dl, int dr,
                                         int row0, int col0, int j0) {
    float *ahi = st, *alo = st + A_FLOATS, *bhi = st + 2 * A_FLOATS, *blo = bhi + B_FLOATS;
    const int kmax = phase == 0 ? dl : dr;
    constexpr int NA = A_FLOATS / TC_THREADS, NB = B_FLOATS / TC_THREADS;
    float xa[NA], xb[NB];
    // lane -> (row & 7, k & 3) so a warp writes 128 contiguous bytes
#pragma unroll
    for (int it = 0; it < NA; ++it) {
        const int e = threadIdx.x + it * TC_THREADS;
        const int lane = e & 31, grp = e >> 5;             // grp = (row>>3)*(TC_K/4) + (k>>2)
        const int row = (grp / (TC_K / 4)) * 8 + (lane >> 2), k = (grp % (TC_K / 4)) * 4 + (lane & 3);
        const int gi = row0 + row, gj = j0 + k;
        xa[it] = 0.f;
        if (gi < dl && gj < kmax) xa[it] = phase == 0 ? H[(int64_t)gi * dl + gj] : W[(int64_t)gi * dr + gj];
    }
#pragma unroll
    for (int it = 0; it < NB; ++it) {
        const int e = threadIdx.x + it * TC_THREADS;
        const int lane = e & 31, grp = e >> 5;
        const int n = (grp / (TC_K / 4)) * 8 + (lane >> 2), k = (grp % (TC_K / 4)) * 4 + (lane & 3);
        const int gc = col0 + n, gj = j0 + k;
        xb[it] = 0.f;
        if (gc < dr && gj < kmax) xb[it] = phase == 0 ? W[(int64_t)gj * dr + gc] : H[(int64_t)gc * dr + gj];
    }
#pragma unroll
    for (int it = 0; it < NA; ++it) {
        const int e = threadIdx.x + it * TC_THREADS;
        const int lane = e & 31, grp = e >> 5;
        const int row = (grp / (TC_K / 4)) * 8 + (lane >> 2), k = (grp % (TC_K / 4)) * 4 + (lane & 3);
        const float h = tf32_round(xa[it]);
        ahi[canon(row, k)] = h;
        alo[canon(row, k)] = xa[it] - h;
    }
#pragma unroll
    for (int it = 0; it < NB; ++it) {
        const int e = threadIdx.x + it * TC_THREADS;
        const int lane = e & 31, grp = e >> 5;
        const int n = (grp / (TC_K / 4)) * 8 + (lane >> 2), k = (grp % (TC_K / 4)) * 4 + (lane & 3);
        const float h = tf32_round(xb[it]);
        bhi[canon(n, k)] = h;
        blo[canon(n, k)] = xb[it] - h;
    }
}

__global__ void __launch_bounds__(TC_THREADS) k_hv_tc(
    const float *__restrict__ v, float *__restrict__ hv, const int4 *__restrict__ tiles,
    const int *__restrict__ dls, const int *__restrict__ drs, const int64_t *__restrict__ off,
    const float *__restrict__ hlp, const int64_t *__restrict__ hl_off,
    const float *__restrict__ hrp, const int64_t *__restrict__ hr_off, int *err, const int *stop) {
    if (stop && *stop) return;   // before any TMEM allocation: uniform exit
    extern __shared__ __align__(1024) uint8_t smem[];
    float *stage[2] = {(float *)smem, (float *)smem + STAGE_FLOATS};
    __shared__ __align__(8) uint64_t mbar[2];
    __shared__ uint32_t tmem_base;
    __shared__ int ok_s;
    const int4 t = tiles[blockIdx.x];
    const int k = t.x, row0 = t.y, col0 = t.z;
    const int dl = dls[k], dr = drs[k];
    const float *W = v + off[k];
    const float *HL = hlp + hl_off[k];
    const float *HR = hrp + hr_off[k];
    const int tid = threadIdx.x;
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar[0])));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar[1])));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        ok_s = 1;
    }
    if (tid < 32) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                     "r"(TC_NCOLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_base;

    // chunk c uses stage c&1 and commits to mbar[c&1]; that barrier has then
    // completed c>>1 earlier phases, so chunk c's completion has parity (c>>1)&1
    const int nk0 = (dl + TC_K - 1) / TC_K, nk1 = (dr + TC_K - 1) / TC_K, nk = nk0 + nk1;
    tc_stage(stage[0], 0, W, HL, dl, dr, row0, col0, 0);
    for (int c = 0; c < nk; ++c) {
        const int buf = c & 1;
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (tid == 0 && ok_s) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const float *st = stage[buf];
            const uint32_t ahi = smem_u32(st), alo = smem_u32(st + A_FLOATS);
            const uint32_t bhi = smem_u32(st + 2 * A_FLOATS), blo = smem_u32(st + 2 * A_FLOATS + B_FLOATS);
            for (int kk = 0; kk < TC_K / 8; ++kk) {
                const uint32_t o = kk * 256;   // 8 TF32 = two cores along K
                const uint32_t acc0 = (c > 0 || kk > 0) ? 1u : 0u;
                mma_tf32(tmem, umma_desc(ahi + o), umma_desc(bhi + o), acc0);
                mma_tf32(tmem, umma_desc(ahi + o), umma_desc(blo + o), 1u);
                mma_tf32(tmem, umma_desc(alo + o), umma_desc(bhi + o), 1u);
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                smem_u32(&mbar[buf])));
        }
        // stage the next chunk into the other buffer while the MMAs run; that
        // buffer was last read by chunk c-1, whose commit must have landed
        if (c + 1 < nk) {
            if (c >= 1) {
                if (tid == 0 && !mbar_wait(smem_u32(&mbar[buf ^ 1]), ((c - 1) >> 1) & 1)) {
                    ok_s = 0;
                    atomicExch(err, 1);
                }
                __syncthreads();
            }
            const int cn = c + 1;
            if (cn < nk0) tc_stage(stage[buf ^ 1], 0, W, HL, dl, dr, row0, col0, cn * TC_K);
            else tc_stage(stage[buf ^ 1], 1, W, HR, dl, dr, row0, col0, (cn - nk0) * TC_K);
        }
    }
    // the last commit covers every earlier MMA of the issuing thread
    if (tid == 0 && ok_s && !mbar_wait(smem_u32(&mbar[(nk - 1) & 1]), ((nk - 1) >> 1) & 1)) {
        ok_s = 0;
        atomicExch(err, 1);
    }
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    // Epilogue, in two passes.  (1) Each warp moves its 32 TMEM lanes (rows)
    // into shared memory (row stride 65 floats: conflict-free), the MMAs being
    // complete so the stage buffers are free.  (2) Lanes run along columns, so
    // the read-add-store of H psi (which holds the A x B terms) is coalesced.
    const int w = tid >> 5, lane = tid & 31;
    float *Dsm = stage[0];                          // 128 x 65 floats < one stage
    if (ok_s) {
        for (int c0 = 0; c0 < TC_BN; c0 += 8) {
            uint32_t r[8];
            asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                         : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                           "=r"(r[7])
                         : "r"(tmem + ((uint32_t)(32 * w) << 16) + (uint32_t)c0));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
            for (int j = 0; j < 8; ++j) Dsm[(32 * w + lane) * (TC_BN + 1) + c0 + j] = __uint_as_float(r[j]);
        }
    }
    __syncthreads();
    if (ok_s) {
        // warp w owns rows w, w+4, ..., lanes columns lane and lane+32; the
        // terms already in H psi are read eight rows at a time, so those loads
        // are in flight together
        float *out = hv + off[k];
        constexpr int RB = 8;
        for (int r0 = w; r0 < TC_M; r0 += 4 * RB) {
            float x[RB][2];
#pragma unroll
            for (int q = 0; q < RB; ++q) {
                const int il = row0 + r0 + 4 * q;
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const int ir = col0 + lane + 32 * h;
                    x[q][h] = (il < dl && ir < dr) ? __ldcg(out + (int64_t)il * dr + ir) : 0.f;
                }
            }
#pragma unroll
            for (int q = 0; q < RB; ++q) {
                const int rr = r0 + 4 * q, il = row0 + rr;
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const int cc = lane + 32 * h, ir = col0 + cc;
                    if (il < dl && ir < dr) out[(int64_t)il * dr + ir] = Dsm[rr * (TC_BN + 1) + cc] + x[q][h];
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (tid < 32) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_NCOLS));
}

int hv_device_tc(Ctx &c, const float *d_v, float *d_hv, const int *stop) {
    DevSb &s = c.sb;
    if (s.ntiles_tc == 0) return NSS_OK;
    static bool attr_set = false;
    if (!attr_set) {
        NSS_CUDA_TRY(c, cudaFuncSetAttribute(k_hv_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM));
        attr_set = true;
    }
    k_hv_tc<<<s.ntiles_tc, TC_THREADS, TC_SMEM, c.stream>>>(
        d_v, d_hv, s.d_tiles_tc, s.d_dls, s.d_drs, s.d_off, s.d_hl32, s.d_hl_off, s.d_hr32, s.d_hr_off,
        s.d_tc_err, stop);
    c.launches += 1;
    NSS_CUDA_TRY(c, cudaGetLastError());
    return NSS_OK;
}

}  // namespace nss
