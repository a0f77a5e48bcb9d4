// Tensor-core sector product of the mixed-precision path (tcgen05 + TMA).
//
// For every sector k routed here it computes the dense part of the direct
// superblock product (src/DMRG_SUPERBLOCK_SETUP.f90:767-796)
//     D_k = H_L(k) W_k + W_k H_R(k)^T ,   W_k = psi_k as row-major [Dl x Dr],
// as a grouped GEMM over work items.  A tile (sector, 128-row block of il,
// BN-column block of ir) runs the K loop of H_L W (K = Dl) followed by that of
// W H_R^T (K = Dr), in 32-wide slabs; long tiles are cut into up to four
// pieces of consecutive slabs, each writing its partial tile to its own
// output plane (no atomics: every plane element has one writer, and the
// plane sum is formed in a fixed order).  The A x B terms of these sectors
// stay on CUDA cores (k_hv_fp32 "terms only" tiles, launched after this
// kernel), which add the planes.  The pieces are dealt to the CTAs longest
// first onto the least loaded CTA, and each CTA runs its own range.
//
// Precision: split TF32.  Every FP32 operand x is split into hi = x rounded
// to TF32 and lo = (x - hi) rounded to TF32 (so the tensor core's reading of
// a TF32 operand drops nothing); each K step issues hi.hi + hi.lo + lo.hi
// (and lo.lo with the context's lolo option) as tcgen05.mma kind::tf32 into
// FP32 accumulators in TMEM: FP32-class products.  hi.hi and hi.lo are ONE
// MMA of N = 2 BN, the B operand being B_hi and B_lo stacked along N; lo.hi
// (and lo.lo) accumulate into its first BN columns.
//
// Operand layout for TMA: every operand is stored "K-chunked": for a block X
// with R rows contracted over K, chunk c (K columns 32c..32c+31) is an
// [R x 32] FP32 slab (128-byte rows, K beyond the block zero), slabs one
// after the other.  All slabs of all sectors, the constant operators and the
// per-call W, live in one [rows x 32] FP32 pool, so ONE 2-D tensor map (box
// 32 x 128 or 32 x BN rows, 128-byte swizzle) loads every tile: the swizzled
// box is exactly the canonical K-major SW128 layout the UMMA descriptors
// read.  The pool holds plain FP32; the hi/lo split happens in shared memory
// (converter warps), which halves the bytes each slab moves from L2.  Rows
// of a box that run past a block belong to the next slab (finite values)
// and only reach output rows / columns beyond the block, which the epilogue
// drops; K padding is zero in every operand.
//   phase 0 (H_L W):    A = H_L rows il, K = j     B = W^T rows ir, K = il
//   phase 1 (W H_R^T):  A = W rows il, K = ir       B = H_R rows ir, K = j
//
// Kernel: persistent, one CTA per SM, 12 warps.  Warp 0 (one lane) issues
// the TMA loads into a ring of shared-memory stages; warps 2-3 split each
// landed stage into its hi and lo planes in place; warp 1 (one lane) issues
// the MMAs of each slab into a fresh TMEM accumulator and commits the stage
// back to the producer and the slab's partial product to the epilogue;
// warps 4-11 (two per TMEM lane quarter, each half of the columns) read the
// partials out of TMEM and sum them in FP32 registers, then store the
// piece's tile (staged in shared memory for whole-segment writes).  The
// accumulator buffers rotate, so the MMAs run ahead of the draining.  The
// per-slab promotion matters: the tensor core's FP32 accumulation does not
// round to nearest, and over a whole K loop of ~350 its error grew to 5x
// that of an FP32 FMA chain (measured RMS 1.8e-6 against 3.6e-7), enough to
// cost the mixed solver a third more iterations; over one slab it stays
// below the FMA chain's.  Every wait is bounded (wait_limit): a wait that
// runs out sets the error word, every role stops, the producer waits for
// the copies it issued, the MMA lane for its MMAs, and the CTA frees its
// TMEM and returns.
#include "sector_mma.cuh"

#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <atomic>
#include <cstring>
#include <vector>

namespace nss {

namespace {

constexpr int MM_THREADS = 448;            // 14 warps
constexpr int MM_CONV0 = 2, MM_NCONV = 4;   // converter warps 2-5
constexpr int MM_EPI0 = 6, MM_NEPI = 8;     // epilogue warps 6-13
constexpr int MM_SMEM_LIMIT = 232448;       // dynamic shared memory of one CTA

// instruction descriptor, kind::tf32: D FP32, A and B TF32, both K-major
__host__ __device__ constexpr uint32_t idesc_tf32(int bn) {
    return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(bn >> 3) << 17) | ((uint32_t)(MM_M >> 4) << 24);
}

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups
// 1024 bytes apart (SBO), start address in 16-byte units
__device__ __forceinline__ uint64_t desc_sw128(uint32_t saddr) {
    uint64_t d = (uint64_t)((saddr & 0x3FFFF) >> 4);
    d |= (uint64_t)1 << 16;                 // LBO (unused for swizzled K-major)
    d |= (uint64_t)(1024 >> 4) << 32;       // SBO
    d |= (uint64_t)1 << 46;                 // descriptor version
    d |= (uint64_t)2 << 61;                 // SWIZZLE_128B
    return d;
}

__device__ __forceinline__ void mma_tf32(uint32_t tmem, uint64_t ad, uint64_t bd, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem),
        "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                 : "memory");
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

// bounded wait for the phase of the given parity; false when it ran out or
// when another role has already given up (*abort)
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, uint32_t spin, volatile int *abort) {
    for (uint32_t it = 0; it <= spin; ++it) {
        uint32_t ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(ok)
            : "r"(bar), "r"(parity)
            : "memory");
        if (ok) return true;
        if ((it & 63u) == 63u && *abort) return false;
    }
    return false;
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, int x, int y, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            dst),
        "l"((uint64_t)map), "r"(x), "r"(y), "r"(bar)
        : "memory");
}

// x rounded to TF32 (10 explicit mantissa bits), to nearest with ties away
// from zero: half a TF32 unit added to the magnitude bits, the 13 dropped
// bits cleared.  Finite inputs (the operands are checked at upload).
__device__ __forceinline__ float tf32_rna(float x) {
    return __uint_as_float((__float_as_uint(x) + 0x1000u) & 0xffffe000u);
}

__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

}  // namespace

// Pack one operator block X [d x d] (row-major FP32) into its K-chunked
// slabs: slab c row r = X[r][32c .. 32c+31] (zero beyond d).  One thread per
// (slab row, K column) element.
__global__ void __launch_bounds__(256) k_pack_h(const float *__restrict__ x, int d, float *__restrict__ dst) {
    const int nch = (d + MM_KC - 1) / MM_KC;
    const int64_t total = (int64_t)nch * d * MM_KC;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
        const int kk = (int)(e % MM_KC);
        const int64_t rr = e / MM_KC;
        const int r = (int)(rr % d), c = (int)(rr / d);
        const int j = c * MM_KC + kk;
        dst[e] = j < d ? x[(int64_t)r * d + j] : 0.f;
    }
}

// Per call: W of every routed sector into its two K-chunked operands.  One
// CTA per 32 x 32 tile of W_k (tile list `wt`: sector, il0, ir0):
//   W1 (phase 1 A): slab c = ir0/32, row il:  W[il][ir0..ir0+31]
//   W0 (phase 0 B): slab c = il0/32, row ir:  W[il0..il0+31][ir]   (transposed through shared memory)
// with zeros beyond the block on the K side.  `scale` multiplies W.
__global__ void __launch_bounds__(256) k_pack_w(const float *__restrict__ v, float scale,
                                                const int4 *__restrict__ wt, const PackSec *__restrict__ sec,
                                                float *__restrict__ pool, const int *stop) {
    if (stop && *stop) return;
    __shared__ float t[32][33];
    const int4 w = wt[blockIdx.x];
    const PackSec s = sec[w.x];
    const int il0 = w.y, ir0 = w.z;
    const float *W = v + s.off;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;   // 8 rows of 32 lanes
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int il = il0 + ty + 8 * q, ir = ir0 + tx;
        const float x = (il < s.dl && ir < s.dr) ? W[(int64_t)il * s.dr + ir] * scale : 0.f;
        t[ty + 8 * q][tx] = x;
        if (il < s.dl)   // W1 row il of slab ir0/32, K column tx (zero beyond Dr)
            pool[((int64_t)s.w1_row + (int64_t)(ir0 / MM_KC) * s.dl + il) * MM_KC + tx] = x;
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int ir = ir0 + ty + 8 * q;
        if (ir < s.dr)   // W0 row ir of slab il0/32, K column tx = il - il0 (zero beyond Dl)
            pool[((int64_t)s.w0_row + (int64_t)(il0 / MM_KC) * s.dr + ir) * MM_KC + tx] = t[tx][ty + 8 * q];
    }
}

template <int BN>
struct MmaCfg {
    static constexpr int A_BYTES = MM_M * 128;                 // one plane of an A box
    static constexpr int B_BYTES = BN * 128;
    static constexpr int STAGE = 2 * A_BYTES + 2 * B_BYTES;    // A hi, A lo, B hi, B lo (B hi, lo adjacent)
    static constexpr int TX = A_BYTES + B_BYTES;               // bytes the TMA lands per stage (FP32 A, B)
    static constexpr int HALF = BN / 2;                        // columns of one epilogue warp
    static constexpr int OUT_LD = 33;                          // staging: 32 rows x 32 columns per pass
    static constexpr int OUT_BYTES = MM_NEPI * 32 * OUT_LD * 4;
    // as many operand stages as fit beside the epilogue's staging
    static constexpr int STAGES = (MM_SMEM_LIMIT - OUT_BYTES - 1024) / STAGE;
    static constexpr int SMEM = STAGES * STAGE + OUT_BYTES + 1024;   // + alignment slack
    static_assert(STAGES >= 2 && SMEM <= MM_SMEM_LIMIT, "shared memory plan");
    static constexpr int ACOLS = 2 * BN;                       // TMEM columns of one slab accumulator
    static constexpr int NBUF = 512 / ACOLS;                   // accumulators in flight (4 or 2)
    static constexpr uint32_t TCOLS = 512;
};

// slab c of a piece: TMA rows of its A and B boxes
__device__ __forceinline__ void item_rows(const MmaItem &m, int c, int &ar, int &br) {
    const int cs = m.c0 + c;
    const bool p0 = cs < m.nk0;
    const int cc = p0 ? cs : cs - m.nk0;
    ar = (p0 ? m.a_row0 : m.a_row1) + cc * m.a_step + m.m0;
    br = (p0 ? m.b_row0 : m.b_row1) + cc * m.b_step + m.n0;
}

template <int BN, int KPS>
__global__ void __launch_bounds__(MM_THREADS, 1) k_sector_mma(const __grid_constant__ CUtensorMap map_a,
                                                               const __grid_constant__ CUtensorMap map_b,
                                                               const MmaItem *__restrict__ items,
                                                               const int2 *__restrict__ ranges,
                                                               float *__restrict__ out, int64_t plane, int lolo,
                                                               uint32_t spin, int *err, const int *stop) {
    using C = MmaCfg<BN>;
    constexpr int S = C::STAGES;
    constexpr int NB = C::NBUF;
    if (stop && *stop) return;   // before any TMEM allocation: uniform exit
    extern __shared__ uint8_t mm_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)mm_raw + 1023) & ~(uintptr_t)1023);
    __shared__ __align__(8) uint64_t full[S], conv[S], empty[S], tfull[NB], tempty[NB], drain;
    __shared__ uint32_t tmem_base;
    __shared__ int abort_s;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int2 rg = ranges[blockIdx.x];
    if (threadIdx.x == 0) {
        for (int s = 0; s < S; ++s) {
            mbar_init(smem_u32(&full[s]), 1);
            mbar_init(smem_u32(&conv[s]), MM_NCONV * 32);   // every converter thread
            mbar_init(smem_u32(&empty[s]), 1);
        }
        for (int a = 0; a < NB; ++a) {
            mbar_init(smem_u32(&tfull[a]), 1);
            mbar_init(smem_u32(&tempty[a]), MM_NEPI);       // one arrival per epilogue warp
        }
        mbar_init(smem_u32(&drain), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&map_a) : "memory");
        asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&map_b) : "memory");
        abort_s = 0;
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                     "r"(C::TCOLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_base;
    volatile int *abort = &abort_s;
    // waits for the CTA's own copies and MMAs before it leaves
    const uint32_t drain_spin = spin > (1u << 22) ? spin : (1u << 22);
    auto give_up = [&]() {
        *abort = 1;
        atomicExch(err, 1);
    };

    if (warp == 0 && lane == 0) {
        // ---- TMA producer: the FP32 A and B boxes of each slab into the hi
        // slots of a stage
        int it = 0;                   // stage fills issued so far
        int last_par[S];
        bool inflight[S];
        for (int s = 0; s < S; ++s) inflight[s] = false;
        bool ok = true;
        for (int i = rg.x; i < rg.y && ok && !*abort; ++i) {
            const MmaItem m = items[i];
            for (int c = 0; c < m.nk; ++c, ++it) {
                const int s = it % S;
                const uint32_t par = (uint32_t)(it / S) & 1u;
                if (!mbar_wait(smem_u32(&empty[s]), par ^ 1u, spin, abort)) { give_up(); ok = false; break; }
                int ar, br;
                item_rows(m, c, ar, br);
                uint8_t *st = smem + (size_t)s * C::STAGE;
                const uint32_t fb = smem_u32(&full[s]);
                mbar_expect_tx(fb, (uint32_t)C::TX);
                tma_load_2d(smem_u32(st), &map_a, 0, ar, fb);
                tma_load_2d(smem_u32(st + 2 * C::A_BYTES), &map_b, 0, br, fb);
                inflight[s] = true;
                last_par[s] = (int)par;
            }
        }
        // no copy of this CTA may still be landing when it leaves: bounded, but
        // by a limit of its own (the CTA's own copies complete whatever the
        // other roles did; the configurable limit may be tiny in tests), and
        // not cut short by the abort flag
        volatile int never = 0;
        for (int s = 0; s < S; ++s)
            if (inflight[s] && !mbar_wait(smem_u32(&full[s]), (uint32_t)last_par[s], drain_spin, &never))
                atomicExch(err, 1);
    } else if (warp >= MM_CONV0 && warp < MM_CONV0 + MM_NCONV) {
        // ---- converters: each landed stage into its hi and lo planes (in
        // place: hi over the FP32 values, lo into the lo slots); the layout is
        // elementwise, so the swizzled boxes stay valid UMMA operands
        const int ct = threadIdx.x - 32 * MM_CONV0;
        int it = 0;
        bool ok = true;
        for (int i = rg.x; i < rg.y && ok && !*abort; ++i) {
            const int nk = items[i].nk;
            for (int c = 0; c < nk; ++c, ++it) {
                const int s = it % S;
                const uint32_t par = (uint32_t)(it / S) & 1u;
                if (!mbar_wait(smem_u32(&full[s]), par, spin, abort)) { give_up(); ok = false; break; }
                uint8_t *st = smem + (size_t)s * C::STAGE;
                float4 *ah = (float4 *)st, *al = (float4 *)(st + C::A_BYTES);
                float4 *bh = (float4 *)(st + 2 * C::A_BYTES), *bl = (float4 *)(st + 2 * C::A_BYTES + C::B_BYTES);
                auto split4 = [](float4 *h, float4 *l, int q) {
                    const float4 x = h[q];
                    float4 a, b;
                    a.x = tf32_rna(x.x); b.x = tf32_rna(x.x - a.x);
                    a.y = tf32_rna(x.y); b.y = tf32_rna(x.y - a.y);
                    a.z = tf32_rna(x.z); b.z = tf32_rna(x.z - a.z);
                    a.w = tf32_rna(x.w); b.w = tf32_rna(x.w - a.w);
                    h[q] = a;
                    l[q] = b;
                };
#pragma unroll 4
                for (int q = ct; q < C::A_BYTES / 16; q += MM_NCONV * 32) split4(ah, al, q);
#pragma unroll 4
                for (int q = ct; q < C::B_BYTES / 16; q += MM_NCONV * 32) split4(bh, bl, q);
                fence_async_smem();   // the tensor core reads these through the async proxy
                mbar_arrive(smem_u32(&conv[s]));
            }
        }
    } else if (warp == 1 && lane == 0) {
        // ---- MMA issuer: every slab into a fresh accumulator buffer, which
        // the epilogue drains into FP32 registers.  Per K step of 8: A_hi x
        // [B_hi; B_lo] (N = 2 BN: hi.hi in the first BN columns, hi.lo in the
        // second), then A_lo x B_hi (and A_lo x B_lo) into the first BN.
        constexpr uint32_t IDESC2 = idesc_tf32(2 * BN), IDESC1 = idesc_tf32(BN);
        int it = 0;                   // slabs issued (= stage fills consumed)
        int gq = 0;                   // accumulator groups (KPS slabs of one piece each)
        bool issued = false, ok = true;
        for (int i = rg.x; i < rg.y && ok && !*abort; ++i) {
            const int nk = items[i].nk;
            for (int c = 0; c < nk; ++c, ++it) {
                const int s = it % S, acc = gq % NB;
                const bool gfirst = c % KPS == 0, glast = c % KPS == KPS - 1 || c == nk - 1;
                const uint32_t par = (uint32_t)(it / S) & 1u;
                const uint32_t tacc = tmem + (uint32_t)(acc * C::ACOLS);
                // the epilogue has drained this buffer (its use NB groups ago)
                if ((gfirst && !mbar_wait(smem_u32(&tempty[acc]), ((uint32_t)(gq / NB) & 1u) ^ 1u, spin, abort)) ||
                    !mbar_wait(smem_u32(&conv[s]), par, spin, abort)) {
                    give_up();
                    ok = false;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t a_hi = smem_u32(smem + (size_t)s * C::STAGE), a_lo = a_hi + C::A_BYTES;
                const uint32_t b_hi = a_hi + 2 * C::A_BYTES, b_lo = b_hi + C::B_BYTES;
#pragma unroll
                for (int kk = 0; kk < MM_KC / 8; ++kk) {
                    const uint32_t o = kk * 32;   // 8 TF32 = 32 bytes along K inside the swizzled row
                    mma_tf32(tacc, desc_sw128(a_hi + o), desc_sw128(b_hi + o), IDESC2, (kk > 0 || !gfirst) ? 1u : 0u);
                    mma_tf32(tacc, desc_sw128(a_lo + o), desc_sw128(b_hi + o), IDESC1, 1u);
                    if (lolo) mma_tf32(tacc, desc_sw128(a_lo + o), desc_sw128(b_lo + o), IDESC1, 1u);
                }
                issued = true;
                mma_commit(smem_u32(&empty[s]));       // the stage is free once these MMAs have read it
                if (glast) {
                    mma_commit(smem_u32(&tfull[acc]));  // ... and the group's partial product is ready
                    ++gq;
                }
            }
        }
        if (issued) {   // every MMA of this lane done before the CTA frees its TMEM
            mma_commit(smem_u32(&drain));
            volatile int never = 0;
            if (!mbar_wait(smem_u32(&drain), 0u, drain_spin, &never)) atomicExch(err, 1);
        }
    } else if (warp >= MM_EPI0) {
        // ---- epilogue: warp w reads TMEM lanes 32 (w % 4) .. +31 (its rows),
        // columns [h BN/2, (h+1) BN/2) of both halves of the accumulator, and
        // sums the slab partials of a piece in FP32 registers; the tensor
        // core's own accumulation then spans one slab only, which keeps the
        // product as accurate as FP32 FMA chains
        const int q = warp & 3, h = (warp - MM_EPI0) >> 2;
        float *stg = (float *)(smem + (size_t)S * C::STAGE) + (size_t)(warp - MM_EPI0) * 32 * C::OUT_LD;
        int gq = 0;
        for (int i = rg.x; i < rg.y && !*abort; ++i) {
            const MmaItem m = items[i];
            float sum[C::HALF];
#pragma unroll
            for (int j = 0; j < C::HALF; ++j) sum[j] = 0.f;
            bool ok = true;
            const int ngr = (m.nk + KPS - 1) / KPS;
            for (int c = 0; c < ngr; ++c, ++gq) {
                const int acc = gq % NB;
                bool got = true;
                if (lane == 0) got = mbar_wait(smem_u32(&tfull[acc]), (uint32_t)(gq / NB) & 1u, spin, abort);
                if (__shfl_sync(0xffffffffu, got ? 1 : 0, 0) == 0) {
                    if (lane == 0) give_up();
                    ok = false;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
                for (int part = 0; part < 2; ++part)
#pragma unroll
                    for (int c0 = 0; c0 < C::HALF; c0 += 32) {   // 32 columns per load, one wait
                        uint32_t r[32];
                        asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
                                     : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
                                     : "r"(tmem + ((uint32_t)(32 * q) << 16) +
                                           (uint32_t)(acc * C::ACOLS + part * BN + h * C::HALF + c0)));
                        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
                        for (int j = 0; j < 32; ++j) sum[c0 + j] += __uint_as_float(r[j]);
                    }
                asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
                __syncwarp();
                if (lane == 0) mbar_arrive(smem_u32(&tempty[acc]));
            }
            if (!ok) break;
            // the warp's 32 rows through shared memory, 32 columns at a time,
            // then row by row with the lanes along the columns: whole 128-byte
            // segments per store (a lane writing its own row touched 32
            // sectors per store)
            float *base = out + (int64_t)m.out * plane + m.off;
#pragma unroll
            for (int c0 = 0; c0 < C::HALF; c0 += 32) {
#pragma unroll
                for (int j = 0; j < 32; ++j) stg[lane * C::OUT_LD + j] = sum[c0 + j];
                __syncwarp();
                const int col = m.n0 + h * C::HALF + c0 + lane;
                for (int r = 0; r < 32; ++r) {
                    const int il = m.m0 + 32 * q + r;
                    if (il >= m.dl) break;
                    if (col < m.dr) base[(int64_t)il * m.dr + col] = stg[r * C::OUT_LD + lane];
                }
                __syncwarp();
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(C::TCOLS));
}

// ---------------------------------------------------------------------------
// Host side

namespace {

// the driver's tensor-map encoder, looked up once (thread-safe: contexts
// of several host threads may plan at the same time)
PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static const PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            return (PFN_cuTensorMapEncodeTiled_v12000)p;
        return (PFN_cuTensorMapEncodeTiled_v12000) nullptr;
    }();
    return fn;
}

template <int BN, int KPS>
int launch_mma(Ctx &c, const CUtensorMap &ma, const CUtensorMap &mb, uint32_t spin, const int *stop) {
    static std::atomic<bool> done{false};
    if (!done.load()) {
        NSS_CUDA_TRY(c, cudaFuncSetAttribute(k_sector_mma<BN, KPS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             MmaCfg<BN>::SMEM));
        done.store(true);
    }
    DevSb &s = c.sb;
    k_sector_mma<BN, KPS><<<s.mma_grid, MM_THREADS, MmaCfg<BN>::SMEM, c.stream>>>(
        ma, mb, s.d_mma_items, s.d_mma_rng, s.d_mma_out, s.n, c.mma_lolo ? 1 : 0, spin, s.d_tc_err, stop);
    return NSS_OK;
}

}  // namespace

void mma_layout(const DevSb &s, int tc_min_dl, int bn, bool split, int nsm, MmaPlan &p) {
    p = MmaPlan{};
    p.bn = bn == 128 ? 128 : 64;
    p.split = split;
    for (int k = 0; k < s.nsb; ++k)
        if (tc_min_dl > 0 && s.dls[k] >= tc_min_dl) p.sectors.push_back(k);
    if (p.sectors.empty()) return;
    // pool rows: [H_L slabs | H_R slabs | W0 slabs | W1 slabs] of every
    // routed sector
    auto slabs = [](int d) { return (d + MM_KC - 1) / MM_KC; };
    int64_t r = 0;
    for (size_t i = 0; i < p.sectors.size(); ++i) {
        const int k = p.sectors[i], dl = s.dls[k], dr = s.drs[k];
        PackSec ps{dl, dr, 0, 0, s.off[k]};
        p.hl_row.push_back((int)r); r += (int64_t)slabs(dl) * dl;
        p.hr_row.push_back((int)r); r += (int64_t)slabs(dr) * dr;
        ps.w0_row = (int)r; r += (int64_t)slabs(dl) * dr;
        ps.w1_row = (int)r; r += (int64_t)slabs(dr) * dl;
        p.ps.push_back(ps);
        for (int a = 0; a < dl; a += 32)
            for (int b = 0; b < dr; b += 32) p.wt.push_back(make_int4((int)i, a, b, 0));
    }
    r += MM_M;   // a box that starts near the end of the pool stays inside it
    p.plane_rows = r;
    // tiles, each a run of slabs (phase 0, then phase 1)
    std::vector<MmaItem> tiles;
    int64_t total = 0;
    for (size_t i = 0; i < p.sectors.size(); ++i) {
        const int k = p.sectors[i], dl = s.dls[k], dr = s.drs[k];
        for (int m0 = 0; m0 < dl; m0 += MM_M)
            for (int n0 = 0; n0 < dr; n0 += p.bn) {
                MmaItem m{};
                m.a_row0 = p.hl_row[i];
                m.b_row0 = p.ps[i].w0_row;
                m.a_row1 = p.ps[i].w1_row;
                m.b_row1 = p.hr_row[i];
                m.a_step = dl;
                m.b_step = dr;
                m.nk0 = slabs(dl);
                m.c0 = 0;
                m.nk = slabs(dl) + slabs(dr);
                m.dl = dl; m.dr = dr; m.m0 = m0; m.n0 = n0; m.off = s.off[k];
                total += m.nk;
                tiles.push_back(m);
            }
    }
    // pieces: a tile longer than the mean load of an SM is cut into up to
    // MM_PLANES runs of consecutive slabs, piece q writing output plane q
    const int64_t target = std::max<int64_t>(2, (total + nsm - 1) / std::max(1, nsm));
    std::vector<MmaItem> pieces;
    p.nplanes = 1;
    for (const MmaItem &t : tiles) {
        const int np = split ? (int)std::min<int64_t>(MM_PLANES, (t.nk + target - 1) / target) : 1;
        p.nplanes = std::max(p.nplanes, np);
        for (int q = 0; q < np; ++q) {
            MmaItem m = t;
            m.c0 = (int)((int64_t)q * t.nk / np);
            m.nk = (int)((int64_t)(q + 1) * t.nk / np) - m.c0;
            m.out = q;
            pieces.push_back(m);
        }
    }
    // longest first onto the least loaded CTA (a piece costs its slabs plus
    // about two slabs of epilogue); each CTA runs its pieces in that order
    std::stable_sort(pieces.begin(), pieces.end(), [](const MmaItem &a, const MmaItem &b) { return a.nk > b.nk; });
    const int G = (int)std::min<size_t>(pieces.size(), (size_t)std::max(1, nsm));
    std::vector<int64_t> load(G, 0);
    std::vector<std::vector<int>> own(G);
    for (size_t e = 0; e < pieces.size(); ++e) {
        int b = 0;
        for (int g = 1; g < G; ++g)
            if (load[g] < load[b]) b = g;
        load[b] += pieces[e].nk + 2;
        own[b].push_back((int)e);
    }
    p.grid = G;
    for (int g = 0; g < G; ++g) {
        const int start = (int)p.items.size();
        for (int e : own[g]) p.items.push_back(pieces[e]);
        p.rng.push_back(make_int2(start, (int)p.items.size()));
    }
}

int mma_finish(Ctx &c, const MmaPlan &p) {
    DevSb &s = c.sb;
    if (p.items.empty()) return NSS_OK;
    const int64_t pl = p.plane_rows * MM_KC;
    NSS_CUDA_TRY(c, cudaMemsetAsync(s.d_mma_pool, 0, (size_t)pl * sizeof(float), c.stream));
    // output planes: a plane element no piece writes stays zero
    NSS_CUDA_TRY(c, cudaMemsetAsync(s.d_mma_out, 0, (size_t)p.nplanes * s.n * sizeof(float), c.stream));
    auto slabs = [](int d) { return (d + MM_KC - 1) / MM_KC; };
    for (size_t i = 0; i < p.sectors.size(); ++i) {
        const int k = p.sectors[i], dl = s.dls[k], dr = s.drs[k];
        float *q = s.d_mma_pool;
        k_pack_h<<<(unsigned)std::min<int64_t>(1024, ((int64_t)slabs(dl) * dl * MM_KC + 255) / 256), 256, 0,
                   c.stream>>>(s.d_hl32 + s.hl_off[k], dl, q + (int64_t)p.hl_row[i] * MM_KC);
        k_pack_h<<<(unsigned)std::min<int64_t>(1024, ((int64_t)slabs(dr) * dr * MM_KC + 255) / 256), 256, 0,
                   c.stream>>>(s.d_hr32 + s.hr_off[k], dr, q + (int64_t)p.hr_row[i] * MM_KC);
        c.launches += 2;
    }
    NSS_CUDA_TRY(c, cudaGetLastError());
    s.mma_nitems = (int)p.items.size();
    s.mma_nwt = (int)p.wt.size();
    s.mma_plane_rows = (int)p.plane_rows;
    s.mma_bn = p.bn;
    s.mma_split = p.split;
    s.mma_nplanes = p.nplanes;
    s.mma_grid = p.grid;
    // two tensor maps over the pool, [plane rows] x 32 FP32 with 128-byte
    // rows and the 128-byte swizzle: boxes of 128 rows (A) and of BN rows (B)
    auto enc = encode_fn();
    if (!enc) {
        c.err = "nss_sb_upload: cuTensorMapEncodeTiled is not available from the driver";
        return NSS_ERR_CUDA;
    }
    const cuuint64_t gdim[2] = {(cuuint64_t)MM_KC, (cuuint64_t)p.plane_rows};
    const cuuint64_t gstride[1] = {(cuuint64_t)MM_KC * sizeof(float)};
    const cuuint32_t estr[2] = {1, 1};
    for (int which = 0; which < 2; ++which) {
        alignas(64) CUtensorMap map;
        const cuuint32_t box[2] = {(cuuint32_t)MM_KC, (cuuint32_t)(which == 0 ? MM_M : p.bn)};
        const CUresult cr = enc(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, (void *)s.d_mma_pool, gdim, gstride, box,
                                estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                                CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (cr != CUDA_SUCCESS) {
            c.err = "nss_sb_upload: cuTensorMapEncodeTiled failed (" + std::to_string((int)cr) + ")";
            return NSS_ERR_CUDA;
        }
        static_assert(sizeof(CUtensorMap) == sizeof(s.mma_map_a), "tensor map storage");
        std::memcpy(which == 0 ? s.mma_map_a : s.mma_map_b, &map, sizeof(map));
    }
    return NSS_OK;
}

// D_k of every routed sector into the output planes (d_mma_out + q n): pack
// W, then the persistent GEMM.  The caller's "terms only" tiles add the
// planes to their A x B terms.
int hv_device_mma(Ctx &c, const float *d_v, const int *stop) {
    DevSb &s = c.sb;
    if (s.mma_nitems == 0) return NSS_OK;
    k_pack_w<<<s.mma_nwt, 256, 0, c.stream>>>(d_v, 1.0f, s.d_mma_wt, s.d_mma_sec, s.d_mma_pool, stop);
    const uint32_t spin = wait_limit();
    alignas(64) CUtensorMap ma, mb;
    std::memcpy(&ma, s.mma_map_a, sizeof(ma));
    std::memcpy(&mb, s.mma_map_b, sizeof(mb));
    int rc;
    if (s.mma_bn == 128)
        rc = c.mma_kps == 2 ? launch_mma<128, 2>(c, ma, mb, spin, stop) : launch_mma<128, 1>(c, ma, mb, spin, stop);
    else
        rc = c.mma_kps == 2 ? launch_mma<64, 2>(c, ma, mb, spin, stop) : launch_mma<64, 1>(c, ma, mb, spin, stop);
    if (rc) return rc;
    c.launches += 2;
    NSS_CUDA_TRY(c, cudaGetLastError());
    return NSS_OK;
}

}  // namespace nss
