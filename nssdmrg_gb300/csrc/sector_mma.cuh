// Tensor-core sector product (k_sector_mma.cu): the work-item and packing
// records shared with the superblock upload (k_matvec.cu), and the host plan
// that sizes the upload arena's tensor-core sections.
#pragma once

#include <cstdint>
#include <vector>

#include "device.cuh"

namespace nss {

constexpr int MM_M = 128;      // UMMA M: rows of il per work item
constexpr int MM_KC = 32;      // K columns per slab (128 bytes of FP32)
constexpr int MM_PLANES = 4;   // output planes: pieces a tile may be cut into

// One work item (piece) of the grouped sector GEMM: slabs [c0, c0 + nk) of
// its tile's sequence, phase 0 (H_L W, slabs 0 .. nk0-1) then phase 1
// (W H_R^T).  Row indices address the [rows x 32] operand pool.
struct MmaItem {
    int a_row0, a_row1;          // A slab of chunk 0, phase 0 / phase 1
    int b_row0, b_row1;          // B slab of chunk 0, phase 0 / phase 1
    int a_step, b_step;          // rows from one chunk's slab to the next (Dl for A, Dr for B)
    int nk0;                     // chunks of phase 0 (the tile's K chunks of H_L W)
    int c0, nk;                  // this piece's slabs
    int dl, dr;                  // the sector
    int m0, n0;                  // output tile origin (il, ir)
    int out;                     // output plane 0 .. MM_PLANES-1
    int64_t off;                 // sector offset in psi
};

// Per routed sector, for the per-call packing of W.
struct PackSec {
    int dl, dr;
    int w0_row, w1_row;          // chunk-0 slab rows of W0 / W1
    int64_t off;
};

// Host plan of the tensor-core path of one superblock.
struct MmaPlan {
    std::vector<int> sectors;          // routed sectors
    std::vector<int> hl_row, hr_row;   // their H_L / H_R slab rows
    std::vector<MmaItem> items;        // grouped by CTA
    std::vector<int2> rng;             // per CTA: its items [x, y)
    std::vector<int4> wt;              // 32x32 tiles of W (routed-sector index, il0, ir0)
    std::vector<PackSec> ps;
    int64_t plane_rows = 0;
    int bn = 64;
    bool split = true;
    int nplanes = 1;                   // output planes in use
    int grid = 0;                      // CTAs
};

// Sectors with Dl >= tc_min_dl and the pool layout, items (tiles cut into
// pieces when split, dealt to nsm CTAs) and W tiles for tile width bn.
void mma_layout(const DevSb &s, int tc_min_dl, int bn, bool split, int nsm, MmaPlan &p);
// After the arena is filled and the FP32 operator blocks exist: zero the
// pool and the output planes, pack H_L / H_R, encode the tensor maps.
int mma_finish(Ctx &c, const MmaPlan &p);

}  // namespace nss
