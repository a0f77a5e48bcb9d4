// Host-side DMRG driver: sites, block enlargement, renormalisation and the
// infinite/finite algorithms (src/BLOCKS/SITES.f90, src/DMRG_CONNECT.f90,
// src/DMRG_RDM.f90:172-404, src/DMRG_MAIN.f90).  Every superblock solve
// (H*psi, Lanczos, RDM, block eigh, truncation) runs on the GPU through the
// same entry points as the C ABI.
#pragma once

#include <memory>

#include "host_setup.hpp"

namespace nss {

struct Ctx;
// the library context behind a C ABI handle (capi.cpp)
Ctx &ctx_of(nss_ctx *ctx);

Block spin_site(int sun);
Block electron_site(double uloc, bool hfmode);

// enlarge_block with link 'n' (src/DMRG_CONNECT.f90:18-291); label 'l' or 'r'.
Block enlarge_block(const Block &blk, const Block &dot, char label, const double *hij);

// Block descriptors <-> Block
Block block_from_desc(const nss_block_desc &d, bool fermion);

struct Driver {
    Ctx *ctx = nullptr;
    nss_dmrg_params p{};
    std::vector<int32_t> msweep;
    std::vector<double> esweep;   // Esweep (default Edmrg for every sweep)
    double hij[4] = {0, 0, 0, 0};
    Block dot, left, right;
    std::vector<nss_step_record> records;
    // bench support: stop before the solve of the last infinite step
    bool stop_before_last_solve = false;
    bool stopped = false;
    std::shared_ptr<SbHost> last_sb;   // superblock of the step stopped at

    int init(Ctx *c, const nss_dmrg_params &params);
    int step(int type, int label, int sweep, int keep_sides = 3);
    int infinite();
    int finite();
    // Build_Op_dmrg + Advance_Op_dmrg: the site operator op (dot basis) at
    // chain position pos, on the last step's enlarged block holding it;
    // *side = 0 (left) or 1 (right)
    Csr site_op_on_block(const Csr &op, int pos, int *side) const;
};

}  // namespace nss
