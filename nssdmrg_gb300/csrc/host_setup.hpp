// Superblock enumeration and direct-mode operator pool (host side).
//
// sb_get_states / sb_build_dims / sb2block_states (src/DMRG_SUPERBLOCK.f90:
// 36-283, src/DMRG_SUPERBLOCK_SETUP.f90:1079-1122) and
// Setup_SuperBlock_{Spin,Fermion}_Direct (src/DMRG_SUPERBLOCK_SETUP.f90:
// 152-693).  The result is the operator pool that the reference keeps in
// module globals (src/DMRG_GLOBAL.f90:119-124); sb_view() exposes it as the
// nss_sb_desc of the C ABI.
#pragma once

#include "host_sparse.hpp"
#include "../../include/nssdmrg.h"

namespace nss {

struct SbHost {
    Qn target;
    int qdim = 1;
    int m_left = 0, m_right = 0;
    std::vector<Qn> qns;                 // sb_sector QN (left QN) per sector
    std::vector<int> dls, drs;
    std::vector<int64_t> offset;
    std::vector<int64_t> sb_states;      // l*m_right + r, 0-based
    std::vector<std::vector<int>> ai, bi;
    std::vector<Csr> hleft, hright;
    int tnso = 0;
    std::vector<Csr> a, b;               // [tnso*nsb], absent: nrow == 0
    std::vector<int> isb2jsb, ishconjg;
    std::vector<int64_t> row_off, col_off;

    int nsb() const { return (int)qns.size(); }
    int64_t n() const { return (int64_t)sb_states.size(); }
};

// Build the superblock of `target` from the enlarged blocks.  hij is the
// 2x2 coupling matrix (HopH), row-major.
SbHost sb_build(const Block &left, const Block &right, const Qn &target, const double *hij);

// Flattened C view of an SbHost; the view owns the pointer arrays it hands out.
struct SbView {
    nss_sb_desc desc{};
    std::vector<nss_csr> hl, hr, a, b;
    std::vector<int32_t> ai, bi;
};
void sb_view(const SbHost &sb, SbView &v);

}  // namespace nss
