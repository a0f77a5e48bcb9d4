// Superblock enumeration and direct-mode operator pool (see host_setup.hpp).
#include "host_setup.hpp"

#include <stdexcept>

namespace nss {

namespace {

Qn qn_sub(const Qn &a, const Qn &b) {
    Qn c(a.size());
    for (size_t i = 0; i < a.size(); ++i) c[i] = a[i] - b[i];
    return c;
}

}  // namespace

SbHost sb_build(const Block &left, const Block &right, const Qn &target, const double *hij) {
    if (left.fermion != right.fermion)
        throw std::runtime_error("Setup_SuperBlock_Direct ERROR: left.Type != right.Type");
    if (left.qdim != right.qdim || (int)target.size() != left.qdim)
        throw std::runtime_error("sb_build: QN dimension mismatch");
    SbHost sb;
    sb.target = target;
    sb.qdim = left.qdim;
    sb.m_left = left.dim;
    sb.m_right = right.dim;
    const Sectors lsec = left.sectors(), rsec = right.sectors();

    // sb_get_states (src/DMRG_SUPERBLOCK.f90:167-283): left sectors in list
    // order, each with its matching right sector target - q; inside a sector
    // the left state is the slow index.
    int64_t pos = 0;
    for (size_t ql = 0; ql < lsec.qns.size(); ++ql) {
        const Qn rq = qn_sub(target, lsec.qns[ql]);
        int rk = rsec.find(rq);
        if (rk < 0) continue;
        const std::vector<int> &lmap = lsec.maps[ql], &rmap = rsec.maps[rk];
        sb.qns.push_back(lsec.qns[ql]);
        sb.dls.push_back((int)lmap.size());
        sb.drs.push_back((int)rmap.size());
        sb.offset.push_back(pos);
        pos += (int64_t)lmap.size() * rmap.size();
        // sb2block_states (src/DMRG_SUPERBLOCK_SETUP.f90:1079-1122): the unique
        // left/right states of the sector, i.e. the two sector maps.
        sb.ai.push_back(lmap);
        sb.bi.push_back(rmap);
    }
    if (pos == 0) throw std::runtime_error("sb_get_states ERROR: total_states=0. There are no SB states.");
    const int nsb = sb.nsb();
    // the states of each sector at its offset (sectors fill in parallel)
    sb.sb_states.resize((size_t)pos);
    parallel_for(nsb, [&](int k) {
        int64_t at = sb.offset[k];
        for (int l : sb.ai[k])
            for (int r : sb.bi[k]) sb.sb_states[(size_t)at++] = (int64_t)l * right.dim + r;
    }, pos > 200000);
    std::map<Qn, int> index;
    for (int k = 0; k < nsb; ++k) index.emplace(sb.qns[k], k);

    const Csr &hl = left.op("H"), &hr = right.op("H");
    sb.hleft.resize(nsb);
    sb.hright.resize(nsb);
    parallel_for(2 * nsb, [&](int t) {
        const int k = t >> 1;
        if (t & 1) sb.hright[k] = csr_filter(hr, sb.bi[k], sb.bi[k]);
        else sb.hleft[k] = csr_filter(hl, sb.ai[k], sb.ai[k]);
    }, hl.nnz() + hr.nnz() > 40000);

    auto set_term = [&](int it, int k, int jsb, int hc, Csr a, Csr b, int64_t ro, int64_t co) {
        int idx = it + sb.tnso * k;
        sb.a[idx] = std::move(a);
        sb.b[idx] = std::move(b);
        sb.isb2jsb[idx] = jsb;
        sb.ishconjg[idx] = hc;
        sb.row_off[idx] = ro;
        sb.col_off[idx] = co;
    };
    auto alloc_terms = [&](int tnso) {
        sb.tnso = tnso;
        sb.a.assign((size_t)tnso * nsb, Csr{});
        sb.b.assign((size_t)tnso * nsb, Csr{});
        sb.isb2jsb.assign((size_t)tnso * nsb, -1);
        sb.ishconjg.assign((size_t)tnso * nsb, 0);
        sb.row_off.assign((size_t)tnso * nsb, 0);
        sb.col_off.assign((size_t)tnso * nsb, 0);
    };

    if (!left.fermion) {
        // Setup_SuperBlock_Spin_Direct (src/DMRG_SUPERBLOCK_SETUP.f90:152-405), OBC.
        alloc_terms(3);
        const Csr &szl = left.op("S_z_n"), &spl = left.op("S_p_n");
        const Csr &szr = right.op("S_z_n");
        const Csr smr = csr_transpose(right.op("S_p_n"));
        // each sector's terms in their own slots (sectors in parallel)
        parallel_for(nsb, [&](int k) {
            set_term(0, k, k, 0, csr_scale(csr_filter(szl, sb.ai[k], sb.ai[k]), hij[0]),
                     csr_filter(szr, sb.bi[k], sb.bi[k]), sb.offset[k], sb.offset[k]);
            Qn qm = sb.qns[k];
            qm[0] -= 1.0;
            auto it = index.find(qm);
            if (it == index.end()) return;
            int j = it->second;
            Csr a2 = csr_scale(csr_filter(spl, sb.ai[k], sb.ai[j]), hij[3]);
            Csr b2 = csr_filter(smr, sb.bi[k], sb.bi[j]);
            Csr a3 = csr_transpose(a2), b3 = csr_transpose(b2);
            set_term(1, k, j, 0, std::move(a2), std::move(b2), sb.offset[k], sb.offset[j]);
            set_term(2, k, j, 1, std::move(a3), std::move(b3), sb.offset[j], sb.offset[k]);
        }, szl.nnz() + spl.nnz() > 20000);
    } else {
        // Setup_SuperBlock_Fermion_Direct (src/DMRG_SUPERBLOCK_SETUP.f90:416-693),
        // Norb=1, OBC (fbc=2): tMap(i,io,jo) counts the non-zero couplings.
        const int nso = 2;
        int tmap[3][2][2] = {};
        int it = 0;
        for (int i = 1; i <= 2; ++i)
            for (int io = 0; io < nso; ++io)
                for (int jo = 0; jo < nso; ++jo)
                    if (hij[io * nso + jo] != 0.0) tmap[i][io][jo] = it++;
        alloc_terms(it);
        const Csr &pl = left.op("P_n");
        Csr cldp[2], cr[2];
        const char *ckey[2] = {"C_l1_s1_n", "C_l1_s2_n"};
        for (int io = 0; io < nso; ++io) {
            cldp[io] = csr_matmul(csr_transpose(left.op(ckey[io])), pl);
            cr[io] = right.op(ckey[io]);
        }
        // each sector's terms in their own slots (sectors in parallel)
        parallel_for(nsb, [&](int k) {
            for (int ispin = 0; ispin < 2; ++ispin) {
                Qn qm = sb.qns[k];
                qm[ispin] -= 1.0;   // qnup = [1,0], qndw = [0,1]
                auto f = index.find(qm);
                if (f == index.end()) continue;
                int j = f->second;
                int io = ispin, jo = ispin;
                double t = hij[io * nso + jo];
                if (t == 0.0) continue;
                Csr a1 = csr_scale(csr_filter(cldp[io], sb.ai[k], sb.ai[j]), t);
                Csr b1 = csr_filter(cr[jo], sb.bi[k], sb.bi[j]);
                Csr a2 = csr_transpose(a1), b2 = csr_transpose(b1);
                set_term(tmap[1][io][jo], k, j, 0, std::move(a1), std::move(b1), sb.offset[k], sb.offset[j]);
                set_term(tmap[2][io][jo], k, j, 1, std::move(a2), std::move(b2), sb.offset[j], sb.offset[k]);
            }
        }, cldp[0].nnz() + cr[0].nnz() > 20000);
    }
    return sb;
}

void sb_view(const SbHost &sb, SbView &v) {
    auto view = [](const Csr &m) {
        nss_csr c;
        c.nrow = m.nrow;
        c.ncol = m.ncol;
        c.rowptr = m.rowptr.data();
        c.colidx = m.col.data();
        c.vals = m.val.data();
        return c;
    };
    const int nsb = sb.nsb();
    v.hl.clear(); v.hr.clear(); v.a.clear(); v.b.clear(); v.ai.clear(); v.bi.clear();
    for (int k = 0; k < nsb; ++k) {
        v.hl.push_back(view(sb.hleft[k]));
        v.hr.push_back(view(sb.hright[k]));
        v.ai.insert(v.ai.end(), sb.ai[k].begin(), sb.ai[k].end());
        v.bi.insert(v.bi.end(), sb.bi[k].begin(), sb.bi[k].end());
    }
    for (size_t i = 0; i < sb.a.size(); ++i) {
        v.a.push_back(view(sb.a[i]));
        v.b.push_back(view(sb.b[i]));
    }
    nss_sb_desc &d = v.desc;
    d.nsb = nsb;
    d.tnso = sb.tnso;
    d.m_left = sb.m_left;
    d.m_right = sb.m_right;
    d.dls = sb.dls.data();
    d.drs = sb.drs.data();
    d.offset = sb.offset.data();
    d.ai = v.ai.data();
    d.bi = v.bi.data();
    d.hleft = v.hl.data();
    d.hright = v.hr.data();
    d.a = v.a.data();
    d.b = v.b.data();
    d.isb2jsb = sb.isb2jsb.data();
    d.ishconjg = sb.ishconjg.data();
    d.row_offset = sb.row_off.data();
    d.col_offset = sb.col_off.data();
}

}  // namespace nss
