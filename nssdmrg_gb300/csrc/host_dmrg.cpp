// Host-side DMRG driver (see host_dmrg.hpp).
#include "host_dmrg.hpp"

#include <chrono>
#include <deque>
#include <thread>
#include <cstdlib>
#include <cmath>
#include <stdexcept>

#include "device.cuh"

namespace nss {

namespace {

Csr dense_csr(int n, std::initializer_list<double> v) {
    std::vector<double> a(v);
    return csr_from_dense(n, n, a.data());
}

}  // namespace

// spin_site (src/BLOCKS/SITES.f90:281-350), zero field.
Block spin_site(int sun) {
    Block b;
    b.length = 1;
    b.qdim = 1;
    b.fermion = false;
    if (sun == 2) {
        b.dim = 2;
        b.basis = {0.5, -0.5};
        b.ops.push_back({"H", Csr{}, "bosonic"});
        b.ops[0].m.init(2, 2);
        b.ops.push_back({"S_z_n", dense_csr(2, {0.5, 0, 0, -0.5}), "bosonic"});
        b.ops.push_back({"S_p_n", dense_csr(2, {0, 1, 0, 0}), "bosonic"});
    } else if (sun == 3) {
        const double r2 = std::sqrt(2.0);
        b.dim = 3;
        b.basis = {1.0, 0.0, -1.0};
        b.ops.push_back({"H", Csr{}, "bosonic"});
        b.ops[0].m.init(3, 3);
        b.ops.push_back({"S_z_n", dense_csr(3, {1, 0, 0, 0, 0, 0, 0, 0, -1}), "bosonic"});
        b.ops.push_back({"S_p_n", dense_csr(3, {0, r2, 0, 0, 0, r2, 0, 0, 0}), "bosonic"});
    } else {
        throw std::runtime_error("spin_site ERROR: SU(N) value not supported");
    }
    return b;
}

// electron_site, Norb=1 (src/BLOCKS/SITES.f90:358-450; src/FOCK/HLOCAL.f90:
// 312-433 local H, :587-615 C with the Jordan-Wigner sign of c() :884-896,
// :735-781 basis QNs and parity).  Fock index m = iup + 2*idw.
Block electron_site(double uloc, bool hfmode) {
    Block b;
    b.length = 1;
    b.dim = 4;
    b.qdim = 2;
    b.fermion = true;
    const int nup[4] = {0, 1, 0, 1}, ndw[4] = {0, 0, 1, 1};
    std::vector<double> h(16, 0.0), cu(16, 0.0), cd(16, 0.0), p(16, 0.0);
    for (int m = 0; m < 4; ++m) {
        double e = uloc * nup[m] * ndw[m];
        if (hfmode) e -= 0.5 * uloc * (nup[m] + ndw[m]);
        h[m * 4 + m] = e;
        p[m * 4 + m] = ((nup[m] + ndw[m]) % 2) ? -1.0 : 1.0;
        b.basis.push_back(nup[m]);
        b.basis.push_back(ndw[m]);
    }
    cu[0 * 4 + 1] = 1.0;    // c_up |up>    = |0>
    cu[2 * 4 + 3] = 1.0;    // c_up |up,dw> = |dw>
    cd[0 * 4 + 2] = 1.0;    // c_dw |dw>    = |0>
    cd[1 * 4 + 3] = -1.0;   // c_dw |up,dw> = -|up>  (one occupied level below)
    b.ops.push_back({"H", csr_from_dense(4, 4, h.data()), "bosonic"});
    b.ops.push_back({"C_l1_s1_n", csr_from_dense(4, 4, cu.data()), "fermionic"});
    b.ops.push_back({"C_l1_s2_n", csr_from_dense(4, 4, cd.data()), "fermionic"});
    b.ops.push_back({"P_n", csr_from_dense(4, 4, p.data()), "psign"});
    return b;
}

namespace {

// The coupling terms of connect_spin_blocks (src/DMRG_CONNECT.f90:394-454)
// and connect_fermion_blocks (:296-389, real, Norb=1), link 'n', as
// coef * kron(X from l, Y from r); transposes and products land in tmp.
void connect_terms(const Block &l, const Block &r, const double *hij, std::deque<Csr> &tmp,
                   std::vector<KronTerm> &terms) {
    if (!l.fermion) {
        const Csr &szl = l.op("S_z_n"), &spl = l.op("S_p_n");
        const Csr &szr = r.op("S_z_n"), &spr = r.op("S_p_n");
        terms.push_back({&szl, &szr, hij[0]});
        tmp.push_back(csr_transpose(spr));
        terms.push_back({&spl, &tmp.back(), hij[3]});
        tmp.push_back(csr_transpose(spl));
        terms.push_back({&tmp.back(), &spr, hij[3]});
        return;
    }
    const Csr &pl = l.op("P_n");
    const char *key[2] = {"C_l1_s1_n", "C_l1_s2_n"};
    for (int io = 0; io < 2; ++io)
        for (int jo = 0; jo < 2; ++jo) {
            const double t = hij[io * 2 + jo];
            if (t == 0.0) continue;
            const Csr &cl = l.op(key[io]), &cr = r.op(key[jo]);
            tmp.push_back(csr_matmul(csr_transpose(cl), pl));
            terms.push_back({&tmp.back(), &cr, t});
            tmp.push_back(csr_matmul(pl, cl));
            const Csr *a2 = &tmp.back();
            tmp.push_back(csr_transpose(cr));
            terms.push_back({a2, &tmp.back(), t});
        }
}

std::vector<double> outsum(const std::vector<double> &a, int na, const std::vector<double> &b, int nb, int q) {
    std::vector<double> c((size_t)na * nb * q);
    for (int i = 0; i < na; ++i)
        for (int j = 0; j < nb; ++j)
            for (int t = 0; t < q; ++t) c[((size_t)i * nb + j) * q + t] = a[(size_t)i * q + t] + b[(size_t)j * q + t];
    return c;
}

}  // namespace

Block enlarge_block(const Block &blk, const Block &dot, char label, const double *hij) {
    const int m = blk.dim, d = dot.dim;
    // the block's metadata and operator list without its matrices, which
    // are all replaced below
    Block out;
    out.length = blk.length;
    out.dim = blk.dim;
    out.qdim = blk.qdim;
    out.fermion = blk.fermion;
    out.omats = blk.omats;
    out.ops.reserve(blk.ops.size());
    for (const Op &o : blk.ops) out.ops.push_back({o.key, Csr{}, o.type});
    // H = H_block x 1 + 1 x H_dot + the coupling terms (left; mirrored on the
    // right), summed in one pass over the output rows
    std::deque<Csr> tmp;
    const Csr id_m = csr_identity(m), id_d = csr_identity(d);
    std::vector<KronTerm> terms;
    const unsigned hw = std::thread::hardware_concurrency();
    const int nth = blk.op("H").nnz() > 20000 ? (int)std::max(1u, std::min(4u, hw / 2)) : 1;
    if (label == 'l') {
        terms.push_back({&blk.op("H"), &id_d, 1.0});
        terms.push_back({&id_m, &dot.op("H"), 1.0});
        connect_terms(blk, dot, hij, tmp, terms);
        out.op("H") = csr_kron_sum(m, d, terms, nth);
    } else {
        terms.push_back({&id_d, &blk.op("H"), 1.0});
        terms.push_back({&dot.op("H"), &id_m, 1.0});
        connect_terms(dot, blk, hij, tmp, terms);
        out.op("H") = csr_kron_sum(d, m, terms, nth);
    }
    // other operators in list order; P is read from the list being updated
    // exactly as the reference loop does (src/DMRG_CONNECT.f90:117-146):
    // the enlarged P once its own entry has been passed, the block's before
    const int ip = blk.find_op("P_n");
    auto p_now = [&](size_t i) -> const Csr & {
        if (ip < 0) throw std::runtime_error("block operator not found: P_n");
        return (size_t)ip < i ? out.ops[ip].m : blk.ops[ip].m;
    };
    for (size_t i = 0; i < blk.ops.size(); ++i) {
        const Op &o = blk.ops[i];
        if (o.key == "H") continue;
        const char t = o.type.empty() ? 'b' : o.type[0];
        if (label == 'l') {
            out.ops[i].m = (t == 'b') ? csr_kron(csr_identity(m), dot.op(o.key)) : csr_kron(p_now(i), dot.op(o.key));
        } else {
            out.ops[i].m = (t == 'p') ? csr_kron(dot.op(o.key), p_now(i)) : csr_kron(dot.op(o.key), csr_identity(m));
        }
    }
    out.length = blk.length + 1;
    out.dim = m * d;
    out.basis = (label == 'l') ? outsum(blk.basis, m, dot.basis, d, blk.qdim)
                               : outsum(dot.basis, d, blk.basis, m, blk.qdim);
    return out;
}

Block block_from_desc(const nss_block_desc &d, bool fermion) {
    Block b;
    b.dim = d.dim;
    b.qdim = d.qdim;
    b.fermion = fermion;
    b.basis.assign(d.basis, d.basis + (size_t)d.dim * d.qdim);
    auto mk = [&](const nss_csr &c) {
        Csr m;
        m.init(c.nrow, c.ncol);
        if (c.nrow != d.dim || c.ncol != d.dim) throw std::runtime_error("block operator has wrong shape");
        int nnz = c.rowptr[c.nrow];
        m.rowptr.assign(c.rowptr, c.rowptr + c.nrow + 1);
        m.col.assign(c.colidx, c.colidx + nnz);
        m.val.assign(c.vals, c.vals + nnz);
        return m;
    };
    b.ops.push_back({"H", mk(d.h), "bosonic"});
    if (!fermion) {
        b.ops.push_back({"S_z_n", mk(d.op[0]), "bosonic"});
        b.ops.push_back({"S_p_n", mk(d.op[1]), "bosonic"});
    } else {
        b.ops.push_back({"C_l1_s1_n", mk(d.op[0]), "fermionic"});
        b.ops.push_back({"C_l1_s2_n", mk(d.op[1]), "fermionic"});
        b.ops.push_back({"P_n", mk(d.op[2]), "psign"});
    }
    return b;
}

// ---------------------------------------------------------------------------
int Driver::init(Ctx *c, const nss_dmrg_params &params) {
    ctx = c;
    p = params;
    if (p.msweep && p.nsweep > 0) msweep.assign(p.msweep, p.msweep + p.nsweep);
    p.msweep = nullptr;
    // Esweep defaults to Edmrg for every sweep (src/INPUT_VARS.f90:203-205)
    esweep.assign(msweep.size(), p.edmrg);
    if (p.esweep && p.nsweep > 0) esweep.assign(p.esweep, p.esweep + p.nsweep);
    p.esweep = nullptr;
    if (p.mdmrg < 0) throw std::invalid_argument("nss_dmrg_create: Mdmrg must not be negative");
    if (p.mdmrg == 0 && !(p.edmrg != 0.0))
        throw std::invalid_argument("Mdmrg=Edmrg=0 can not fix a threshold for the RDM");
    if (p.lanc_neigen <= 0) p.lanc_neigen = 2;
    if (p.lanc_niter <= 0) p.lanc_niter = 512;
    if (p.lanc_tolerance <= 0) p.lanc_tolerance = 1e-12;
    if (p.deg_evals_threshold <= 0) p.deg_evals_threshold = 0.1;
    switch (p.model) {
    case NSS_MODEL_HEISENBERG_HALF:
        dot = spin_site(2);
        break;
    case NSS_MODEL_HEISENBERG_ONE:
        dot = spin_site(3);
        break;
    case NSS_MODEL_HUBBARD:
        dot = electron_site(p.u, p.hfmode != 0);
        break;
    default:
        c->err = "nss_dmrg_create: unknown model";
        return NSS_ERR_INVALID;
    }
    if (p.model == NSS_MODEL_HUBBARD) {
        hij[0] = -p.t; hij[1] = 0; hij[2] = 0; hij[3] = -p.t;    // Hlr = diag(ts,ts), ts=-t
    } else {
        hij[0] = p.jz; hij[1] = 0; hij[2] = 0; hij[3] = p.jxy / 2.0;   // Hlr = diag(Jp, Jx/2)
    }
    // the site block's rotation list starts with the identity
    // (constructor_from_site, src/BLOCKS/BLOCKS.f90:140-142)
    dot.omats = {std::make_shared<const Csr>(csr_identity(dot.dim))};
    left = dot;
    right = dot;
    return NSS_OK;
}

int nss_solve_step(Ctx &c, const SbHost &sb, const nss_dmrg_params &p, int mstates, double estates,
                   bool renormalize, Block &left, Block &right, nss_step_record &rec, int keep_sides);

// step_dmrg (src/DMRG_MAIN.f90:262-433), OBC link 'n'.  keep_sides: bit 0
// left, bit 1 right; a side left out is not renormalised (its block is
// replaced from the stored list before the next step uses it), its spectrum,
// truncation error and entropies are still formed
int Driver::step(int type, int label, int sweep, int keep_sides) {
    const auto t_step = std::chrono::steady_clock::now();
    // Mstates/Estates of step_dmrg (src/DMRG_MAIN.f90:288-295): Mdmrg/Edmrg
    // while growing, Msweep/Esweep of the sweep afterwards
    const int mstates = (type == 0) ? p.mdmrg : msweep.at(sweep - 1);
    const double estates = (type == 0) ? p.edmrg : esweep.at(sweep - 1);
    using clk = std::chrono::steady_clock;
    auto ms_since = [](clk::time_point t) { return std::chrono::duration<double, std::milli>(clk::now() - t).count(); };
    // the two enlargements are independent
    run_pair([&] { left = enlarge_block(left, dot, 'l', hij); },
             [&] { right = enlarge_block(right, dot, 'r', hij); },
             (int64_t)left.op("H").nnz() + right.op("H").nnz() > 20000);
    const double ms_enlarge = ms_since(t_step);
    const int current_l = left.length + right.length;
    // sb_set_current_qn, QNtype local: int(target_qn * L * Norb), truncated
    Qn target(left.qdim);
    for (int i = 0; i < left.qdim; ++i) target[i] = std::trunc(p.dmrg_qn[i] * current_l * 1.0);
    const auto t_sb = clk::now();
    SbHost sb = sb_build(left, right, target, hij);
    const double ms_sb = ms_since(t_sb);
    bool renorm;
    if (type == 0) renorm = left.length != p.ldmrg;
    else renorm = !(left.length == p.ldmrg + 1 && label == 1);
    nss_step_record rec{};
    rec.type = type;
    rec.left_length = left.length;
    rec.right_length = right.length;
    rec.current_l = current_l;
    rec.n = sb.n();
    rec.nsb = sb.nsb();
    if (stop_before_last_solve && type == 0 && left.length == p.ldmrg) {
        last_sb = std::make_shared<SbHost>(std::move(sb));
        SbView v;
        sb_view(*last_sb, v);
        int rc = sb_upload(*ctx, &v.desc, true);
        stopped = true;
        return rc;
    }
    rec.ms_build = ms_since(t_step);
    rec.host_phase_ms[0] = ms_enlarge;
    rec.host_phase_ms[1] = ms_sb;
    int rc = nss_solve_step(*ctx, sb, p, mstates, estates, renorm, left, right, rec, keep_sides);
    if (rc) return rc;
    rec.ms_step = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_step).count();
    records.push_back(rec);
    return NSS_OK;
}

// Build_Op_dmrg (src/DMRG_MEASURE.f90:288-386) and Advance_Op_dmrg
// (:398-486), OBC: the site sits at index i of the block holding it (i = pos
// on the left, N+1-pos on the right); it enters as Id(D) x Op on the left
// (Op x Id(D) on the right) of the enlarged length-i block, D the states of
// the length-(i-1) block, and is rotated with omat(i), ..., omat(Lside-1)
// and enlarged by the site after each rotation.
Csr Driver::site_op_on_block(const Csr &op, int pos, int *side) const {
    const int L = left.length, R = right.length, N = L + R;
    if (pos < 1 || pos > N) throw std::runtime_error("Build_op_dmrg error: Pos not in [1,Ldmrg]");
    const bool rgt = pos > L;
    const Block &b = rgt ? right : left;
    const int i = rgt ? N + 1 - pos : pos, iend = (rgt ? R : L) - 1;
    if ((int)b.omats.size() < std::max(iend, i - 1))
        throw std::runtime_error("Init_Measure_DMRG: No rotation matrices are present (run with save_umat)");
    if (op.nrow != dot.dim || op.ncol != dot.dim) throw std::runtime_error("measure: operator is not d x d");
    Csr oi = op;
    if (i > 1) {
        const int D = b.omats[i - 2]->ncol;
        oi = rgt ? csr_kron(op, csr_identity(D)) : csr_kron(csr_identity(D), op);
    }
    for (int it = i; it <= iend; ++it) {
        const Csr &u = *b.omats[it - 1];
        if (u.nrow != oi.nrow) throw std::runtime_error("Advance_Op_DMRG: rotation does not match the operator");
        oi = csr_matmul(csr_matmul(csr_transpose(u), oi), u);
        oi = rgt ? csr_kron(csr_identity(dot.dim), oi) : csr_kron(oi, csr_identity(dot.dim));
    }
    *side = rgt ? 1 : 0;
    return oi;
}

int Driver::infinite() {
    while (left.length < p.ldmrg) {
        int rc = step(0, 0, 0);
        if (rc || stopped) return rc;
    }
    return NSS_OK;
}

// finite_DMRG (src/DMRG_MAIN.f90:168-241), OBC
int Driver::finite() {
    const int fN = 2 * p.ldmrg;
    std::vector<Block> lb(fN + 2), rb(fN + 2);
    lb[1] = left;
    rb[1] = right;
    while (left.length < p.ldmrg) {
        int rc = step(0, 0, 0);
        if (rc) return rc;
        lb[left.length] = left;
        rb[right.length] = right;
    }
    // the environment block of a step is loaded from the stored list; its
    // renormalised copy is only used when the sweep turns on it (the last
    // step of each half sweep) or when the run ends there
    const int nsw = (int)msweep.size();
    for (int im = 1; im <= nsw; ++im) {
        while (left.length < fN) {
            right = rb[fN - left.length];
            int rc = step(1, 1, im, left.length + 1 < fN ? 1 : 3);
            if (rc) return rc;
            lb[left.length] = left;
        }
        while (right.length < fN) {
            left = lb[fN - right.length];
            int rc = step(1, 2, im, right.length + 1 < fN ? 2 : 3);
            if (rc) return rc;
            rb[right.length] = right;
        }
        while (left.length <= p.ldmrg) {
            right = rb[fN - left.length];
            const bool last = left.length + 1 > p.ldmrg && im == nsw;
            int rc = step(1, 1, im, last ? 3 : 1);
            if (rc) return rc;
            lb[left.length] = left;
        }
    }
    return NSS_OK;
}

namespace {

// U (column-major m_block x m_s, dense) -> CSR, dropping exact zeros
Csr u_to_csr(const std::vector<double> &u, int nrow, int ncol) {
    Csr c;
    c.init(nrow, ncol);
    std::vector<std::vector<std::pair<int, double>>> rows(nrow);
    for (int j = 0; j < ncol; ++j)
        for (int i = 0; i < nrow; ++i) {
            double v = u[(size_t)j * nrow + i];
            if (v != 0.0) rows[i].push_back({j, v});
        }
    for (int i = 0; i < nrow; ++i) {
        for (auto &e : rows[i]) {
            c.col.push_back(e.first);
            c.val.push_back(e.second);
        }
        c.rowptr[i + 1] = (int)c.col.size();
    }
    return c;
}

// operators_renormalization (src/DMRG_RDM.f90:355-404): O <- U^T O U, and the
// new basis from the kept blocks' QNs (:244-251).
void renormalize(Block &blk, const Csr &u, const std::vector<Qn> &kept_qn) {
    const Csr ut = csr_transpose(u);
    for (auto &o : blk.ops) o.m = csr_matmul(csr_matmul(ut, o.m), u);
    blk.dim = u.ncol;
    blk.basis.clear();
    for (const Qn &q : kept_qn) blk.basis.insert(blk.basis.end(), q.begin(), q.end());
}

}  // namespace

int nss_solve_step(Ctx &c, const SbHost &sb, const nss_dmrg_params &p, int mstates, double estates, bool renorm, Block &left,
                   Block &right, nss_step_record &rec, int keep_sides) {
    const auto t_up = std::chrono::steady_clock::now();
    SbView v;
    sb_view(sb, v);
    int rc;
    {
        ServeLock g(c);   // a served request's device phases take turns with the others'
        rc = sb_upload(c, &v.desc, true);
    }
    if (rc) return rc;
    rec.host_phase_ms[2] = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_up).count();
    const int64_t n = sb.n();
    const int neigen = (int)std::min<int64_t>(n, p.lanc_neigen);
    const int nitermax = (int)std::min<int64_t>(n, p.lanc_niter);
    double ev[4] = {0, 0, 0, 0};
    int numop = 0;
    cudaEvent_t e0, e1, em;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventCreate(&em);
    cudaEventRecord(e0, c.stream);
    if (c.serve && p.precision == NSS_PREC_MIXED && neigen == 1) {
        // served: the solve joins the server's batch engine with the other requests'
        rc = serve_solve(c, nitermax, p.lanc_tolerance, p.seed, ev, &numop);
    } else {
        ServeLock g(c);
        rc = lanczos_eigh(c, neigen, nitermax, p.lanc_tolerance, p.seed, p.precision, ev, &numop);
    }
    if (rc) return rc;
    serve_count(c);
    ServeLock g_rdm(c);   // the RDM and the device renormalisation below
    cudaEventRecord(em, c.stream);
    nss_rdm_side side[2];
    // operator renormalisation: QN-block GEMMs on the device for blocks of
    // at least 256 states (below that the host's sparse products are as
    // fast as the transfers); env NSS_RENORM=host / device forces one
    const char *rh = std::getenv("NSS_RENORM");
    const bool force_host = rh && std::string(rh) == "host", force_dev = rh && std::string(rh) == "device";
    const bool dev_renorm =
        renorm && !force_host && (force_dev || std::max(sb.m_left, sb.m_right) >= 256);
    std::vector<double> u_l, u_r;
    std::vector<int32_t> k_l, k_r;
    // m_s is known only after the truncation kernel: size for the maximum
    // (the dense U only for the host renormalisation)
    const bool ren_l = renorm && (keep_sides & 1), ren_r = renorm && (keep_sides & 2);
    if (renorm && !dev_renorm) {
        if (ren_l) u_l.resize((size_t)sb.m_left * sb.m_left);
        if (ren_r) u_r.resize((size_t)sb.m_right * sb.m_right);
    }
    k_l.resize(sb.m_left);
    k_r.resize(sb.m_right);
    KeptLayout kl[2];
    rc = rdm_run(c, c.lz.evecs, mstates, estates, p.deg_evals_threshold, side, nullptr, nullptr,
                 ren_l ? k_l.data() : nullptr, ren_r ? k_r.data() : nullptr,
                 (ren_l && !dev_renorm) ? u_l.data() : nullptr, (ren_r && !dev_renorm) ? u_r.data() : nullptr,
                 dev_renorm ? kl : nullptr, renorm ? keep_sides : 3);
    if (rc) return rc;
    cudaEventRecord(e1, c.stream);
    cudaEventSynchronize(e1);
    float ms = 0.f, ms_e = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventElapsedTime(&ms_e, e0, em);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaEventDestroy(em);
    rec.ms_solve = ms;
    rec.ms_eigh = ms_e;
    for (int i = 0; i < 6; ++i) rec.rdm_phase_ms[i] = c.rdm_phase_ms[i];
    for (int i = 0; i < 4; ++i) rec.rdm_path_blocks[i] = c.rdm_path_blocks[i];
    rec.rdm_max_block = c.rdm_max_block;
    rec.rdm_own_blocks = c.rdm_own_blocks;
    rec.rdm_fallback_blocks = c.rdm_fallback_blocks;
    rec.numop = numop;
    for (int e = 0; e < 2; ++e) rec.energy[e] = (e < neigen) ? ev[e] / rec.current_l : 0.0;
    rec.entropy_left = side[0].entropy;
    rec.entropy_right = side[1].entropy;
    rec.sn_left = side[0].s_number;
    rec.sc_left = side[0].s_config;
    rec.sn_right = side[1].s_number;
    rec.sc_right = side[1].s_config;
    rec.m_left = left.dim;
    rec.m_right = right.dim;
    if (renorm) {
        std::vector<Qn> ql, qr;
        if (ren_l)
            for (int j = 0; j < side[0].m_s; ++j) ql.push_back(sb.qns[k_l[j]]);
        if (ren_r)
            for (int j = 0; j < side[1].m_s; ++j) {
                Qn q = sb.target;
                for (size_t t = 0; t < q.size(); ++t) q[t] -= sb.qns[k_r[j]][t];
                qr.push_back(q);
            }
        const auto t_r = std::chrono::steady_clock::now();
        for (double &x : c.renorm_phase_ms) x = 0.0;
        if (dev_renorm) {
            if (p.save_umat) {
                // put_omat(str(length), trRho) (src/DMRG_RDM.f90:225, :298)
                Csr ul, ur;
                if (ren_l) {
                    if ((rc = kept_u_csr(c, kl[0], left.dim, ul))) return rc;
                    left.omats.push_back(std::make_shared<const Csr>(std::move(ul)));
                }
                if (ren_r) {
                    if ((rc = kept_u_csr(c, kl[1], right.dim, ur))) return rc;
                    right.omats.push_back(std::make_shared<const Csr>(std::move(ur)));
                }
            }
            Block *bl[2] = {ren_l ? &left : nullptr, ren_r ? &right : nullptr};
            const std::vector<Qn> *kq[2] = {&ql, &qr};
            if ((rc = renorm_device(c, kl, bl, kq))) return rc;
            rec.nnz_u = 0;
            for (int s2 = 0; s2 < 2; ++s2)
                for (int j = 0; j < kl[s2].ms; ++j) rec.nnz_u += kl[s2].dims[kl[s2].q[j]];
        } else {
            Csr cul, cur;
            // the two blocks are independent (a thread pays off from ~10^4 entries)
            run_pair(
                [&] {
                    if (!ren_l) return;
                    cul = u_to_csr(u_l, sb.m_left, side[0].m_s);
                    renormalize(left, cul, ql);
                },
                [&] {
                    if (!ren_r) return;
                    cur = u_to_csr(u_r, sb.m_right, side[1].m_s);
                    renormalize(right, cur, qr);
                },
                (int64_t)sb.m_left * side[0].m_s + (int64_t)sb.m_right * side[1].m_s > 8000);
            rec.nnz_u = (ren_l ? cul.nnz() : 0) + (ren_r ? cur.nnz() : 0);
            if (p.save_umat) {
                if (ren_l) left.omats.push_back(std::make_shared<const Csr>(cul));
                if (ren_r) right.omats.push_back(std::make_shared<const Csr>(cur));
            }
        }
        rec.nnz_ops = 0;
        for (const auto &o : left.ops) rec.nnz_ops += o.m.nnz();
        for (const auto &o : right.ops) rec.nnz_ops += o.m.nnz();
        rec.ms_renorm = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_r).count();
        for (int i = 0; i < 3; ++i) rec.host_phase_ms[3 + i] = c.renorm_phase_ms[i];
        rec.trunc_left = side[0].trunc_err;
        rec.trunc_right = side[1].trunc_err;
        // a side not renormalised reports the dimension it would have had
        rec.m_left = ren_l ? left.dim : side[0].m_s;
        rec.m_right = ren_r ? right.dim : side[1].m_s;
    }
    return NSS_OK;
}

}  // namespace nss
