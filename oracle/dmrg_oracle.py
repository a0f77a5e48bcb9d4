"""numpy/scipy restatement of the nssDMRG superblock path (oracle; test only).

Every function names the reference routine it follows (paths relative to the
reference project root).  Indices are 0-based here; the reference is 1-based.
The restatement keeps the reference's ordering rules exactly, because sector
order, offsets and state maps must match bit-for-bit:

* a sector list is ordered by first occurrence of each QN tuple in the basis,
  and each map is the ascending list of basis positions with that QN
  (src/LIST/LIST_SECTORS.f90:174-217, src/LIST/QN_TUPLE_BASIS.f90:305-322);
* QN tuples are float64 and compared with exact equality
  (src/LIST/LIST_SECTORS.f90:192);
* the enlarged basis of a left block is ``outsum(self, dot)`` and of a right
  block ``outsum(dot, self)`` (src/DMRG_CONNECT.f90:253-264,
  src/LIST/QN_TUPLE_BASIS.f90:371-394).

Third-party arithmetic that the reference takes from SciFortran (not in the
reference tree, unpinned version): ``sp_eigh`` (ARPACK Lanczos) is restated by
``scipy.sparse.linalg.eigsh`` (ARPACK) or a dense LAPACK ``eigh`` below the
Lanczos threshold; the block ``eigh`` (LAPACK dsyev family) by
``numpy.linalg.eigh``; ``sort_quicksort`` by a stable ascending sort followed by
a reversal.  Tie order among exactly equal RDM eigenvalues is therefore a
documented choice, not a pinned one.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

TINY = np.finfo(np.float64).tiny  # Fortran tiny(1d0)


# ----------------------------------------------------------------------------
# Parameters (src/INPUT_VARS.f90 defaults; test drivers override some)
# ----------------------------------------------------------------------------
@dataclass
class Params:
    Ldmrg: int = 10
    Mdmrg: int = 64
    Msweep: tuple = ()
    Edmrg: float = 0.0                 # INPUT_VARS.f90:18, used when Mdmrg == 0
    Esweep: tuple = ()                 # :35, default Edmrg per sweep
    dmrg_qn: tuple = (0.0,)            # DMRG_QN, QNtype=local
    norb: int = 1
    lanc_neigen: int = 2               # INPUT_VARS.f90:275
    lanc_ncv_factor: int = 10          # :277
    lanc_ncv_add: int = 0              # :279
    lanc_niter: int = 512              # :281
    lanc_tolerance: float = 1e-12      # :285
    lanc_dim_threshold: int = 1024     # :287
    deg_evals_threshold: float = 0.1   # :260
    seed: int = 1234

    @property
    def fNlat(self):
        return 2 * self.Ldmrg


def csr(a):
    return sp.csr_matrix(np.asarray(a, dtype=np.float64))


def eye(n):
    return sp.identity(n, dtype=np.float64, format="csr")


def kron(a, b):
    """sp_kron_matrix (src/MATRIX/MATRIX_SPARSE.f90:832-876): row index
    (i-1)*B.Nrow+k, column (j-1)*B.Ncol+l -- the standard Kronecker order."""
    return sp.kron(a, b, format="csr")


# ----------------------------------------------------------------------------
# Sector lists (src/LIST/LIST_SECTORS.f90)
# ----------------------------------------------------------------------------
class Sectors:
    """sectors_list: QN tuples in first-occurrence order, ascending maps."""

    def __init__(self, basis: np.ndarray):
        basis = np.asarray(basis, dtype=np.float64)
        self.qns: list[tuple] = []
        maps: dict[tuple, list] = {}
        for i, row in enumerate(basis):
            q = tuple(float(x) for x in row)
            if q not in maps:
                maps[q] = []
                self.qns.append(q)
            maps[q].append(i)
        self.maps = {q: np.asarray(v, dtype=np.int64) for q, v in maps.items()}

    def has(self, q) -> bool:
        return tuple(float(x) for x in q) in self.maps

    def map(self, q) -> np.ndarray:
        return self.maps[tuple(float(x) for x in q)]

    def index(self, q) -> int:
        return self.qns.index(tuple(float(x) for x in q))

    def __len__(self):
        return len(self.qns)


# ----------------------------------------------------------------------------
# Sites and blocks (src/BLOCKS/SITES.f90, src/BLOCKS/BLOCKS.f90)
# ----------------------------------------------------------------------------
@dataclass
class Block:
    length: int
    dim: int
    sitetype: str                      # "spin" | "fermion"
    basis: np.ndarray                  # [dim, qdim] float64 QN per state
    ops: dict = field(default_factory=dict)   # key -> (csr, type), ordered
    # omatrices (src/BLOCKS/BLOCKS.f90:21): omats[i] is the rotation of the
    # block of length i+1; a site block starts with its identity (:140-142)
    omats: list = field(default_factory=list)

    def op(self, key):
        return self.ops[key][0]

    def copy(self):
        return Block(self.length, self.dim, self.sitetype, self.basis.copy(),
                     {k: (v[0].copy(), v[1]) for k, v in self.ops.items()}, list(self.omats))

    def sectors(self) -> Sectors:
        return Sectors(self.basis)


def spin_site(sun: int = 2, hvec=(0.0, 0.0)) -> Block:
    """spin_site (src/BLOCKS/SITES.f90:281-350): Sz, S+ and a field term."""
    if sun == 2:
        sz = np.diag([0.5, -0.5])
        spl = np.array([[0.0, 1.0], [0.0, 0.0]])
        h = hvec[0] * np.array([[0.0, 1.0], [1.0, 0.0]]) + hvec[1] * np.diag([1.0, -1.0])
        qn = [[0.5], [-0.5]]
    elif sun == 3:
        sz = np.diag([1.0, 0.0, -1.0])
        spl = np.zeros((3, 3))
        spl[0, 1] = spl[1, 2] = math.sqrt(2.0)
        sx = np.array([[0, 1, 0], [1, 0, 1], [0, 1, 0]], dtype=float) / math.sqrt(2.0)
        h = hvec[0] * sx + hvec[1] * sz
        qn = [[1.0], [0.0], [-1.0]]
    else:
        raise ValueError("spin_site: SU(N) value not supported")
    d = sz.shape[0]
    ops = {"H": (csr(h), "bosonic"), "S_z_n": (csr(sz), "bosonic"),
           "S_p_n": (csr(spl), "bosonic")}
    return Block(1, d, "spin", np.array(qn, dtype=np.float64), ops)


def electron_site(uloc: float = 0.0, hfmode: bool = True, hloc=None) -> Block:
    """electron_site with Norb=1 (src/BLOCKS/SITES.f90:358-450).

    Fock index m = iup + 2*idw (src/FOCK/HLOCAL.f90:229-238); basis QN
    [nup, ndw] in the same order (Build_BasisStates :735-757); local H from
    build_Hlocal_operator :312-433 (HF shift -U/2 (n_up+n_dw) when hfmode);
    C operators with the Jordan-Wigner sign of c() :884-896; P = (-1)^N
    (Build_FermionicSign :768-781).
    """
    hloc = np.zeros((2, 2)) if hloc is None else np.asarray(hloc, float)
    nup = np.array([0, 1, 0, 1])
    ndw = np.array([0, 0, 1, 1])
    diag = hloc[0, 0] * nup + hloc[1, 1] * ndw + uloc * nup * ndw
    if hfmode:
        diag = diag - 0.5 * uloc * (nup + ndw)
    h = np.diag(diag.astype(float))

    def c_op(alfa):  # alfa: bit position 0 (up) or 1 (dw)
        c = np.zeros((4, 4))
        for m in range(4):
            if not (m >> alfa) & 1:
                continue
            sgn = 1.0
            for l in range(alfa):
                if (m >> l) & 1:
                    sgn = -sgn
            c[m & ~(1 << alfa), m] = sgn
        return c

    p = np.diag([(-1.0) ** (nup[m] + ndw[m]) for m in range(4)])
    ops = {"H": (csr(h), "bosonic"),
           "C_l1_s1_n": (csr(c_op(0)), "fermionic"),
           "C_l1_s2_n": (csr(c_op(1)), "fermionic"),
           "P_n": (csr(p), "psign")}
    basis = np.stack([nup, ndw], axis=1).astype(np.float64)
    return Block(1, 4, "fermion", basis, ops)


# ----------------------------------------------------------------------------
# Block enlargement and block-block coupling (src/DMRG_CONNECT.f90)
# ----------------------------------------------------------------------------
def connect_spin_blocks(left: Block, right: Block, hij) -> sp.csr_matrix:
    """connect_spin_blocks (src/DMRG_CONNECT.f90:394-454), link 'n'."""
    szl, spl = left.op("S_z_n"), left.op("S_p_n")
    szr, spr = right.op("S_z_n"), right.op("S_p_n")
    return (hij[0, 0] * kron(szl, szr) + hij[1, 1] * kron(spl, spr.T.tocsr())
            + hij[1, 1] * kron(spl.T.tocsr(), spr))


def c_key(iorb, ispin):
    """'C'//okey(iorb,ispin,ilink='n') (src/AUX_FUNCS.f90:68-117)."""
    return f"C_l{iorb}_s{ispin}_n"


def connect_fermion_blocks(left: Block, right: Block, hij, norb=1) -> sp.csr_matrix:
    """connect_fermion_blocks (src/DMRG_CONNECT.f90:296-389), real case:
    sum_ab H(a,b) [(C_La^+ P_L) x C_Rb + (P_L C_La) x C_Rb^+]."""
    nso = 2 * norb
    cl, cr = {}, {}
    for ispin in (1, 2):
        for iorb in range(1, norb + 1):
            io = iorb + (ispin - 1) * norb
            cl[io] = left.op(c_key(iorb, ispin))
            cr[io] = right.op(c_key(iorb, ispin))
    pl = left.op("P_n")
    h2 = sp.csr_matrix((left.dim * right.dim, left.dim * right.dim))
    for io in range(1, nso + 1):
        for jo in range(1, nso + 1):
            t = hij[io - 1, jo - 1]
            if t == 0.0:
                continue
            h2 = h2 + t * kron((cl[io].T @ pl).tocsr(), cr[jo])
            h2 = h2 + t * kron((pl @ cl[io]).tocsr(), cr[jo].T.tocsr())
    return h2.tocsr()


def connect(left, right, hij, norb=1):
    if left.sitetype == "spin":
        return connect_spin_blocks(left, right, hij)
    return connect_fermion_blocks(left, right, hij, norb)


def enlarge_block(blk: Block, dot: Block, label: str, hij, norb=1) -> Block:
    """enlarge_block with link 'n' (src/DMRG_CONNECT.f90:18-291).

    H is rebuilt first from the old operators; the other operators are then
    enlarged in list order, reading the sign operator P from the list as it
    is being updated (exactly as the reference loop :117-146 does)."""
    m, d = blk.dim, dot.dim
    out = blk.copy()
    if label == "l":
        hb = kron(blk.op("H"), eye(d))
        hd = kron(eye(m), dot.op("H"))
        h2 = connect(blk, dot, hij, norb)
    else:
        hb = kron(eye(d), blk.op("H"))
        hd = kron(dot.op("H"), eye(m))
        h2 = connect(dot, blk, hij, norb)
    out.ops["H"] = ((hb + hd + h2).tocsr(), "bosonic")
    for key in list(blk.ops.keys()):
        if key == "H":
            continue
        otype = out.ops[key][1][0].lower()
        if otype not in ("b", "f", "p"):
            raise ValueError("enlarge_block: wrong operator type")
        if label == "l":
            eo = eye(m) if otype == "b" else out.ops["P_n"][0]
            new = kron(eo, dot.op(key))
        else:
            eo = out.ops["P_n"][0] if otype == "p" else eye(m)
            new = kron(dot.op(key), eo)
        out.ops[key] = (new.tocsr(), out.ops[key][1])
    out.length = blk.length + 1
    out.dim = m * d
    if label == "l":
        out.basis = outsum(blk.basis, dot.basis)
    else:
        out.basis = outsum(dot.basis, blk.basis)
    return out


def outsum(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """outsum_tbasis (src/LIST/QN_TUPLE_BASIS.f90:371-394): io=j+(i-1)*Nb."""
    return (a[:, None, :] + b[None, :, :]).reshape(a.shape[0] * b.shape[0], -1)


# ----------------------------------------------------------------------------
# Superblock enumeration and dims (src/DMRG_SUPERBLOCK.f90)
# ----------------------------------------------------------------------------
@dataclass
class Superblock:
    target: np.ndarray          # current_target_QN
    sb_states: np.ndarray       # 0-based l*rDim + r, in superblock order
    qns: list                   # sb_sector QN (left QN) per sector, in order
    maps: list                  # sb_sector map (0-based positions) per sector
    Dls: np.ndarray
    Drs: np.ndarray
    Offset: np.ndarray
    AI: list                    # left states per sector (sorted)
    BI: list                    # right states per sector (sorted)

    @property
    def N(self):
        return int(self.sb_states.size)


def current_target_qn(p: Params, current_L: int) -> np.ndarray:
    """sb_set_current_qn, QNtype local (src/DMRG_SUPERBLOCK.f90:717-726):
    int(target_qn*current_L*Norb), Fortran int() truncating toward zero."""
    return np.trunc(np.asarray(p.dmrg_qn, dtype=np.float64) * current_L * p.norb)


def sb_get_states(left: Block, right: Block, target) -> Superblock:
    """sb_get_states (src/DMRG_SUPERBLOCK.f90:167-283) + sb_build_dims
    (:36-121) + sb2block_states (src/DMRG_SUPERBLOCK_SETUP.f90:1079-1122)."""
    lsec, rsec = left.sectors(), right.sectors()
    rdim = right.dim
    target = np.asarray(target, dtype=np.float64)
    states, qns, maps, dls, drs, ai, bi = [], [], [], [], [], [], []
    pos = 0
    for lqn in lsec.qns:
        rqn = target - np.asarray(lqn)
        if not rsec.has(rqn):
            continue
        lmap, rmap = lsec.map(lqn), rsec.map(rqn)
        blk = (rmap[None, :] + lmap[:, None] * rdim).reshape(-1)
        states.append(blk)
        qns.append(lqn)
        maps.append(np.arange(pos, pos + blk.size))
        pos += blk.size
        dls.append(lmap.size)
        drs.append(rmap.size)
        ai.append(lmap)
        bi.append(rmap)
    if pos == 0:
        raise RuntimeError("sb_get_states ERROR: total_states=0")
    dls = np.asarray(dls, np.int64)
    drs = np.asarray(drs, np.int64)
    off = np.concatenate([[0], np.cumsum(dls * drs)[:-1]]).astype(np.int64)
    return Superblock(target, np.concatenate(states), qns, maps, dls, drs, off, ai, bi)


# ----------------------------------------------------------------------------
# Direct-mode setup (src/DMRG_SUPERBLOCK_SETUP.f90:152-693)
# ----------------------------------------------------------------------------
@dataclass
class Term:
    it: int          # 1-based term index within the sector (tMap)
    isb: int         # sector whose loop creates the term (0-based)
    jsb: int         # isb2jsb
    hconj: int       # IsHconjg
    A: sp.csr_matrix
    B: sp.csr_matrix
    row_offset: int
    col_offset: int


@dataclass
class DirectSetup:
    sb: Superblock
    Hleft: list
    Hright: list
    terms: list      # flat list, ordered by (isb, it) as the reference loops
    tNso: int


def _filt(a, rows, cols):
    """sp_filter_matrix_1/2 (src/MATRIX/MATRIX_SPARSE.f90:478-628)."""
    return a[rows][:, cols].tocsr()


def setup_direct(left: Block, right: Block, sb: Superblock, hij, norb=1) -> DirectSetup:
    hl, hr = left.op("H"), right.op("H")
    hleft = [_filt(hl, sb.AI[k], sb.AI[k]) for k in range(len(sb.qns))]
    hright = [_filt(hr, sb.BI[k], sb.BI[k]) for k in range(len(sb.qns))]
    index = {q: k for k, q in enumerate(sb.qns)}
    terms = []
    if left.sitetype == "spin":
        # Setup_SuperBlock_Spin_Direct :152-405 (OBC: tNso=3)
        tnso = 3
        szl, spl = left.op("S_z_n"), left.op("S_p_n")
        szr, spr = right.op("S_z_n"), right.op("S_p_n")
        for isb, qn in enumerate(sb.qns):
            ai, bi, off = sb.AI[isb], sb.BI[isb], int(sb.Offset[isb])
            terms.append(Term(1, isb, isb, 0, hij[0, 0] * _filt(szl, ai, ai),
                              _filt(szr, bi, bi), off, off))
            qm = tuple(float(x) for x in np.asarray(qn) - 1.0)
            if qm not in index:
                continue
            jsb = index[qm]
            aj, bj, offj = sb.AI[jsb], sb.BI[jsb], int(sb.Offset[jsb])
            a2 = (hij[1, 1] * _filt(spl, ai, aj)).tocsr()
            b2 = _filt(spr.T.tocsr(), bi, bj)
            terms.append(Term(2, isb, jsb, 0, a2, b2, off, offj))
            terms.append(Term(3, isb, jsb, 1, a2.T.tocsr(), b2.T.tocsr(), offj, off))
    else:
        # Setup_SuperBlock_Fermion_Direct :416-693 (OBC: fbc=2)
        nso = 2 * norb
        tmap, it = {}, 0
        for i in (1, 2):
            for io in range(1, nso + 1):
                for jo in range(1, nso + 1):
                    if hij[io - 1, jo - 1] == 0.0:
                        continue
                    it += 1
                    tmap[(i, io, jo)] = it
        tnso = it
        pl = left.op("P_n")
        cl = {}
        cr = {}
        for ispin in (1, 2):
            for iorb in range(1, norb + 1):
                io = iorb + (ispin - 1) * norb
                cl[io] = (left.op(c_key(iorb, ispin)).T @ pl).tocsr()
                cr[io] = right.op(c_key(iorb, ispin))
        qnup = np.array([1.0, 0.0])
        qndw = np.array([0.0, 1.0])
        for isb, qn in enumerate(sb.qns):
            ai, bi, off = sb.AI[isb], sb.BI[isb], int(sb.Offset[isb])
            for ispin in (1, 2):
                dq = qnup if ispin == 1 else qndw
                qm = tuple(float(x) for x in np.asarray(qn) - dq)
                if qm not in index:
                    continue
                jsb = index[qm]
                aj, bj, offj = sb.AI[jsb], sb.BI[jsb], int(sb.Offset[jsb])
                for iorb in range(1, norb + 1):
                    for jorb in range(1, norb + 1):
                        io = iorb + (ispin - 1) * norb
                        jo = jorb + (ispin - 1) * norb
                        if hij[io - 1, jo - 1] == 0.0:
                            continue
                        a1 = (hij[io - 1, jo - 1] * _filt(cl[io], ai, aj)).tocsr()
                        b1 = _filt(cr[jo], bi, bj)
                        terms.append(Term(tmap[(1, io, jo)], isb, jsb, 0, a1, b1, off, offj))
                        terms.append(Term(tmap[(2, io, jo)], isb, jsb, 1,
                                          a1.T.tocsr(), b1.T.tocsr(), offj, off))
        terms.sort(key=lambda t: (t.isb, t.it))
    return DirectSetup(sb, hleft, hright, terms, tnso)


# ----------------------------------------------------------------------------
# The direct matvec (src/DMRG_SUPERBLOCK_SETUP.f90:740-865)
# ----------------------------------------------------------------------------
def spmatvec_direct(ds: DirectSetup, v: np.ndarray) -> np.ndarray:
    """spMatVec_direct_main, vectorised.

    Sector k of v is Psi_k[Dr_k x Dl_k] column-major (i = ir + il*Dr + off),
    i.e. the row-major array W_k[il, ir].  Then
      1_L x H_R : W <- W + W H_R^T        (:767-779)
      H_L x 1_R : W <- W + H_L W          (:784-796)
      A x B     : W_row += A W_col B^T    (:808-857, W_col at ColOffset)
    """
    sb = ds.sb
    hv = np.zeros_like(v)
    for k in range(len(sb.qns)):
        dl, dr, off = int(sb.Dls[k]), int(sb.Drs[k]), int(sb.Offset[k])
        w = v[off:off + dl * dr].reshape(dl, dr)
        out = (ds.Hright[k] @ w.T).T + ds.Hleft[k] @ w
        hv[off:off + dl * dr] += out.reshape(-1)
    for t in ds.terms:
        na, ma = t.A.shape
        nb, mb = t.B.shape
        wq = v[t.col_offset:t.col_offset + ma * mb].reshape(ma, mb)
        out = t.A @ (t.B @ wq.T).T                     # [na, nb]
        hv[t.row_offset:t.row_offset + na * nb] += np.asarray(out).reshape(-1)
    return hv


def spmatvec_direct_loops(ds: DirectSetup, v: np.ndarray) -> np.ndarray:
    """spMatVec_direct_main in the reference loop order (pure Python; only
    for small cases -- the C restatement in spmatvec_ref.c is the fast one)."""
    sb = ds.sb
    hv = np.zeros_like(v)
    for k in range(len(sb.qns)):
        dl, dr, off = int(sb.Dls[k]), int(sb.Drs[k]), int(sb.Offset[k])
        hr, hl = ds.Hright[k], ds.Hleft[k]
        for il in range(dl):
            for ir in range(dr):
                i = ir + il * dr + off
                for jj in range(hr.indptr[ir], hr.indptr[ir + 1]):
                    hv[i] += hr.data[jj] * v[hr.indices[jj] + il * dr + off]
        for ir in range(dr):
            for il in range(dl):
                i = ir + il * dr + off
                for jj in range(hl.indptr[il], hl.indptr[il + 1]):
                    hv[i] += hl.data[jj] * v[ir + hl.indices[jj] * dr + off]
        for t in [t for t in ds.terms if t.isb == k]:
            A, B = t.A, t.B
            C = np.zeros((B.shape[0], A.shape[1]))
            for aj in range(A.shape[1]):
                for bi in range(B.shape[0]):
                    for jb in range(B.indptr[bi], B.indptr[bi + 1]):
                        C[bi, aj] += B.data[jb] * v[B.indices[jb] + aj * B.shape[1] + t.col_offset]
            for bi in range(B.shape[0]):
                for ai in range(A.shape[0]):
                    i = bi + ai * B.shape[0] + t.row_offset
                    for ja in range(A.indptr[ai], A.indptr[ai + 1]):
                        hv[i] += A.data[ja] * C[bi, A.indices[ja]]
    return hv


def sparse_superblock_h(left: Block, right: Block, sb: Superblock, hij, norb=1):
    """Setup_SuperBlock_Sparse (src/DMRG_SUPERBLOCK_SETUP.f90:46-88): the
    superblock H restricted to sb_states, built independently of the
    direct setup (used for the dense path and as a cross-check)."""
    h2 = connect(left, right, hij, norb)
    full = (h2 + kron(left.op("H"), eye(right.dim)) + kron(eye(left.dim), right.op("H"))).tocsr()
    s = sb.sb_states
    return full[s][:, s].tocsr()


# ----------------------------------------------------------------------------
# Eigensolve (src/DMRG_SUPERBLOCK.f90:335-474)
# ----------------------------------------------------------------------------
def sb_diag(left, right, sb, ds, p: Params, hij, norb=1, rng=None):
    m_sb = sb.N
    neigen = min(m_sb, p.lanc_neigen)
    nitermax = min(m_sb, p.lanc_niter)
    nblock = min(m_sb, p.lanc_ncv_factor * p.lanc_neigen + p.lanc_ncv_add)
    lanc = not (neigen == m_sb or m_sb <= p.lanc_dim_threshold)
    if lanc:
        rng = np.random.default_rng(p.seed) if rng is None else rng
        v0 = rng.uniform(-1.0, 1.0, m_sb)
        op = spla.LinearOperator((m_sb, m_sb), matvec=lambda x: spmatvec_direct(ds, x),
                                 dtype=np.float64)
        ncv = max(nblock, neigen + 1)
        ev, evec = spla.eigsh(op, k=neigen, which="SA", ncv=min(ncv, m_sb - 1), v0=v0,
                              tol=p.lanc_tolerance, maxiter=max(nitermax, 10 * m_sb))
        order = np.argsort(ev)
        return ev[order], evec[:, order], "lanczos"
    h = sparse_superblock_h(left, right, sb, hij, norb).toarray()
    ev, evec = np.linalg.eigh(h)
    return ev[:neigen], evec[:, :neigen], "dense"


# ----------------------------------------------------------------------------
# Reduced density matrices (src/DMRG_RDM.f90, src/MATRIX/MATRIX_BLOCKS.f90)
# ----------------------------------------------------------------------------
@dataclass
class RhoBlocks:
    qns: list          # per block QN
    maps: list         # per block: block-state indices (ascending)
    evals: list        # per block eigenvalues (eigh order, tiny-clamped)
    evecs: list        # per block eigenvectors (columns)
    evalues: np.ndarray   # all eigenvalues, descending
    eorder: np.ndarray    # 0-based global position (block-concatenated) per rank

    def find(self, pos):
        acc = 0
        for q, e in enumerate(self.evals):
            if pos < acc + e.size:
                return q, pos - acc
            acc += e.size
        raise IndexError(pos)


def build_density_matrices(sb: Superblock, psi: np.ndarray, lsec: Sectors, rsec: Sectors):
    """sb_get_rdm + build_density_matrix (src/DMRG_RDM.f90:18-162):
    Psi[il, ir] = psi(map(ir + il*Nr)); rho_L = Psi Psi^T, rho_R = Psi^T Psi.
    Blocks are appended in sb_sector order (left: QN q, right: target - q)."""
    left, right = [], []
    for k, q in enumerate(sb.qns):
        nl, nr = int(sb.Dls[k]), int(sb.Drs[k])
        w = psi[sb.maps[k]].reshape(nl, nr)
        rl = w @ w.T
        rr = w.T @ w
        rq = tuple(float(x) for x in sb.target - np.asarray(q))
        left.append((q, lsec.map(q), rl))
        right.append((rq, rsec.map(rq), rr))
    return left, right


def eigh_blocks(blocks) -> RhoBlocks:
    """eigh_blocks_matrix (src/MATRIX/MATRIX_BLOCKS.f90:589-657) with the
    defaults QNtruncation_error=0, QNtruncation_dim=1: per-block LAPACK eigh,
    negative eigenvalues -> tiny(1d0), ascending sort then reversal."""
    qns, maps, evals, evecs = [], [], [], []
    for q, m, rho in blocks:
        e, u = np.linalg.eigh(rho)
        e = np.where(e < 0.0, TINY, e)
        qns.append(q)
        maps.append(m)
        evals.append(e)
        evecs.append(u)
    allv = np.concatenate(evals)
    order = np.argsort(allv, kind="stable")
    evalues = allv[order][::-1].copy()
    eorder = order[::-1].copy()
    return RhoBlocks(qns, maps, evals, evecs, evalues, eorder)


def truncation(rho: RhoBlocks, mstates: int, m_block: int, deg_thr: float, estates: float = 0.0):
    """renormalize_block selection (src/DMRG_RDM.f90:204-221): m_s=min(M,m,#λ)
    when Mstates != 0, else (Estates != 0) the first minimum of
    |1 - cumulate(λ)(i) - Estates| (:206-208, cumulate_D in
    src/AUX_FUNCS.f90:133-143: running sums left to right); then extended
    over every later λ within deg_thr (relative) of λ(m_s); truncation error
    1 - sum(λ(1:m_s)).  λ<0 clipped to 0 (:88,:97)."""
    lam = np.where(rho.evalues < 0.0, 0.0, rho.evalues)
    if mstates != 0:
        m_s = min(mstates, m_block, lam.size)
    elif estates != 0.0:
        m_s = int(np.argmin(np.abs(1.0 - np.cumsum(lam) - estates))) + 1
    else:
        raise ValueError("Mdmrg=Edmrg=0 can not fix a threshold for the RDM")
    e_ = lam[m_s - 1]
    ext = 0
    with np.errstate(divide="ignore", invalid="ignore"):
        for i in range(m_s, lam.size):
            if abs(e_ - lam[i]) / e_ <= deg_thr:
                ext += 1
    m_s += ext
    eps = 1.0 - float(np.sum(lam[:m_s]))
    return m_s, eps


def rotation_matrix(rho: RhoBlocks, n: int, m: int) -> sp.csr_matrix:
    """sparse_blocks_matrix (src/MATRIX/MATRIX_BLOCKS.f90:556-576): column j is
    the eigenvector of rank j scattered onto its block map."""
    rows, cols, vals = [], [], []
    for j in range(m):
        q, pos = rho.find(int(rho.eorder[j]))
        vec = rho.evecs[q][:, pos]
        rows.append(rho.maps[q])
        cols.append(np.full(vec.size, j))
        vals.append(vec)
    return sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                         shape=(n, m))


def kept_qns(rho: RhoBlocks, m: int) -> np.ndarray:
    """rho%qn(m=im) for im=1..m_s (src/DMRG_RDM.f90:244-251)."""
    return np.array([rho.qns[rho.find(int(rho.eorder[j]))[0]] for j in range(m)],
                    dtype=np.float64)


def renormalize(blk: Block, u: sp.csr_matrix, qns: np.ndarray) -> Block:
    """operators_renormalization (src/DMRG_RDM.f90:355-404): O <- U^T O U;
    the rotation is stored as put_omat(str(length), trRho) does (:225, :298)."""
    out = blk.copy()
    ut = u.T.tocsr()
    for key, (o, t) in blk.ops.items():
        out.ops[key] = ((ut @ o @ u).tocsr(), t)
    out.dim = u.shape[1]
    out.basis = np.asarray(qns, dtype=np.float64).reshape(out.dim, -1)
    out.omats = list(blk.omats) + [u.tocsr()]
    return out


def odotv_direct(ops, v, label, sb: "Superblock"):
    """OdotV_direct (src/DMRG_MEASURE.f90:653-705), loop for loop: ops[k] is
    the block operator filtered to sector k's left ('l') or right ('r')
    states; sector k of v is Psi[il, ir] at ir + il*Drs + Offset (0-based)."""
    ov = np.zeros_like(v)
    for k in range(len(sb.Dls)):
        dl, dr, off = int(sb.Dls[k]), int(sb.Drs[k]), int(sb.Offset[k])
        o = sp.csr_matrix(ops[k])
        if label == "l":
            for ir in range(dr):
                for il in range(dl):
                    i = ir + il * dr + off
                    for p in range(o.indptr[il], o.indptr[il + 1]):
                        ov[i] += o.data[p] * v[ir + o.indices[p] * dr + off]
        else:
            for il in range(dl):
                for ir in range(dr):
                    i = ir + il * dr + off
                    for p in range(o.indptr[ir], o.indptr[ir + 1]):
                        ov[i] += o.data[p] * v[o.indices[p] + il * dr + off]
    return ov


def odotv_vectorised(ops, v, label, sb: "Superblock"):
    """The same product per sector as a matrix product (O Psi or Psi O^T)."""
    ov = np.zeros_like(v)
    for k in range(len(sb.Dls)):
        dl, dr, off = int(sb.Dls[k]), int(sb.Drs[k]), int(sb.Offset[k])
        psi = v[off:off + dl * dr].reshape(dl, dr)
        o = sp.csr_matrix(ops[k])
        ov[off:off + dl * dr] = (o @ psi if label == "l" else (o @ psi.T).T).ravel()
    return ov


def filter_sectors(oi, label, sb: "Superblock"):
    """sp_filter(Oi, LI(isb)%states) / RI per sector (src/DMRG_MEASURE.f90:617-625)."""
    oi = sp.csr_matrix(oi)
    maps = sb.AI if label == "l" else sb.BI
    return [oi[np.asarray(m)][:, np.asarray(m)].tocsr() for m in maps]


def average_op(oi, label, sb: "Superblock", psi):
    """Average_Op_dmrg (src/DMRG_MEASURE.f90:595-646): psi . OdotV(filtered Oi)."""
    return float(np.dot(psi, odotv_vectorised(filter_sectors(oi, label, sb), psi, label, sb)))


def entropy(lam: np.ndarray) -> float:
    """write_entanglement (src/DMRG_MAIN.f90:511-518): -sum λ log(λ+1e-32)."""
    lam = np.where(lam < 0.0, 0.0, lam)
    return float(-np.sum(lam * np.log(lam + 1e-32)))


def qn_entropies(rho: RhoBlocks) -> tuple[float, float]:
    """write_entanglement (src/DMRG_MAIN.f90:523-561): the entropy split over
    the QN blocks of rho, P_q = sum of block q's (tiny-clamped) eigenvalues,
    S_q = sum_i (l_i/P_q) log(l_i/P_q + 1e-32); returns
    S_N = -sum_q P_q log(P_q + 1e-32) and S_c = -sum_q P_q S_q."""
    sn = sc = 0.0
    for e in rho.evals:
        p = float(np.sum(e))
        with np.errstate(divide="ignore", invalid="ignore"):
            o = e / p
            sq = float(np.sum(o * np.log(o + 1e-32)))
        sn -= p * np.log(p + 1e-32)
        sc -= p * sq
    return float(sn), float(sc)


# ----------------------------------------------------------------------------
# DMRG driver (src/DMRG_MAIN.f90)
# ----------------------------------------------------------------------------
@dataclass
class StepRecord:
    kind: str
    left_length: int
    right_length: int
    current_L: int
    N: int
    nsb: int
    energies: np.ndarray     # gs_energy / current_L / Norb
    gs_energy: np.ndarray    # raw eigenvalues
    solver: str
    entropy_left: float
    entropy_right: float
    trunc_left: float = 0.0
    trunc_right: float = 0.0
    m_left: int = 0
    m_right: int = 0


class DMRG:
    """init_dmrg / infinite_DMRG / finite_DMRG / step_dmrg
    (src/DMRG_MAIN.f90:22-72, :140-159, :168-241, :262-433), OBC only."""

    def __init__(self, hij, dot: Block, p: Params, left: Block | None = None,
                 right: Block | None = None, keep_setups=False):
        self.hij = np.asarray(hij, dtype=np.float64)
        self.dot = dot
        self.p = p
        if not dot.omats:
            dot.omats = [sp.identity(dot.dim, format="csr")]
        self.left = (left or dot).copy()
        self.right = (right or dot).copy()
        self.records: list[StepRecord] = []
        self.keep_setups = keep_setups
        self.setups = []
        self.rng = np.random.default_rng(p.seed)

    def step(self, kind="i", label=0, sweep=None):
        p = self.p
        if kind == "i":
            mstates, estates = p.Mdmrg, p.Edmrg
        else:
            mstates = (p.Msweep or (p.Mdmrg,))[sweep - 1]
            estates = (p.Esweep or (p.Edmrg,) * max(1, len(p.Msweep)))[sweep - 1]
        m_left0, m_right0 = self.left.dim, self.right.dim
        self.left = enlarge_block(self.left, self.dot, "l", self.hij, p.norb)
        self.right = enlarge_block(self.right, self.dot, "r", self.hij, p.norb)
        current_L = self.left.length + self.right.length
        target = current_target_qn(p, current_L)
        sb = sb_get_states(self.left, self.right, target)
        ds = setup_direct(self.left, self.right, sb, self.hij, p.norb)
        ev, evec, solver = sb_diag(self.left, self.right, sb, ds, p, self.hij, p.norb, self.rng)
        if self.keep_setups:
            self.setups.append((self.left.copy(), self.right.copy(), sb, ds, ev, evec))
        self.last_sb, self.last_psi = sb, evec[:, 0].copy()
        lsec, rsec = self.left.sectors(), self.right.sectors()
        lblocks, rblocks = build_density_matrices(sb, evec[:, 0], lsec, rsec)
        rho_l, rho_r = eigh_blocks(lblocks), eigh_blocks(rblocks)
        if kind == "i":
            renorm = self.left.length != p.Ldmrg
        else:
            renorm = not (self.left.length == p.Ldmrg + 1 and label == 1)
        rec = StepRecord(kind, self.left.length, self.right.length, current_L, sb.N,
                         len(sb.qns), ev / current_L / p.norb, ev, solver,
                         entropy(rho_l.evalues), entropy(rho_r.evalues))
        rec.m_left, rec.m_right = self.left.dim, self.right.dim
        if renorm:
            for side in ("l", "r"):
                blk = self.left if side == "l" else self.right
                rho = rho_l if side == "l" else rho_r
                m_s, eps = truncation(rho, mstates, blk.dim, p.deg_evals_threshold, estates)
                u = rotation_matrix(rho, blk.dim, m_s)
                nb = renormalize(blk, u, kept_qns(rho, m_s))
                if side == "l":
                    self.left, rec.trunc_left, rec.m_left = nb, eps, m_s
                else:
                    self.right, rec.trunc_right, rec.m_right = nb, eps, m_s
        self.records.append(rec)
        return rec

    def site_op(self, op, pos):
        """Build_Op_dmrg + Advance_Op_dmrg, OBC (src/DMRG_MEASURE.f90:288-486):
        the site operator op at chain position pos (1-based) on the last
        step's enlarged block holding it; returns (operator, 'l' | 'r')."""
        L, R = self.left.length, self.right.length
        n = L + R
        if pos < 1 or pos > n:
            raise ValueError("Build_op_dmrg error: Pos not in [1,Ldmrg]")
        label = "r" if pos > L else "l"
        blk = self.right if label == "r" else self.left
        i = n + 1 - pos if label == "r" else pos
        iend = (R if label == "r" else L) - 1
        d = self.dot.dim
        oi = sp.csr_matrix(op)
        if i > 1:
            big_d = blk.omats[i - 2].shape[1]
            oi = kron(oi, eye(big_d)) if label == "r" else kron(eye(big_d), oi)
        for it in range(i, iend + 1):
            u = blk.omats[it - 1]
            oi = (u.T @ oi @ u).tocsr()
            oi = kron(eye(d), oi) if label == "r" else kron(oi, eye(d))
        return oi, label

    def measure(self, op, positions):
        """Measure_DMRG_scalar (src/DMRG_MEASURE.f90:172-220) in the ground
        state of the last step."""
        sb, psi = self.last_sb, self.last_psi
        out = []
        for pos in positions:
            oi, label = self.site_op(op, pos)
            out.append(average_op(oi, label, sb, psi))
        return np.array(out)

    def infinite(self):
        while self.left.length < self.p.Ldmrg:
            self.step("i")

    def finite(self):
        p = self.p
        fN = p.fNlat
        blocks = {1: {1: self.left.copy()}, 2: {1: self.right.copy()}}
        while self.left.length < p.Ldmrg:
            self.step("i")
            blocks[1][self.left.length] = self.left.copy()
            blocks[2][self.right.length] = self.right.copy()
        for im in range(1, len(p.Msweep) + 1):
            while self.left.length < fN:
                self.right = blocks[2][fN - self.left.length].copy()
                self.step("f", 1, im)
                blocks[1][self.left.length] = self.left.copy()
            while self.right.length < fN:
                self.left = blocks[1][fN - self.right.length].copy()
                self.step("f", 2, im)
                blocks[2][self.right.length] = self.right.copy()
            while self.left.length <= p.Ldmrg:
                self.right = blocks[2][fN - self.left.length].copy()
                self.step("f", 1, im)
                blocks[1][self.left.length] = self.left.copy()


# ----------------------------------------------------------------------------
# Model presets used by the reference's test drivers
# ----------------------------------------------------------------------------
def heisenberg_hij(jz=1.0, jxy=1.0):
    """Hlr = diag([Jp, Jx/2]) (test/src/Spin1d_SU2/spinSU2_1d.f90:236)."""
    return np.diag([jz, jxy / 2.0])


def hubbard_hij(t=1.0):
    """Hlr = diag([ts, ts]) with ts = -t (test/src/Hubbard1d/hm_1d.f90:104)."""
    return np.diag([-t, -t])
