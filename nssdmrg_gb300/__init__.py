"""GB300-native superblock eigensolver for nssDMRG.

A thin Python view of the C ABI in ``include/nssdmrg.h`` (``libnssdmrg.so``,
built by ``nssdmrg_gb300.build``).  The names mirror the reference library's
Fortran procedures that the ABI replaces:

* ``Superblock.upload``      -- the operator pool of Setup_SuperBlock_Direct
* ``Superblock.setup``       -- sb_get_states + sb_build_dims + Setup_SuperBlock_Direct
* ``Superblock.spmatvec``    -- spMatVec_direct_main (the sparse_HxV callback)
* ``Superblock.sb_diag``     -- sb_diag's Lanczos branch (replaces sp_eigh)
* ``Superblock.sb_get_rdm``  -- sb_get_rdm + block eigh + truncation choice
* ``DMRG``                   -- init_dmrg / run_DMRG (infinite, finite)

There is no CPU fallback: every call goes to the CUDA library, and loading
fails loudly when the library is missing.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from pathlib import Path

import numpy as np

_HERE = Path(__file__).resolve().parent
LIB_PATH = _HERE / "libnssdmrg.so"

NSS_OK = 0
NSS_ERR_INVALID = -1
NSS_ERR_CUDA = -2
NSS_ERR_NOMEM = -3
NSS_ERR_STATE = -4
NSS_ERR_NOCONV = -5
NSS_ERR_ASYMMETRIC = -6
NSS_PREC_FP64 = 0
NSS_PREC_MIXED = 1
NSS_SITE_SPIN = 0
NSS_SITE_FERMION = 1
MODEL_HEISENBERG_HALF = 0
MODEL_HEISENBERG_ONE = 1
MODEL_HUBBARD = 2


class NssError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"nssdmrg error {code}: {msg}")
        self.code = code


class Csr(C.Structure):
    _fields_ = [("nrow", C.c_int32), ("ncol", C.c_int32), ("rowptr", C.POINTER(C.c_int32)),
                ("colidx", C.POINTER(C.c_int32)), ("vals", C.POINTER(C.c_double))]


class SbDesc(C.Structure):
    _fields_ = [("nsb", C.c_int32), ("tnso", C.c_int32), ("m_left", C.c_int32), ("m_right", C.c_int32),
                ("dls", C.POINTER(C.c_int32)), ("drs", C.POINTER(C.c_int32)), ("offset", C.POINTER(C.c_int64)),
                ("ai", C.POINTER(C.c_int32)), ("bi", C.POINTER(C.c_int32)),
                ("hleft", C.POINTER(Csr)), ("hright", C.POINTER(Csr)),
                ("a", C.POINTER(Csr)), ("b", C.POINTER(Csr)),
                ("isb2jsb", C.POINTER(C.c_int32)), ("ishconjg", C.POINTER(C.c_int32)),
                ("row_offset", C.POINTER(C.c_int64)), ("col_offset", C.POINTER(C.c_int64))]


class RdmSide(C.Structure):
    _fields_ = [("nevals", C.c_int32), ("m_s", C.c_int32), ("trunc_err", C.c_double), ("entropy", C.c_double),
                ("s_number", C.c_double), ("s_config", C.c_double)]


class BlockDesc(C.Structure):
    _fields_ = [("dim", C.c_int32), ("qdim", C.c_int32), ("basis", C.POINTER(C.c_double)),
                ("h", Csr), ("op", Csr * 3)]


class DmrgParams(C.Structure):
    _fields_ = [("model", C.c_int32), ("jz", C.c_double), ("jxy", C.c_double), ("t", C.c_double),
                ("u", C.c_double), ("hfmode", C.c_int32), ("dmrg_qn", C.c_double * 2), ("ldmrg", C.c_int32),
                ("mdmrg", C.c_int32), ("nsweep", C.c_int32), ("msweep", C.POINTER(C.c_int32)),
                ("lanc_neigen", C.c_int32), ("lanc_niter", C.c_int32), ("lanc_tolerance", C.c_double),
                ("deg_evals_threshold", C.c_double), ("seed", C.c_uint64), ("precision", C.c_int32),
                ("save_umat", C.c_int32), ("edmrg", C.c_double), ("esweep", C.POINTER(C.c_double))]


class Served(C.Structure):
    _fields_ = [("id", C.c_int32), ("status", C.c_int32), ("energy", C.c_double), ("wait_s", C.c_double),
                ("service_s", C.c_double), ("footprint_est", C.c_size_t), ("peak_bytes", C.c_size_t)]


class StepRecord(C.Structure):
    _fields_ = [("type", C.c_int32), ("left_length", C.c_int32), ("right_length", C.c_int32),
                ("current_l", C.c_int32), ("n", C.c_int64), ("nsb", C.c_int32), ("numop", C.c_int32),
                ("energy", C.c_double * 2), ("entropy_left", C.c_double), ("entropy_right", C.c_double),
                ("trunc_left", C.c_double), ("trunc_right", C.c_double), ("m_left", C.c_int32),
                ("m_right", C.c_int32), ("ms_solve", C.c_double), ("ms_eigh", C.c_double),
                ("ms_step", C.c_double), ("ms_build", C.c_double), ("ms_renorm", C.c_double),
                ("nnz_u", C.c_int64), ("nnz_ops", C.c_int64), ("rdm_own_blocks", C.c_int32),
                ("rdm_fallback_blocks", C.c_int32), ("sn_left", C.c_double), ("sc_left", C.c_double),
                ("sn_right", C.c_double), ("sc_right", C.c_double), ("rdm_phase_ms", C.c_double * 6),
                ("rdm_path_blocks", C.c_int32 * 4), ("rdm_max_block", C.c_int32),
                ("host_phase_ms", C.c_double * 6)]


_lib = None


def lib():
    """Load libnssdmrg.so (raises when it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise ImportError(f"{LIB_PATH} is missing: run nssdmrg_gb300.build.build() first "
                          "(there is no CPU fallback)")
    L = C.CDLL(str(LIB_PATH))
    P, I32, I64, D = C.c_void_p, C.c_int32, C.c_int64, C.c_double
    sig = {
        "nss_create": (P, [C.c_int, C.c_size_t]),
        "nss_destroy": (None, [P]),
        "nss_last_error": (C.c_char_p, [P]),
        "nss_sb_upload": (C.c_int, [P, C.POINTER(SbDesc)]),
        "nss_sb_free": (C.c_int, [P]),
        "nss_sb_dim": (I64, [P]),
        "nss_sb_shape": (C.c_int, [P, C.POINTER(I32), C.POINTER(I32), C.POINTER(I32), C.POINTER(I64)]),
        "nss_sb_flops": (C.c_int, [P, C.POINTER(D), C.POINTER(D)]),
        "nss_kernel_launches": (I64, [P]),
        "nss_sb_upload_bytes": (I64, [P]),
        "nss_stream": (P, [P]),
        "nss_hv": (C.c_int, [P, I64, P, P]),
        "nss_hv_device": (C.c_int, [P, I64, P, P]),
        "nss_hv_device_f32": (C.c_int, [P, I64, P, P]),
        "nss_sb_energy_noalloc": (C.c_int, [P, I64, P, C.POINTER(D)]),
        "nss_tridiag_lowest": (C.c_int, [C.c_int, P, P, C.c_int, D, P, P, P]),
        "nss_arrow_lowest": (C.c_int, [C.c_int, D, P, P, P, D, C.POINTER(D), P, C.POINTER(D)]),
        "nss_tridiag_eig": (C.c_int, [C.c_int, P, P, P, P]),
        "nss_restart_rewrite": (C.c_int, [C.c_char_p, C.c_char_p]),
        "nss_kron_sum": (C.c_int, [I32, I32, I32, P, C.POINTER(Csr), C.POINTER(Csr), C.c_int, I64,
                                   C.POINTER(I64), P, P, P]),
        "nss_eigh": (C.c_int, [P, C.c_int, C.c_int, C.c_int, D, C.c_uint64, C.c_int, P, P, C.POINTER(C.c_int)]),
        "nss_tune_info": (C.c_int, [P, C.POINTER(C.c_int), C.POINTER(C.c_double), C.POINTER(C.c_int)]),
        "nss_tune_reset": (None, []),
        "nss_server_create": (P, [C.c_int, C.c_size_t]),
        "nss_server_footprint": (C.c_size_t, [C.POINTER(DmrgParams)]),
        "nss_server_submit": (C.c_int, [P, C.POINTER(DmrgParams), C.POINTER(C.c_int)]),
        "nss_server_poll": (C.c_int, [P, C.c_int, C.POINTER(Served)]),
        "nss_server_stats": (C.c_int, [P, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_size_t),
                                       C.POINTER(C.c_size_t), C.POINTER(C.c_int64), C.POINTER(C.c_double)]),
        "nss_server_destroy": (None, [P]),
        "nss_server_solves": (C.c_int64, [P]),
        "nss_rdm": (C.c_int, [P, P, C.c_int, D, C.POINTER(RdmSide), P, P, P, P, P, P]),
        "nss_rdm_estates": (C.c_int, [P, P, C.c_int, D, D, C.POINTER(RdmSide), P, P, P, P, P, P]),
        "nss_eigh_batch": (C.c_int, [P, C.c_int, C.c_int, D, P, P, P]),
        "nss_time_chunks": (C.c_int, [P, C.c_int]),
        "nss_chunk_stats": (C.c_int, [P, C.POINTER(D), C.POINTER(C.c_int), C.POINTER(I64), C.POINTER(D)]),
        "nss_chunk_cache": (C.c_int, [P, C.POINTER(C.c_int), C.POINTER(I64)]),
        "nss_graph_stats": (C.c_int, [P, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
        "nss_batch_create": (P, [P]),
        "nss_batch_add": (C.c_int, [P, P, C.c_uint64, C.c_int, D, C.POINTER(C.c_int)]),
        "nss_batch_step": (C.c_int, [P, C.c_int, C.POINTER(C.c_int), P, P, P]),
        "nss_batch_inflight": (C.c_int, [P]),
        "nss_batch_destroy": (None, [P]),
        "nss_sb_setup": (C.c_int, [P, C.c_int, C.POINTER(BlockDesc), C.POINTER(BlockDesc), P, P]),
        "nss_sb_counts": (C.c_int, [P, C.POINTER(I32), C.POINTER(I32), C.POINTER(I64)]),
        "nss_sb_tables": (C.c_int, [P, P, P, P, P, P]),
        "nss_dmrg_create": (P, [P, C.POINTER(DmrgParams)]),
        "nss_dmrg_destroy": (None, [P]),
        "nss_dmrg_infinite": (C.c_int, [P]),
        "nss_dmrg_finite": (C.c_int, [P]),
        "nss_dmrg_prepare_last": (C.c_int, [P]),
        "nss_dmrg_export_superblock": (C.c_int, [P, C.POINTER(SbDesc)]),
        "nss_rdm_stats": (C.c_int, [P, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]),
        "nss_rdm_fallback_reasons": (C.c_int, [P, C.POINTER(C.c_int64)]),
        "nss_refine_stats": (C.c_int, [P, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int64)]),
        "nss_dmrg_nrecords": (C.c_int, [P]),
        "nss_dmrg_measure": (C.c_int, [P, C.POINTER(Csr), C.POINTER(C.c_int32), C.c_int, C.POINTER(C.c_double)]),
        "nss_dmrg_save_blocks": (C.c_int, [P, C.c_char_p, C.c_char_p]),
        "nss_dmrg_load_blocks": (C.c_int, [P, C.c_char_p, C.c_char_p]),
        "nss_odotv": (C.c_int, [P, C.c_char, C.POINTER(Csr), C.POINTER(C.c_double), C.POINTER(C.c_double)]),
        "nss_average_op": (C.c_int, [P, C.c_char, C.POINTER(Csr), C.POINTER(C.c_double), C.POINTER(C.c_double)]),
        "nss_dmrg_records": (C.c_int, [P, C.POINTER(StepRecord), C.c_int]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def _p(a: np.ndarray, t):
    return a.ctypes.data_as(C.POINTER(t))


def tridiag_lowest(a, b, ne: int = 1, b_last: float = 0.0):
    """Lowest `ne` eigenpairs of the symmetric tridiagonal matrix (diagonal a,
    off-diagonal b) with the host solver nss_eigh uses on the Lanczos matrix.
    Returns (theta[ne], s[ne, m], resid[ne]), resid = |b_last * s[:, -1]|."""
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    m = a.size
    theta = np.zeros(ne)
    s = np.zeros((ne, m))
    resid = np.zeros(ne)
    rc = lib().nss_tridiag_lowest(m, _ptr(a), _ptr(b) if b.size else None, ne, float(b_last), _ptr(theta),
                                  _ptr(s), _ptr(resid))
    if rc != 0:
        raise NssError(rc, lib().nss_last_error(None).decode())
    return theta, s, resid


def restart_rewrite(in_path, out_path):
    """Read a block restart file (older operator names included) and write it
    in the current layout; no GPU needed."""
    rc = lib().nss_restart_rewrite(str(in_path).encode(), str(out_path).encode())
    if rc:
        raise NssError(rc, lib().nss_last_error(None).decode())


def tridiag_eig(d, e):
    """All eigenpairs of a symmetric tridiagonal matrix (host implicit QL):
    (evals ascending, Z with Z[:, j] the eigenvector of evals[j])."""
    d = np.ascontiguousarray(d, np.float64)
    e = np.ascontiguousarray(e, np.float64)
    n = d.size
    ev = np.empty(n)
    Z = np.empty((n, n))   # filled column-major: Z.T[j] is column j
    rc = lib().nss_tridiag_eig(n, _ptr(d), _ptr(e) if n > 1 else None, _ptr(ev), _ptr(Z))
    if rc:
        raise NssError(rc, lib().nss_last_error(None).decode())
    return ev, Z.T.copy()


def kron_sum(terms, nthreads: int = 0):
    """sum_t coef_t * kron(A_t, B_t) on the host, as enlarge_block builds the
    enlarged H; terms = [(coef, A, B), ...] with scipy sparse A (na x na) and
    B (nb x nb).  Returns (indptr, indices, data) of the na*nb square CSR."""
    if not terms:
        raise ValueError("kron_sum: no terms")
    na, nb = terms[0][1].shape[0], terms[0][2].shape[0]
    keep = _Keep()
    coef = keep.arr([t[0] for t in terms], np.float64)
    ca = (Csr * len(terms))(*[keep.csr(t[1]) for t in terms])
    cb = (Csr * len(terms))(*[keep.csr(t[2]) for t in terms])
    nnz = C.c_int64()
    args = (na, nb, len(terms), _ptr(coef), ca, cb, nthreads)
    rc = lib().nss_kron_sum(*args, 0, C.byref(nnz), None, None, None)
    if rc:
        raise NssError(rc, lib().nss_last_error(None).decode())
    rp = np.empty(na * nb + 1, np.int32)
    ci = np.empty(nnz.value, np.int32)
    va = np.empty(nnz.value, np.float64)
    rc = lib().nss_kron_sum(*args, nnz.value, C.byref(nnz), _ptr(rp), _ptr(ci), _ptr(va))
    if rc:
        raise NssError(rc, lib().nss_last_error(None).decode())
    return rp, ci, va


def arrow_lowest(theta0: float, m, a, b, b_last: float = 0.0):
    """Lowest eigenpair of [[theta0, m^T], [m, tridiag(a, b)]] with the host
    solver of the mixed-precision refinement.  Returns (lam, c, resid)."""
    m = np.ascontiguousarray(m, dtype=np.float64)
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    k = a.size
    lam = C.c_double(0.0)
    res = C.c_double(0.0)
    c = np.zeros(k + 1)
    rc = lib().nss_arrow_lowest(k, float(theta0), _ptr(m) if k else None, _ptr(a) if k else None,
                                _ptr(b) if b.size else None, float(b_last), C.byref(lam), _ptr(c), C.byref(res))
    if rc != 0:
        raise NssError(rc, lib().nss_last_error(None).decode())
    return lam.value, c, res.value


def eigh_batch(superblocks, nitermax: int = 512, tol: float = 1e-12, seeds=None):
    """Ground states of several Superblocks (one context each) solved together
    by the batched persistent kernel (mixed precision).  Returns (energies,
    numops); each Superblock keeps its ground state for sb_get_rdm."""
    nb = len(superblocks)
    ctxs = (C.c_void_p * nb)(*[sb._ctx for sb in superblocks])
    sd = np.ascontiguousarray(seeds if seeds is not None else np.arange(1, nb + 1), dtype=np.uint64)
    ev = np.zeros(nb)
    nops = np.zeros(nb, dtype=np.int32)
    rc = lib().nss_eigh_batch(ctxs, nb, int(nitermax), float(tol), _ptr(sd), _ptr(ev), _ptr(nops))
    if rc != 0:
        raise NssError(rc, lib().nss_last_error(superblocks[0]._ctx).decode())
    return ev, nops


class BatchEngine:
    """Continuous batching of ground-state solves (mixed precision): add()
    a Superblock (its context must hold the superblock) between step()
    calls; each step() runs one round of the batched persistent kernel and
    returns the solves that finished: [(id, energy, numop)], id < 0 on
    failure."""

    def __init__(self, host: "Superblock"):
        self.host = host
        self._b = lib().nss_batch_create(host._ctx)
        if not self._b:
            raise NssError(NSS_ERR_INVALID, lib().nss_last_error(host._ctx).decode())

    def add(self, sb: "Superblock", seed: int = 1234, nitermax: int = 512, tol: float = 1e-12) -> int:
        i = C.c_int(0)
        rc = lib().nss_batch_add(self._b, sb._ctx, int(seed), int(nitermax), float(tol), C.byref(i))
        if rc != 0:
            raise NssError(rc, lib().nss_last_error(self.host._ctx).decode())
        return i.value

    def step(self, max_done: int = 256):
        nd = C.c_int(0)
        ids = np.zeros(max_done, dtype=np.int32)
        en = np.zeros(max_done)
        nops = np.zeros(max_done, dtype=np.int32)
        rc = lib().nss_batch_step(self._b, max_done, C.byref(nd), _ptr(ids), _ptr(en), _ptr(nops))
        if rc != 0:
            raise NssError(rc, lib().nss_last_error(self.host._ctx).decode())
        return [(int(ids[q]), float(en[q]), int(nops[q])) for q in range(nd.value)]

    @property
    def inflight(self) -> int:
        return lib().nss_batch_inflight(self._b)

    def close(self):
        if getattr(self, "_b", None):
            lib().nss_batch_destroy(self._b)
            self._b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class _Keep:
    """Keeps numpy buffers alive while a ctypes descriptor points at them."""

    def __init__(self):
        self.refs = []

    def arr(self, a, dtype):
        a = np.ascontiguousarray(a, dtype=dtype)
        self.refs.append(a)
        return a

    def csr(self, m) -> Csr:
        """scipy.sparse matrix (or None = absent block) -> nss_csr."""
        c = Csr()
        if m is None:
            c.nrow = 0
            c.ncol = 0
            return c
        m = m.tocsr()
        rp = self.arr(m.indptr, np.int32)
        ci = self.arr(m.indices, np.int32)
        va = self.arr(m.data, np.float64)
        c.nrow, c.ncol = m.shape
        c.rowptr = _p(rp, C.c_int32)
        c.colidx = _p(ci, C.c_int32)
        c.vals = _p(va, C.c_double)
        return c


@dataclass
class RdmResult:
    m_s: tuple
    trunc_err: tuple
    entropy: tuple
    lambdas: tuple       # descending eigenvalues, left and right
    kept_blocks: tuple   # rho block (= sector) of each kept state
    u: tuple             # rotation matrices [m_block x m_s]
    s_number: tuple = (0.0, 0.0)   # S_N per side (number entropy over QN blocks)
    s_config: tuple = (0.0, 0.0)   # S_c per side (configurational entropy)


class Superblock:
    """One GPU context holding one superblock (the reference's H*v pool)."""

    def __init__(self, device: int = 0, hbm_budget: int = 0):
        L = lib()
        self._ctx = L.nss_create(device, hbm_budget)
        if not self._ctx:
            raise NssError(NSS_ERR_CUDA, L.nss_last_error(None).decode())
        self._keep = None
        self.m_left = self.m_right = 0

    def close(self):
        if self._ctx:
            lib().nss_destroy(self._ctx)
            self._ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc != NSS_OK:
            raise NssError(rc, lib().nss_last_error(self._ctx).decode())

    @property
    def n(self) -> int:
        return int(lib().nss_sb_dim(self._ctx))

    # -- the operator pool as the reference keeps it (DMRG_GLOBAL.f90:119-124)
    def upload(self, dls, drs, offset, hleft, hright, terms, tnso, m_left, m_right, ai=None, bi=None):
        """terms: list of (it, k, jsb, hconj, A, B, row_offset, col_offset)
        with it 0-based; A/B scipy sparse matrices."""
        keep = _Keep()
        nsb = len(dls)
        d = SbDesc()
        d.nsb, d.tnso, d.m_left, d.m_right = nsb, tnso, m_left, m_right
        dl = keep.arr(dls, np.int32)
        dr = keep.arr(drs, np.int32)
        off = keep.arr(offset, np.int64)
        d.dls, d.drs, d.offset = _p(dl, C.c_int32), _p(dr, C.c_int32), _p(off, C.c_int64)
        if ai is not None:
            a_ = keep.arr(np.concatenate(ai), np.int32)
            b_ = keep.arr(np.concatenate(bi), np.int32)
            d.ai, d.bi = _p(a_, C.c_int32), _p(b_, C.c_int32)
        hl = (Csr * nsb)(*[keep.csr(h) for h in hleft])
        hr = (Csr * nsb)(*[keep.csr(h) for h in hright])
        nt = max(1, tnso * nsb)
        A = (Csr * nt)()
        B = (Csr * nt)()
        isb = np.full(nt, -1, np.int32)
        hc = np.zeros(nt, np.int32)
        ro = np.zeros(nt, np.int64)
        co = np.zeros(nt, np.int64)
        for (it, k, jsb, hconj, a, b, r_off, c_off) in terms:
            idx = it + tnso * k
            A[idx] = keep.csr(a)
            B[idx] = keep.csr(b)
            isb[idx], hc[idx], ro[idx], co[idx] = jsb, hconj, r_off, c_off
        keep.refs += [hl, hr, A, B]
        isb, hc, ro, co = (keep.arr(isb, np.int32), keep.arr(hc, np.int32), keep.arr(ro, np.int64),
                           keep.arr(co, np.int64))
        d.hleft = C.cast(hl, C.POINTER(Csr))
        d.hright = C.cast(hr, C.POINTER(Csr))
        d.a = C.cast(A, C.POINTER(Csr))
        d.b = C.cast(B, C.POINTER(Csr))
        d.isb2jsb, d.ishconjg = _p(isb, C.c_int32), _p(hc, C.c_int32)
        d.row_offset, d.col_offset = _p(ro, C.c_int64), _p(co, C.c_int64)
        self._check(lib().nss_sb_upload(self._ctx, C.byref(d)))
        self.m_left, self.m_right = m_left, m_right

    def time_chunks(self, enable: bool = True):
        """CUDA-event timing of the persistent Lanczos kernel in later solves."""
        self._check(lib().nss_time_chunks(self._ctx, int(enable)))

    def chunk_stats(self):
        """(ms, launches, iterations, sum of m) of the persistent kernel in
        the last solve (with time_chunks enabled)."""
        ms, nl, it, cols = C.c_double(), C.c_int(), C.c_int64(), C.c_double()
        self._check(lib().nss_chunk_stats(self._ctx, C.byref(ms), C.byref(nl), C.byref(it), C.byref(cols)))
        return ms.value, nl.value, it.value, cols.value

    def graph_stats(self):
        """(chunks replayed as CUDA graphs, graphs captured) in the last solve."""
        r, cpt = C.c_int(), C.c_int()
        self._check(lib().nss_graph_stats(self._ctx, C.byref(r), C.byref(cpt)))
        return r.value, cpt.value

    def chunk_cache(self):
        """(basis vectors cached per CTA, rows per CTA) of the persistent
        kernel's shared-memory row cache in this context's workspace."""
        vc, rows = C.c_int(), C.c_int64()
        self._check(lib().nss_chunk_cache(self._ctx, C.byref(vc), C.byref(rows)))
        return vc.value, rows.value

    def odotv(self, label, ops, v):
        """OdotV_direct: (O x 1) v for label 'l', (1 x O) v for 'r'; ops[k]
        is the block operator filtered to sector k's states (scipy sparse)."""
        keep = _Keep()
        arr = (Csr * len(ops))(*[keep.csr(m) for m in ops])
        v = keep.arr(v, np.float64)
        ov = np.empty_like(v)
        self._check(lib().nss_odotv(self._ctx, label.encode()[:1], arr, _p(v, C.c_double), _p(ov, C.c_double)))
        return ov

    def average_op(self, label, op, psi=None):
        """Average_Op_dmrg: <psi| O |psi> for a whole block operator O (scipy
        sparse, m_block x m_block) on side 'l' or 'r'; psi None = the ground
        state of the last sb_diag."""
        keep = _Keep()
        c = keep.csr(op)
        pp = _p(keep.arr(psi, np.float64), C.c_double) if psi is not None else None
        val = C.c_double()
        self._check(lib().nss_average_op(self._ctx, label.encode()[:1], C.byref(c), pp, C.byref(val)))
        return val.value

    def rdm_stats(self):
        """(own-eigensolver blocks, library blocks, own blocks recomputed by
        the library) of the last sb_get_rdm."""
        a, b, c = C.c_int(), C.c_int(), C.c_int()
        self._check(lib().nss_rdm_stats(self._ctx, C.byref(a), C.byref(b), C.byref(c)))
        return a.value, b.value, c.value

    def refine_stats(self):
        """(passes, cluster size, FP64 fallbacks so far) of the mixed
        method's refinement in the last sb_diag."""
        a, b, f = C.c_int(), C.c_int(), C.c_int64()
        self._check(lib().nss_refine_stats(self._ctx, C.byref(a), C.byref(b), C.byref(f)))
        return a.value, b.value, f.value

    def rdm_fallback_reasons(self):
        """Counts of own-path blocks sent back to the library, by reason:
        (not positive definite, gap < 32 eps, Rayleigh iteration unsettled,
        Gram-Schmidt remainder < 1/2, cluster too large)."""
        out = (C.c_int64 * 5)()
        self._check(lib().nss_rdm_fallback_reasons(self._ctx, out))
        return tuple(out)

    def upload_desc(self, desc: SbDesc):
        self._check(lib().nss_sb_upload(self._ctx, C.byref(desc)))
        self.m_left, self.m_right = desc.m_left, desc.m_right

    def setup(self, site_type, left, right, target, hij):
        """Block-level setup.  left/right: dicts with 'basis' [dim,qdim],
        'H' and the model operators (spin: S_z_n, S_p_n; fermion: C_l1_s1_n,
        C_l1_s2_n, P_n) as scipy sparse matrices."""
        keep = _Keep()

        def bd(blk):
            b = BlockDesc()
            basis = keep.arr(blk["basis"], np.float64)
            b.dim, b.qdim = basis.shape
            b.basis = _p(basis, C.c_double)
            b.h = keep.csr(blk["H"])
            keys = ("S_z_n", "S_p_n") if site_type == NSS_SITE_SPIN else ("C_l1_s1_n", "C_l1_s2_n", "P_n")
            for i, k in enumerate(keys):
                b.op[i] = keep.csr(blk[k])
            return b

        L, R = bd(left), bd(right)
        t = keep.arr(target, np.float64)
        h = keep.arr(np.asarray(hij, np.float64).reshape(-1), np.float64)
        self._check(lib().nss_sb_setup(self._ctx, site_type, C.byref(L), C.byref(R), _ptr(t), _ptr(h)))
        self.m_left, self.m_right = L.dim, R.dim

    def tables(self):
        """Sector tables of the last setup(): qns, Dls, Drs, Offset, sb_states."""
        L = lib()
        nsb, qdim, n = C.c_int32(), C.c_int32(), C.c_int64()
        self._check(L.nss_sb_counts(self._ctx, C.byref(nsb), C.byref(qdim), C.byref(n)))
        qns = np.zeros((nsb.value, qdim.value))
        dls = np.zeros(nsb.value, np.int32)
        drs = np.zeros(nsb.value, np.int32)
        off = np.zeros(nsb.value, np.int64)
        st = np.zeros(n.value, np.int64)
        self._check(L.nss_sb_tables(self._ctx, _ptr(qns), _ptr(dls), _ptr(drs), _ptr(off), _ptr(st)))
        return qns, dls, drs, off, st

    def shape(self):
        """(nsb, m_left, m_right, N) of the uploaded superblock, as the library holds it."""
        a, b, c, d = C.c_int32(), C.c_int32(), C.c_int32(), C.c_int64()
        self._check(lib().nss_sb_shape(self._ctx, C.byref(a), C.byref(b), C.byref(c), C.byref(d)))
        return a.value, b.value, c.value, d.value

    def flops(self):
        """(dense, ab) algorithmic FLOPs of one H*v."""
        d, a = C.c_double(), C.c_double()
        self._check(lib().nss_sb_flops(self._ctx, C.byref(d), C.byref(a)))
        return d.value, a.value

    @property
    def stream(self) -> int:
        """cudaStream_t of the context (for torch.cuda.ExternalStream)."""
        return int(lib().nss_stream(self._ctx) or 0)

    @property
    def upload_bytes(self) -> int:
        return int(lib().nss_sb_upload_bytes(self._ctx))

    @property
    def launches(self) -> int:
        return int(lib().nss_kernel_launches(self._ctx))

    def hv_device(self, d_v: int, d_hv: int):
        """H*v on device pointers (e.g. torch tensors' data_ptr())."""
        self._check(lib().nss_hv_device(self._ctx, self.n, C.c_void_p(d_v), C.c_void_p(d_hv)))

    def tune_info(self):
        """(candidate, ms per H*psi of candidates 0..2, solves of each) of the
        tile tuner for the uploaded superblock's shape class."""
        cand = C.c_int()
        ms = (C.c_double * 3)()
        n = (C.c_int * 3)()
        self._check(lib().nss_tune_info(self._ctx, C.byref(cand), ms, n))
        return cand.value, list(ms), list(n)

    def energy_noalloc(self, d_psi: int) -> float:
        """<psi|H|psi>/<psi|psi> of a device vector, allocating nothing (for
        callers that cannot allocate device memory at that point)."""
        e = C.c_double()
        self._check(lib().nss_sb_energy_noalloc(self._ctx, self.n, C.c_void_p(d_psi), C.byref(e)))
        return e.value

    def hv_device_f32(self, d_v: int, d_hv: int):
        """The mixed path's FP32 H*v on device pointers."""
        self._check(lib().nss_hv_device_f32(self._ctx, self.n, C.c_void_p(d_v), C.c_void_p(d_hv)))

    # -- sparse_HxV
    def spmatvec(self, v: np.ndarray) -> np.ndarray:
        v = np.ascontiguousarray(v, np.float64)
        hv = np.empty_like(v)
        self._check(lib().nss_hv(self._ctx, v.size, _ptr(v), _ptr(hv)))
        return hv

    def sb_diag(self, neigen=1, nitermax=512, tol=1e-12, seed=1234, precision=NSS_PREC_FP64,
                want_vectors=True, ncv=0):
        ev = np.zeros(max(1, neigen))
        n = self.n
        vec = np.zeros((max(1, neigen), n)) if want_vectors else None
        numop = C.c_int()
        self._check(lib().nss_eigh(self._ctx, neigen, nitermax, ncv, tol, seed, precision, _ptr(ev),
                                   _ptr(vec) if vec is not None else None, C.byref(numop)))
        ne = min(neigen, n)
        return ev[:ne], (vec[:ne].T if vec is not None else None), numop.value

    def sb_get_rdm(self, mstates, deg_thr=0.1, psi=None, want_u=True, estates=0.0) -> RdmResult:
        """sb_get_rdm + eigh + the truncation choice; mstates=0 with
        estates != 0 selects the error-threshold rule (Edmrg)."""
        out = (RdmSide * 2)()
        _, ml, mr, n = self.shape()     # output buffers sized from the uploaded superblock
        if psi is not None and np.asarray(psi).size != n:
            raise NssError(NSS_ERR_INVALID, "psi has the wrong length")
        lam_l, lam_r = np.zeros(ml), np.zeros(mr)
        kl, kr = np.zeros(ml, np.int32), np.zeros(mr, np.int32)
        ul = np.zeros(ml * ml) if want_u else None
        ur = np.zeros(mr * mr) if want_u else None
        p = np.ascontiguousarray(psi, np.float64) if psi is not None else None
        self._check(lib().nss_rdm_estates(self._ctx, _ptr(p) if p is not None else None, mstates, estates, deg_thr, out,
                                  _ptr(lam_l), _ptr(lam_r), _ptr(kl), _ptr(kr),
                                  _ptr(ul) if want_u else None, _ptr(ur) if want_u else None))
        ms = (out[0].m_s, out[1].m_s)
        us = (None, None)
        if want_u:
            us = (ul[: ml * ms[0]].reshape(ms[0], ml).T, ur[: mr * ms[1]].reshape(ms[1], mr).T)
        return RdmResult(ms, (out[0].trunc_err, out[1].trunc_err), (out[0].entropy, out[1].entropy),
                         (lam_l[: out[0].nevals], lam_r[: out[1].nevals]), (kl[: ms[0]], kr[: ms[1]]), us,
                         (out[0].s_number, out[1].s_number), (out[0].s_config, out[1].s_config))


def dmrg_params(model, ldmrg, mdmrg, msweep=(), jz=1.0, jxy=1.0, t=1.0, u=0.0, hfmode=True, dmrg_qn=(0.0, 0.0),
                lanc_neigen=1, lanc_niter=512, lanc_tolerance=1e-12, deg_evals_threshold=0.1, seed=1234,
                precision=NSS_PREC_FP64, save_umat=False, edmrg=0.0, esweep=()):
    """nss_dmrg_params (and the arrays it points to, which must outlive it)."""
    p = DmrgParams()
    p.model, p.jz, p.jxy, p.t, p.u, p.hfmode = model, jz, jxy, t, u, int(hfmode)
    p.dmrg_qn[0] = dmrg_qn[0]
    p.dmrg_qn[1] = dmrg_qn[1] if len(dmrg_qn) > 1 else 0.0
    p.ldmrg, p.mdmrg = ldmrg, mdmrg
    ms = np.ascontiguousarray(msweep, np.int32) if len(msweep) else np.zeros(1, np.int32)
    p.nsweep = len(msweep)
    p.msweep = _p(ms, C.c_int32)
    p.lanc_neigen, p.lanc_niter, p.lanc_tolerance = lanc_neigen, lanc_niter, lanc_tolerance
    p.deg_evals_threshold, p.seed, p.precision = deg_evals_threshold, seed, precision
    p.save_umat = int(save_umat)
    p.edmrg = edmrg
    es = np.ascontiguousarray(esweep, np.float64) if len(esweep) else None
    if es is not None:
        if len(es) != len(msweep):
            raise NssError(NSS_ERR_INVALID, "esweep needs one entry per sweep")
        p.esweep = _p(es, C.c_double)
    return p, ms, es


class Server:
    """Whole DMRG runs served as requests (nss_server_*): admission by HBM
    footprint, one worker context per running request, the mixed ground-state
    solves of all running requests batched in one engine."""

    def __init__(self, device: int = 0, hbm_budget: int = 0):
        self._s = lib().nss_server_create(device, hbm_budget)
        if not self._s:
            raise NssError(NSS_ERR_CUDA, lib().nss_last_error(None).decode())
        self._keep = {}

    @staticmethod
    def footprint(**kw) -> int:
        p, ms, es = dmrg_params(**kw)
        return int(lib().nss_server_footprint(C.byref(p)))

    def submit(self, **kw) -> int:
        """Queue one run (keyword arguments as for DMRG); returns its id."""
        p, ms, es = dmrg_params(**kw)
        rid = C.c_int()
        rc = lib().nss_server_submit(self._s, C.byref(p), C.byref(rid))
        if rc != NSS_OK:
            raise NssError(rc, "nss_server_submit: invalid request")
        return rid.value

    def poll(self, max_n: int = 256):
        out = (Served * max_n)()
        n = lib().nss_server_poll(self._s, max_n, out)
        return [{k: getattr(r, k) for k, _ in Served._fields_} for r in out[:max(n, 0)]]

    def stats(self):
        q, r, iu, pk, rounds, mb = C.c_int(), C.c_int(), C.c_size_t(), C.c_size_t(), C.c_int64(), C.c_double()
        lib().nss_server_stats(self._s, C.byref(q), C.byref(r), C.byref(iu), C.byref(pk), C.byref(rounds),
                               C.byref(mb))
        return {"queued": q.value, "running": r.value, "in_use": iu.value, "peak_in_use": pk.value,
                "rounds": rounds.value, "mean_batch": mb.value, "solves": int(lib().nss_server_solves(self._s))}

    def close(self):
        """Wait for every submitted request and release the server; its last
        counters stay in `last_stats`."""
        if self._s:
            self.last_stats = self.stats()
            lib().nss_server_destroy(self._s)
            self._s = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class DMRG:
    """init_dmrg / run_DMRG with every superblock solve on the GPU."""

    def __init__(self, model, ldmrg, mdmrg, msweep=(), jz=1.0, jxy=1.0, t=1.0, u=0.0, hfmode=True,
                 dmrg_qn=(0.0, 0.0), lanc_neigen=1, lanc_niter=512, lanc_tolerance=1e-12,
                 deg_evals_threshold=0.1, seed=1234, precision=NSS_PREC_FP64, device=0, sb=None,
                 save_umat=False, edmrg=0.0, esweep=()):
        self.sb = sb or Superblock(device)
        p, self._ms, self._es = dmrg_params(model, ldmrg, mdmrg, msweep, jz, jxy, t, u, hfmode, dmrg_qn, lanc_neigen,
                                            lanc_niter, lanc_tolerance, deg_evals_threshold, seed, precision,
                                            save_umat, edmrg, esweep)
        self._p = p
        self._d = lib().nss_dmrg_create(self.sb._ctx, C.byref(p))
        if not self._d:
            raise NssError(NSS_ERR_INVALID, lib().nss_last_error(self.sb._ctx).decode())

    def close(self):
        if getattr(self, "_d", None):
            lib().nss_dmrg_destroy(self._d)
            self._d = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def infinite(self):
        self.sb._check(lib().nss_dmrg_infinite(self._d))
        return self.records()

    def finite(self):
        self.sb._check(lib().nss_dmrg_finite(self._d))
        return self.records()

    def prepare_last(self):
        self.sb._check(lib().nss_dmrg_prepare_last(self._d))

    def save_blocks(self, left=None, right=None):
        """write_block of the current left / right block to restart files."""
        enc = lambda x: None if x is None else str(x).encode()
        self.sb._check(lib().nss_dmrg_save_blocks(self._d, enc(left), enc(right)))

    def load_blocks(self, left=None, right=None):
        """load_block: replace the current left / right block from restart
        files (the reference's own, older operator names included)."""
        enc = lambda x: None if x is None else str(x).encode()
        self.sb._check(lib().nss_dmrg_load_blocks(self._d, enc(left), enc(right)))

    def measure(self, op, pos):
        """Measure_DMRG for one site operator op (d x d, dense or scipy
        sparse, dot basis) at the 1-based chain positions pos, after a run
        with save_umat=True: <gs|O(pos)|gs> per position."""
        import scipy.sparse as sp
        keep = _Keep()
        c = keep.csr(sp.csr_matrix(np.asarray(op.todense() if hasattr(op, "todense") else op, np.float64)))
        pos = keep.arr(pos, np.int32)
        out = np.empty(len(pos))
        self.sb._check(lib().nss_dmrg_measure(self._d, C.byref(c), _p(pos, C.c_int32), len(pos),
                                              _p(out, C.c_double)))
        return out

    def export_superblock(self) -> SbDesc:
        d = SbDesc()
        self.sb._check(lib().nss_dmrg_export_superblock(self._d, C.byref(d)))
        return d

    def records(self):
        L = lib()
        n = L.nss_dmrg_nrecords(self._d)
        arr = (StepRecord * max(1, n))()
        L.nss_dmrg_records(self._d, arr, n)
        out = []
        for r in arr[:n]:
            out.append({k: (list(getattr(r, k)) if k in ("energy", "rdm_phase_ms", "rdm_path_blocks", "host_phase_ms") else getattr(r, k))
                        for k, _ in StepRecord._fields_})
        return out
