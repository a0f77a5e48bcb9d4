"""ctypes view of the oracle's C restatement (libnss_oracle.so).

Test infrastructure and the timed CPU baseline only.  Defines its own
mirror of the nss_sb_desc layout of include/nssdmrg.h so that the oracle
does not depend on the shipped package.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB = Path(__file__).resolve().parent / "libnss_oracle.so"


class _Csr(C.Structure):
    _fields_ = [("nrow", C.c_int32), ("ncol", C.c_int32), ("rowptr", C.c_void_p),
                ("colidx", C.c_void_p), ("vals", C.c_void_p)]


class _Desc(C.Structure):
    _fields_ = [("nsb", C.c_int32), ("tnso", C.c_int32), ("m_left", C.c_int32), ("m_right", C.c_int32),
                ("dls", C.c_void_p), ("drs", C.c_void_p), ("offset", C.c_void_p), ("ai", C.c_void_p),
                ("bi", C.c_void_p), ("hleft", C.c_void_p), ("hright", C.c_void_p), ("a", C.c_void_p),
                ("b", C.c_void_p), ("isb2jsb", C.c_void_p), ("ishconjg", C.c_void_p),
                ("row_offset", C.c_void_p), ("col_offset", C.c_void_p)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not LIB.exists():
            from . import build
            build.build()
        L = C.CDLL(str(LIB))
        L.ref_hv_serial.argtypes = [C.POINTER(_Desc), C.c_void_p, C.c_void_p]
        L.ref_hv_omp.argtypes = [C.POINTER(_Desc), C.c_void_p, C.c_void_p, C.c_int]
        L.ref_lanczos.argtypes = [C.POINTER(_Desc), C.c_int, C.c_int, C.c_double, C.c_uint64, C.c_int,
                                  C.c_void_p, C.POINTER(C.c_int)]
        L.ref_lanczos.restype = C.c_int
        L.ref_lanczos_vec.argtypes = [C.POINTER(_Desc), C.c_int, C.c_int, C.c_double, C.c_uint64, C.c_int,
                                      C.c_void_p, C.c_void_p, C.POINTER(C.c_int)]
        L.ref_lanczos_vec.restype = C.c_int
        L.ref_max_threads.restype = C.c_int
        _lib = L
    return _lib


class RefSuperblock:
    """Holds a C descriptor built from an oracle DirectSetup (or from raw
    descriptor pointers of another library, see from_desc)."""

    def __init__(self, ds=None, m_left=0, m_right=0):
        self._keep = []
        self.desc = _Desc()
        if ds is not None:
            self._from_setup(ds, m_left, m_right)

    def _arr(self, a, dt):
        a = np.ascontiguousarray(a, dtype=dt)
        self._keep.append(a)
        return a.ctypes.data

    def _csr(self, m):
        c = _Csr()
        if m is None:
            return c
        m = m.tocsr()
        c.nrow, c.ncol = m.shape
        c.rowptr = self._arr(m.indptr, np.int32)
        c.colidx = self._arr(m.indices, np.int32)
        c.vals = self._arr(m.data, np.float64)
        return c

    def _from_setup(self, ds, m_left, m_right):
        sb = ds.sb
        nsb, tnso = len(sb.qns), ds.tNso
        d = self.desc
        d.nsb, d.tnso, d.m_left, d.m_right = nsb, tnso, m_left, m_right
        d.dls = self._arr(sb.Dls, np.int32)
        d.drs = self._arr(sb.Drs, np.int32)
        d.offset = self._arr(sb.Offset, np.int64)
        hl = (_Csr * nsb)(*[self._csr(h) for h in ds.Hleft])
        hr = (_Csr * nsb)(*[self._csr(h) for h in ds.Hright])
        nt = max(1, nsb * tnso)
        A, B = (_Csr * nt)(), (_Csr * nt)()
        ro, co = np.zeros(nt, np.int64), np.zeros(nt, np.int64)
        for t in ds.terms:
            idx = (t.it - 1) + tnso * t.isb
            A[idx], B[idx] = self._csr(t.A), self._csr(t.B)
            ro[idx], co[idx] = t.row_offset, t.col_offset
        self._keep += [hl, hr, A, B]
        d.hleft, d.hright = C.addressof(hl), C.addressof(hr)
        d.a, d.b = C.addressof(A), C.addressof(B)
        d.row_offset = self._arr(ro, np.int64)
        d.col_offset = self._arr(co, np.int64)
        self.n = int(np.sum(np.asarray(sb.Dls, np.int64) * np.asarray(sb.Drs, np.int64)))

    @classmethod
    def from_desc_struct(cls, desc, n):
        """Wrap a descriptor struct with the same layout owned by someone else."""
        self = cls()
        C.memmove(C.byref(self.desc), C.byref(desc), C.sizeof(_Desc))
        self.n = n
        return self

    def hv(self, v, nthreads=1):
        v = np.ascontiguousarray(v, np.float64)
        out = np.empty_like(v)
        if nthreads > 1:
            lib().ref_hv_omp(C.byref(self.desc), v.ctypes.data, out.ctypes.data, nthreads)
        else:
            lib().ref_hv_serial(C.byref(self.desc), v.ctypes.data, out.ctypes.data)
        return out

    def lanczos(self, neigen=1, nitermax=512, tol=1e-12, seed=1234, nthreads=1):
        ev = np.zeros(max(1, neigen))
        numop = C.c_int()
        rc = lib().ref_lanczos(C.byref(self.desc), neigen, nitermax, tol, seed, nthreads, ev.ctypes.data,
                               C.byref(numop))
        return ev[:neigen], numop.value, rc

    def lanczos_vectors(self, neigen=1, nitermax=512, tol=1e-12, seed=1234, nthreads=1):
        """As lanczos, plus the unit Ritz vectors as the columns of an n x neigen array."""
        ev = np.zeros(max(1, neigen))
        vec = np.zeros((max(1, neigen), self.n))
        numop = C.c_int()
        rc = lib().ref_lanczos_vec(C.byref(self.desc), neigen, nitermax, tol, seed, nthreads, ev.ctypes.data,
                                   vec.ctypes.data, C.byref(numop))
        return ev[:neigen], vec[:neigen].T.copy(), numop.value, rc
