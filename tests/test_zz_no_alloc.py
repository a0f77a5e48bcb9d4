"""The allocation-free energy entry point (nss_sb_energy_noalloc).

It exists for callers that cannot allocate device memory when they need the
energy of a state: its scratch is a static device array, so it must agree
with the ordinary path, H*psi through nss_hv followed by two dot products,
on consecutive calls that reuse that array.  Tolerance: FP64 sums in two
different orders, 1e-12 relative.  This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

from conftest import load_npz
from oracle import dmrg_oracle as O
from tests.golden.blockio import unpack_block

pytestmark = pytest.mark.gpu


def _superblock(nss, name):
    z = load_npz(name)
    l, r = unpack_block("eleft", z), unpack_block("eright", z)
    sb = O.sb_get_states(l, r, z["target"])
    ds = O.setup_direct(l, r, sb, z["hij"])
    s = nss.Superblock()
    terms = [(t.it - 1, t.isb, t.jsb, t.hconj, t.A, t.B, t.row_offset, t.col_offset) for t in ds.terms]
    s.upload(sb.Dls, sb.Drs, sb.Offset, ds.Hleft, ds.Hright, terms, ds.tNso, l.dim, r.dim, sb.AI, sb.BI)
    return s


@pytest.mark.parametrize("name", ["kat_hubbard.npz", "c2_small.npz"])
def test_energy_noalloc_matches_hv_path_twice(name):
    import torch
    import nssdmrg_gb300 as nss
    s = _superblock(nss, name)
    rng = np.random.default_rng(21)
    for call in range(2):
        psi = rng.standard_normal(s.n)
        ref = float(psi @ s.spmatvec(psi)) / float(psi @ psi)
        d_psi = torch.from_numpy(psi).cuda()
        e = s.energy_noalloc(d_psi.data_ptr())
        torch.cuda.synchronize()
        assert abs(e - ref) <= 1e-12 * abs(ref), (call, e, ref)


def test_energy_noalloc_rejects_bad_calls():
    """No superblock, a wrong length and a zero vector are refused with the
    library's status codes; nothing runs on the GPU for the first two."""
    import torch
    import nssdmrg_gb300 as nss
    empty = nss.Superblock()
    d = torch.ones(8, dtype=torch.float64, device="cuda")
    with pytest.raises(nss.NssError) as ei:
        empty.energy_noalloc(d.data_ptr())
    assert ei.value.code == nss.NSS_ERR_STATE
    s = _superblock(nss, "kat_spin.npz")
    L = nss.lib()
    e = ctypes.c_double()
    rc = L.nss_sb_energy_noalloc(s._ctx, s.n + 1, ctypes.c_void_p(d.data_ptr()), ctypes.byref(e))
    assert rc == nss.NSS_ERR_INVALID
    z = torch.zeros(s.n, dtype=torch.float64, device="cuda")
    with pytest.raises(nss.NssError) as ei:
        s.energy_noalloc(z.data_ptr())
    assert ei.value.code == nss.NSS_ERR_INVALID and "zero norm" in str(ei.value)


def test_energy_noalloc_two_contexts_one_device():
    """Two contexts on one device share the static array; used one after the
    other, each gets its own superblock's energy."""
    import torch
    import nssdmrg_gb300 as nss
    a = _superblock(nss, "kat_spin.npz")
    b = _superblock(nss, "kat_hubbard.npz")
    rng = np.random.default_rng(5)
    for _ in range(2):
        for s in (a, b):
            psi = rng.standard_normal(s.n)
            ref = float(psi @ s.spmatvec(psi)) / float(psi @ psi)
            e = s.energy_noalloc(torch.from_numpy(psi).cuda().data_ptr())
            assert abs(e - ref) <= 1e-12 * abs(ref), (e, ref)
