"""Uploads back to back on one context.

An upload copies the operator pool to the device from a pinned staging
buffer with an asynchronous copy; the next upload reuses that buffer.  Two
uploads with no solve between them, of different superblocks and of
different sizes, must leave the context holding exactly the last one: its
ground-state energy equals the oracle's.
"""
import numpy as np
import pytest

from conftest import load_npz
from oracle import dmrg_oracle as O
from tests.golden.blockio import unpack_block

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def nss():
    import nssdmrg_gb300 as nss
    nss.lib()
    return nss


def _desc(name):
    z = load_npz(name)
    l, r = unpack_block("eleft", z), unpack_block("eright", z)
    sb = O.sb_get_states(l, r, z["target"])
    ds = O.setup_direct(l, r, sb, z["hij"])
    terms = [(t.it - 1, t.isb, t.jsb, t.hconj, t.A, t.B, t.row_offset, t.col_offset) for t in ds.terms]
    args = (ds.sb.Dls, ds.sb.Drs, ds.sb.Offset, ds.Hleft, ds.Hright, terms, ds.tNso, l.dim, r.dim, ds.sb.AI,
            ds.sb.BI)
    return args, z["oracle_gs_energy"][0]


def test_back_to_back_uploads_keep_the_last(nss):
    small, e_small = _desc("kat_spin.npz")
    big, e_big = _desc("c2_small.npz")
    s = nss.Superblock()
    for first, (last, e_last) in ((small, (big, e_big)), (big, (small, e_small)), (big, (big, e_big))):
        s.upload(*first)
        s.upload(*last)
        ev, _, _ = s.sb_diag(neigen=1, tol=1e-12, want_vectors=False)
        np.testing.assert_allclose(ev[0], e_last, rtol=1e-10, atol=0)
    s.close()
