"""Batched ground-state solves (nss_eigh_batch): several superblocks, one
context each, advanced together by one persistent launch per group of
iterations.  Each result must equal that context's own solve within the
solver tolerance, alone or in the mix."""
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


def _fixture_sb(nss, name):
    z = load_npz(name)
    l, r = unpack_block("eleft", z), unpack_block("eright", z)
    sbo = O.sb_get_states(l, r, z["target"])
    ds = O.setup_direct(l, r, sbo, z["hij"])
    s = nss.Superblock()
    terms = [(t.it - 1, t.isb, t.jsb, t.hconj, t.A, t.B, t.row_offset, t.col_offset) for t in ds.terms]
    s.upload(sbo.Dls, sbo.Drs, sbo.Offset, ds.Hleft, ds.Hright, terms, ds.tNso, l.dim, r.dim, sbo.AI, sbo.BI)
    return s


@pytest.fixture(scope="module")
def superblocks(nss):
    sbs = [_fixture_sb(nss, n) for n in ("kat_spin.npz", "kat_hubbard.npz", "c2_small.npz")]
    # superblocks produced by the infinite algorithm (kept alive with their drivers)
    drivers = []
    for model, L2, m, u in ((nss.MODEL_HUBBARD, 8, 64, 2.0), (nss.MODEL_HUBBARD, 10, 96, 6.0),
                            (nss.MODEL_HEISENBERG_ONE, 8, 48, 0.0), (nss.MODEL_HEISENBERG_HALF, 12, 64, 0.0)):
        qn = (0.5, 0.5) if model == nss.MODEL_HUBBARD else (0.0,)
        d = nss.DMRG(model, L2, m, u=u, hfmode=False, dmrg_qn=qn, lanc_neigen=1)
        d.prepare_last()
        drivers.append(d)
        sbs.append(d.sb)
    return sbs, drivers


def test_batch_matches_single_solves(nss, superblocks):
    sbs, _ = superblocks
    single = []
    for s in sbs:
        ev, _, _ = s.sb_diag(neigen=1, tol=1e-12, want_vectors=False, precision=nss.NSS_PREC_MIXED)
        single.append(ev[0])
    ref64 = []
    for s in sbs:
        ev, _, _ = s.sb_diag(neigen=1, tol=1e-12, want_vectors=False)
        ref64.append(ev[0])
    eb, nops = nss.eigh_batch(sbs, tol=1e-12)
    single, ref64 = np.array(single), np.array(ref64)
    assert np.all(nops > 0)
    np.testing.assert_allclose(eb, single, rtol=1e-10, atol=0)
    np.testing.assert_allclose(eb, ref64, rtol=1e-10, atol=0)


def test_batch_leaves_ground_states_for_rdm(nss, superblocks):
    """After the batch, each context's RDM (from the batched ground state)
    matches the one after its own FP64 solve."""
    sbs, _ = superblocks
    s = sbs[-1]
    s.sb_diag(neigen=1, tol=1e-12, want_vectors=False)
    ref = s.sb_get_rdm(32, 0.1)
    nss.eigh_batch(sbs, tol=1e-12)
    got = s.sb_get_rdm(32, 0.1)
    assert got.m_s == ref.m_s
    assert abs(got.entropy[0] - ref.entropy[0]) <= 1e-8 * abs(ref.entropy[0])


def test_batch_one_and_repeat(nss, superblocks):
    """A batch of one, and the same batch twice (the state of the previous
    batch must not leak into the next)."""
    sbs, _ = superblocks
    e1, _ = nss.eigh_batch(sbs[:1], tol=1e-12)
    e2, _ = nss.eigh_batch(sbs[:1], tol=1e-12)
    ev, _, _ = sbs[0].sb_diag(neigen=1, tol=1e-12, want_vectors=False)
    np.testing.assert_allclose(e1, ev[:1], rtol=1e-10)
    np.testing.assert_allclose(e2, ev[:1], rtol=1e-10)


def test_continuous_batching(nss, superblocks):
    """Solves join the engine while others are in flight and leave when
    done; every result equals the context's own solve."""
    sbs, _ = superblocks
    ref = []
    for s in sbs:
        ev, _, _ = s.sb_diag(neigen=1, tol=1e-12, want_vectors=False)
        ref.append(ev[0])
    eng = nss.BatchEngine(sbs[0])
    ids = {}
    ids[eng.add(sbs[0], seed=11)] = 0
    ids[eng.add(sbs[3], seed=12)] = 3
    got = {}
    pending = [1, 2, 4, 5, 6]
    rounds = 0
    while eng.inflight or pending:
        if pending and rounds % 3 == 1:
            k = pending.pop(0)
            ids[eng.add(sbs[k], seed=20 + k)] = k
        for i, e, nop in eng.step():
            assert i > 0 and nop > 0
            got[ids[i]] = e
        rounds += 1
        assert rounds < 10000
    eng.close()
    assert sorted(got) == list(range(len(sbs)))
    for k, e in got.items():
        assert abs(e - ref[k]) <= 1e-10 * abs(ref[k]), (k, e, ref[k])
