"""The tile tuner of the mixed path (tile_tune.cpp): per shape class of
superblock it plans the first uploads with each candidate (CUDA cores, tensor
cores with 64- and 128-column tiles), records the converged mixed solves'
device time per H*psi product, and then keeps the fastest.  Whatever the
plan, the energy is the FP64 one to 1e-10."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def nss():
    import nssdmrg_gb300 as nss
    nss.lib()
    return nss


def test_tuner_tries_each_candidate_then_keeps_the_fastest(nss, monkeypatch):
    monkeypatch.delenv("NSS_TC_MIN_DL", raising=False)
    monkeypatch.delenv("NSS_TC_AUTO", raising=False)
    # spin-1 chain L=32, m=256, last infinite step: sectors up to ~190 states
    d = nss.DMRG(nss.MODEL_HEISENBERG_ONE, 16, 256, dmrg_qn=(0.0, 0.0), lanc_neigen=1)
    d.prepare_last()
    desc = d.export_superblock()
    e64, _, _ = d.sb.sb_diag(neigen=1, tol=1e-12, want_vectors=False)
    nss.lib().nss_tune_reset()
    seen = []
    for visit in range(5):
        s = nss.Superblock()
        s.upload_desc(desc)
        cand, _, _ = s.tune_info()
        ev, _, _ = s.sb_diag(neigen=1, tol=1e-12, precision=nss.NSS_PREC_MIXED, want_vectors=False)
        assert abs(ev[0] - e64[0]) <= 1e-10 * abs(e64[0]), (cand, ev[0], e64[0])
        seen.append(cand)
        _, ms, n = s.tune_info()
        s.close()
    print("candidates", seen, "ms per H*psi", ms, "solves", n)
    assert seen[:3] == [0, 1, 2]
    best = int(np.argmin(ms))
    assert seen[3:] == [best, best]
    assert n == [1 + 2 * (best == 0), 1 + 2 * (best == 1), 1 + 2 * (best == 2)]


def test_small_sectors_stay_on_cuda_cores(nss, monkeypatch):
    """A superblock without a sector of 32 left states has one candidate."""
    monkeypatch.delenv("NSS_TC_MIN_DL", raising=False)
    monkeypatch.delenv("NSS_TC_AUTO", raising=False)
    d = nss.DMRG(nss.MODEL_HEISENBERG_HALF, 6, 16, dmrg_qn=(0.0, 0.0), lanc_neigen=1)
    d.prepare_last()
    desc = d.export_superblock()
    assert max(desc.dls[k] for k in range(desc.nsb)) < 32
    s = nss.Superblock()
    s.upload_desc(desc)
    assert s.tune_info()[0] == 0
