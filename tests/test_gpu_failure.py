"""Failure paths, exercised without a GPU fault.

* A bounded device wait that runs out: env NSS_WAIT_LIMIT shortens the poll
  limit of every grid barrier (a test knob), so the cooperative Lanczos
  kernels and the whole-GPU tridiagonalisation give up at their first wait.
  The kernels return (no trap), the entry point reports NSS_ERR_CUDA with
  the reason, and the same context then solves correctly.
* A context over its HBM budget: NSS_ERR_NOMEM, and the context stays usable
  once the budget allows.
* Too few iterations: NSS_ERR_NOCONV.
* A NaN in an uploaded operator: refused with NSS_ERR_INVALID.
"""
import numpy as np
import pytest
import scipy.sparse as sp

from conftest import load_npz
from oracle import dmrg_oracle as O
from tests.golden.blockio import unpack_block

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def nss():
    import nssdmrg_gb300 as nss
    nss.lib()
    return nss


def _setup(name):
    z = load_npz(name)
    l, r = unpack_block("eleft", z), unpack_block("eright", z)
    sb = O.sb_get_states(l, r, z["target"])
    ds = O.setup_direct(l, r, sb, z["hij"])
    return z, l, r, sb, ds


def _upload(s, l, r, sb, ds, hleft=None):
    terms = [(t.it - 1, t.isb, t.jsb, t.hconj, t.A, t.B, t.row_offset, t.col_offset) for t in ds.terms]
    s.upload(sb.Dls, sb.Drs, sb.Offset, hleft or ds.Hleft, ds.Hright, terms, ds.tNso, l.dim, r.dim, sb.AI, sb.BI)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_barrier_wait_runs_out_then_context_recovers(nss, monkeypatch, precision):
    z, l, r, sb, ds = _setup("c2_small.npz")
    s = nss.Superblock()
    _upload(s, l, r, sb, ds)
    prec = nss.NSS_PREC_FP64 if precision == "fp64" else nss.NSS_PREC_MIXED
    monkeypatch.setenv("NSS_WAIT_LIMIT", "0")
    with pytest.raises(nss.NssError) as ei:
        s.sb_diag(neigen=1, tol=1e-12, precision=prec, want_vectors=False)
    assert ei.value.code == nss.NSS_ERR_CUDA and "timed out" in str(ei.value), str(ei.value)
    monkeypatch.delenv("NSS_WAIT_LIMIT")
    ev, _, _ = s.sb_diag(neigen=1, tol=1e-12, precision=prec, want_vectors=False)
    ref = z["oracle_gs_energy"][0]
    assert abs(ev[0] - ref) <= 1e-10 * abs(ref)


def test_whole_gpu_reduction_wait_runs_out_then_recovers(nss, monkeypatch):
    """The whole-GPU Householder tier (forced onto every rho block above the
    one-CTA size with NSS_TRD_CL_SHARED_MAX=0, NSS_TRD_GRID_MIN=1; the spin-1
    chain L=32, m=256 has blocks of ~190 states) with a poll limit of zero:
    its group barriers give up, nss_rdm reports it, and the next call on the
    context reproduces the unforced result."""
    d = nss.DMRG(nss.MODEL_HEISENBERG_ONE, 16, 256, dmrg_qn=(0.0, 0.0), lanc_neigen=1)
    d.prepare_last()
    s = d.sb
    s.sb_diag(neigen=1, tol=1e-12, want_vectors=False)
    ref = s.sb_get_rdm(64, 0.1, want_u=False)
    monkeypatch.setenv("NSS_TRD_CL_SHARED_MAX", "0")
    monkeypatch.setenv("NSS_TRD_GRID_MIN", "1")
    monkeypatch.setenv("NSS_WAIT_LIMIT", "0")
    with pytest.raises(nss.NssError) as ei:
        s.sb_get_rdm(64, 0.1, want_u=False)
    assert ei.value.code == nss.NSS_ERR_CUDA and "timed out" in str(ei.value), str(ei.value)
    monkeypatch.delenv("NSS_WAIT_LIMIT")
    res = s.sb_get_rdm(64, 0.1, want_u=False)
    for side in (0, 1):
        np.testing.assert_allclose(res.lambdas[side], ref.lambdas[side], rtol=0, atol=1e-13)
    assert list(res.m_s) == list(ref.m_s)
    d.close()


def test_hbm_budget_refusal(nss):
    """A context whose budget cannot hold the solve's Krylov basis returns
    NSS_ERR_NOMEM from the solve; the upload itself fits.  (N = 12 066: the
    operator pool takes well under 8 MiB, an FP64 basis of 513 vectors 50 MB.)"""
    z, l, r, sb, ds = _setup("c2_small.npz")
    s = nss.Superblock(0, hbm_budget=8 << 20)
    _upload(s, l, r, sb, ds)
    with pytest.raises(nss.NssError) as ei:
        s.sb_diag(neigen=1, nitermax=512, tol=1e-12, want_vectors=False)
    assert ei.value.code == nss.NSS_ERR_NOMEM, str(ei.value)
    tiny = nss.Superblock(0, hbm_budget=1024)
    with pytest.raises(nss.NssError) as ei:
        _upload(tiny, l, r, sb, ds)
    assert ei.value.code == nss.NSS_ERR_NOMEM, str(ei.value)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_iteration_cap_reports_no_convergence(nss, precision):
    z, l, r, sb, ds = _setup("c2_small.npz")
    s = nss.Superblock()
    _upload(s, l, r, sb, ds)
    prec = nss.NSS_PREC_FP64 if precision == "fp64" else nss.NSS_PREC_MIXED
    with pytest.raises(nss.NssError) as ei:
        s.sb_diag(neigen=1, nitermax=6, tol=1e-12, precision=prec, want_vectors=False)
    assert ei.value.code == nss.NSS_ERR_NOCONV, str(ei.value)
    ev, _, _ = s.sb_diag(neigen=1, tol=1e-12, precision=prec, want_vectors=False)
    assert abs(ev[0] - z["oracle_gs_energy"][0]) <= 1e-10 * abs(z["oracle_gs_energy"][0])


@pytest.mark.parametrize("value", [np.nan, np.inf])
def test_non_finite_operator_is_refused(nss, value):
    z, l, r, sb, ds = _setup("kat_spin.npz")
    bad = [h.copy().tocsr() for h in ds.Hleft]
    k = int(np.argmax([h.nnz for h in bad]))
    bad[k].data[bad[k].nnz // 2] = value
    s = nss.Superblock()
    with pytest.raises(nss.NssError) as ei:
        _upload(s, l, r, sb, ds, hleft=bad)
    assert ei.value.code == nss.NSS_ERR_INVALID and "non-finite" in str(ei.value), str(ei.value)
    # the context holds no superblock afterwards and takes a good one
    _upload(s, l, r, sb, ds)
    ev, _, _ = s.sb_diag(neigen=2, tol=1e-12)
    np.testing.assert_allclose(ev / (l.length + r.length), z["golden_energy"], rtol=1e-12, atol=0)


def test_tensor_core_pipeline_wait_runs_out_then_recovers(nss, monkeypatch):
    """The tensor-core sector GEMM's mbarrier waits with a poll limit of zero
    (every sector of 32 left states or more routed to it): its roles give up,
    the CTAs still wait for their own copies and MMAs and free their TMEM, the
    solve reports the time-out, and the next solve on the context is right."""
    z, l, r, sb, ds = _setup("c2_small.npz")
    assert max(sb.Dls) >= 32
    monkeypatch.setenv("NSS_TC_MIN_DL", "32")
    s = nss.Superblock()
    _upload(s, l, r, sb, ds)
    monkeypatch.setenv("NSS_WAIT_LIMIT", "0")
    with pytest.raises(nss.NssError) as ei:
        s.sb_diag(neigen=1, tol=1e-12, precision=nss.NSS_PREC_MIXED, want_vectors=False)
    assert ei.value.code == nss.NSS_ERR_CUDA and "timed out" in str(ei.value), str(ei.value)
    monkeypatch.delenv("NSS_WAIT_LIMIT")
    ev, _, _ = s.sb_diag(neigen=1, tol=1e-12, precision=nss.NSS_PREC_MIXED, want_vectors=False)
    ref = z["oracle_gs_energy"][0]
    assert abs(ev[0] - ref) <= 1e-10 * abs(ref)


def test_batch_round_wait_runs_out_drops_solves(nss, monkeypatch):
    """A continuous-batching round whose grid barrier gives up: the step
    reports NSS_ERR_CUDA and the engine drops every solve in flight, so a
    dropped context may be freed at once; the engine then solves a context
    that joins again, to the oracle's energy."""
    z, l, r, sb, ds = _setup("c2_small.npz")
    host, other = nss.Superblock(), nss.Superblock()
    _upload(host, l, r, sb, ds)
    _upload(other, l, r, sb, ds)
    eng = nss.BatchEngine(host)
    eng.add(host, seed=1)
    eng.add(other, seed=2)
    monkeypatch.setenv("NSS_WAIT_LIMIT", "0")
    with pytest.raises(nss.NssError) as ei:
        eng.step()
    assert ei.value.code == nss.NSS_ERR_CUDA and "timed out" in str(ei.value), str(ei.value)
    assert eng.inflight == 0
    monkeypatch.delenv("NSS_WAIT_LIMIT")
    other.close()
    eng.add(host, seed=3)
    done = []
    for _ in range(10000):
        done += eng.step()
        if eng.inflight == 0:
            break
    eng.close()
    assert len(done) == 1 and done[0][0] > 0
    ref = z["oracle_gs_energy"][0]
    assert abs(done[0][1] - ref) <= 1e-10 * abs(ref)
    host.close()
