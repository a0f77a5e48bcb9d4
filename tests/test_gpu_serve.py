"""Serving whole DMRG runs (nss_server_*): requests of different models,
lengths and bond dimensions run concurrently, their mixed ground-state solves
batched in one engine and their admission bounded by the HBM footprint
estimate.  Every request's result must equal the same run made alone
(nss_dmrg_finite on a context of its own) to 1e-10 relative: batching and
interleaving change the order of the device work, not the arithmetic of a
request."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def nss():
    import nssdmrg_gb300 as nss
    nss.lib()
    return nss


def _requests(nss, precision):
    H, S1, HU = nss.MODEL_HEISENBERG_HALF, nss.MODEL_HEISENBERG_ONE, nss.MODEL_HUBBARD
    common = dict(lanc_neigen=1, lanc_tolerance=1e-12, precision=precision)
    return [
        dict(model=H, ldmrg=8, mdmrg=32, msweep=(32, 32), jz=0.8, jxy=0.8, dmrg_qn=(0.0, 0.0), **common),
        dict(model=HU, ldmrg=6, mdmrg=48, msweep=(48, 48), u=3.0, hfmode=False, dmrg_qn=(0.5, 0.5), **common),
        dict(model=S1, ldmrg=8, mdmrg=40, msweep=(40, 40), dmrg_qn=(0.0, 0.0), **common),
        dict(model=H, ldmrg=12, mdmrg=64, msweep=(64, 64), jz=1.3, jxy=1.3, dmrg_qn=(0.0, 0.0), **common),
        dict(model=HU, ldmrg=8, mdmrg=64, msweep=(64, 64), u=6.5, hfmode=False, dmrg_qn=(0.5, 0.5), **common),
    ]


def _alone(nss, kw):
    d = nss.DMRG(**kw)
    recs = d.finite()
    e = recs[-1]["energy"][0]
    d.close()
    return e


def _serve(nss, reqs, budget):
    srv = nss.Server(0, hbm_budget=budget)
    ids = [srv.submit(**kw) for kw in reqs]
    done = {}
    t0 = time.time()
    while len(done) < len(ids) and time.time() - t0 < 300:
        for r in srv.poll():
            done[r["id"]] = r
        time.sleep(0.01)
    stats = srv.stats()
    srv.close()
    return ids, done, stats


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_served_runs_equal_runs_alone(nss, precision):
    prec = nss.NSS_PREC_MIXED if precision == "mixed" else nss.NSS_PREC_FP64
    reqs = _requests(nss, prec)
    ids, done, stats = _serve(nss, reqs, budget=1 << 40)
    assert len(done) == len(reqs)
    for rid, kw in zip(ids, reqs):
        r = done[rid]
        assert r["status"] == 0, r
        e = _alone(nss, kw)
        assert abs(r["energy"] - e) <= 1e-10 * abs(e), (kw, r["energy"], e)
    if precision == "mixed":
        # the requests ran together: the engine's rounds carried several solves
        assert stats["mean_batch"] > 1.0, stats


def test_admission_respects_the_hbm_budget(nss):
    """With a budget that fits the largest request but not two of them, the
    estimated footprints in flight never exceed it, and every request still
    completes; each request's measured device peak stays within its
    estimate."""
    reqs = _requests(nss, nss.NSS_PREC_MIXED)
    fps = [nss.Server.footprint(**kw) for kw in reqs]
    budget = max(fps) + min(fps) // 2
    ids, done, stats = _serve(nss, reqs, budget)
    assert len(done) == len(reqs)
    assert stats["peak_in_use"] <= budget, (stats, budget)
    for rid in ids:
        r = done[rid]
        assert r["status"] == 0
        assert r["peak_bytes"] <= r["footprint_est"], r
