"""Measurements on the GPU: OdotV_direct / Average_Op_dmrg through the C ABI
against the oracle's restatement, and whole Measure_DMRG runs (Build_Op,
Advance_Op over the stored rotations, Average_Op) against the reference's
golden files and the oracle.

Tolerances: the product O v and <psi|O|psi> at 1e-12 relative (FP64, a
different summation order); sz.check at 1e-8 and n / d / s2z.check at 1e-6,
the reference's own asserts (spinSU2_1d.f90:60, hm_1d.f90:139-147); the
oracle's U=4 measurements at 1e-9 (the two runs' ground states agree to
rounding, with an energy difference of ~1e-14 per site).
"""
import json
import os

import numpy as np
import pytest
import scipy.sparse as sp

from conftest import GOLDEN, load_npz
from oracle import dmrg_oracle as O
from test_gpu_parity import _setup, _upload

pytestmark = pytest.mark.gpu

MODELS = {"heisenberg_half": 0, "heisenberg_one": 1, "hubbard": 2}


@pytest.fixture(scope="module")
def nss():
    import nssdmrg_gb300 as nss
    nss.lib()
    return nss


def _site_ops(model):
    """The operators the reference's test drivers measure: S_z, and n,
    n_up n_dw, (n_up - n_dw)^2 from N_s = C_s^+ C_s of the dot."""
    if model == "heisenberg_half":
        return {"sz": np.diag([0.5, -0.5])}
    dot = O.electron_site(0.0, True)
    nup = (dot.op("C_l1_s1_n").T @ dot.op("C_l1_s1_n")).toarray()
    ndw = (dot.op("C_l1_s2_n").T @ dot.op("C_l1_s2_n")).toarray()
    return {"n": nup + ndw, "d": nup @ ndw, "s2z": (nup - ndw) @ (nup - ndw)}


@pytest.mark.parametrize("name", ["kat_spin.npz", "kat_hubbard.npz", "c2_small.npz"])
def test_odotv_and_average_match_oracle(nss, name):
    z = load_npz(name)
    l, r, sb, ds = _setup(z)
    s = nss.Superblock()
    _upload(nss, s, l, r, ds)
    rng = np.random.default_rng(17)
    v = rng.standard_normal(sb.N)
    v /= np.linalg.norm(v)
    for label in ("l", "r"):
        dims = sb.Dls if label == "l" else sb.Drs
        ops = [sp.random(int(d), int(d), density=0.25, random_state=rng, format="csr") for d in dims]
        got = s.odotv(label, ops, v)
        ref = O.odotv_vectorised(ops, v, label, sb)
        assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()
        # a whole block operator, filtered by the uploaded sector maps
        mb = l.dim if label == "l" else r.dim
        a = sp.random(mb, mb, density=0.05, random_state=rng, format="csr")
        oi = (a + a.T).tocsr()
        val = s.average_op(label, oi, psi=v)
        ref_val = O.average_op(oi, label, sb, v)
        assert abs(val - ref_val) <= 1e-12 * max(1.0, abs(ref_val)), (label, val, ref_val)


def test_odotv_rejects_bad_operators(nss):
    z = load_npz("kat_spin.npz")
    l, r, sb, ds = _setup(z)
    s = nss.Superblock()
    _upload(nss, s, l, r, ds)
    ops = [sp.identity(int(d), format="csr") for d in sb.Dls]
    ops[0] = sp.identity(int(sb.Dls[0]) + 1, format="csr")
    with pytest.raises(nss.NssError):
        s.odotv("l", ops, np.zeros(sb.N))
    with pytest.raises(nss.NssError):
        s.odotv("x", [sp.identity(int(d), format="csr") for d in sb.Dls], np.zeros(sb.N))


@pytest.mark.parametrize("key", ["spin_L40_M20", "hubbard_L40_M40"])
def test_measure_matches_reference_checks(nss, trajectories, key):
    t = trajectories[key]
    d = nss.DMRG(MODELS[t["model"]], t["ldmrg"], t["mdmrg"], u=t.get("u", 0.0), hfmode=t.get("hfmode", True),
                 dmrg_qn=tuple(t["dmrg_qn"]) + ((0.0,) if len(t["dmrg_qn"]) == 1 else ()),
                 lanc_neigen=t["neigen"], lanc_tolerance=1e-12, save_umat=True)
    d.infinite()
    tol = 1e-8 if t["model"] == "heisenberg_half" else 1e-6
    for name, op in _site_ops(t["model"]).items():
        got = d.measure(op, np.arange(1, t["ldmrg"] + 1))
        np.testing.assert_allclose(got, np.array(t["measure"][name]), rtol=0, atol=tol, err_msg=name)


@pytest.mark.parametrize("renorm", ["host", "device"])
def test_measure_matches_oracle_u4(nss, renorm):
    """Hubbard U=4, HFMODE=F, L=20, M=64: n_up n_dw varies along the open
    chain; every site, the right half through the right block's rotations,
    with the rotations taken from the host or the device renormalisation."""
    m = json.loads((GOLDEN / "measure_runs.json").read_text())["hubbard_U4_L20_M64"]
    old = os.environ.get("NSS_RENORM")
    try:
        os.environ["NSS_RENORM"] = renorm
        d = nss.DMRG(MODELS[m["model"]], m["ldmrg"], m["mdmrg"], u=m["u"], hfmode=m["hfmode"],
                     dmrg_qn=tuple(m["dmrg_qn"]), lanc_neigen=1, lanc_tolerance=1e-12, save_umat=True)
        recs = d.infinite()
    finally:
        if old is None:
            os.environ.pop("NSS_RENORM", None)
        else:
            os.environ["NSS_RENORM"] = old
    assert abs(recs[-1]["energy"][0] - m["energy_last"][0]) <= 1e-11
    for name, op in m["ops"].items():
        got = d.measure(np.array(op), np.array(m["pos"]))
        np.testing.assert_allclose(got, np.array(m["measure"][name]), rtol=0, atol=1e-9, err_msg=name)


def test_measure_without_rotations_fails(nss):
    d = nss.DMRG(0, 6, 16, dmrg_qn=(0.0, 0.0), lanc_neigen=1)
    d.infinite()
    with pytest.raises(nss.NssError):
        d.measure(np.diag([0.5, -0.5]), [1])
