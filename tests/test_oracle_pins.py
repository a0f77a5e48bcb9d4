"""The CPU oracle against the reference's own golden files (no GPU).

Pins: test/src/Spin1d_SU2/energy.check (asserted by the reference at 1e-12),
test/src/Hubbard1d/energy.check and Sentropy.check, the 39-step from-scratch
trajectories L40.energy.check / L40.Sentropy.check of both test models, and
the published U=2 Hubbard trajectory .plot/Hubbard/U2 (HFMODE=F), all
converted into tests/golden by make_golden.py.
"""
import numpy as np
import pytest
import scipy.sparse as sp

from conftest import load_npz
from oracle import dmrg_oracle as O
from oracle.restart_io import parse_block
from tests.golden.blockio import restart_text, unpack_block


def _kat_run(name):
    z = load_npz(f"kat_{name}.npz")
    left, right = unpack_block("left", z), unpack_block("right", z)
    ldmrg, mdmrg, neigen = (int(x) for x in z["params"])
    if name == "spin":
        p = O.Params(Ldmrg=ldmrg, Mdmrg=mdmrg, lanc_neigen=neigen, lanc_ncv_factor=5,
                     lanc_dim_threshold=128, dmrg_qn=(0.0,))
        run = O.DMRG(O.heisenberg_hij(), O.spin_site(2), p, left, right, keep_setups=True)
    else:
        p = O.Params(Ldmrg=ldmrg, Mdmrg=mdmrg, lanc_neigen=neigen, lanc_ncv_factor=10,
                     lanc_dim_threshold=128, dmrg_qn=(0.5, 0.5))
        run = O.DMRG(O.hubbard_hij(), O.electron_site(0.0, True), p, left, right, keep_setups=True)
    rec = run.step("i")
    return z, run, rec


def test_kat_spin_energy_matches_energy_check():
    z, run, rec = _kat_run("spin")
    # spinSU2_1d.f90:246-255 asserts at 1e-12
    np.testing.assert_allclose(rec.energies, z["golden_energy"], rtol=1e-12, atol=0)
    assert rec.solver == "lanczos"


def test_kat_hubbard_energy_matches_energy_check():
    z, run, rec = _kat_run("hubbard")
    # hm_1d.f90:139-147 asserts at 1e-6; the restatement holds 1e-12
    np.testing.assert_allclose(rec.energies, z["golden_energy"], rtol=1e-12, atol=0)


def test_kat_superblock_tables_are_reproducible():
    z, run, rec = _kat_run("spin")
    l, r, sb, ds, ev, evec = run.setups[0]
    np.testing.assert_array_equal(sb.sb_states, z["sb_states"])
    np.testing.assert_array_equal(sb.Dls, z["sb_dls"])
    np.testing.assert_array_equal(sb.Offset, z["sb_offset"])


@pytest.mark.parametrize("name", ["spin", "hubbard"])
def test_direct_matvec_equals_independent_kron_hamiltonian(name):
    """spMatVec_direct_main == the sparse superblock H of
    Setup_SuperBlock_Sparse built from full Kronecker products."""
    z, run, rec = _kat_run(name)
    l, r, sb, ds, ev, evec = run.setups[0]
    h = O.sparse_superblock_h(l, r, sb, run.hij)
    v = z["v"]
    ref = h @ v
    np.testing.assert_allclose(O.spmatvec_direct(ds, v), ref, rtol=0, atol=1e-12 * np.abs(ref).max())
    np.testing.assert_allclose(z["hv"], ref, rtol=0, atol=1e-12 * np.abs(ref).max())
    # Hermiticity of the direct operator
    u = np.random.default_rng(3).standard_normal(sb.N)
    assert abs(u @ O.spmatvec_direct(ds, v) - v @ O.spmatvec_direct(ds, u)) < 1e-10 * np.abs(ref).max()


def test_loop_order_restatement_matches_vectorised():
    z, run, rec = _kat_run("spin")
    l, r, sb, ds, ev, evec = run.setups[0]
    v = z["v"]
    a = O.spmatvec_direct_loops(ds, v)
    b = O.spmatvec_direct(ds, v)
    np.testing.assert_allclose(a, b, rtol=0, atol=1e-13 * np.abs(b).max())


_L40_RUNS = {}


def _l40_run(trajectories, key):
    if key not in _L40_RUNS:
        t = trajectories[key]
        if t["model"] == "heisenberg_half":
            p = O.Params(Ldmrg=t["ldmrg"], Mdmrg=t["mdmrg"], lanc_neigen=2, lanc_ncv_factor=5,
                         lanc_dim_threshold=128, dmrg_qn=(0.0,))
            run = O.DMRG(O.heisenberg_hij(), O.spin_site(2), p)
        else:
            p = O.Params(Ldmrg=t["ldmrg"], Mdmrg=t["mdmrg"], lanc_neigen=1, lanc_ncv_factor=10,
                         lanc_dim_threshold=128, dmrg_qn=(0.5, 0.5))
            run = O.DMRG(O.hubbard_hij(), O.electron_site(t["u"], t["hfmode"]), p)
        run.infinite()
        _L40_RUNS[key] = run
    return _L40_RUNS[key]


def measure_ops(model):
    """The site operators the reference's test drivers measure: S_z
    (spinSU2_1d.f90:41), and n, n_up n_dw, (n_up - n_dw)^2 built from the
    dot's C operators as N_s = C_s^+ C_s (hm_1d.f90:62-76)."""
    if model == "heisenberg_half":
        return {"sz": np.diag([0.5, -0.5])}
    dot = O.electron_site(0.0, True)
    nup = (dot.op("C_l1_s1_n").T @ dot.op("C_l1_s1_n")).toarray()
    ndw = (dot.op("C_l1_s2_n").T @ dot.op("C_l1_s2_n")).toarray()
    return {"n": nup + ndw, "d": nup @ ndw, "s2z": (nup - ndw) @ (nup - ndw)}


@pytest.mark.parametrize("key", ["spin_L40_M20", "hubbard_L40_M40"])
def test_l40_trajectory(trajectories, key):
    t = trajectories[key]
    run = _l40_run(trajectories, key)
    e = np.array([r.energies for r in run.records])
    ref = np.array(t["energy"])
    np.testing.assert_allclose(e, ref, rtol=1e-11, atol=0)
    s = np.array([r.entropy_left for r in run.records])
    # The golden entropy files were written by an older revision that wrote
    # the previous step's entropy again at the last (non-truncating) step, so
    # the last row repeats the one before; every other row is pinned.
    np.testing.assert_allclose(s[:-1], np.array(t["entropy"])[:-1], rtol=0, atol=1e-9)
    assert t["entropy"][-1] == t["entropy"][-2]


def test_hubbard_sentropy_check_is_the_step_that_wrote_the_restart_blocks(trajectories):
    z = load_npz("kat_hubbard.npz")
    # Sentropy.check = entropy of the step that grew the blocks to length 39
    assert z["golden_sentropy"][0] == trajectories["hubbard_L40_M40"]["entropy"][37]


def test_u2_hfmode_false_trajectory_first_steps(trajectories):
    """U != 0 with the plain U n_up n_dw interaction (HFMODE=F); the first 40
    of the 99 published steps, past step 28 where the degeneracy extension
    decides (the run used deg_evals_threshold = 0.01)."""
    t = trajectories["hubbard_U2_L100_M50"]
    nsteps = 40
    p = O.Params(Ldmrg=nsteps + 1, Mdmrg=t["mdmrg"], lanc_neigen=1, lanc_ncv_factor=10,
                 lanc_dim_threshold=128, dmrg_qn=(0.5, 0.5), deg_evals_threshold=t["deg_evals_threshold"])
    run = O.DMRG(O.hubbard_hij(), O.electron_site(t["u"], t["hfmode"]), p)
    for _ in range(nsteps):
        run.step("i")
    e = np.array([r.energies[0] for r in run.records])
    np.testing.assert_allclose(e, np.array(t["energy"])[:nsteps, 0], rtol=1e-10, atol=0)


def test_restart_reader_maps_legacy_operator_names():
    text = """ 1
 2
 SPIN
 S
 1
 2
 1
 1
 0.5
 1
 1
 1
 -0.5
 1
 2
 3
 H
 bosonic
 2 2
 1
 1 0.25
 1
 2 -0.25
 S_z
 bosonic
 2 2
 1
 1 0.5
 1
 2 -0.5
 S_p
 bosonic
 2 2
 1
 2 1.0
 0
 0
"""
    b = parse_block(text)
    assert list(b.ops) == ["H", "S_z_n", "S_p_n"]
    assert b.op("S_p_n").toarray().tolist() == [[0.0, 1.0], [0.0, 0.0]]
    assert b.basis[:, 0].tolist() == [0.5, -0.5]


def test_truncation_degeneracy_extension():
    """renormalize_block keeps every later eigenvalue within 10 % of lambda(m_s)."""
    ev = np.array([0.5, 0.2, 0.1, 0.095, 0.0951, 0.05, 0.004, 0.0009])
    rho = O.RhoBlocks([(0.0,)], [np.arange(ev.size)], [ev[::-1].copy()], [np.eye(ev.size)],
                      ev.copy(), np.arange(ev.size)[::-1].copy())
    m_s, eps = O.truncation(rho, 3, 8, 0.1)
    assert m_s == 5
    assert abs(eps - (1.0 - ev[:5].sum())) < 1e-15


def test_electron_site_signs():
    s = O.electron_site(4.0, False)
    cu, cd, p = s.op("C_l1_s1_n").toarray(), s.op("C_l1_s2_n").toarray(), s.op("P_n").toarray()
    # anticommutation {c_up, c_dw^+} = 0 and {c_s, c_s^+} = 1 on the 4-state Fock space
    assert np.allclose(cu @ cd.T + cd.T @ cu, 0)
    assert np.allclose(cu @ cu.T + cu.T @ cu, np.eye(4))
    assert np.allclose(cd @ cd.T + cd.T @ cd, np.eye(4))
    assert np.allclose(p, np.diag([1, -1, -1, 1]))
    assert np.allclose(np.diag(s.op("H").toarray()), [0, 0, 0, 4.0])


@pytest.mark.parametrize("name", ["kat_spin.npz", "kat_hubbard.npz", "c2_small.npz"])
def test_qn_entropy_split_adds_up(name):
    """write_entanglement's S_N + S_c equals the von Neumann entropy of the
    same blocks (an identity of the restatement, src/DMRG_MAIN.f90:510-561),
    and a single block has S_N = 0."""
    z = load_npz(name)
    psi, dls, drs, off = z["psi"], z["sb_dls"], z["sb_drs"], z["sb_offset"]
    blocks = []
    for k in range(len(dls)):
        w = psi[off[k]:off[k] + dls[k] * drs[k]].reshape(dls[k], drs[k])
        blocks.append(((k,), np.arange(dls[k]), w @ w.T))
    rho = O.eigh_blocks(blocks)
    sn, sc = O.qn_entropies(rho)
    s = O.entropy(rho.evalues)
    assert abs((sn + sc) - s) <= 1e-12 * max(1.0, abs(s))
    one = O.eigh_blocks([((0,), np.arange(4), np.diag([0.5, 0.3, 0.2, 0.0]))])
    sn1, sc1 = O.qn_entropies(one)
    assert abs(sn1) < 1e-15 and abs(sc1 - O.entropy(one.evalues)) < 1e-15


@pytest.mark.parametrize("key", ["spin_L40_M20", "hubbard_L40_M40"])
def test_l40_measurements_match_checks(trajectories, key):
    """Measure_DMRG (Build_Op, Advance_Op, Average_Op, OdotV_direct) after the
    L=40 runs against sz.check (asserted at 1e-8 by spinSU2_1d.f90:60) and
    n / d / s2z.check (1e-6, hm_1d.f90:139-147)."""
    t = trajectories[key]
    run = _l40_run(trajectories, key)
    tol = 1e-8 if t["model"] == "heisenberg_half" else 1e-6
    for name, op in measure_ops(t["model"]).items():
        got = run.measure(op, range(1, t["ldmrg"] + 1))
        ref = np.array(t["measure"][name])
        assert got.shape == ref.shape
        np.testing.assert_allclose(got, ref, rtol=0, atol=tol, err_msg=name)


def test_odotv_loop_restatement_matches_vectorised():
    """OdotV_direct's loop nest against the per-sector matrix product, both
    sides, random sparse sector operators on the spin KAT superblock."""
    z, run, rec = _kat_run("spin")
    left, right, sb, ds, ev, evec = run.setups[-1]
    rng = np.random.default_rng(3)
    v = rng.standard_normal(sb.N)
    for label in ("l", "r"):
        dims = sb.Dls if label == "l" else sb.Drs
        ops = [sp.random(int(d), int(d), density=0.3, random_state=rng, format="csr") for d in dims]
        a = O.odotv_direct(ops, v, label, sb)
        b = O.odotv_vectorised(ops, v, label, sb)
        np.testing.assert_allclose(a, b, rtol=0, atol=1e-13 * np.abs(b).max())


@pytest.mark.parametrize("name", ["spin", "hubbard"])
@pytest.mark.parametrize("legacy", [False, True])
def test_restart_text_writer_round_trips_through_the_reader(name, legacy):
    """The fixtures' blocks written in the restart layout (as the GPU tests
    feed them to the library's reader) read back exactly with the oracle's
    reader, legacy operator names included."""
    z = load_npz(f"kat_{name}.npz")
    for side in ("left", "right"):
        b = unpack_block(side, z)
        r = parse_block(restart_text(b, legacy=legacy))
        assert (r.length, r.dim, r.sitetype) == (b.length, b.dim, b.sitetype)
        np.testing.assert_array_equal(r.basis, b.basis)
        assert list(r.ops) == list(b.ops)
        for k in b.ops:
            assert r.ops[k][1] == b.ops[k][1]
            assert (r.op(k) != b.op(k)).nnz == 0


def test_error_threshold_rule_by_hand():
    """The Edmrg rule of renormalize_block (src/DMRG_RDM.f90:206-208) on a
    small spectrum worked out by hand: 1 - cumulate(lambda) = .5, .2, .05,
    .01, .001, 0; closest to Estates = 0.012 is the fourth (|.01 - .012|);
    no eigenvalue after it lies within 10 % of 0.04."""
    from oracle import dmrg_oracle as O
    lam = np.array([0.5, 0.3, 0.15, 0.04, 0.009, 0.001])
    rho = O.RhoBlocks([(0.0,)], [np.arange(6)], [lam[::-1].copy()], [np.eye(6)], lam.copy(), np.arange(6)[::-1])
    m_s, eps = O.truncation(rho, 0, 6, 0.1, 0.012)
    assert m_s == 4 and abs(eps - 0.01) < 1e-15
    # Mstates != 0 ignores Estates; both zero is the reference's stop
    assert O.truncation(rho, 2, 6, 0.1, 0.012)[0] == 2
    with pytest.raises(ValueError):
        O.truncation(rho, 0, 6, 0.1, 0.0)
