"""Generate the golden fixtures of this folder from the reference project.

Reads the reference's own test fixtures and published result files (restart
blocks, energy.check, Sentropy.check, L40.*.check, .plot/*.dmrg) and runs the
CPU oracle on them.  Needs the reference tree (default path below, or the
first command-line argument); the GPU host never runs this script, it only
reads what it wrote.

    python -m tests.golden.make_golden [/path/to/reference]
"""
from __future__ import annotations

import json
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import dmrg_oracle as O          # noqa: E402
from oracle.restart_io import read_block     # noqa: E402
from tests.golden.blockio import pack_block  # noqa: E402

OUT = Path(__file__).resolve().parent


def kat(ref: Path, model: str):
    """One iDMRG step from the shipped length-39 restart blocks."""
    d = ref / "test" / "src" / ("Spin1d_SU2" if model == "spin" else "Hubbard1d")
    left = read_block(str(d / "block_left.restart"))
    right = read_block(str(d / "block_right.restart"))
    if model == "spin":
        p = O.Params(Ldmrg=40, Mdmrg=20, lanc_neigen=2, lanc_ncv_factor=5, lanc_dim_threshold=128,
                     dmrg_qn=(0.0,))
        hij, dot = O.heisenberg_hij(), O.spin_site(2)
        golden_e = np.loadtxt(d / "energy.check")[1:3]
    else:
        p = O.Params(Ldmrg=40, Mdmrg=40, lanc_neigen=1, lanc_ncv_factor=10, lanc_dim_threshold=128,
                     dmrg_qn=(0.5, 0.5))
        hij, dot = O.hubbard_hij(), O.electron_site(0.0, True)
        golden_e = np.atleast_1d(np.loadtxt(d / "energy.check"))
    run = O.DMRG(hij, dot, p, left, right, keep_setups=True)
    rec = run.step("i")
    l, r, sb, ds, ev, evec = run.setups[0]
    rng = np.random.default_rng(7)
    v = rng.standard_normal(sb.N)
    hv = O.spmatvec_direct(ds, v)
    lblocks, rblocks = O.build_density_matrices(sb, evec[:, 0], l.sectors(), r.sectors())
    rho_l, rho_r = O.eigh_blocks(lblocks), O.eigh_blocks(rblocks)
    ms_l, eps_l = O.truncation(rho_l, p.Mdmrg, l.dim, p.deg_evals_threshold)
    ms_r, eps_r = O.truncation(rho_r, p.Mdmrg, r.dim, p.deg_evals_threshold)
    out = {}
    pack_block("left", left, out)
    pack_block("right", right, out)
    pack_block("eleft", l, out)
    pack_block("eright", r, out)
    out.update({
        "hij": hij, "target": sb.target, "golden_energy": golden_e,
        "sb_qns": np.array(sb.qns), "sb_dls": sb.Dls, "sb_drs": sb.Drs, "sb_offset": sb.Offset,
        "sb_states": sb.sb_states, "v": v, "hv": hv, "oracle_energy": rec.energies,
        "oracle_gs_energy": rec.gs_energy, "psi": evec[:, 0],
        "lam_left": rho_l.evalues, "lam_right": rho_r.evalues,
        "ms": np.array([ms_l, ms_r]), "trunc": np.array([eps_l, eps_r]),
        "entropy": np.array([rec.entropy_left, rec.entropy_right]),
        "params": np.array([p.Ldmrg, p.Mdmrg, p.lanc_neigen]),
        "dmrg_qn": np.array(p.dmrg_qn),
    })
    if model == "hubbard":
        out["golden_sentropy"] = np.atleast_1d(np.loadtxt(d / "Sentropy.check"))
    np.savez_compressed(OUT / f"kat_{model}.npz", **out)
    print(model, "KAT: N", sb.N, "E", rec.energies, "golden", golden_e)


def trajectories(ref: Path):
    t = ref / "test" / "src"
    pl = ref / ".plot"
    out = {}
    e = np.loadtxt(t / "Spin1d_SU2" / "L40.energy.check")
    s = np.loadtxt(t / "Spin1d_SU2" / "L40.Sentropy.check")
    out["spin_L40_M20"] = {"model": "heisenberg_half", "ldmrg": 40, "mdmrg": 20, "neigen": 2,
                           "dmrg_qn": [0.0], "left_length": e[:, 0].astype(int).tolist(),
                           "energy": e[:, 1:3].tolist(), "entropy": s.tolist(),
                           "source": "test/src/Spin1d_SU2/L40.energy.check, L40.Sentropy.check"}
    # Measure_DMRG of S_z at sites 1..40 after that run (spinSU2_1d.f90:41, asserted at 1e-8)
    out["spin_L40_M20"]["measure"] = {"sz": np.loadtxt(t / "Spin1d_SU2" / "sz.check").tolist(),
                                      "source": "test/src/Spin1d_SU2/sz.check"}
    e = np.loadtxt(t / "Hubbard1d" / "L40.energy.check")
    s = np.loadtxt(t / "Hubbard1d" / "L40.Sentropy.check")
    out["hubbard_L40_M40"] = {"model": "hubbard", "ldmrg": 40, "mdmrg": 40, "neigen": 1, "u": 0.0,
                              "hfmode": True, "dmrg_qn": [0.5, 0.5],
                              "left_length": list(range(2, 41)), "energy": e[:, None].tolist(),
                              "entropy": s.tolist(),
                              "source": "test/src/Hubbard1d/L40.energy.check, L40.Sentropy.check"}
    # Measure_DMRG of n, n_up n_dw and (n_up - n_dw)^2 at sites 1..40 (hm_1d.f90:62-76,
    # asserted at 1e-6)
    out["hubbard_L40_M40"]["measure"] = {k: np.loadtxt(t / "Hubbard1d" / f"{k}.check").tolist()
                                         for k in ("n", "d", "s2z")}
    out["hubbard_L40_M40"]["measure"]["source"] = "test/src/Hubbard1d/{n,d,s2z}.check"
    e = np.loadtxt(pl / "Hubbard" / "U2" / "energyVSleft.length_L100_M50_iDMRG.dmrg")
    s = np.loadtxt(pl / "Hubbard" / "U2" / "SentropyVSleft.length_L100_M50_iDMRG.dmrg")
    # This published run used deg_evals_threshold = 0.01 (its DMRG.conf does
    # not set it; the current default is 0.1): with 0.01 all 99 steps are
    # reproduced to 6e-15, with 0.1 the curve departs at step 28, where a
    # multiplet 7.3 % below lambda(m_s) is kept.  The spin L=300 curve in
    # .plot/HeisenbergSU2.3 matches no threshold of the current algorithm
    # past step 7 (an older revision) and is not used.
    out["hubbard_U2_L100_M50"] = {"model": "hubbard", "ldmrg": 100, "mdmrg": 50, "neigen": 1, "u": 2.0,
                                  "hfmode": False, "dmrg_qn": [0.5, 0.5], "deg_evals_threshold": 0.01,
                                  "left_length": e[:, 0].astype(int).tolist(), "energy": e[:, 1:2].tolist(),
                                  "entropy": s[:, 1].tolist(),
                                  "source": ".plot/Hubbard/U2/energyVSleft.length_L100_M50_iDMRG.dmrg"}
    (OUT / "trajectories.json").write_text(json.dumps(out))
    print("trajectories:", {k: len(v["energy"]) for k, v in out.items()})


def oracle_runs():
    """Oracle trajectories for cases the reference publishes nothing on."""
    res = {}
    t0 = time.time()
    p = O.Params(Ldmrg=10, Mdmrg=64, lanc_neigen=1, dmrg_qn=(0.0,), Msweep=(64, 64, 64))
    run = O.DMRG(O.heisenberg_hij(), O.spin_site(2), p)
    run.finite()
    res["c1_spin_L20_M64_3sweeps"] = {
        "model": "heisenberg_half", "ldmrg": 10, "mdmrg": 64, "msweep": [64, 64, 64], "neigen": 1,
        "dmrg_qn": [0.0],
        "kind": [r.kind for r in run.records], "left_length": [r.left_length for r in run.records],
        "energy": [r.energies.tolist() for r in run.records],
        "entropy": [r.entropy_left for r in run.records], "N": [r.N for r in run.records],
        "trunc": [r.trunc_left for r in run.records]}
    print("C1 oracle", time.time() - t0)
    t0 = time.time()
    p = O.Params(Ldmrg=10, Mdmrg=64, lanc_neigen=1, dmrg_qn=(0.5, 0.5))
    run = O.DMRG(O.hubbard_hij(1.0), O.electron_site(4.0, False), p)
    run.infinite()
    res["hubbard_U4_L20_M64"] = {
        "model": "hubbard", "ldmrg": 10, "mdmrg": 64, "neigen": 1, "u": 4.0, "hfmode": False,
        "dmrg_qn": [0.5, 0.5], "left_length": [r.left_length for r in run.records],
        "energy": [r.energies.tolist() for r in run.records],
        "entropy": [r.entropy_left for r in run.records], "N": [r.N for r in run.records],
        "trunc": [r.trunc_left for r in run.records]}
    print("Hubbard U4 oracle", time.time() - t0)
    p = O.Params(Ldmrg=8, Mdmrg=48, lanc_neigen=1, dmrg_qn=(0.0,))
    run = O.DMRG(O.heisenberg_hij(), O.spin_site(3), p)
    run.infinite()
    res["spin1_L16_M48"] = {
        "model": "heisenberg_one", "ldmrg": 8, "mdmrg": 48, "neigen": 1, "dmrg_qn": [0.0],
        "left_length": [r.left_length for r in run.records],
        "energy": [r.energies.tolist() for r in run.records],
        "entropy": [r.entropy_left for r in run.records], "N": [r.N for r in run.records],
        "trunc": [r.trunc_left for r in run.records]}
    # the error-threshold truncation (Mdmrg = 0, Edmrg != 0; src/DMRG_RDM.f90:206-208):
    # spin-1 L=20 grown at Edmrg=1e-6, then one finite sweep at Esweep=1e-7
    p = O.Params(Ldmrg=10, Mdmrg=0, Edmrg=1e-6, Msweep=(0,), Esweep=(1e-7,), lanc_neigen=1, dmrg_qn=(0.0,))
    run = O.DMRG(O.heisenberg_hij(), O.spin_site(3), p)
    run.finite()
    res["spin1_L20_E1e-6_sweep_E1e-7"] = {
        "model": "heisenberg_one", "ldmrg": 10, "mdmrg": 0, "edmrg": 1e-6, "msweep": [0], "esweep": [1e-7],
        "neigen": 1, "dmrg_qn": [0.0],
        "kind": [r.kind for r in run.records], "left_length": [r.left_length for r in run.records],
        "energy": [r.energies.tolist() for r in run.records],
        "entropy": [r.entropy_left for r in run.records], "N": [r.N for r in run.records],
        "trunc": [r.trunc_left for r in run.records], "m_left": [r.m_left for r in run.records]}
    p = O.Params(Ldmrg=8, Mdmrg=0, Edmrg=1e-5, lanc_neigen=1, dmrg_qn=(0.5, 0.5))
    run = O.DMRG(O.hubbard_hij(1.0), O.electron_site(4.0, False), p)
    run.infinite()
    res["hubbard_U4_L16_E1e-5"] = {
        "model": "hubbard", "ldmrg": 8, "mdmrg": 0, "edmrg": 1e-5, "neigen": 1, "u": 4.0, "hfmode": False,
        "dmrg_qn": [0.5, 0.5], "left_length": [r.left_length for r in run.records],
        "energy": [r.energies.tolist() for r in run.records],
        "entropy": [r.entropy_left for r in run.records], "N": [r.N for r in run.records],
        "trunc": [r.trunc_left for r in run.records], "m_left": [r.m_left for r in run.records]}
    (OUT / "oracle_runs.json").write_text(json.dumps(res))


def measure_runs():
    """Oracle measurements (Measure_DMRG, src/DMRG_MEASURE.f90:148-705) where
    the values are not fixed by symmetry: Hubbard U=4, HFMODE=F, L=20, M=64,
    whose open ends make n_up n_dw vary along the chain, at every site (the
    right half through the right block's rotations)."""
    p = O.Params(Ldmrg=10, Mdmrg=64, lanc_neigen=1, dmrg_qn=(0.5, 0.5))
    run = O.DMRG(O.hubbard_hij(1.0), O.electron_site(4.0, False), p)
    run.infinite()
    dot = run.dot
    nup = (dot.op("C_l1_s1_n").T @ dot.op("C_l1_s1_n")).toarray()
    ndw = (dot.op("C_l1_s2_n").T @ dot.op("C_l1_s2_n")).toarray()
    ops = {"n": nup + ndw, "d": nup @ ndw, "s2z": (nup - ndw) @ (nup - ndw)}
    pos = list(range(1, 21))
    res = {"hubbard_U4_L20_M64": {"model": "hubbard", "ldmrg": 10, "mdmrg": 64, "u": 4.0, "hfmode": False,
                                  "dmrg_qn": [0.5, 0.5], "neigen": 1, "pos": pos,
                                  "energy_last": run.records[-1].energies.tolist(),
                                  "ops": {k: v.tolist() for k, v in ops.items()},
                                  "measure": {k: run.measure(v, pos).tolist() for k, v in ops.items()}}}
    (OUT / "measure_runs.json").write_text(json.dumps(res))
    print("measure runs", {k: v["measure"]["d"][:3] for k, v in res.items()})


def c2_small():
    """A U=4, HFMODE=F Hubbard superblock (L=24, M=96) with oracle outputs."""
    p = O.Params(Ldmrg=12, Mdmrg=96, lanc_neigen=1, dmrg_qn=(0.5, 0.5))
    run = O.DMRG(O.hubbard_hij(1.0), O.electron_site(4.0, False), p, keep_setups=True)
    run.infinite()
    l, r, sb, ds, ev, evec = run.setups[-1]
    rng = np.random.default_rng(11)
    v = rng.standard_normal(sb.N)
    out = {}
    pack_block("eleft", l, out)
    pack_block("eright", r, out)
    lblocks, rblocks = O.build_density_matrices(sb, evec[:, 0], l.sectors(), r.sectors())
    rho_l = O.eigh_blocks(lblocks)
    out.update({"hij": O.hubbard_hij(1.0), "target": sb.target, "sb_qns": np.array(sb.qns),
                "sb_dls": sb.Dls, "sb_drs": sb.Drs, "sb_offset": sb.Offset, "sb_states": sb.sb_states,
                "v": v, "hv": O.spmatvec_direct(ds, v), "oracle_gs_energy": ev, "psi": evec[:, 0],
                "lam_left": rho_l.evalues, "entropy": np.array([run.records[-1].entropy_left])})
    np.savez_compressed(OUT / "c2_small.npz", **out)
    print("c2_small N", sb.N, "nsb", len(sb.qns))


if __name__ == "__main__":
    if len(sys.argv) < 2:
        sys.exit("usage: make_golden.py <reference checkout> [kat] [trajectories] [c2_small] [oracle_runs] [measure_runs]")
    ref = Path(sys.argv[1])
    parts = set(sys.argv[2:]) or {"kat", "trajectories", "c2_small", "oracle_runs", "measure_runs"}
    if "kat" in parts:
        kat(ref, "spin")
        kat(ref, "hubbard")
    if "trajectories" in parts:
        trajectories(ref)
    if "c2_small" in parts:
        c2_small()
    if "oracle_runs" in parts:
        oracle_runs()
    if "measure_runs" in parts:
        measure_runs()
