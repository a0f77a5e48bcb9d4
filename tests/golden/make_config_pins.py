"""Oracle results at the benchmark configurations (golden fixture writer).

Runs the oracle's own infinite algorithm (oracle.dmrg_oracle, numpy/scipy)
up to the last infinite step of two benchmark chains and stops before that
step's solve, as nss_dmrg_prepare_last does on the GPU side:

  hubbard_L32_M256   Hubbard, t=1, U=4 (HFMODE=F), half filling, Ldmrg=16, Mdmrg=256
  spin1_L64_M512     spin-1 Heisenberg, J=1, Sz=0, Ldmrg=32, Mdmrg=512

That superblock is then solved by the oracle's C restatement of
spMatVec_direct_main + Lanczos (FP64, OpenMP, Ritz vector returned), and its
reduced density matrices are formed, diagonalised and truncated by the
oracle's restatement of sb_get_rdm / eigh_blocks / renormalize_block
(src/DMRG_RDM.f90:18-221, src/MATRIX/MATRIX_BLOCKS.f90:589-657) with the
entanglement entropy of write_entanglement (src/DMRG_MAIN.f90:501-518).

Writes config_pins.json next to this file: sector tables (Dls, Drs, Offset,
AI, BI), E, and per side all rho eigenvalues (descending), m_s, the
truncation error and the entropy.  Needs no reference checkout.

    python -m tests.golden.make_config_pins [hubbard_L32_M256] [spin1_L64_M512]
"""
from __future__ import annotations

import json
import os
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import dmrg_oracle as O            # noqa: E402
from oracle.cref import RefSuperblock          # noqa: E402

OUT = Path(__file__).resolve().parent / "config_pins.json"

CASES = {
    "hubbard_L32_M256": {"model": "hubbard", "ldmrg": 16, "mdmrg": 256, "u": 4.0, "hfmode": False,
                         "dmrg_qn": [0.5, 0.5]},
    "spin1_L64_M512": {"model": "heisenberg_one", "ldmrg": 32, "mdmrg": 512, "dmrg_qn": [0.0]},
}


def last_superblock(case):
    if case["model"] == "hubbard":
        hij, dot = O.hubbard_hij(1.0), O.electron_site(case["u"], case["hfmode"])
    else:
        hij, dot = O.heisenberg_hij(1.0, 1.0), O.spin_site(3)
    p = O.Params(Ldmrg=case["ldmrg"], Mdmrg=case["mdmrg"], lanc_neigen=1, dmrg_qn=tuple(case["dmrg_qn"]))
    run = O.DMRG(hij, dot, p)
    while run.left.length < p.Ldmrg - 1:
        run.step("i")
    left = O.enlarge_block(run.left, run.dot, "l", run.hij)
    right = O.enlarge_block(run.right, run.dot, "r", run.hij)
    target = O.current_target_qn(p, left.length + right.length)
    sb = O.sb_get_states(left, right, target)
    ds = O.setup_direct(left, right, sb, run.hij)
    return p, left, right, sb, ds


def rdm_side(blocks, mstates, m_block, deg):
    rho = O.eigh_blocks(blocks)
    m_s, eps = O.truncation(rho, mstates, m_block, deg)
    return {"lambda": [float(x) for x in rho.evalues], "m_s": int(m_s), "trunc_err": float(eps),
            "entropy": float(O.entropy(rho.evalues))}


def pin(name):
    case = CASES[name]
    t0 = time.perf_counter()
    p, left, right, sb, ds = last_superblock(case)
    t_build = time.perf_counter() - t0
    ref = RefSuperblock(ds, left.dim, right.dim)
    t0 = time.perf_counter()
    ev, vec, numop, rc = ref.lanczos_vectors(neigen=1, nitermax=512, tol=1e-12, seed=7,
                                             nthreads=os.cpu_count() or 1)
    t_solve = time.perf_counter() - t0
    assert rc == 0, "oracle Lanczos did not converge"
    psi = vec[:, 0]
    hv = ref.hv(psi, nthreads=os.cpu_count() or 1)
    resid = float(np.linalg.norm(hv - ev[0] * psi))
    lb, rb = O.build_density_matrices(sb, psi, left.sectors(), right.sectors())
    out = dict(case)
    out.update({
        "L": left.length + right.length, "N": int(sb.N), "nsb": len(sb.qns),
        "qns": [[float(x) for x in q] for q in sb.qns],
        "dls": [int(x) for x in sb.Dls], "drs": [int(x) for x in sb.Drs],
        "offset": [int(x) for x in sb.Offset],
        "ai": [int(x) for a in sb.AI for x in a], "bi": [int(x) for b in sb.BI for x in b],
        "m_left": int(left.dim), "m_right": int(right.dim),
        "energy": float(ev[0]), "numop": int(numop), "residual": resid,
        "left": rdm_side(lb, p.Mdmrg, left.dim, p.deg_evals_threshold),
        "right": rdm_side(rb, p.Mdmrg, right.dim, p.deg_evals_threshold),
        "seconds": {"build": round(t_build, 1), "solve": round(t_solve, 1)},
    })
    return out


if __name__ == "__main__":
    names = sys.argv[1:] or list(CASES)
    pins = json.loads(OUT.read_text()) if OUT.exists() else {}
    for nm in names:
        pins[nm] = pin(nm)
        r = pins[nm]
        print(nm, "N", r["N"], "E", r["energy"], "m_s", r["left"]["m_s"], r["right"]["m_s"],
              "eps", r["left"]["trunc_err"], "S", r["left"]["entropy"], r["seconds"], flush=True)
        OUT.write_text(json.dumps(pins, indent=0))
