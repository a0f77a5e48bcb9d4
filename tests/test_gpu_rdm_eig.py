"""The library's own FP64 block eigensolver of the reduced density matrices
(Householder tridiagonalisation, Sturm bisection, twisted-factorisation
vectors of the kept states) against numpy's eigh on the same blocks and
against the Jacobi / batched-cuSOLVER path (env NSS_RDM_EIG=library), through
the C ABI.

Tolerances: eigenvalues at 1e-13 absolute (rho has unit trace, so this is
~500 ulps of the largest eigenvalue; both paths are backward stable with
errors of a few n * eps); kept vectors orthonormal to 1e-12; the kept
subspace (projector U U^T) equal to the library path's within
100 eps ||rho|| / gap, gap the smallest distance between a kept and a
discarded eigenvalue of one block: any backward-stable eigensolver fixes
the kept space only to eps ||rho|| / gap (Davis-Kahan); truncation error and
entropy as the oracle tests.
"""
import os

import numpy as np
import pytest

from conftest import load_npz
from test_gpu_parity import _setup, _upload

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def nss():
    import nssdmrg_gb300 as nss
    nss.lib()
    return nss


def _rdm(s, mst, psi, library):
    old = os.environ.get("NSS_RDM_EIG")
    try:
        if library:
            os.environ["NSS_RDM_EIG"] = "library"
        else:
            os.environ.pop("NSS_RDM_EIG", None)
        res = s.sb_get_rdm(mst, 0.1, psi=psi)
        return res, s.rdm_stats()
    finally:
        if old is None:
            os.environ.pop("NSS_RDM_EIG", None)
        else:
            os.environ["NSS_RDM_EIG"] = old


def _blocks_of(psi, dls, drs, off):
    out = [[], []]
    for k in range(len(dls)):
        W = psi[off[k]:off[k] + dls[k] * drs[k]].reshape(dls[k], drs[k])
        out[0].append(W @ W.T)
        out[1].append(W.T @ W)
    return out


def _edge_gap(blocks, ms):
    """Smallest gap between a kept and a discarded eigenvalue of one block
    when the ms largest eigenvalues over all blocks are kept."""
    allw = sorted(((w, b) for b, blk in enumerate(blocks) for w in np.linalg.eigvalsh(blk)), key=lambda t: -t[0])
    kept, disc = allw[:ms], allw[ms:]
    lo = {}
    for w, b in kept:
        lo[b] = min(lo.get(b, np.inf), w)
    g = np.inf
    for w, b in disc:
        if b in lo:
            g = min(g, lo[b] - w)
    return g, allw[0][0]


def _check_against(res_own, res_lib, blocks):
    for side in (0, 1):
        np.testing.assert_allclose(res_own.lambdas[side], res_lib.lambdas[side], rtol=0, atol=1e-13)
        assert res_own.m_s[side] == res_lib.m_s[side]
        assert abs(res_own.trunc_err[side] - res_lib.trunc_err[side]) <= 1e-13
        assert abs(res_own.entropy[side] - res_lib.entropy[side]) <= 1e-11 * abs(res_lib.entropy[side]) + 1e-14
        u, ul = res_own.u[side], res_lib.u[side]
        assert np.abs(u.T @ u - np.eye(u.shape[1])).max() <= 1e-12
        kb, kbl = np.asarray(res_own.kept_blocks[side]), np.asarray(res_lib.kept_blocks[side])
        assert sorted(kb.tolist()) == sorted(kbl.tolist())
        # per kept block: the kept columns span the same subspace, and each
        # column is an eigenvector of the block (residual vs the block rho)
        gap, lmax = _edge_gap(blocks[side], res_own.m_s[side])
        tol = max(1e-12, 100 * 2.0**-52 * lmax / gap)
        assert np.abs(u @ u.T - ul @ ul.T).max() <= tol, (gap, tol)


@pytest.mark.parametrize("name", ["kat_spin.npz", "kat_hubbard.npz", "c2_small.npz"])
def test_own_eigensolver_matches_library_and_numpy(nss, name):
    z = load_npz(name)
    l, r, sb, ds = _setup(z)
    s = nss.Superblock()
    _upload(nss, s, l, r, ds)
    mst = int(z["params"][1]) if "params" in z else 128
    own, st_own = _rdm(s, mst, z["psi"], library=False)
    lib, st_lib = _rdm(s, mst, z["psi"], library=True)
    assert st_own[0] > 0 and st_own[1] == 0, st_own
    assert st_lib[0] == 0 and st_lib[1] > 0, st_lib
    blocks = _blocks_of(z["psi"], z["sb_dls"], z["sb_drs"], z["sb_offset"])
    _check_against(own, lib, blocks)
    # eigenvalues against numpy on the same blocks
    for side in (0, 1):
        ref = np.sort(np.concatenate([np.linalg.eigvalsh(b) for b in blocks[side]]))[::-1]
        ref = np.where(ref < 0, 0.0, ref)
        np.testing.assert_allclose(own.lambdas[side], ref, rtol=0, atol=1e-13)


def _synthetic_psi(dls, drs, off, n, rng, mode):
    """psi whose sector blocks have prescribed singular values: exact pairs
    (degenerate rho eigenvalues), pairs split at 1e-7 relative (a relative
    cluster) or a graded spectrum with random factors."""
    psi = np.zeros(n)
    for k in range(len(dls)):
        dl, dr = int(dls[k]), int(drs[k])
        kk = min(dl, dr)
        U, _ = np.linalg.qr(rng.standard_normal((dl, dl)))
        V, _ = np.linalg.qr(rng.standard_normal((dr, dr)))
        base = np.exp(-0.35 * np.arange(kk)) * (1.0 + 0.3 * rng.random(kk))
        if mode == "pairs":
            base[1::2] = base[0::2][: len(base[1::2])]
        elif mode == "near_pairs":
            base[1::2] = base[0::2][: len(base[1::2])] * (1.0 + 1e-7)
        W = (U[:, :kk] * base) @ V[:, :kk].T
        psi[off[k]:off[k] + dl * dr] = W.ravel()
    return psi / np.linalg.norm(psi)


@pytest.mark.parametrize("mode", ["graded", "pairs", "near_pairs"])
def test_own_eigensolver_degenerate_spectra(nss, mode):
    z = load_npz("c2_small.npz")
    l, r, sb, ds = _setup(z)
    s = nss.Superblock()
    _upload(nss, s, l, r, ds)
    rng = np.random.default_rng({"graded": 1, "pairs": 2, "near_pairs": 3}[mode])
    psi = _synthetic_psi(z["sb_dls"], z["sb_drs"], z["sb_offset"], len(z["psi"]), rng, mode)
    own, st_own = _rdm(s, 96, psi, library=False)
    lib, _ = _rdm(s, 96, psi, library=True)
    assert st_own[0] > 0
    _check_against(own, lib, _blocks_of(psi, z["sb_dls"], z["sb_drs"], z["sb_offset"]))


def test_own_eigensolver_rank_deficient_blocks_fall_back(nss):
    """Keeping every state of rank-deficient blocks asks for vectors of
    numerically zero eigenvalues, which the own path leaves to the library:
    the result must still be an orthonormal eigenbasis."""
    z = load_npz("kat_spin.npz")
    l, r, sb, ds = _setup(z)
    s = nss.Superblock()
    _upload(nss, s, l, r, ds)
    own, st_own = _rdm(s, 10_000, z["psi"], library=False)
    lib, _ = _rdm(s, 10_000, z["psi"], library=True)
    for side in (0, 1):
        u = own.u[side]
        assert np.abs(u.T @ u - np.eye(u.shape[1])).max() <= 1e-12
        np.testing.assert_allclose(own.lambdas[side], lib.lambdas[side], rtol=0, atol=1e-13)
        assert own.m_s[side] == lib.m_s[side]


@pytest.mark.parametrize("name", ["kat_spin.npz", "kat_hubbard.npz", "c2_small.npz"])
def test_qn_entropy_split_matches_oracle(nss, name):
    """S_N and S_c (write_entanglement, src/DMRG_MAIN.f90:523-561) from the
    device eigenvalues against the oracle's restatement on numpy's
    eigenvalues of the same blocks, at the entropy's 1e-11 relative."""
    from oracle import dmrg_oracle as O
    z = load_npz(name)
    l, r, sb, ds = _setup(z)
    s = nss.Superblock()
    _upload(nss, s, l, r, ds)
    mst = int(z["params"][1]) if "params" in z else 128
    res = s.sb_get_rdm(mst, 0.1, psi=z["psi"], want_u=False)
    blocks = _blocks_of(z["psi"], z["sb_dls"], z["sb_drs"], z["sb_offset"])
    for side in (0, 1):
        rho = O.eigh_blocks([((k,), np.arange(b.shape[0]), b) for k, b in enumerate(blocks[side])])
        sn, sc = O.qn_entropies(rho)
        assert abs(res.s_number[side] - sn) <= 1e-11 * abs(sn) + 1e-14, (side, res.s_number[side], sn)
        assert abs(res.s_config[side] - sc) <= 1e-11 * abs(sc) + 1e-14, (side, res.s_config[side], sc)
        assert abs(res.s_number[side] + res.s_config[side] - res.entropy[side]) <= 1e-12


@pytest.mark.parametrize("cluster_mem", ["shared", "global", "grid"])
def test_big_blocks_through_blocked_reduction(nss, cluster_mem, monkeypatch):
    """Rho blocks above 160 states are reduced by a thread-block cluster,
    with the block in the cluster's shared memory or (env
    NSS_TRD_CL_SHARED_MAX=0, as for blocks too large for it) in a global
    copy, or (NSS_TRD_GRID_MIN, as for blocks of 1400 states and more) by
    the whole GPU, then the same bisection and twisted vectors: against the
    library eigensolver on the spin-1 chain's last infinite step (L=32,
    m=256, blocks up to ~190)."""
    monkeypatch.delenv("NSS_TRD_GRID_MIN", raising=False)
    if cluster_mem in ("global", "grid"):
        monkeypatch.setenv("NSS_TRD_CL_SHARED_MAX", "0")
    else:
        monkeypatch.delenv("NSS_TRD_CL_SHARED_MAX", raising=False)
    if cluster_mem == "grid":
        monkeypatch.setenv("NSS_TRD_GRID_MIN", "1")
    d = nss.DMRG(nss.MODEL_HEISENBERG_ONE, 16, 256, dmrg_qn=(0.0,), lanc_neigen=1, lanc_tolerance=1e-12)
    d.prepare_last()
    s = d.sb
    desc = d.export_superblock()
    assert max(desc.dls[k] for k in range(desc.nsb)) > 160
    ev, vec, _ = s.sb_diag(neigen=1, nitermax=300, tol=1e-12, seed=5, want_vectors=True)
    psi = np.ascontiguousarray(vec[:, 0])
    # the cut at 64 states lies well above the rounding level of this
    # spectrum (at 256 it falls among eigenvalues of 1e-15, where rounding
    # decides the degeneracy extension)
    own, st_own = _rdm(s, 64, psi, library=False)
    lib, _ = _rdm(s, 64, psi, library=True)
    monkeypatch.delenv("NSS_TRD_CL_SHARED_MAX", raising=False)
    monkeypatch.delenv("NSS_TRD_GRID_MIN", raising=False)
    assert st_own[0] > 0 and st_own[1] == 0, st_own
    dls = np.array([desc.dls[k] for k in range(desc.nsb)])
    drs = np.array([desc.drs[k] for k in range(desc.nsb)])
    off = np.array([desc.offset[k] for k in range(desc.nsb)])
    _check_against(own, lib, _blocks_of(psi, dls, drs, off))


@pytest.mark.parametrize("mode", ["inverse_iteration", "host_ql"])
@pytest.mark.parametrize("name", ["kat_hubbard.npz", "c2_small.npz"])
def test_flagged_block_paths_match_library(nss, name, mode):
    """The in-house fallbacks for flagged blocks, forced onto every block:
    inverse iteration with Gram-Schmidt inside near clusters (k_vec_fb,
    NSS_RDM_REDO_ALL=1), and implicit QL of the block's tridiagonal matrix on
    the host with the device back-transformation (NSS_RDM_QL_ALL=1), against
    the library path on the same blocks."""
    z = load_npz(name)
    l, r, sb, ds = _setup(z)
    s = nss.Superblock()
    _upload(nss, s, l, r, ds)
    mst = int(z["params"][1]) if "params" in z else 128
    os.environ["NSS_RDM_REDO_ALL"] = "1"
    if mode == "host_ql":
        os.environ["NSS_RDM_QL_ALL"] = "1"
    try:
        own, st_own = _rdm(s, mst, z["psi"], library=False)
    finally:
        os.environ.pop("NSS_RDM_REDO_ALL", None)
        os.environ.pop("NSS_RDM_QL_ALL", None)
    lib, _ = _rdm(s, mst, z["psi"], library=True)
    assert st_own[2] == 0, st_own           # none left to the library
    _check_against(own, lib, _blocks_of(z["psi"], z["sb_dls"], z["sb_drs"], z["sb_offset"]))
