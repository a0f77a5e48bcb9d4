"""CUDA path against the oracle on identical inputs, through the C ABI.

Tolerances: H*v and rho eigenvalues are FP64 sums in a different order than
the oracle's, bounded here at 1e-12 relative to the largest entry; energies
at 1e-12 relative (the reference's own assertion for the spin model).
Sector enumeration and block indexing are integer work: bit-exact.
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


def _setup(z):
    l, r = unpack_block("eleft", z), unpack_block("eright", z)
    sb = O.sb_get_states(l, r, z["target"])
    ds = O.setup_direct(l, r, sb, z["hij"])
    return l, r, sb, ds


def _upload(nss, sbo, l, r, ds):
    terms = [(t.it - 1, t.isb, t.jsb, t.hconj, t.A, t.B, t.row_offset, t.col_offset) for t in ds.terms]
    sbo.upload(ds.sb.Dls, ds.sb.Drs, ds.sb.Offset, ds.Hleft, ds.Hright, terms, ds.tNso, l.dim, r.dim,
               ds.sb.AI, ds.sb.BI)


def _blocks(blk):
    d = {"basis": blk.basis}
    for k, (m, _) in blk.ops.items():
        d[k] = m
    return d


@pytest.mark.parametrize("name", ["kat_spin.npz", "kat_hubbard.npz", "c2_small.npz"])
def test_hv_upload_path_matches_oracle(nss, name):
    z = load_npz(name)
    l, r, sb, ds = _setup(z)
    s = nss.Superblock()
    _upload(nss, s, l, r, ds)
    assert s.n == sb.N
    hv = s.spmatvec(z["v"])
    ref = z["hv"]
    assert np.abs(hv - ref).max() <= 1e-12 * np.abs(ref).max()


@pytest.mark.parametrize("name", ["kat_spin.npz", "kat_hubbard.npz", "c2_small.npz"])
def test_block_setup_enumeration_is_bit_exact(nss, name):
    z = load_npz(name)
    l, r = unpack_block("eleft", z), unpack_block("eright", z)
    s = nss.Superblock()
    st = nss.NSS_SITE_FERMION if l.sitetype == "fermion" else nss.NSS_SITE_SPIN
    s.setup(st, _blocks(l), _blocks(r), z["target"], z["hij"])
    qns, dls, drs, off, states = s.tables()
    np.testing.assert_array_equal(qns, z["sb_qns"])
    np.testing.assert_array_equal(dls, z["sb_dls"])
    np.testing.assert_array_equal(drs, z["sb_drs"])
    np.testing.assert_array_equal(off, z["sb_offset"])
    np.testing.assert_array_equal(states, z["sb_states"])
    hv = s.spmatvec(z["v"])
    assert np.abs(hv - z["hv"]).max() <= 1e-12 * np.abs(z["hv"]).max()


def test_hv_is_linear_and_symmetric(nss):
    z = load_npz("c2_small.npz")
    l, r, sb, ds = _setup(z)
    s = nss.Superblock()
    _upload(nss, s, l, r, ds)
    rng = np.random.default_rng(5)
    u, v = rng.standard_normal(sb.N), rng.standard_normal(sb.N)
    hu, hv = s.spmatvec(u), s.spmatvec(v)
    huv = s.spmatvec(2.0 * u - 3.0 * v)
    scale = np.abs(hu).max() + np.abs(hv).max()
    assert np.abs(huv - (2.0 * hu - 3.0 * hv)).max() <= 1e-12 * scale
    assert abs(u @ hv - v @ hu) <= 1e-11 * scale * np.sqrt(sb.N)


@pytest.mark.parametrize("name,neigen", [("kat_spin.npz", 2), ("kat_hubbard.npz", 1)])
def test_eigh_matches_energy_check(nss, name, neigen):
    z = load_npz(name)
    l, r, sb, ds = _setup(z)
    s = nss.Superblock()
    _upload(nss, s, l, r, ds)
    ev, vec, numop = s.sb_diag(neigen=neigen, tol=1e-12)
    current_l = l.length + r.length
    np.testing.assert_allclose(ev / current_l, z["golden_energy"], rtol=1e-12, atol=0)
    # the Ritz vectors are normalised eigenvectors to the tolerance
    hv = s.spmatvec(vec[:, 0])
    assert np.linalg.norm(hv - ev[0] * vec[:, 0]) <= 1e-9 * abs(ev[0])
    assert abs(np.linalg.norm(vec[:, 0]) - 1.0) < 1e-12
    assert 0 < numop <= 512


@pytest.mark.parametrize("name", ["kat_spin.npz", "kat_hubbard.npz"])
def test_rdm_of_given_state_matches_oracle(nss, name):
    z = load_npz(name)
    l, r, sb, ds = _setup(z)
    s = nss.Superblock()
    _upload(nss, s, l, r, ds)
    mst = int(z["params"][1])
    res = s.sb_get_rdm(mst, 0.1, psi=z["psi"])
    np.testing.assert_allclose(res.lambdas[0], z["lam_left"], rtol=0, atol=1e-13)
    np.testing.assert_allclose(res.lambdas[1], z["lam_right"], rtol=0, atol=1e-13)
    assert list(res.m_s) == [int(x) for x in z["ms"]]
    np.testing.assert_allclose(res.trunc_err, z["trunc"], rtol=0, atol=1e-13)
    np.testing.assert_allclose(res.entropy, z["entropy"], rtol=1e-11, atol=0)
    # U has orthonormal columns and spans kept blocks only
    for side in (0, 1):
        u = res.u[side]
        assert np.allclose(u.T @ u, np.eye(u.shape[1]), atol=1e-12)


@pytest.mark.parametrize("name", ["kat_spin.npz", "kat_hubbard.npz", "c2_small.npz"])
def test_full_solve_entropy_matches_oracle(nss, name):
    z = load_npz(name)
    l, r, sb, ds = _setup(z)
    s = nss.Superblock()
    _upload(nss, s, l, r, ds)
    ev, vec, _ = s.sb_diag(neigen=1, tol=1e-12, want_vectors=False)
    np.testing.assert_allclose(ev[0], z["oracle_gs_energy"][0], rtol=1e-12, atol=0)
    res = s.sb_get_rdm(64, 0.1)
    np.testing.assert_allclose(res.lambdas[0], z["lam_left"], rtol=0, atol=1e-10)
    np.testing.assert_allclose(res.entropy[0], z["entropy"][0], rtol=1e-9, atol=0)


def test_errors_are_status_codes(nss):
    s = nss.Superblock()
    with pytest.raises(nss.NssError) as e:
        s.spmatvec(np.zeros(4))
    assert e.value.code == nss.NSS_ERR_STATE
    z = load_npz("kat_spin.npz")
    l, r, sb, ds = _setup(z)
    bad = list(ds.sb.Offset)
    bad[1] += 1
    terms = [(t.it - 1, t.isb, t.jsb, t.hconj, t.A, t.B, t.row_offset, t.col_offset) for t in ds.terms]
    with pytest.raises(nss.NssError) as e:
        s.upload(ds.sb.Dls, ds.sb.Drs, bad, ds.Hleft, ds.Hright, terms, ds.tNso, l.dim, r.dim)
    assert e.value.code == nss.NSS_ERR_INVALID
    _upload(nss, s, l, r, ds)
    with pytest.raises(nss.NssError) as e:
        s.spmatvec(np.zeros(sb.N + 1))
    assert e.value.code == nss.NSS_ERR_INVALID


def test_tiny_superblock_exhausts_krylov_space(nss):
    """First iDMRG step: N=6; the Krylov space is the whole space."""
    dot = O.spin_site(2)
    l = O.enlarge_block(dot, dot, "l", O.heisenberg_hij())
    r = O.enlarge_block(dot, dot, "r", O.heisenberg_hij())
    sb = O.sb_get_states(l, r, np.array([0.0]))
    ds = O.setup_direct(l, r, sb, O.heisenberg_hij())
    s = nss.Superblock()
    _upload(nss, s, l, r, ds)
    ev, vec, numop = s.sb_diag(neigen=2, tol=1e-12)
    h = O.sparse_superblock_h(l, r, sb, O.heisenberg_hij()).toarray()
    ref = np.linalg.eigvalsh(h)[:2]
    np.testing.assert_allclose(ev, ref, rtol=1e-12, atol=1e-12)
    assert numop <= sb.N


@pytest.mark.parametrize("name,neigen", [("kat_spin.npz", 2), ("kat_hubbard.npz", 1), ("c2_small.npz", 1)])
def test_mixed_precision_energy_within_1e10(nss, name, neigen):
    """Mixed method: FP32 H*psi and Krylov basis, FP64 alpha/beta, FP64
    Rayleigh-quotient refinement; |dE|/|E| <= 1e-10 against the FP64 oracle."""
    z = load_npz(name)
    l, r, sb, ds = _setup(z)
    s = nss.Superblock()
    _upload(nss, s, l, r, ds)
    ev, vec, numop = s.sb_diag(neigen=neigen, tol=1e-12, precision=nss.NSS_PREC_MIXED)
    ref = z["oracle_gs_energy"][:neigen]
    np.testing.assert_allclose(ev, ref, rtol=1e-10, atol=0)
    # the refined Ritz vector is an eigenvector to FP32-level accuracy
    hv = s.spmatvec(vec[:, 0])
    assert np.linalg.norm(hv - ev[0] * vec[:, 0]) <= 1e-5 * abs(ev[0])
    res = s.sb_get_rdm(64, 0.1)
    assert abs(res.entropy[0] - z["entropy"][0]) <= 1e-5 * abs(z["entropy"][0])


@pytest.fixture(scope="module")
def c2_superblock(nss):
    """Last infinite step of the Hubbard L=32, U=4, M=256 chain (the
    benchmark superblock: N=65 900, sectors up to 120 x 120).  Its context
    sends sectors with Dl >= 64 to the tensor-core kernel (the default
    threshold would leave it unused at this size)."""
    import os
    old = os.environ.get("NSS_TC_MIN_DL")
    os.environ["NSS_TC_MIN_DL"] = "64"
    try:
        d = nss.DMRG(nss.MODEL_HUBBARD, 16, 256, u=4.0, hfmode=False, dmrg_qn=(0.5, 0.5), lanc_neigen=1)
    finally:
        if old is None:
            del os.environ["NSS_TC_MIN_DL"]
        else:
            os.environ["NSS_TC_MIN_DL"] = old
    d.prepare_last()
    return d


def test_fp32_and_tensor_core_products_match_fp64(nss, c2_superblock):
    """The mixed path's product (tcgen05 3xTF32 tiles for sectors with
    Dl >= 64, FP32 CUDA-core tiles for the rest) against the FP64 product on
    the same superblock: FP32-class accuracy, 4e-6 of the largest entry
    (a few hundred FP32 products per output, with cancellation; the solve
    below does not depend on it, its vector is refined against FP64)."""
    import torch
    sb = c2_superblock.sb
    n = sb.n
    g = torch.Generator(device="cuda").manual_seed(3)
    v64 = torch.rand(n, dtype=torch.float64, device="cuda", generator=g) * 2 - 1
    v32 = v64.float()
    h64 = torch.empty_like(v64)
    h32 = torch.empty_like(v32)
    sb.hv_device(v64.data_ptr(), h64.data_ptr())
    sb.hv_device_f32(v32.data_ptr(), h32.data_ptr())
    torch.cuda.synchronize()
    err = (h32.double() - h64).abs().max().item() / h64.abs().max().item()
    assert err <= 4e-6, err
    # the mixed solve on this superblock: |dE|/|E| <= 1e-10 against FP64
    e64, _, _ = sb.sb_diag(neigen=1, tol=1e-12, want_vectors=False)
    emx, _, _ = sb.sb_diag(neigen=1, tol=1e-12, want_vectors=False, precision=nss.NSS_PREC_MIXED)
    assert abs(emx[0] - e64[0]) <= 1e-10 * abs(e64[0])


@pytest.fixture(scope="module")
def spin1_superblock_desc(nss):
    """Last infinite step of the spin-1 chain L=32, m=256 (sectors up to ~190
    states: two 128-row tiles per sector on the tensor cores)."""
    d = nss.DMRG(nss.MODEL_HEISENBERG_ONE, 16, 256, dmrg_qn=(0.0, 0.0), lanc_neigen=1)
    d.prepare_last()
    yield d.export_superblock()
    d.close()


@pytest.mark.parametrize("bn,split", [(64, 1), (64, 0), (128, 1), (128, 0)])
@pytest.mark.parametrize("case", ["hubbard_L32_M256", "spin1_L32_M256"])
def test_tensor_core_tiles_match_fp64(nss, c2_superblock, spin1_superblock_desc, monkeypatch, case, bn, split):
    """The TMA-fed tcgen05 sector GEMM (3xTF32, every sector with Dl >= 32
    routed to it) for each tile width and K-loop split, against the FP64
    product on the same superblock: FP32-class accuracy, 4e-6 of the largest
    entry (few-hundred-term FP32 sums with cancellation)."""
    import torch
    desc = c2_superblock.export_superblock() if case.startswith("hubbard") else spin1_superblock_desc
    monkeypatch.setenv("NSS_TC_MIN_DL", "32")
    monkeypatch.setenv("NSS_TC_BN", str(bn))
    monkeypatch.setenv("NSS_TC_SPLIT", str(split))
    s = nss.Superblock()
    s.upload_desc(desc)
    ref = nss.Superblock()
    monkeypatch.setenv("NSS_TC_MIN_DL", "0")
    ref.upload_desc(desc)
    n = s.n
    g = torch.Generator(device="cuda").manual_seed(7)
    for call in range(2):
        v64 = torch.rand(n, dtype=torch.float64, device="cuda", generator=g) * 2 - 1
        v32 = v64.float()
        h64 = torch.empty_like(v64)
        h32 = torch.empty_like(v32)
        c32 = torch.empty_like(v32)
        s.hv_device(v64.data_ptr(), h64.data_ptr())
        s.hv_device_f32(v32.data_ptr(), h32.data_ptr())
        ref.hv_device_f32(v32.data_ptr(), c32.data_ptr())
        torch.cuda.synchronize()
        scale = h64.abs().max().item()
        err = (h32.double() - h64).abs().max().item() / scale
        err_cc = (c32.double() - h64).abs().max().item() / scale
        print(f"{case} bn={bn} split={split}: tensor-core {err:.2e}, CUDA-core {err_cc:.2e}")
        assert err <= 4e-6, err


def test_precision_modes_alternate_on_one_context(nss):
    """FP64 and mixed solves share a context's buffers; switching back and
    forth must re-shape them (the FP64 basis is larger than the mixed
    path's FP64 scratch)."""
    z = load_npz("c2_small.npz")
    l, r, sb, ds = _setup(z)
    s = nss.Superblock()
    _upload(nss, s, l, r, ds)
    ref = z["oracle_gs_energy"][0]
    for prec in (nss.NSS_PREC_MIXED, nss.NSS_PREC_FP64, nss.NSS_PREC_MIXED, nss.NSS_PREC_FP64):
        ev, _, _ = s.sb_diag(neigen=1, tol=1e-12, want_vectors=False, precision=prec)
        assert abs(ev[0] - ref) <= 1e-10 * abs(ref)


@pytest.mark.parametrize("name", ["kat_spin.npz", "kat_hubbard.npz", "c2_small.npz"])
@pytest.mark.parametrize("estates", [1e-3, 1e-5, 1e-8])
def test_rdm_error_threshold_rule_matches_oracle(nss, name, estates):
    """The Edmrg rule (Mstates = 0, Estates != 0; src/DMRG_RDM.f90:206-208 and
    :279-281): m_s is the first minimum of |1 - cumulate(lambda) - Estates|,
    then the degeneracy extension.  On a given state against the oracle's
    restatement: m_s exact, truncation error to 1e-13."""
    z = load_npz(name)
    l, r, sb, ds = _setup(z)
    s = nss.Superblock()
    _upload(nss, s, l, r, ds)
    psi = z["psi"]
    res = s.sb_get_rdm(0, 0.1, psi=psi, want_u=True, estates=estates)
    lb, rb = O.build_density_matrices(sb, psi, l.sectors(), r.sectors())
    for side, blocks, dim in ((0, lb, l.dim), (1, rb, r.dim)):
        rho = O.eigh_blocks(blocks)
        m_s, eps = O.truncation(rho, 0, dim, 0.1, estates)
        assert res.m_s[side] == m_s, (side, res.m_s[side], m_s)
        assert abs(res.trunc_err[side] - eps) <= 1e-13, (side, res.trunc_err[side], eps)
        u = res.u[side]
        assert u.shape == (dim, m_s)
        assert np.allclose(u.T @ u, np.eye(m_s), atol=1e-12)


def test_rdm_without_threshold_is_refused(nss):
    """Mstates = Estates = 0 stops the reference ("Mdmrg=Edmrg=0 can not fix
    a threshold for the RDM"); here it is NSS_ERR_INVALID."""
    z = load_npz("kat_spin.npz")
    l, r, sb, ds = _setup(z)
    s = nss.Superblock()
    _upload(nss, s, l, r, ds)
    with pytest.raises(nss.NssError) as ei:
        s.sb_get_rdm(0, 0.1, psi=z["psi"], estates=0.0)
    assert ei.value.code == nss.NSS_ERR_INVALID and "Edmrg" in str(ei.value)
