"""Row cache of the persistent Lanczos kernel (k_chunk32).

Each CTA keeps its rows of the work vector and of the first basis vectors
in shared memory; columns beyond the cache come from global memory.  The
cached dots run one warp per column (another summation order than the
multi-column form of the uncached path), so a mixed solve with the cache
(default) and without it (NSS_CHUNK_CACHE=0) agree to rounding: the same
energy to 1e-12 relative, both within 1e-10 of the FP64 solve, product
counts within 10 %.  Two superblocks: the Hubbard L=32 m=256 benchmark
superblock (434 rows per CTA: the whole basis of a solve fits the cache)
and the spin-1 L=64 m=512 one (2.6k rows per CTA: about a dozen vectors
cached, the rest from global memory).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def nss():
    import nssdmrg_gb300 as nss
    nss.lib()
    return nss


def _desc(nss, case):
    if case == "hubbard_L32_M256":
        d = nss.DMRG(nss.MODEL_HUBBARD, 16, 256, u=4.0, hfmode=False, dmrg_qn=(0.5, 0.5), lanc_neigen=1)
    else:
        d = nss.DMRG(nss.MODEL_HEISENBERG_ONE, 32, 512, dmrg_qn=(0.0, 0.0), lanc_neigen=1)
    d.prepare_last()
    return d   # the exported description points into the run's tables: keep it open


@pytest.mark.parametrize("case", ["hubbard_L32_M256", "spin1_L64_M512"])
def test_row_cache_matches_uncached(nss, monkeypatch, case):
    run = _desc(nss, case)
    desc = run.export_superblock()
    monkeypatch.setenv("NSS_TC_MIN_DL", "0")   # all sectors on CUDA cores: the persistent kernel runs
    out = {}
    for cache in ("0", "1"):
        monkeypatch.setenv("NSS_CHUNK_CACHE", cache)
        s = nss.Superblock()
        s.upload_desc(desc)
        ev, _, numop = s.sb_diag(neigen=1, tol=1e-12, precision=nss.NSS_PREC_MIXED, want_vectors=False)
        out[cache] = (ev.copy(), numop, s.chunk_cache())
        if cache == "1":
            e64, _, _ = s.sb_diag(neigen=1, tol=1e-12, want_vectors=False)
        s.close()
    run.close()
    (e0, n0, c0), (e1, n1, c1) = out["0"], out["1"]
    print(f"{case}: E {e1[0]!r} / {e0[0]!r}, products {n1} / {n0}, cache {c1} / {c0}")
    assert c0 == (0, 0) and c1[0] > 0          # the cached run did use the cache
    assert abs(e1[0] - e0[0]) <= 1e-12 * abs(e0[0])
    for e in (e0, e1):
        assert abs(e[0] - e64[0]) <= 1e-10 * abs(e64[0])
    # the spin-1 superblock's end-spin pair makes the refinement's path (and
    # its product count) follow rounding: measured 230 against 217
    assert abs(n1 - n0) <= 0.1 * max(n0, n1)


def test_contexts_of_different_sizes_interleave(nss, monkeypatch):
    """The persistent kernels' shared-memory limit is a per-kernel setting
    shared by every context: a context set up for a small superblock (small
    row cache) must not shrink it under one set up for a large superblock."""
    from conftest import load_npz
    from oracle import dmrg_oracle as O
    from tests.golden.blockio import unpack_block
    monkeypatch.setenv("NSS_TC_MIN_DL", "0")
    big = _desc(nss, "hubbard_L32_M256")
    sb_big = nss.Superblock()
    sb_big.upload_desc(big.export_superblock())
    z = load_npz("kat_spin.npz")
    l, r = unpack_block("eleft", z), unpack_block("eright", z)
    sb = O.sb_get_states(l, r, z["target"])
    ds = O.setup_direct(l, r, sb, z["hij"])
    small = nss.Superblock()
    terms = [(t.it - 1, t.isb, t.jsb, t.hconj, t.A, t.B, t.row_offset, t.col_offset) for t in ds.terms]
    small.upload(ds.sb.Dls, ds.sb.Drs, ds.sb.Offset, ds.Hleft, ds.Hright, terms, ds.tNso, l.dim, r.dim,
                 ds.sb.AI, ds.sb.BI)
    e1, _, _ = sb_big.sb_diag(neigen=1, tol=1e-12, precision=nss.NSS_PREC_MIXED)
    e2, _, _ = small.sb_diag(neigen=1, tol=1e-12, precision=nss.NSS_PREC_MIXED)
    e3, _, _ = sb_big.sb_diag(neigen=1, tol=1e-12, precision=nss.NSS_PREC_MIXED)
    np.testing.assert_array_equal(e1, e3)
    np.testing.assert_allclose(e2, z["oracle_gs_energy"][:1], rtol=1e-10, atol=0)
    small.close()
    sb_big.close()
    big.close()
