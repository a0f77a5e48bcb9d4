"""CUDA-graph replay of the Lanczos chunks.

Where an iteration is several launches (the FP64 method, and the mixed
method's FP32 phase when sectors run on the tensor-core GEMM) the first
chunk of four iterations runs as launches and is captured; later chunks
replay the graph, with the step counter and the input vector of H*psi on the
device.  The replayed iterations are the same kernels on the same data, so
a solve gives bit-identical eigenvalues, vectors and product counts with
graphs (default) and without them (NSS_GRAPH=0).
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


def _upload(nss, name):
    z = load_npz(name)
    l, r = unpack_block("eleft", z), unpack_block("eright", z)
    sb = O.sb_get_states(l, r, z["target"])
    ds = O.setup_direct(l, r, sb, z["hij"])
    s = nss.Superblock()
    terms = [(t.it - 1, t.isb, t.jsb, t.hconj, t.A, t.B, t.row_offset, t.col_offset) for t in ds.terms]
    s.upload(ds.sb.Dls, ds.sb.Drs, ds.sb.Offset, ds.Hleft, ds.Hright, terms, ds.tNso, l.dim, r.dim,
             ds.sb.AI, ds.sb.BI)
    return s, z


@pytest.mark.parametrize("name", ["kat_spin.npz", "c2_small.npz"])
def test_fp64_chunks_replayed_as_graphs_match_launches(nss, monkeypatch, name):
    out = {}
    for g in ("0", "1"):
        monkeypatch.setenv("NSS_GRAPH", g)
        s, z = _upload(nss, name)
        ev, vec, numop = s.sb_diag(neigen=1, tol=1e-12)
        out[g] = (ev.copy(), vec.copy(), numop, s.graph_stats())
        s.close()
    (e0, v0, n0, g0), (e1, v1, n1, g1) = out["0"], out["1"]
    print(f"{name}: {n1} products, graphs {g1}")
    assert g0 == (0, 0)
    assert g1[1] == 1 and g1[0] >= 1          # captured once, replayed
    assert n0 == n1
    np.testing.assert_array_equal(e0, e1)
    np.testing.assert_array_equal(v0, v1)
    np.testing.assert_allclose(e1, z["oracle_gs_energy"][:1], rtol=1e-12, atol=0)


def test_tensor_core_fp32_phase_replayed_as_graphs(nss, monkeypatch):
    """The mixed method's FP32 phase with every sector of >= 32 left states on
    the tensor-core GEMM (a fork onto the side stream inside each H*psi) on
    the spin-1 L=32 m=256 superblock."""
    d = nss.DMRG(nss.MODEL_HEISENBERG_ONE, 16, 256, dmrg_qn=(0.0, 0.0), lanc_neigen=1)
    d.prepare_last()
    desc = d.export_superblock()
    monkeypatch.setenv("NSS_TC_MIN_DL", "32")
    out = {}
    for g in ("0", "1"):
        monkeypatch.setenv("NSS_GRAPH", g)
        s = nss.Superblock()
        s.upload_desc(desc)
        ev, _, numop = s.sb_diag(neigen=1, tol=1e-12, precision=nss.NSS_PREC_MIXED, want_vectors=False)
        out[g] = (ev.copy(), numop, s.graph_stats())
        s.close()
    d.close()
    (e0, n0, g0), (e1, n1, g1) = out["0"], out["1"]
    print(f"spin1_L32_M256 mixed TC: {n1} products, graphs {g1}")
    assert g0 == (0, 0) and g1[0] >= 1
    assert n0 == n1
    np.testing.assert_array_equal(e0, e1)
