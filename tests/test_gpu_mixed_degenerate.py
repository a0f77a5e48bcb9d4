"""The mixed method on superblocks with a near-degenerate ground state.

An open spin-1 chain carries a spin-1/2 at each end; in the Sz=0 sector
their singlet and triplet are split by ~exp(-L/6): 2.6e-4 at L=48 and
1.8e-5 at L=64 (2e-7 of |E|), close to what FP32 arithmetic resolves.  The
mixed result must still meet the FP64 residual test (tol 1e-12) and agree
with the FP64 method to 1e-13 relative, from several start vectors, on the
last infinite step of L=48, m=128 and L=64, m=512 (N ~ 2.6e4 and 4e5).
The FP64 residual ||H psi - E psi|| / |E| of the returned vector is
recomputed here with the FP64 direct product.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def nss():
    import nssdmrg_gb300 as nss
    nss.lib()
    return nss


@pytest.mark.parametrize("ldmrg,m", [(24, 128), (32, 512)])
def test_mixed_resolves_edge_state_pair(nss, ldmrg, m):
    d = nss.DMRG(nss.MODEL_HEISENBERG_ONE, ldmrg, m, dmrg_qn=(0.0, 0.0), lanc_neigen=1, lanc_niter=200,
                 lanc_tolerance=1e-12, precision=nss.NSS_PREC_FP64)
    d.prepare_last()
    s = d.sb
    ev64, _, _ = s.sb_diag(neigen=2, nitermax=300, tol=1e-12, seed=3, precision=nss.NSS_PREC_FP64)
    gap = (ev64[1] - ev64[0]) / abs(ev64[0])
    assert gap < 1e-5, gap          # a near-degenerate pair indeed
    clusters = []
    for seed in (3, 4, 5):
        ev, vec, _ = s.sb_diag(neigen=1, nitermax=300, tol=1e-12, seed=seed, precision=nss.NSS_PREC_MIXED,
                               want_vectors=True)
        v = np.ascontiguousarray(vec[:, 0])
        hv = s.spmatvec(v)
        assert np.linalg.norm(hv - ev[0] * v) <= 1e-11 * abs(ev[0])
        assert abs(ev[0] - ev64[0]) <= 1e-13 * abs(ev64[0]), (seed, ev[0], ev64[0])
        passes, cluster, fallbacks = s.refine_stats()
        clusters.append(cluster)
        assert fallbacks == 0
    assert max(clusters) >= 2       # the pair was refined together
