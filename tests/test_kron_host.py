"""Host Kronecker sums of enlarge_block (nss_kron_sum), on CPU.

H = Hb + Hd + H2 of enlarge_block (src/DMRG_CONNECT.f90:75-107) is a sum of
coefficient-weighted Kronecker products (sp_kron_matrix,
src/MATRIX/MATRIX_SPARSE.f90:832-876).  Against scipy's kron summed term by
term the product is bit-exact: each entry of one term comes from a single
pair of factors, and the terms are added in the same order.  Against the
oracle's enlarge_block, which groups the connection terms first, the bar is
1e-14 relative."""
import numpy as np
import pytest
import scipy.sparse as sp

import nssdmrg_gb300 as nss
from oracle import dmrg_oracle as O


def _dense(rp, ci, va, n):
    return sp.csr_matrix((va, ci, rp), shape=(n, n)).toarray()


def _scipy_sum(terms):
    out = None
    for c, a, b in terms:
        t = c * sp.kron(a, b, format="csr")
        out = t if out is None else out + t
    return out.toarray()


@pytest.mark.parametrize("na,nb,nterms", [(1, 1, 1), (7, 3, 4), (40, 9, 6), (123, 4, 3)])
def test_random_terms_bit_exact(na, nb, nterms):
    rng = np.random.default_rng(na * 100 + nb)
    terms = [(float(rng.standard_normal()),
              sp.random(na, na, density=0.3, random_state=rng, format="csr"),
              sp.random(nb, nb, density=0.5, random_state=rng, format="csr")) for _ in range(nterms)]
    ref = _scipy_sum(terms)
    one = nss.kron_sum(terms, nthreads=1)
    many = nss.kron_sum(terms, nthreads=5)
    for k in range(3):
        assert np.array_equal(one[k], many[k])
    assert np.array_equal(_dense(*one, na * nb), ref)
    # rows are well formed and columns unique within a row
    rp, ci, _ = one
    assert rp[0] == 0 and np.all(np.diff(rp) >= 0) and rp[-1] == ci.size
    for i in range(na * nb):
        row = ci[rp[i]:rp[i + 1]]
        assert np.unique(row).size == row.size


def test_cancelling_entries_stay():
    """Like sp_sum, an entry present in a term stays when the sum cancels it."""
    a = sp.csr_matrix(np.array([[0.0, 1.0], [1.0, 0.0]]))
    b = sp.identity(3, format="csr")
    rp, ci, va = nss.kron_sum([(1.0, a, b), (-1.0, a, b)])
    assert ci.size == 6 and np.all(va == 0.0)


@pytest.mark.parametrize("sun", [2, 3])
def test_enlarged_spin_hamiltonian_matches_oracle(sun):
    hij = np.diag([1.0, 0.5])
    dot = O.spin_site(sun)
    blk = dot
    for _ in range(3):
        blk = O.enlarge_block(blk, dot, "l", hij)
    ref = O.enlarge_block(blk, dot, "l", hij).op("H").toarray()
    m, d = blk.dim, dot.dim
    spl, spd = blk.op("S_p_n"), dot.op("S_p_n")
    terms = [(1.0, blk.op("H"), sp.identity(d, format="csr")),
             (1.0, sp.identity(m, format="csr"), dot.op("H")),
             (hij[0, 0], blk.op("S_z_n"), dot.op("S_z_n")),
             (hij[1, 1], spl, spd.T.tocsr()),
             (hij[1, 1], spl.T.tocsr(), spd)]
    got = _dense(*nss.kron_sum(terms), m * d)
    assert np.abs(got - ref).max() <= 1e-14 * np.abs(ref).max()


def test_bad_terms_are_rejected():
    a = sp.identity(3, format="csr")
    with pytest.raises(nss.NssError):
        nss.kron_sum([(1.0, a, sp.identity(2, format="csr")), (1.0, sp.identity(4, format="csr"), a)])
    bad = sp.csr_matrix((np.ones(1), np.array([5]), np.array([0, 1, 1, 1])), shape=(3, 3))
    bad.indices[0] = 5   # column outside the block
    with pytest.raises(nss.NssError):
        nss.kron_sum([(1.0, bad, a)])
