"""Host tridiagonal solver of the Lanczos check (nss_tridiag_lowest), on CPU.

nss_eigh hands T_m to this solver every few Lanczos steps (the reference
hands it to ARPACK, src/DMRG_SUPERBLOCK.f90:412-425); here it is compared
with LAPACK's tridiagonal eigensolver through scipy."""
import numpy as np
import pytest

scipy_linalg = pytest.importorskip("scipy.linalg")

import nssdmrg_gb300 as nss


def _check(a, b, ne, tol_rel=1e-13):
    m = a.size
    b_last = 0.37
    theta, s, resid = nss.tridiag_lowest(a, b, ne, b_last)
    ref = scipy_linalg.eigh_tridiagonal(a, b, eigvals_only=True)
    tn = max(np.abs(ref).max(), 1e-300)
    assert np.allclose(theta, ref[:ne], rtol=0, atol=tol_rel * tn), (theta, ref[:ne])
    T = np.diag(a) + np.diag(b, 1) + np.diag(b, -1)
    for e in range(ne):
        v = s[e]
        assert abs(np.linalg.norm(v) - 1.0) < 1e-13
        assert np.linalg.norm((T / tn) @ v - (theta[e] / tn) * v) <= 1e-12
        assert v[np.argmax(np.abs(v))] > 0
        assert resid[e] == pytest.approx(abs(b_last * v[-1]), rel=1e-14, abs=1e-300)
    if ne > 1:
        G = s @ s.T
        assert np.abs(G - np.eye(ne)).max() < 1e-10


@pytest.mark.parametrize("m", [1, 2, 3, 7, 40, 133, 512])
@pytest.mark.parametrize("ne", [1, 4])
def test_random_tridiagonal(m, ne):
    rng = np.random.default_rng(m * 10 + ne)
    a = rng.standard_normal(m) * 3.0 - 10.0
    b = np.abs(rng.standard_normal(max(m - 1, 0)))
    _check(a, b, min(ne, m))


def test_lanczos_matrix():
    """T_m of a Lanczos run on a dense symmetric matrix (well-separated low end
    plus a dense bulk), the shape nss_eigh produces."""
    rng = np.random.default_rng(7)
    n, m = 400, 90
    Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
    ev = np.concatenate([[-30.0, -29.5, -29.4], rng.uniform(-20, 20, n - 3)])
    H = (Q * ev) @ Q.T
    V = np.zeros((m + 1, n))
    a = np.zeros(m)
    b = np.zeros(m)
    V[0] = rng.standard_normal(n)
    V[0] /= np.linalg.norm(V[0])
    for j in range(m):
        w = H @ V[j]
        a[j] = V[j] @ w
        w -= a[j] * V[j] + (b[j - 1] * V[j - 1] if j else 0)
        w -= V[: j + 1].T @ (V[: j + 1] @ w)
        b[j] = np.linalg.norm(w)
        V[j + 1] = w / b[j]
    _check(a, b[:-1], 3)
    theta, _, _ = nss.tridiag_lowest(a, b[:-1], 3, b[-1])
    assert np.allclose(theta, ev[:3], rtol=1e-12)


def test_degenerate_blocks():
    """Zero couplings (a restarted Lanczos) give exactly repeated eigenvalues."""
    a = np.array([1.0, 2.0, 1.0, 2.0, 1.0, 2.0])
    b = np.array([0.5, 0.0, 0.5, 0.0, 0.5])
    _check(a, b, 4, tol_rel=1e-14)


def test_scaled_extremes():
    rng = np.random.default_rng(3)
    for scale in (1e-200, 1e-8, 1e8, 1e200):
        a = rng.standard_normal(50) * scale
        b = np.abs(rng.standard_normal(49)) * scale
        _check(a, b, 2)


def test_invalid_arguments():
    with pytest.raises(nss.NssError):
        nss.tridiag_lowest(np.zeros(3), np.zeros(2), ne=4)


def _arrow_dense(theta0, m, a, b):
    k = a.size
    M = np.zeros((k + 1, k + 1))
    M[0, 0] = theta0
    M[0, 1:] = m
    M[1:, 0] = m
    M[1:, 1:] = np.diag(a) + np.diag(b, 1) + np.diag(b, -1)
    return M


@pytest.mark.parametrize("k", [0, 1, 5, 60, 200])
def test_arrowhead_refinement_matrix(k):
    """The small problem of the anchored refinement: an FP64 anchor (row 0)
    close to the ground state, coupled by a small m to its Krylov
    complement."""
    rng = np.random.default_rng(k + 11)
    theta0 = -20.0
    a = rng.uniform(-15.0, 5.0, k)
    b = np.abs(rng.standard_normal(max(k - 1, 0)))
    m = rng.standard_normal(k) * 1e-6
    if k:
        m[0] = 3e-6
    lam, c, resid = nss.arrow_lowest(theta0, m, a, b, 0.25)
    M = _arrow_dense(theta0, m, a, b)
    w, v = np.linalg.eigh(M)
    assert lam == pytest.approx(w[0], rel=1e-15, abs=1e-14)
    ref = v[:, 0] * np.sign(v[0, 0])
    assert np.abs(c - ref).max() < 1e-12
    assert abs(np.linalg.norm(c) - 1.0) < 1e-14
    if k:
        assert resid == pytest.approx(0.25 * abs(c[-1]), rel=1e-14, abs=1e-300)


def test_arrowhead_strong_coupling():
    rng = np.random.default_rng(5)
    k = 40
    a = rng.uniform(-2.0, 2.0, k)
    b = np.abs(rng.standard_normal(k - 1))
    m = rng.standard_normal(k)
    lam, c, _ = nss.arrow_lowest(0.5, m, a, b)
    w, v = np.linalg.eigh(_arrow_dense(0.5, m, a, b))
    assert lam == pytest.approx(w[0], rel=1e-13)
    assert np.abs(np.abs(c) - np.abs(v[:, 0])).max() < 1e-10


@pytest.mark.parametrize("n", [1, 2, 5, 40, 305])
@pytest.mark.parametrize("kind", ["random", "clustered"])
def test_tridiag_eig_matches_lapack(n, kind):
    """Host implicit QL (nss_tridiag_eig, the flagged-rho-block fallback)
    against LAPACK's tridiagonal eigensolver: eigenvalues at 1e-13 of the
    norm, eigenvectors orthonormal to 1e-12 with residuals below 1e-12 of the
    norm, also for a third of the diagonal in an exactly degenerate cluster
    (the noise-level states the truncation keeps)."""
    rng = np.random.default_rng(n + (0 if kind == "random" else 1000))
    d = rng.standard_normal(n)
    e = rng.standard_normal(max(n - 1, 0))
    if kind == "clustered" and n > 3:
        k = n // 3
        d[:k] = 1e-17 * np.arange(k)
        e[:k] = 0.0
    ev, Z = nss.tridiag_eig(d, e)
    ref = scipy_linalg.eigh_tridiagonal(d, e, eigvals_only=True)
    T = np.diag(d) + np.diag(e, 1) + np.diag(e, -1)
    tn = max(np.abs(ref).max(), 1e-300)
    assert np.all(np.diff(ev) >= 0)
    np.testing.assert_allclose(ev, ref, rtol=0, atol=1e-13 * tn)
    assert np.abs(Z.T @ Z - np.eye(n)).max() <= 1e-12
    assert np.abs(T @ Z - Z * ev).max() <= 1e-12 * tn
