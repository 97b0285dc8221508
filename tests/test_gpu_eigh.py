"""The device Hermitian eigensolver behind the dense paths, the block eigensolver's projected
matrices and RIXS, against numpy's LAPACK (eigenvalues ascending, eigenvectors as columns):
one-block cyclic Jacobi (k <= 40) and the tridiagonal reduction above it (Householder,
bisection, inverse iteration), degenerate multiplets, tight clusters, real tridiagonal and
diagonal matrices, eigenvalues only and the lowest few eigenvectors."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def api():
    from quanty_gb300 import build
    build.build()
    from quanty_gb300 import api
    return api


@pytest.mark.parametrize("k", [1, 2, 3, 8, 39, 40, 41, 60, 257, 700])
def test_random_hermitian(api, k):
    rng = np.random.default_rng(k)
    B = rng.normal(size=(k, k)) + 1j * rng.normal(size=(k, k))
    A = (B + B.conj().T) / 2
    nv = min(k, 20)
    w, v = api.hermitian_eigh(A, nv)
    scale = max(1.0, np.abs(np.linalg.eigvalsh(A)).max())
    assert np.abs(w - np.linalg.eigvalsh(A)).max() < 1e-13 * scale
    assert np.abs(A @ v - v * w[:nv]).max() < 1e-12 * scale
    assert np.abs(v.conj().T @ v - np.eye(nv)).max() < 1e-13


@pytest.mark.parametrize("k", [30, 120, 600])
def test_degenerate_multiplets(api, k):
    rng = np.random.default_rng(1)
    Q, _ = np.linalg.qr(rng.normal(size=(k, k)) + 1j * rng.normal(size=(k, k)))
    d = np.repeat(np.arange(k // 6, dtype=float) * 0.5, 6)[:k]
    A = Q @ np.diag(d) @ Q.conj().T
    A = (A + A.conj().T) / 2
    w, v = api.hermitian_eigh(A, k)
    assert np.abs(w - np.sort(d)).max() < 1e-13 * max(1, d.max())
    assert np.abs(A @ v - v * w).max() < 1e-12 * max(1, d.max())
    assert np.abs(v.conj().T @ v - np.eye(k)).max() < 1e-13


def test_tridiagonal_and_diagonal(api):
    rng = np.random.default_rng(2)
    k = 90
    T = np.diag(rng.normal(size=k)) + np.diag(rng.normal(size=k - 1), 1)
    T = T + np.triu(T, 1).T
    w, v = api.hermitian_eigh(T.astype(complex), k)
    assert np.abs(w - np.linalg.eigvalsh(T)).max() < 1e-13
    assert np.abs(T @ v - v * w).max() < 1e-13
    D = np.diag([3.0, -1.0, 2.0, 0.0])
    w, v = api.hermitian_eigh(D.astype(complex), 4)
    assert list(w) == [-1.0, 0.0, 2.0, 3.0]


def test_clusters_and_partial_vectors(api):
    """Eigenvalues in groups of eight within 1e-9 of one another (one inverse-iteration cluster
    each), the eigenvalues alone, and the lowest eigenvectors only."""
    rng = np.random.default_rng(5)
    k = 400
    Q, _ = np.linalg.qr(rng.normal(size=(k, k)) + 1j * rng.normal(size=(k, k)))
    d = np.sort(np.repeat(rng.normal(size=k // 8), 8) + 1e-9 * rng.normal(size=k))
    A = Q @ np.diag(d) @ Q.conj().T
    A = (A + A.conj().T) / 2
    w, v = api.hermitian_eigh(A, k)
    assert np.abs(w - d).max() < 1e-13 * np.abs(d).max()
    assert np.abs(A @ v - v * w).max() < 1e-12 * np.abs(d).max()
    assert np.abs(v.conj().T @ v - np.eye(k)).max() < 1e-13
    w0, _ = api.hermitian_eigh(A, 0)
    assert np.array_equal(w0, w)
    w16, v16 = api.hermitian_eigh(A, 16)
    assert np.array_equal(w16, w) and v16.shape == (k, 16)
    assert np.abs(A @ v16 - v16 * w[:16]).max() < 1e-12 * np.abs(d).max()
