"""The host-side Hermitian eigensolver (Householder + implicit QL) behind the block Lanczos
and RIXS projected matrices: pure host code in libqgpu.so, checked against numpy."""
import ctypes
import os

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    from quanty_gb300 import build, qgpu
    if not os.path.exists(os.path.join(ROOT, "quanty_gb300", "libqgpu.so")):
        build.build()
    return qgpu.load()


def eigh(lib, A, nv):
    k = A.shape[0]
    a = np.ascontiguousarray(A, dtype=np.complex128)
    w = np.zeros(k)
    v = np.zeros((k, max(nv, 1)), dtype=np.complex128)
    assert lib.qg_hermitian_eigh(k, a.ctypes.data, w.ctypes.data, v.ctypes.data, nv) == 0
    return w, v[:, :nv]


@pytest.mark.parametrize("k", [1, 2, 3, 8, 60, 257])
def test_random_hermitian(lib, k):
    rng = np.random.default_rng(k)
    B = rng.normal(size=(k, k)) + 1j * rng.normal(size=(k, k))
    A = (B + B.conj().T) / 2
    nv = min(k, 20)
    w, v = eigh(lib, A, nv)
    scale = max(1.0, np.abs(np.linalg.eigvalsh(A)).max())
    assert np.abs(w - np.linalg.eigvalsh(A)).max() < 1e-13 * scale
    assert np.abs(A @ v - v * w[:nv]).max() < 1e-12 * scale
    assert np.abs(v.conj().T @ v - np.eye(nv)).max() < 1e-13


def test_degenerate_clusters(lib):
    rng = np.random.default_rng(1)
    Q, _ = np.linalg.qr(rng.normal(size=(40, 40)) + 1j * rng.normal(size=(40, 40)))
    d = np.repeat([1.0, 2.0, 2.0, 2.0, 5.0], 8)
    A = Q @ np.diag(d) @ Q.conj().T
    A = (A + A.conj().T) / 2
    w, v = eigh(lib, A, 40)
    assert np.abs(w - np.sort(d)).max() < 1e-13
    assert np.abs(A @ v - v * w).max() < 1e-13
    assert np.abs(v.conj().T @ v - np.eye(40)).max() < 1e-13


def test_tridiagonal_and_diagonal(lib):
    rng = np.random.default_rng(2)
    k = 90
    T = np.diag(rng.normal(size=k)) + np.diag(rng.normal(size=k - 1), 1)
    T = T + np.triu(T, 1).T
    w, v = eigh(lib, T.astype(complex), k)
    assert np.abs(w - np.linalg.eigvalsh(T)).max() < 1e-13
    assert np.abs(T @ v - v * w).max() < 1e-13
    D = np.diag([3.0, -1.0, 2.0, 0.0])
    w, v = eigh(lib, D.astype(complex), 4)
    assert list(w) == [-1.0, 0.0, 2.0, 3.0]


def test_bad_arguments(lib):
    a = np.zeros(4, dtype=np.complex128)
    w = np.zeros(2)
    assert lib.qg_hermitian_eigh(0, a.ctypes.data, w.ctypes.data, None, 0) != 0
    assert lib.qg_hermitian_eigh(2, a.ctypes.data, w.ctypes.data, None, 3) != 0
