"""Tensor spectra (CreateSpectra with Tensor = true): the 3 x 3 matrix of dipole spectra of the
ground state against the reference's files for the same calls (tests/golden/gen/tensor.lua),
dense branch and block-Lanczos branch, 1e-8 relative to the largest element.  The block
Lanczos runs with a complete Krylov space (200 blocks of 3) and with incomplete ones (5 and 8
blocks), where the result depends on the block recursion itself; its pole range (the
eigenvalues of the whole block tridiagonal matrix) sets the automatic window."""
import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def api():
    from quanty_gb300 import build
    build.build()
    from quanty_gb300 import api
    return api


CALLS = {
    "tensor_dense": {"Tensor": True, "Method": "Dense", "NE": 40, "Emin": -5, "Emax": 15, "Gamma": 0.6},
    "tensor_dense_defaults": {"Tensor": True, "Method": "Dense", "NE": 24},
    "tensor_lanczos": {"Tensor": True, "Method": "Lanczos", "NE": 40, "Emin": -5, "Emax": 15, "Gamma": 0.6,
                       "Epsilon": 0.0},
    "tensor_lanczos_short": {"Tensor": True, "Method": "Lanczos", "NTri": 5, "NE": 40, "Emin": -5, "Emax": 15,
                             "Gamma": 0.6, "Epsilon": 0.0},
    "tensor_lanczos_short_auto": {"Tensor": True, "Method": "Lanczos", "NTri": 8, "NE": 32},
}


@pytest.mark.parametrize("key", list(CALLS))
def test_tensor_spectra_match_reference(api, key):
    g = golden("tensor.json")
    HX = api.Operator.from_fixture(g["HX"])
    Ts = [api.Operator.from_fixture(g[t]) for t in ("Tx", "Ty", "Tz")]
    psi = api.Wavefunction.from_fixture(g["psi"])
    S, _ = api.CreateSpectra(HX, Ts, [psi], CALLS[key])
    R = api.Spectra.from_text(g[key])
    assert S.G.shape == R.G.shape == (9, CALLS[key]["NE"] + 1)
    for a, b in ((S.Emin, R.Emin), (S.Emax, R.Emax), (S.Gamma, R.Gamma)):
        assert abs(a - b) <= 1e-8 * max(1.0, abs(b))
    assert abs(S.EminPole - R.EminPole) < 1e-8 and abs(S.EmaxPole - R.EmaxPole) < 1e-8
    assert np.max(np.abs(S.G - R.G)) < 1e-8 * np.max(np.abs(R.G))
    # the matrix is Hermitian in the sense G_ji(w) = G_ij(w) with the roles of bra and ket
    # exchanged: its Hermitian part -Im is positive semi-definite at every frequency
    M = S.G.reshape(3, 3, -1)
    for k in range(0, M.shape[2], 7):
        A = (M[:, :, k] - M[:, :, k].conj().T) / 2j
        assert np.min(np.linalg.eigvalsh(-A)) > -1e-10 * np.max(np.abs(A))
