"""Eigensystem on the GPU: restarted block Lanczos against the Mathematica eigenvalues of
TestScripts/Eigensystem.Quanty and the reference's ground energies (1e-10 eV)."""
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


def test_fshell_atom_eigenvalues(api):
    g = golden("fshell_eigen.json")
    H = api.Operator.from_fixture(g["H"])
    psis, E = api.Eigensystem(H, [14, 0, ["11111111111111", 6, 6]], 10, {"Zero": 1e-14})
    assert np.max(np.abs(E - np.array(g["expected_mathematica"]))) < 1e-10
    # eigenvectors: <psi|H|psi> = E and orthonormal
    for p, e in zip(psis, E):
        assert abs(p.norm() - 1) < 1e-10
        assert abs(api.PsiOperatorPsi(H, p).real - e) < 1e-10


@pytest.mark.parametrize("fx,key", [("c0_xas.json", "energies_dense"), ("c1_lf.json", "energies_krylov")])
def test_ground_energies(api, fx, key):
    g = golden(fx)
    H = api.Operator.from_fixture(g["H"])
    R = [len(g["restrictions"][0][0]), 0] + [list(r) for r in g["restrictions"]]
    psis, E = api.Eigensystem(H, R, 3, {"Zero": 1e-14, "DenseBorder": 0})  # block Lanczos
    assert np.max(np.abs(E - np.array(g[key]))) < 1e-10, (E, g[key])


@pytest.mark.parametrize("fx", ["c0_xas.json", "c1_lf.json"])
def test_dense_eigensystem(api, fx):
    """Bases within DenseBorder take the dense branch (BlockLanczosGroundStateConserveBasisDense,
    Core/BlockLanczos.cpp:370): the reference's dense energies to 1e-10 eV."""
    g = golden(fx)
    H = api.Operator.from_fixture(g["H"])
    R = [H.nf, 0] + [list(r) for r in g["restrictions"]]
    psis, E = api.Eigensystem(H, R, 3, {"DenseBorder": 100000})
    assert np.max(np.abs(np.array(E) - np.array(g["energies_dense"]))) < 1e-10
    for p, e in zip(psis, E):
        assert abs(api.PsiOperatorPsi(H, p).real / p.norm() ** 2 - e) < 1e-10


def test_basis_grows_beyond_the_start_restrictions(api):
    """Start restrictions that allow only d8 L10 on the ligand-field ion: without the
    Restrictions option the basis grows under the hybridisation into d9 L9 and d10 L8, as the
    reference's growth loop does; with it the states stay confined; the second call form starts
    from given states and replaces them by as many eigenstates (1e-10 eV against the reference)."""
    g = golden("eigen_growth.json")
    H = api.Operator.from_fixture(golden("c1_lf.json")["H"])
    Rn = [26, 0] + [list(r) for r in g["start_restrictions"]]
    _, E = api.Eigensystem(H, Rn, 3)
    assert np.max(np.abs(np.array(E) - np.array(g["energies_grown"]))) < 1e-10
    psis, E = api.Eigensystem(H, Rn, 3, {"Restrictions": Rn})
    assert np.max(np.abs(np.array(E) - np.array(g["energies_confined"]))) < 1e-10
    out, E = api.Eigensystem(H, psis)
    assert len(out) == 3
    assert np.max(np.abs(np.array(E) - np.array(g["energies_from_states"]))) < 1e-10
