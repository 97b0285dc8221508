"""CreateResonantSpectra on the GPU against the reference's RIXS spectra (1e-8 relative) on
the 16-orbital 2p -> 3d case: the dense branch the reference takes below DenseBorder, with
lists of absorption operators, emission operators and initial states and with automatic
energy ranges; the tensor form of the dense branch; the Krylov branch with lists; the Krylov
tensor form (block Lanczos in both stages) at complete and incomplete Krylov spaces."""
import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu
SPEC_TOL = 1e-8


@pytest.fixture(scope="module")
def api():
    from quanty_gb300 import build
    build.build()
    from quanty_gb300 import api
    return api


CASES = [
    # key, T1, T2, initial states, options on top of the fixture's energy grid
    ("dense_lists", ("Tx", "Ty"), ("Txd", "Tyd", "Tzd"), 2, {}),
    ("dense_auto", ("Tx",), ("Txd", "Tyd"), 1, None),
    ("dense_tensor", ("Tx", "Ty"), ("Txd", "Tyd"), 1, {"Tensor": True}),
    ("dense_tensor_psi", ("Tx",), ("Tyd",), 2, {"Tensor": True}),
    ("krylov_lists", ("Tx", "Ty"), ("Txd", "Tyd"), 2, {"DenseBorder": 0, "Epsilon": 0.0}),
    ("krylov_tensor", ("Tx", "Ty"), ("Txd", "Tyd"), 1,
     {"DenseBorder": 0, "Epsilon": 0.0, "Tensor": True, "NTri1": 40, "NTri2": 40}),
    # incomplete Krylov spaces (8 intermediate and 20 final vectors): the spectra depend on
    # both block recursions, not only on the Hamiltonians
    ("krylov_tensor_short", ("Tx", "Ty"), ("Txd", "Tyd"), 1,
     {"DenseBorder": 0, "Epsilon": 0.0, "Tensor": True, "NTri1": 4, "NTri2": 5}),
    ("krylov_tensor_short_auto", ("Tx", "Ty"), ("Txd",), 1,
     {"auto": True, "NE1": 3, "NE2": 48, "DenseBorder": 0, "Epsilon": 0.0, "Tensor": True, "NTri1": 6,
      "NTri2": 8}),
]


@pytest.mark.parametrize("key,t1,t2,npsi,extra", CASES, ids=[c[0] for c in CASES])
def test_rixs_matches_reference(api, key, t1, t2, npsi, extra):
    g = golden("rixs.json")
    op = lambda k: api.Operator.from_fixture(g[k])  # noqa: E731
    psis = [api.Wavefunction.from_fixture(p) for p in g["psi"][:npsi]]
    if extra is None:  # automatic intermediate and final energy ranges
        o = {"NE1": 4, "Gamma1": 0.8, "NE2": 64, "Gamma2": 0.3}
    elif extra.get("auto"):  # automatic ranges and default broadenings
        o = {k: v for k, v in extra.items() if k != "auto"}
    else:
        o = dict(g["opts"], **extra)
    T1 = [op(t) for t in t1] if len(t1) > 1 else op(t1[0])
    G, st = api.CreateResonantSpectra(op("HX"), op("H"), T1, [op(t) for t in t2],
                                      psis if npsi > 1 else psis[0], o)
    ref = g[key]
    R = np.array(ref["re"]) + 1j * np.array(ref["im"])
    assert G.shape == R.shape
    err = float(np.max(np.abs(G - R)) / np.max(np.abs(R)))
    assert err < SPEC_TOL, (key, err)
    assert abs(st["emin2"] - ref["emin"]) < 1e-10 and abs(st["emax2"] - ref["emax"]) < 1e-10
    assert st["method"] == ("dense" if key.startswith("dense") else "krylov_tensor" if "tensor" in key else "krylov")
