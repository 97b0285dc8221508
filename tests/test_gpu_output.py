"""Spectra computed here, written in the reference's file format, against the files the
reference wrote for the same calls (tests/golden/gen/print_fmt.lua): the same layout, the same
windows (given and defaulted from the pole range), values to 1e-8 relative."""
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
    "print_lanczos": (2, {"Emin": -10, "Emax": 20, "NE": 16, "Gamma": 0.5, "Method": "Lanczos", "Epsilon": 0.0}),
    "print_defaults": (1, {"NE": 12, "Method": "Lanczos", "Epsilon": 0.0}),
    "print_dense": (1, {"NE": 12, "Method": "Dense"}),
}


@pytest.mark.parametrize("key", list(CALLS))
def test_spectra_files_match_reference(api, key):
    g = golden("print_fmt.json")
    HX = api.Operator.from_fixture(g["HX"])
    Tz = api.Operator.from_fixture(g["Tz"])
    npsi, o = CALLS[key]
    psis = [api.Wavefunction.from_fixture(p) for p in g["psi"][:npsi]]
    S, _ = api.CreateSpectra(HX, [Tz], psis, o)
    text = S.Print()
    ref_text = g[key]
    mine, ref = text.splitlines(), ref_text.splitlines()
    assert len(mine) == len(ref) and mine[0] == ref[0] and mine[4] == ref[4]
    assert [len(a) for a in mine] == [len(b) for b in ref]
    R, M = api.Spectra.from_text(ref_text), api.Spectra.from_text(text)
    for a, b in ((M.Emin, R.Emin), (M.Emax, R.Emax), (M.Gamma, R.Gamma), (M.EminPole, R.EminPole),
                 (M.EmaxPole, R.EmaxPole)):
        assert abs(a - b) <= 1e-8 * max(1.0, abs(b))
    assert np.max(np.abs(M.G - R.G)) < 1e-8 * np.max(np.abs(R.G))
