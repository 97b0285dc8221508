"""The whole-calculation timing script the bench runs under the reference binary computes the
calculation the fixtures hold: its ground energies equal the fixture's dense Eigensystem
energies and its spectra, summed over the three degenerate states, equal the fixture's
(whose states were the reference's Krylov ones: only the sum over the manifold is fixed).
Runs only where the reference binary has been built (oracle/build_ref.sh)."""
import numpy as np
import pytest

from conftest import golden


def test_lf_timing_script_matches_fixture():
    from oracle import ref_quanty
    if not ref_quanty.available():
        pytest.skip("reference binary not built")
    from quanty_gb300.api import Spectra
    r = ref_quanty.time_lf(reps=1, threads=1)
    g = golden("c1_lf.json")
    assert np.max(np.abs(np.sort(r["energies"]) - np.sort(g["energies_dense"]))) < 1e-10
    assert len(r["eigensystem_s"]) == 1 and r["spectra_s"][0] > 0
    S = Spectra.from_text(r["spectra_text"])
    fx = g["spec_eps0"]
    G = np.array(fx["re"]) + 1j * np.array(fx["im"])
    assert S.G.shape == G.shape == (9, 2049)
    a, b = S.G.reshape(3, 3, -1).sum(axis=1), G.reshape(3, 3, -1).sum(axis=1)
    assert np.max(np.abs(a - b)) <= 1e-8 * np.max(np.abs(b))
