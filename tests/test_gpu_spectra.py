"""Lanczos tridiagonalisation and continued-fraction spectra on the GPU against the reference:
the golden response functions of TestScripts/CreateSpectra.Quanty (1e-12 at its omega list)
and the XAS spectra of the 16- and 26-orbital cases (1e-8 relative)."""
import math

import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu
EPS_DEFAULT = math.sqrt(np.finfo(float).eps) / 100
SPEC_TOL = 1e-8


@pytest.fixture(scope="module")
def api():
    from quanty_gb300 import build
    build.build()
    from quanty_gb300 import api
    return api


def spec_err(G, ref):
    return float(np.max(np.abs(G - ref)) / np.max(np.abs(ref)))


def test_chain_golden_response_functions(api):
    g = golden("chain_spectra.json")
    for c in g["combos"]:
        H = api.Operator.from_fixture(g[c["H"]])
        T = api.Operator.from_fixture(g[c["T"]])
        psi = api.Wavefunction.from_fixture(g[c["psi"]])
        E0 = api.PsiOperatorPsi(H, psi).real
        Tpsi = api.OperatorPsi(T, psi)
        a, b = api.LanczosTriDiagonalize(H, Tpsi, 200, EPS_DEFAULT, EPS_DEFAULT)
        a_sh = np.r_[0.0, a[1:] - E0]
        ref = c["ref_tri"]
        assert np.allclose(a_sh[1:12], ref["a"][1:12], atol=1e-10)
        assert np.allclose(b[:12], ref["b"][:12], atol=1e-10)
        got = [api.TriDiagonalMatrixToSpectrum(0.0, a_sh, b, w, w + 1.0, 1, g["gamma"])[0, 0] for w in g["omega"]]
        gold = [complex(*z) for z in c["golden_G"]]
        assert max(abs(x - y) for x, y in zip(got, gold)) < g["threshold"], (c["H"], c["T"], c["psi"])


@pytest.mark.parametrize("fx,eps_key", [("c0_xas.json", "eps0"), ("c0_xas.json", "epsdefault"), ("c1_lf.json", "eps0")])
@pytest.mark.parametrize("batched", [True, False])
def test_xas_spectra_match_reference(api, fx, eps_key, batched):
    g = golden(fx)
    HX = api.Operator.from_fixture(g["HX"])
    Ts = [api.Operator.from_fixture(g[t]) for t in ("Tx", "Ty", "Tz")]
    psis = [api.Wavefunction.from_fixture(p) for p in g["psi"]]
    o = dict(g["spectra_opts"])
    o["Method"] = "Lanczos"
    if eps_key == "eps0":
        o["Epsilon"] = 0.0
    else:
        o.pop("Epsilon", None)
    S, tri = api.CreateSpectra(HX, Ts, psis, o, batched=batched)
    ref = g["spec_" + eps_key]
    for s in range(9):
        R = np.array(ref["re"][s]) + 1j * np.array(ref["im"][s])
        assert spec_err(S.G[s], R) < SPEC_TOL, (fx, eps_key, s, spec_err(S.G[s], R))
        rt = g["tri_" + eps_key][s]
        assert abs(tri[s][1][0] - rt["b"][0]) < 1e-12
        assert abs(tri[s][0][1] - rt["a"][1]) < 1e-10


def test_cf_kernel_matches_oracle(api, oracle_mod):
    rng = np.random.default_rng(3)
    ntri, ns, ne = 150, 7, 777
    a = np.c_[np.zeros(ns), rng.normal(size=(ns, ntri))]
    b = np.abs(rng.normal(size=(ns, ntri))) + 0.1
    e0 = rng.normal(size=ns)
    G = api.TriDiagonalMatrixToSpectrum(e0, a, b, -7.0, 9.0, ne, 0.37)
    for s in range(ns):
        want = oracle_mod.cf_spectrum(a[s], b[s], e0[s], -7.0, 16.0 / ne, ne, 0.37)
        assert spec_err(G[s], want) < 1e-13


def test_lanczos_matches_oracle_coefficients(api, oracle_mod):
    """The device recursion follows the oracle's (reference) recursion step by step while the
    Krylov space is far from exhausted."""
    O = oracle_mod
    g = golden("c1_lf.json")
    HX = api.Operator.from_fixture(g["HX"])
    T = api.Operator.from_fixture(g["Tz"])
    psi = api.Wavefunction.from_fixture(g["psi"][0])
    Tpsi = api.OperatorPsi(T, psi)
    a, b = api.LanczosTriDiagonalize(HX, Tpsi, 40, 0.0, 0.5)
    ao, bo = O.lanczos_tridiag(O.Op(g["HX"]), O.WF(26, Tpsi.det, Tpsi.val), 40, 0.0, 0.5)
    assert np.allclose(a[:20], ao[:20], atol=1e-10)
    assert np.allclose(b[:20], bo[:20], atol=1e-10)


@pytest.mark.parametrize("key,eps", [("rixs", 0.0), ("rixs_default", EPS_DEFAULT)])
def test_rixs_matches_reference(api, key, eps):
    """CreateResonantSpectra on the d8 case: all incident energies and final-state Lanczos runs
    batched, against the reference's RIXS spectra (1e-8)."""
    g = golden("c0_xas.json")
    o = dict(g["rixs_opts"], Epsilon=eps, NTri1=100, NTri2=100, DenseBorder=0)
    G, st = api.CreateResonantSpectra(api.Operator.from_fixture(g["HX"]), api.Operator.from_fixture(g["H"]),
                                      api.Operator.from_fixture(g["Tx"]), [api.Operator.from_fixture(g["Tyd"])],
                                      api.Wavefunction.from_fixture(g["psi"][0]), o)
    ref = g[key]
    R = np.array(ref["re"]) + 1j * np.array(ref["im"])
    assert G.shape == R.shape
    assert spec_err(G, R) < SPEC_TOL, spec_err(G, R)


@pytest.mark.parametrize("dense_border", [0, 1513])
def test_rixs_with_empty_final_basis_gives_zero(api, dense_border):
    """Emission operators that lead out of the final-state restrictions: no determinant is
    reachable, so every RIXS spectrum vanishes (no error), in the Krylov and the dense branch."""
    g = golden("c0_xas.json")
    HX = api.Operator.from_fixture(g["HX"])
    Ts = [api.Operator.from_fixture(g[t]) for t in ("Tx", "Ty", "Tz")]
    psi = api.Wavefunction.from_fixture(g["psi"][0])
    o = {"NTri1": 20, "NTri2": 20, "NE1": 4, "Gamma1": 0.4, "NE2": 50, "Gamma2": 0.2,
         "Emin1": -5.0, "Emax1": 5.0, "Emin2": -2.0, "Emax2": 8.0,
         "Restrictions2": [16, 0, ["1111110000000000", 6, 6]], "DenseBorder": dense_border}
    G, st = api.CreateResonantSpectra(HX, HX, Ts[2], Ts, psi, o)  # T2 = absorption again: 2p4
    assert G.shape == (3 * 5, 51) and np.all(G == 0)


def test_dense_spectra_match_reference(api):
    """The dense branch (Method Dense): poles of H on the union basis, against the reference's
    dense spectra of the same call (1e-8 relative)."""
    g = golden("c0_xas.json")
    HX = api.Operator.from_fixture(g["HX"])
    Ts = [api.Operator.from_fixture(g[t]) for t in ("Tx", "Ty", "Tz")]
    psis = [api.Wavefunction.from_fixture(p) for p in g["psi"]]
    o = dict(g["spectra_opts"])
    o["Method"] = "Dense"
    S, poles = api.CreateSpectra(HX, Ts, psis, o)
    ref = g["spec_dense"]
    for s in range(9):
        R = np.array(ref["re"][s]) + 1j * np.array(ref["im"][s])
        assert spec_err(S.G[s], R) < SPEC_TOL, (s, spec_err(S.G[s], R))
    # the same call through Lanczos at epsilon 0 (exact on this basis)
    o["Method"] = "Lanczos"
    o["Epsilon"] = 0.0
    SL, _ = api.CreateSpectra(HX, Ts, psis, o)
    assert spec_err(S.G, SL.G) < SPEC_TOL
    # default options choose the dense branch on this small basis
    S2, poles2 = api.CreateSpectra(HX, Ts, psis, dict(g["spectra_opts"]))
    assert np.array_equal(S2.G, S.G) and len(poles2[0]) == 2


def test_operator_dense_matches_oracle(api, oracle_mod):
    g = golden("c0_xas.json")
    HX = api.Operator.from_fixture(g["HX"])
    psi = api.Wavefunction.from_fixture(g["psi"][0])
    b = api.closure(HX, psi.det, HX.nf)
    M = api.OperatorToDeterminantMatrix(HX, b)
    dets = b.dets_bytes()
    op = oracle_mod.Op({"nf": HX.nf, "terms": [[list(t[0]), t[1].real, t[1].imag] for t in HX.terms]})
    want = oracle_mod.dense_matrix(op, oracle_mod.WF(HX.nf, dets, np.zeros(len(dets))))
    assert np.max(np.abs(M - want)) < 1e-13 * np.max(np.abs(want))
    assert np.max(np.abs(M - M.conj().T)) < 1e-13 * np.max(np.abs(M))


def test_poles_kernel_matches_oracle(api, oracle_mod):
    rng = np.random.default_rng(4)
    ns, npole, ne = 5, 300, 901
    a = rng.normal(size=(ns, npole)) * 4
    b = np.abs(rng.normal(size=(ns, npole)))
    e0 = rng.normal(size=ns)
    G = api.ListOfPolesToSpectrum(e0, a, b, -9.0, 11.0, ne, 0.42)
    for s in range(ns):
        want = oracle_mod.poles_spectrum(a[s], b[s], e0[s], -9.0, 20.0 / ne, ne, 0.42)
        assert spec_err(G[s], want) < 1e-13


def test_lanczos_with_stored_krylov_vectors(api):
    """qg_lanczos_tridiag with krylov_dev: the coefficients are bitwise those of the run that
    keeps no vectors (the same kernels; that run replays a two-step graph, this one captures
    every step), and the stored vectors start orthonormal."""
    import torch
    from quanty_gb300 import workloads
    eng = api.engine()
    H, R, s0, info = workloads.anderson_impurity(nshell=2, hole_max=2, particle_max=2)
    b = api.closure(H, api.dets_to_bytes([s0], H.nf), H.nf, R)
    rng = np.random.default_rng(41)
    x = torch.from_numpy(rng.normal(size=(b.n, 1)) + 1j * rng.normal(size=(b.n, 1))).cuda()
    ntri = 25
    a0, b0 = api.lanczos_block(H, b, x.clone(), ntri, 0.0, 0.0, eng)
    K = torch.zeros((ntri, b.n), dtype=torch.complex128, device="cuda")
    a1, b1 = api.lanczos_block(H, b, x.clone(), ntri, 0.0, 0.0, eng, krylov=K)
    assert np.array_equal(a0, a1) and np.array_equal(b0, b1)
    torch.cuda.synchronize()
    G = (K[:6].conj() @ K[:6].T).cpu().numpy()
    assert np.max(np.abs(G - np.eye(6))) < 1e-10


def test_krylov_basis_option(api):
    """CreateSpectra with KrylovBasis: the Lanczos branch returns the reference's non-empty
    Krylov vectors (LanczosTriDiagonalizeKrylov; their count and the leading ones element by
    element, 1e-10) with its spectra (1e-8); the dense branch returns the eigenstates of H
    (energies 1e-10 eV)."""
    g = golden("krylov_basis.json")
    r = golden("rixs.json")
    HX, Tz = api.Operator.from_fixture(r["HX"]), api.Operator.from_fixture(g["Tz"])
    psi1 = api.Wavefunction.from_fixture(r["psi"][0])
    o = {"NE": 32, "Emin": -10, "Emax": 20, "Gamma": 0.5}
    ref = np.array(g["lanczos_one"]["re"]) + 1j * np.array(g["lanczos_one"]["im"])
    S, tri, K = api.CreateSpectra(HX, Tz, psi1, dict(o, Method="Lanczos", KrylovBasis=True, NTri=80))
    assert spec_err(S.G, ref) < SPEC_TOL
    assert len(K) == len(g["krylov_one"])
    for fx, k in list(zip(g["krylov_one"], K))[:12]:
        R = api.Wavefunction.from_fixture(fx)
        d = {bytes(x): v for x, v in zip(k.det, k.val)}
        assert len(k.val) == len(R.val)
        assert np.max(np.abs(np.array([d[bytes(x)] for x in R.det]) - R.val)) < 1e-10 * np.max(np.abs(R.val))
    ref = np.array(g["dense_states"]["re"]) + 1j * np.array(g["dense_states"]["im"])
    S, poles, K = api.CreateSpectra(HX, Tz, psi1, dict(o, Method="Dense", KrylovBasis=True))
    assert spec_err(S.G, ref) < SPEC_TOL
    E = np.array([api.PsiOperatorPsi(HX, k).real for k in K])
    assert len(E) == len(g["dense_energies"]) and np.max(np.abs(E - np.array(g["dense_energies"]))) < 1e-10
