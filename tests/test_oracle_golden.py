"""Pin the CPU oracle (oracle/qoracle.c) against the reference.

The fixtures come from the reference Quanty binary (tests/golden/make_fixtures.py) and from
the known answers in the reference's own tests: the golden tridiagonal tables of
TestScripts/CreateSpectra.Quanty (checked at 1e-12 there) and the Mathematica eigenvalues of
TestScripts/Eigensystem.Quanty.
"""
import math

import numpy as np
import pytest

from conftest import golden

EPS_DEFAULT = math.sqrt(np.finfo(float).eps) / 100   # Core/StructDef.cpp:306


def rel_err(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


@pytest.mark.parametrize("case", [c["name"] for c in golden("hpsi_cases.json")["cases"]])
def test_operator_psi_matches_reference_order_and_values(oracle_mod, case):
    O = oracle_mod
    c = next(c for c in golden("hpsi_cases.json")["cases"] if c["name"] == case)
    H = O.Op(c["H"])
    psi = O.WF.from_fixture(c["psi"])
    out = O.operator_psi(H, psi)
    ref = O.WF.from_fixture(c["Hpsi"])
    # single-threaded reference: the basis order is the (determinant, term) visiting order
    assert np.array_equal(out.det, ref.det)
    assert rel_err(out.val, ref.val) < 1e-12
    outr = O.operator_psi(H, psi, c["restrictions"])
    refr = O.WF.from_fixture(c["Hpsir"])
    assert np.array_equal(outr.det, refr.det)
    assert rel_err(outr.val, refr.val) < 1e-12


@pytest.mark.parametrize("case", [c["name"] for c in golden("hpsi_cases.json")["cases"]])
def test_conserve_basis_is_projection_of_growing(oracle_mod, case):
    O = oracle_mod
    c = next(c for c in golden("hpsi_cases.json")["cases"] if c["name"] == case)
    H = O.Op(c["H"])
    psi = O.WF.from_fixture(c["psi"])
    y = O.apply_conserve(H, psi)
    ref = O.WF.from_fixture(c["Hpsi"]).as_dict()
    want = np.array([ref.get(bytes(r), 0.0) for r in psi.det])
    assert rel_err(y, want) < 1e-12


def test_ladder_sign_examples(oracle_mod):
    O = oracle_mod
    # c^dag_1 c^dag_0 c_1 c_0 on |1100> gives -|1100> (orbital 0 first, MSB-first bytes)
    d = O.dets_to_bytes(["1100"], 4)[0].copy()
    ops = np.array([0, 1, 0 | O.CREATION, 1 | O.CREATION], dtype=np.uint16)
    assert O.lib().qo_ladder(O._p(d), O._p(ops), 4) == -1
    assert O.bytes_to_dets([d], 4) == ["1100"]
    # c^dag_9 c_2 on 10 orbitals: crosses bytes; sign = (-1)^(#occupied between)
    d = O.dets_to_bytes(["1110000010"], 10)[0].copy()
    ops = np.array([2, 9 | O.CREATION], dtype=np.uint16)
    s = O.lib().qo_ladder(O._p(d), O._p(ops), 2)
    assert O.bytes_to_dets([d], 10) == ["1100000011"]
    # c_2: two occupied below (0,1) -> +; c^dag_9: occupied below 9 are 0,1,8 -> -
    assert s == -1


def test_chain_golden_tables(oracle_mod):
    """TestScripts/CreateSpectra.Quanty: Lanczos on the impurity + 5-site chain reproduces the
    golden response functions at the test's omega list to the test's 1e-12."""
    O = oracle_mod
    g = golden("chain_spectra.json")
    for c in g["combos"]:
        H = O.Op(g[c["H"]])
        T = O.Op(g[c["T"]])
        psi = O.WF.from_fixture(g[c["psi"]])
        Tpsi = O.operator_psi(T, psi)
        a, b = O.lanczos_tridiag(H, Tpsi, 200, EPS_DEFAULT, EPS_DEFAULT)
        # CreateSpectra returns the table shifted by -<psi|H|psi> (ShiftTriDiagonalMatrix)
        E0 = _expectation(O, H, psi)
        ref = c["ref_tri"]
        k = 12
        assert np.allclose(a[1:k] - E0, ref["a"][1:k], atol=1e-10)
        assert np.allclose(b[:k], ref["b"][:k], atol=1e-10)
        gamma = g["gamma"]
        shifted = a - np.r_[0, np.full(len(a) - 1, E0)]
        got = [O.cf_spectrum(shifted, b, 0.0, w, 0.0, 0, gamma)[0] for w in g["omega"]]
        gold = [complex(*z) for z in c["golden_G"]]
        assert max(abs(x - y) for x, y in zip(got, gold)) < g["threshold"]


def _expectation(O, H, psi):
    """<psi|H|psi> with the reference's growing-basis H*psi and hashed dot."""
    Hpsi = O.operator_psi(H, psi).as_dict()
    return float(np.real(sum(np.conj(v) * Hpsi.get(bytes(r), 0.0) for r, v in zip(psi.det, psi.val))))


def test_fshell_eigenvalues_match_mathematica(oracle_mod):
    """TestScripts/Eigensystem.Quanty f-shell atom: exact diagonalisation on the closed basis
    reproduces the Mathematica eigenvalues."""
    O = oracle_mod
    g = golden("fshell_eigen.json")
    H = O.Op(g["H"])
    basis = O.enumerate_restricted(14, g["restrictions"])
    assert len(basis.val) == math.comb(14, 6)
    w, _ = O.exact_eigensystem(H, basis, 10)
    assert np.max(np.abs(w - np.array(g["expected_mathematica"]))) < 1e-10
    assert np.max(np.abs(w - np.array(g["energies_tight"]))) < 1e-10


@pytest.mark.parametrize("fx", ["c0_xas.json", "c1_lf.json"])
def test_xas_spectra_match_reference(oracle_mod, fx):
    O = oracle_mod
    g = golden(fx)
    HX = O.Op(g["HX"])
    opts = g["spectra_opts"]
    ntri = opts.get("NTri", 200)
    emin, emax, ne, gamma = opts["Emin"], opts["Emax"], opts["NE"], opts["Gamma"]
    de = (emax - emin) / ne
    spec = g["spec_eps0"]
    k = 0
    for T in ("Tx", "Ty", "Tz"):
        Top = O.Op(g[T])
        for p in g["psi"]:
            psi = O.WF.from_fixture(p)
            E0 = _expectation(O, HX, psi)
            Tpsi = O.operator_psi(Top, psi)
            a, b = O.lanczos_tridiag(HX, Tpsi, ntri, 0.0, max(gamma, 0.0))
            G = O.cf_spectrum(a, b, E0, emin, de, ne, gamma)
            ref = np.array(spec["re"][k]) + 1j * np.array(spec["im"][k])
            assert rel_err(G, ref) < 1e-8, (T, k, rel_err(G, ref))
            ta = g["tri_eps0"][k]
            assert abs(b[0] - ta["b"][0]) < 1e-12
            assert abs(a[1] - E0 - ta["a"][1]) < 1e-10
            k += 1


def test_dense_spectra_match_reference(oracle_mod):
    """The dense branch restated (CreateSpectra, LuaInterface/ssp.cpp:2347-2460): H on the
    union basis of all T psi closed under H, its eigensystem, poles weighted by |<E_k|T psi>|^2
    (Core/BasicMath/BasicMath_CompactMatrixVector.cpp:3990), summed Lorentzians
    (Core/Spectral.cpp:1576-1588); against the reference's dense spectra of the same call."""
    O = oracle_mod
    g = golden("c0_xas.json")
    HX = O.Op(g["HX"])
    opts = g["spectra_opts"]
    emin, emax, ne, gamma = opts["Emin"], opts["Emax"], opts["NE"], opts["Gamma"]
    psis = [O.WF.from_fixture(p) for p in g["psi"]]
    Tpsi, E0 = [], []
    for T in ("Tx", "Ty", "Tz"):
        Top = O.Op(g[T])
        for psi in psis:
            Tpsi.append(O.operator_psi(Top, psi))
            E0.append(_expectation(O, HX, psi))
    seed = O.linear_combination(HX.nf, Tpsi, [1.0] * len(Tpsi))
    basis = O.closure(HX, seed)
    M = O.dense_matrix(HX, basis)
    w, V = np.linalg.eigh(M)
    index = {bytes(r): i for i, r in enumerate(basis.det)}
    for k, tp in enumerate(Tpsi):
        x = np.zeros(len(basis.val), dtype=np.complex128)
        for r, v in zip(tp.det, tp.val):
            x[index[bytes(r)]] += v
        weights = np.abs(V.conj().T @ x) ** 2
        G = O.poles_spectrum(w, weights, E0[k], emin, (emax - emin) / ne, ne, gamma)
        ref = np.array(g["spec_dense"]["re"][k]) + 1j * np.array(g["spec_dense"]["im"][k])
        assert rel_err(G, ref) < 1e-8, (k, rel_err(G, ref))


def test_ground_energies_match_reference(oracle_mod):
    O = oracle_mod
    for fx in ("c0_xas.json", "c1_lf.json"):
        g = golden(fx)
        H = O.Op(g["H"])
        basis = _sector(O, g)
        w, _ = O.exact_eigensystem(H, basis, 3)
        assert np.max(np.abs(w - np.array(g["energies_krylov"]))) < 1e-10, (fx, w, g["energies_krylov"])


def _sector(O, g):
    """All determinants of the restricted sector, built from combinations (2^26 is too many
    to scan in Python)."""
    import itertools
    nf = g["H"]["nf"]
    groups = []
    for mask, lo, hi in g["restrictions"]:
        assert lo == hi
        groups.append(([i for i, ch in enumerate(mask) if ch == "1"], lo))
    dets = []
    for combo in itertools.product(*[itertools.combinations(idx, n) for idx, n in groups]):
        s = ["0"] * nf
        for part in combo:
            for i in part:
                s[i] = "1"
        dets.append("".join(s))
    return O.WF(nf, O.dets_to_bytes(dets, nf), np.ones(len(dets)))


@pytest.mark.parametrize("key,eps", [("rixs", 0.0), ("rixs_default", EPS_DEFAULT)])
def test_rixs_matches_reference(oracle_mod, key, eps):
    """CreateResonantSpectra (Core/ResonantSpectra.cpp:6): Krylov-projected intermediate-state
    resolvent and per-incident-energy Lanczos, against the reference's spectra."""
    O = oracle_mod
    g = golden("c0_xas.json")
    o = dict(g["rixs_opts"], Epsilon=eps, NTri1=100, NTri2=100)
    G = O.resonant_spectra(O.Op(g["HX"]), O.Op(g["H"]), O.Op(g["Tx"]), [O.Op(g["Tyd"])],
                           O.WF.from_fixture(g["psi"][0]), o)
    ref = g[key]
    R = np.array(ref["re"]) + 1j * np.array(ref["im"])
    assert rel_err(G, R) < 1e-8


@pytest.mark.parametrize("key", ["tensor_dense", "tensor_dense_defaults"])
def test_dense_tensor_spectra_match_reference(oracle_mod, key):
    """Tensor spectra, dense branch restated: G_ij(w) = sum_k conj(c_ki) c_kj / (w - (E_k - E0)
    + i Gamma/2), c_ki = <E_k|T_i psi>, spectrum i*3 + j (LuaInterface/ssp.cpp:2480-2530,
    Core/BasicMath/BasicMath_CompactMatrixVector.cpp:4064, BasicMath_BlockTypeConversion.cpp:588)."""
    from quanty_gb300 import api  # Spectra.from_text only (host code)
    O = oracle_mod
    g = golden("tensor.json")
    HX = O.Op(g["HX"])
    psi = O.WF.from_fixture(g["psi"])
    E0 = _expectation(O, HX, psi)
    Tpsi = [O.operator_psi(O.Op(g[T]), psi) for T in ("Tx", "Ty", "Tz")]
    seed = O.linear_combination(HX.nf, Tpsi, [1.0] * 3)
    basis = O.closure(HX, seed)
    w, V = np.linalg.eigh(O.dense_matrix(HX, basis))
    index = {bytes(r): i for i, r in enumerate(basis.det)}
    X = np.zeros((len(basis.val), 3), dtype=np.complex128)
    for s, tp in enumerate(Tpsi):
        for r, v in zip(tp.det, tp.val):
            X[index[bytes(r)], s] += v
    C = V.conj().T @ X
    ref = api.Spectra.from_text(g[key])
    assert abs(ref.EminPole - (w[0] - E0)) < 1e-8 and abs(ref.EmaxPole - (w[-1] - E0)) < 1e-8
    de = (ref.Emax - ref.Emin) / ref.NE
    for i in range(3):
        for j in range(3):
            wt = np.conj(C[:, i]) * C[:, j]
            G = (O.poles_spectrum(w - E0, wt.real, 0.0, ref.Emin, de, ref.NE, ref.Gamma)
                 + 1j * O.poles_spectrum(w - E0, wt.imag, 0.0, ref.Emin, de, ref.NE, ref.Gamma))
            R = ref.G[i * 3 + j]
            assert np.max(np.abs(G - R)) < 1e-8 * np.max(np.abs(ref.G)), (i, j)


def _rixs_inputs(O, g, t1, t2, npsi):
    return ([O.Op(g[t]) for t in t1], [O.Op(g[t]) for t in t2],
            [O.WF.from_fixture(p) for p in g["psi"][:npsi]])


def _spectra_of(ref):
    return np.array(ref["re"]) + 1j * np.array(ref["im"])


@pytest.mark.parametrize("key,t1,t2,npsi,tensor,auto", [
    ("dense_lists", ("Tx", "Ty"), ("Txd", "Tyd", "Tzd"), 2, False, False),
    ("dense_auto", ("Tx",), ("Txd", "Tyd"), 1, False, True),
    ("dense_tensor", ("Tx", "Ty"), ("Txd", "Tyd"), 1, True, False),
    ("dense_tensor_psi", ("Tx",), ("Tyd",), 2, True, False),
])
def test_dense_rixs_matches_reference(oracle_mod, key, t1, t2, npsi, tensor, auto):
    """Dense RIXS restated (ResonantSpectraDense / ResonantSpectraDenseTensor,
    Core/ResonantSpectra.cpp:290, :665): lists of absorption and emission operators and of
    initial states, the spectrum order of both forms, the automatic energy ranges."""
    O = oracle_mod
    g = golden("rixs.json")
    T1s, T2s, psis = _rixs_inputs(O, g, t1, t2, npsi)
    o = {"NE1": 4, "Gamma1": 0.8, "NE2": 64, "Gamma2": 0.3} if auto else dict(g["opts"])
    G, st = O.resonant_spectra_dense(O.Op(g["HX"]), O.Op(g["H"]), T1s, T2s, psis, o, tensor=tensor)
    ref = g[key]
    assert G.shape == (ref["nspec"], 65)
    assert rel_err(G, _spectra_of(ref)) < 1e-8
    assert abs(st["emin2"] - ref["emin"]) < 1e-10 and abs(st["emax2"] - ref["emax"]) < 1e-10
    assert abs(st["gamma2"] - ref["gamma"]) < 1e-12


def test_krylov_rixs_lists_and_tensor_match_reference(oracle_mod):
    """Krylov branch: lists of T1 and psi run one ResonantSpectra per (psi, T1) pair, blocks in
    that order (LuaInterface/ssp.cpp:3401-3424); the Krylov tensor form at complete Krylov
    spaces equals the dense tensor restatement in the Krylov branch's index order."""
    O = oracle_mod
    g = golden("rixs.json")
    T1s, T2s, psis = _rixs_inputs(O, g, ("Tx", "Ty"), ("Txd", "Tyd"), 2)
    o = dict(g["opts"], Epsilon=0.0, NTri1=100, NTri2=100)
    G = np.concatenate([O.resonant_spectra(O.Op(g["HX"]), O.Op(g["H"]), T, T2s, p, o) for p in psis for T in T1s])
    assert rel_err(G, _spectra_of(g["krylov_lists"])) < 1e-8
    Gt, _ = O.resonant_spectra_dense(O.Op(g["HX"]), O.Op(g["H"]), T1s, T2s, psis[:1], dict(g["opts"]),
                                     tensor=True, krylov_layout=True)
    assert rel_err(Gt, _spectra_of(g["krylov_tensor"])) < 1e-8


def test_eigensystem_growth_matches_reference(oracle_mod):
    """Eigensystem grows the basis under H within the Restrictions option only
    (Core/BlockLanczos.cpp:5843-5884): from the d8 L10 start determinants of the ligand-field
    ion the unrestricted closure holds d9 L9 and d10 L8 and gives the reference's energies; the
    closure confined to the start windows gives the confined energies."""
    import itertools
    O = oracle_mod
    g = golden("eigen_growth.json")
    H = O.Op(golden("c1_lf.json")["H"])
    dets = []
    for holes in itertools.combinations(range(6, 16), 2):
        s = ["1"] * 26
        for h in holes:
            s[h] = "0"
        dets.append("".join(s))
    seed = O.WF(26, O.dets_to_bytes(dets, 26), np.ones(len(dets)))
    for key, R in (("energies_grown", None), ("energies_confined", g["start_restrictions"])):
        w, _ = O.exact_eigensystem(H, O.closure(H, seed, R), 3)
        assert np.max(np.abs(w - np.array(g[key]))) < 1e-10, key


def test_krylov_basis_matches_reference(oracle_mod):
    """The Krylov-basis Lanczos (LanczosTriDiagonalizeKrylov, Core/Lanczos.cpp:5405) restated:
    the reference's non-empty Krylov vectors of CreateSpectra's KrylovBasis option (their count,
    the leading ones element by element) and, for the dense branch, the eigenstate energies."""
    O = oracle_mod
    g = golden("krylov_basis.json")
    r = golden("rixs.json")
    HX = O.Op(r["HX"])
    t = O.operator_psi(O.Op(g["Tz"]), O.WF.from_fixture(r["psi"][0]))
    a, b, K = O.lanczos_krylov(HX, t, 80, EPS_DEFAULT)
    K = [k for k in K if len(k.val) and np.any(k.val != 0)]
    assert len(K) == len(g["krylov_one"])
    for ref, k in list(zip(g["krylov_one"], K))[:12]:
        R = O.WF.from_fixture(ref)
        d = k.as_dict()
        assert rel_err([d[bytes(x)] for x in R.det], R.val) < 1e-10
    w, _ = O.exact_eigensystem(HX, O.closure(HX, t), len(g["dense_energies"]))
    assert np.max(np.abs(w - np.array(g["dense_energies"]))) < 1e-10


def test_zero_valued_strings_insert_targets_as_the_reference(oracle_mod):
    """OperatorPsi inserts the target of every applicable string whatever its value: the zero
    constant of "OppT = 0 + ..." (TestScripts/CreateResonantSpectra.Quanty's operator) puts
    psi0's own determinants into OppT * psi0 with amplitude 0."""
    O = oracle_mod
    g = golden("rixs_onebody.json")
    out = O.operator_psi(O.Op(g["OppT"]), O.WF.from_fixture(g["psi0"]))
    ref = O.WF.from_fixture(g["Tpsi0"])
    assert sorted(map(bytes, out.det)) == sorted(map(bytes, ref.det))
    d = out.as_dict()
    assert rel_err([d[bytes(r)] for r in ref.det], ref.val) < 1e-14
    assert sum(1 for v in ref.val if v == 0) == len(g["psi0"]["dets"])


def test_one_particle_rixs_of_the_reference_test(oracle_mod):
    """The one-particle RIXS model of TestScripts/CreateResonantSpectra.Quanty (a list of six
    one-particle states and a superposition): dense and Krylov branches restated, against the
    reference (1e-8)."""
    O = oracle_mod
    g = golden("rixs_onebody.json")
    H1, H0, T, T2 = (O.Op(g[k]) for k in ("H1", "H0", "OppT", "T2"))
    psis = [O.WF.from_fixture(p) for p in g["psilist"]]
    p0 = O.WF.from_fixture(g["psi0"])
    o = dict(g["opts"])

    def spec(k):
        return np.array(g[k]["re"]) + 1j * np.array(g[k]["im"])

    G, _ = O.resonant_spectra_dense(H1, H0, [T], [T2], psis, o)
    assert rel_err(G, spec("list_dense")) < 1e-8
    G = np.concatenate([O.resonant_spectra(H1, H0, T, [T2], p, o) for p in psis])
    assert rel_err(G, spec("list_krylov")) < 1e-8
    G, _ = O.resonant_spectra_dense(H1, H0, [T], [T2], [p0], o)
    assert rel_err(G, spec("psi0_dense")) < 1e-8
    assert rel_err(O.resonant_spectra(H1, H0, T, [T2], p0, o), spec("psi0_krylov")) < 1e-8
