"""Output formats, byte for byte against files the reference wrote (tests/golden/gen/print_fmt.lua):
spectra files (Spectra.Print, IO/StreamPrint.cpp:4) and io.put wavefunction records
(LuaInterface/lua_extensions/get_put.cpp:588-634).  Host code only."""
import numpy as np
import pytest

from conftest import golden


@pytest.mark.parametrize("key", ["print_lanczos", "print_defaults", "print_dense"])
def test_spectra_file_round_trip_is_byte_identical(key):
    from quanty_gb300 import api
    text = golden("print_fmt.json")[key]
    S = api.Spectra.from_text(text)
    assert S.Print() == text


def test_spectra_file_layout_for_many_spectra():
    from quanty_gb300 import api
    G = np.arange(12 * 5, dtype=float).reshape(12, 5) * (1 - 0.5j)
    text = api.Spectra(G, -1.0, 3.0, 4, 0.1, -0.5, 2.5).Print()
    lines = text.splitlines()
    assert lines[0] == "#Spectra: 12"
    assert lines[4].startswith("Energy               Re[0]                  Im[0]                ")
    assert "  Re[10]                 Im[10]               " in lines[4]
    assert len(lines) == 5 + 5
    assert all(len(ln) == 19 + 12 * 46 for ln in lines[5:])
    S = api.Spectra.from_text(text)
    assert np.array_equal(S.G, G) and S.Emin == -1.0 and S.Gamma == 0.1 and S.EmaxPole == 2.5


@pytest.mark.parametrize("key", ["put_psi1", "put_psi2"])
def test_wavefunction_put_round_trip_is_byte_identical(key):
    from quanty_gb300 import api, quanty_text
    text = golden("print_fmt.json")[key]
    var = key[4:]
    d = quanty_text.parse_wavefunction(text)
    assert quanty_text.format_wavefunction(d, var) == text
    psi = api.Wavefunction.from_put(text)
    assert psi.put(var, complex_values=d["complex"], nbitskey=d["nbitskey"]) == text


def test_complex_wavefunction_text():
    from quanty_gb300 import api
    psi = api.NewWavefunction(4, 0, [["1100", 0.5 - 0.25j], ["0011", -1.0]])
    t = psi.put("psi")
    assert t.startswith("psi = NewWavefunction( 4, 0,{\n")
    assert '{"1100", 5.0000000000000000E-01 - I *  2.5000000000000000E-01}' in t
    assert '{"0011",-1.0000000000000000E+00 + I *  0.0000000000000000E+00}' in t
    back = api.Wavefunction.from_put(t)
    assert np.array_equal(back.val, psi.val) and back.dets() == psi.dets()


def test_pole_range_extremes_match_dense_eigenvalues():
    """The pole range of CreateSpectra takes the extreme eigenvalues of each tridiagonal matrix
    by bisection; they equal a dense eigensolve's to rounding, including chains of length one
    and two and matrices with repeated or tiny off-diagonal entries."""
    from quanty_gb300.api import _tri_extremes
    rng = np.random.default_rng(5)
    cases = [(rng.normal(size=m), rng.normal(size=m - 1)) for m in (1, 2, 3, 17, 200)]
    cases.append((np.full(50, 2.0), np.full(49, 1e-12)))
    cases.append((np.linspace(-3, 3, 40), np.ones(39)))
    for a, b in cases:
        lo, hi = _tri_extremes(a, b)
        if len(a) == 1:
            w = a
        else:
            w = np.linalg.eigvalsh(np.diag(a) + np.diag(b, 1) + np.diag(b, -1))
        scale = max(1.0, float(np.max(np.abs(w))))
        assert abs(lo - w[0]) <= 1e-12 * scale and abs(hi - w[-1]) <= 1e-12 * scale


def test_spectra_method_options_follow_the_reference():
    """Method / ForceDenseMethod of CreateSpectra (LuaInterface/ssp.cpp:2029-2058): Dense or
    ForceDenseMethod force the dense branch, Lanczos forces the Krylov branch, Auto (or nothing)
    decides by DenseBorder; contradicting or unknown choices are errors raised before any
    device work."""
    import pytest
    from quanty_gb300 import api
    m = lambda **k: api._spectra_method(api._opts(k))  # noqa: E731
    assert m() == "" and m(Method="Auto") == "" and m(Method="auto") == ""
    assert m(Method="Dense") == "dense" and m(ForceDenseMethod=True) == "dense"
    assert m(Method="DENSE", ForceDenseMethod=True) == "dense"
    assert m(Method="Lanczos") == "lanczos"
    with pytest.raises(ValueError, match="contradict"):
        m(Method="Lanczos", ForceDenseMethod=True)
    with pytest.raises(ValueError, match="unknown Method"):
        m(Method="Arnoldi")
    with pytest.raises(NotImplementedError):
        m(Method="Mesh")
    for opt in ({"GridPoints": [0.0, 1.0]}, {"NTriFull": 10}, {"NonCrossing": True}, {"NBathExcitations": 2}):
        with pytest.raises(NotImplementedError, match="self-energy"):
            m(**opt)
    assert m(NBathExcitations=1, NonCrossing=False) == ""
    with pytest.raises(ValueError, match="unknown Method"):  # checked before the GPU is needed
        api.CreateSpectra(None, [], [], {"Method": "Arnoldi"})


def test_option_names_accept_the_reference_aliases():
    """Lower-case option names the reference's option tables also accept
    (LuaInterface/ssp.cpp:1958-1980, :3118-3125, :4063-4075)."""
    from quanty_gb300 import api
    o = api._opts({"epsilon": 0.0, "zero": 1e-12, "restrictions": [1], "restrictions1": [2], "restrictions2": [3]})
    assert (o["Epsilon"], o["Zero"], o["Restrictions"], o["Restrictions1"], o["Restrictions2"]) == (0.0, 1e-12, [1], [2], [3])
    o = api._opts([("NE", 10), ("Gamma", 0.2)])  # the ordered-pairs form of a Lua option table
    assert o["NE"] == 10 and o["Gamma"] == 0.2 and o["NTri"] == 200


def test_wavefunction_arithmetic_follows_the_reference(monkeypatch):
    """The Lua metamethods of wavefunctions (LuaInterface/Wavefunction.cpp): sums on the union
    basis in the reference's order (left operand's determinants first), scaling by real and
    complex numbers, <a|b> with the left side conjugated and returned as a real number when its
    imaginary part vanishes, <psi|O as O^dag|psi>, and the elementwise forms over lists."""
    import numpy as np
    from quanty_gb300 import api
    from oracle import oracle as O
    from conftest import golden
    g = golden("rixs.json")
    p1, p2 = (api.Wavefunction.from_fixture(p) for p in g["psi"])
    t = api.Wavefunction(16, p2.det[::3], np.linspace(1, 2, len(p2.det[::3])) * 1j)
    for a, b, c in ((p1, p2, 0.5), (p1, t, -2.0), (t, p1, 1.5 - 0.5j)):
        s = a + c * b
        ref = O.linear_combination(16, [O.WF(16, a.det, a.val), O.WF(16, b.det, b.val)], [1.0, c])
        assert np.array_equal(s.det, ref.det) and np.allclose(s.val, ref.val, rtol=0, atol=1e-15)
        d = a * b
        want = sum(np.conj(x) * ref_b for x, ref_b in
                   ((a.as_dict()[k], b.as_dict()[k]) for k in a.as_dict() if k in b.as_dict()))
        assert abs(d - want) < 1e-14
    assert isinstance(p1 * p1, float) and abs(p1 * p1 - 1) < 1e-12
    assert isinstance(p1 * (1j * p1), complex) and abs((p1 * (1j * p1)) - 1j) < 1e-12
    assert np.allclose((p1 - p1).val, 0) and np.allclose((-p1).val, -p1.val)
    assert np.allclose((np.float64(2.0) * p1).val, 2 * p1.val) and np.allclose((p1 / 4).val, p1.val / 4)
    assert [w.N for w in p1 + [p1, t]] == [p1.N, (p1 + t).N]
    seen = {}
    monkeypatch.setattr(api, "OperatorPsi", lambda O_, psi: seen.setdefault("call", (O_, psi)))
    Tz = api.Operator.from_fixture(golden("krylov_basis.json")["Tz"])
    p1 * Tz
    O_, psi = seen["call"]
    assert psi is p1 and O_.terms == Tz.dagger().terms


def test_wavefunction_in_place_methods():
    """psi.Chop(), psi.Conjugate() and psi.Norm() as the reference's Lua methods: truncation at
    |a|^2 > border^2 (default 10 DBL_EPSILON), conjugation, normalisation."""
    import numpy as np
    from quanty_gb300 import api
    psi = api.NewWavefunction(4, 0, [["1100", 1e-17], ["1010", 2j], ["0011", 1e-3]])
    psi.Chop()
    assert psi.dets() == ["1010", "0011"]
    psi.Chop(1e-3)
    assert psi.dets() == ["1010"]
    psi.Conjugate()
    assert psi.val[0] == -2j
    psi.Norm()
    assert abs(psi.norm() - 1) < 1e-15 and psi.val[0] == -1j
