"""CPU checks of the boundary: the C-ABI library builds and exports every symbol the header
declares, and the host-side layout conversions match the reference's byte layout."""
import ctypes
import os

import numpy as np
import pytest

from conftest import ROOT, golden


@pytest.fixture(scope="session")
def libpath():
    from quanty_gb300 import build
    return build.build()


def test_library_exports_every_header_symbol(libpath):
    from quanty_gb300 import qgpu
    names = qgpu.header_symbols()
    assert len(names) >= 25
    lib = ctypes.CDLL(libpath)
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # the binding declares exactly the header's functions
    L = qgpu.load(libpath)
    for n in names:
        assert getattr(L, n).argtypes is not None, n


def test_det_bytes_roundtrip_matches_reference_layout():
    from quanty_gb300 import api
    from oracle import oracle as O
    rng = np.random.default_rng(1)
    for nf in (1, 7, 8, 9, 16, 26, 63, 64, 70, 127):
        dets = ["".join(rng.choice(["0", "1"], nf)) for _ in range(20)]
        b = api.dets_to_bytes(dets, nf)
        assert np.array_equal(b, O.dets_to_bytes(dets, nf))
        assert api.bytes_to_dets(b, nf) == dets


def test_new_operator_matches_io_put_convention():
    """NewOperator(NF,0,{{0,-0,1,-1,v}}) is c0^dag c0 c1^dag c1: the rightmost factor acts first."""
    from quanty_gb300 import api
    op = api.NewOperator(4, 0, [[0, -0.0, 1, -1, 2.0]])
    assert op.terms[0][0] == (1, 1 | api.CREATION, 0, 0 | api.CREATION)
    # a fixture operator converts term for term
    g = golden("chain_spectra.json")
    o = api.Operator.from_fixture(g["TDn"])
    assert o.nf == g["TDn"]["nf"] and len(o.terms) == len(g["TDn"]["terms"])


def test_restriction_parsing_and_enumeration():
    from quanty_gb300 import api
    R = api.parse_restrictions([16, 0, ["111111 0000000000", 6, 6], ["000000 1111111111", 8, 8]])
    assert R == [("1111110000000000", 6, 6), ("0000001111111111", 8, 8)]
    d = api.enumerate_restricted(16, R)
    assert len(d) == 45
    R = api.parse_restrictions([14, 0, ["11111111111111", 6, 6]])
    assert len(api.enumerate_restricted(14, R)) == 3003


def test_python_binding_fails_loudly_without_library(tmp_path):
    from quanty_gb300 import qgpu
    with pytest.raises(RuntimeError):
        qgpu._lib_backup = qgpu._lib
        try:
            qgpu._lib = None
            qgpu.load(str(tmp_path / "missing.so"))
        finally:
            qgpu._lib = qgpu._lib_backup
