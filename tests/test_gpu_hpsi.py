"""H*psi on the GPU against the reference fixtures and the CPU oracle (bit-exact determinant
sets and signs, amplitudes to 1e-12 relative)."""
import math

import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu

TOL = 1e-12  # amplitudes, relative to the largest


def rel_err(a, b):
    a, b = np.asarray(a), np.asarray(b)
    if a.size == 0 and b.size == 0:
        return 0.0
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.fixture(scope="module")
def api():
    from quanty_gb300 import build
    build.build()
    from quanty_gb300 import api
    return api


CASES = [c["name"] for c in golden("hpsi_cases.json")["cases"]]


def _case(name):
    return next(c for c in golden("hpsi_cases.json")["cases"] if c["name"] == name)


@pytest.mark.parametrize("case", CASES)
def test_operator_psi_matches_reference(api, case):
    c = _case(case)
    H = api.Operator.from_fixture(c["H"])
    psi = api.Wavefunction.from_fixture(c["psi"])
    if H.nf > 127:
        with pytest.raises(api.qgpu.QGError) as e:
            api.OperatorPsi(H, psi)
        assert e.value.status == 4
        return
    for key, res in (("Hpsi", None), ("Hpsir", c["restrictions"])):
        out = api.OperatorPsi(H, psi, res)
        ref = api.Wavefunction.from_fixture(c[key])
        assert sorted(map(bytes, out.det)) == sorted(map(bytes, ref.det))  # bit-exact set
        rd = ref.as_dict()
        want = np.array([rd[bytes(r)] for r in out.det])
        assert rel_err(out.val, want) < TOL, key


@pytest.mark.parametrize("case", [n for n in CASES if _case(n)["H"]["nf"] <= 127])
def test_conserve_basis_matches_reference(api, case):
    c = _case(case)
    H = api.Operator.from_fixture(c["H"])
    psi = api.Wavefunction.from_fixture(c["psi"])
    y = api.OperatorPsiConserveBasis(H, psi)
    rd = api.Wavefunction.from_fixture(c["Hpsi"]).as_dict()
    want = np.array([rd.get(bytes(r), 0.0) for r in psi.det])
    assert rel_err(y.val, want) < TOL


def _random_operator(api, nf, n2, n4, rng, complex_values=True):
    """Distinct actions only (no two strings that the device would merge), so connection
    counts compare one to one with the oracle's per-string loop."""
    terms, seen = [], set()
    while len(terms) < n2:
        i, j = (int(v) for v in rng.choice(nf, 2, replace=False))
        if (i, j) in seen:
            continue
        seen.add((i, j))
        terms.append(([j, i | api.CREATION], complex(rng.normal(), rng.normal() if complex_values else 0)))
    while len(terms) < n2 + n4:
        i, j, k, l = (int(v) for v in rng.choice(nf, 4, replace=False))
        key = (min(i, j), max(i, j), min(k, l), max(k, l))
        if key in seen:
            continue
        seen.add(key)
        terms.append(([l, k, j | api.CREATION, i | api.CREATION],
                      complex(rng.normal(), rng.normal() if complex_values else 0)))
    terms.append(([], 0.3))
    return api.Operator(nf, terms)


@pytest.mark.parametrize("nf,nel", [(20, 10), (64, 12), (86, 43), (127, 60)])
def test_apply_matches_oracle_on_closed_sets(api, oracle_mod, nf, nel):
    """Seeded random operators on bases grown by the device closure; the oracle's push-form
    H*psi (reference ConserveBasis semantics) on the same basis and amplitudes."""
    O = oracle_mod
    rng = np.random.default_rng(nf)
    H = _random_operator(api, nf, 3 * nf, 2 * nf, rng)
    occ = rng.choice(nf, nel, replace=False)
    s = ["0"] * nf
    for i in occ:
        s[i] = "1"
    b = api.closure(H, api.dets_to_bytes(["".join(s)], nf), nf, None, 2)
    dets = b.dets_bytes()
    assert len(dets) > 100
    x = rng.normal(size=len(dets)) + 1j * rng.normal(size=len(dets))
    psi = api.Wavefunction(nf, dets, x)
    y = api.OperatorPsiConserveBasis(H, psi)
    op = O.Op({"nf": nf, "terms": [[list(t[0]), t[1].real, t[1].imag] for t in H.terms]})
    want = O.apply_conserve(op, O.WF(nf, dets, x))
    assert rel_err(y.val, want) < TOL
    # the device's connection count equals the oracle's
    assert api.count_nnz(H, b) == O.count_nnz(op, O.WF(nf, dets, x))


def test_apply_with_all_ones_low_key_word(api, oracle_mod):
    """nf = 70 with orbitals 16..69 filled: a determinant with orbitals 6..15 also filled has
    all 64 bits of its low device word set (orbitals 6..69).  Such keys sit in the hash table
    beside the others, and lookups whose probe chains pass their slots must keep probing.
    Growth, fixed-basis H*psi and the connection count against the oracle."""
    O = oracle_mod
    nf = 70
    rng = np.random.default_rng(70)
    terms, seen = [], set()
    while len(terms) < 60:  # one-body moves and pair terms among orbitals 0..15
        i, j = (int(v) for v in rng.choice(16, 2, replace=False))
        if (i, j) not in seen:
            seen.add((i, j))
            terms.append(([j, i | api.CREATION], complex(rng.normal(), rng.normal())))
    for _ in range(20):
        i, j, k, l = (int(v) for v in rng.choice(16, 4, replace=False))
        terms.append(([l, k, j | api.CREATION, i | api.CREATION], complex(rng.normal(), 0.0)))
    H = api.Operator(nf, terms)
    seed = "1" * 2 + "0" * 4 + "1" * 64  # orbitals 0, 1 and 6..69: low word all ones
    b = api.closure(H, api.dets_to_bytes([seed], nf), nf, None, -1)
    dets = b.dets_bytes()
    full = [r for r in dets if all(r[i >> 3] & (128 >> (i & 7)) for i in range(6, 70))]
    assert len(dets) == math.comb(16, 12) and len(full) == math.comb(6, 2)
    assert (b.find(dets) == np.arange(len(dets))).all()  # every key found at its row
    x = rng.normal(size=len(dets)) + 1j * rng.normal(size=len(dets))
    psi = api.Wavefunction(nf, dets, x)
    y = api.OperatorPsiConserveBasis(H, psi)
    op = O.Op({"nf": nf, "terms": [[list(t[0]), t[1].real, t[1].imag] for t in H.terms]})
    want = O.apply_conserve(op, O.WF(nf, dets, x))
    assert rel_err(y.val, want) < TOL
    assert api.count_nnz(H, b) == O.count_nnz(op, O.WF(nf, dets, x))
    out = api.OperatorPsi(H, api.Wavefunction(nf, [dets[0]], [1.0]))
    ref = O.operator_psi(op, O.WF(nf, [dets[0]], [1.0]))
    assert sorted(map(bytes, out.det)) == sorted(map(bytes, ref.det))


def test_multivector_apply_equals_single(api):
    import torch
    rng = np.random.default_rng(5)
    nf = 30
    H = _random_operator(api, nf, 60, 60, rng)
    b = api.closure(H, api.dets_to_bytes(["1" * 8 + "0" * 22], nf), nf, None, 2)
    eng = api.engine()
    n = b.n
    X = torch.from_numpy(rng.normal(size=(n, 11)) + 1j * rng.normal(size=(n, 11))).cuda()
    Y = eng.empty(n, 11)
    eng.check(eng.L.qg_apply(eng.ctx, H.handle(), b.h, b.h, api._ptr(X), api._ptr(Y), 11))
    for k in (0, 5, 10):
        xk = X[:, k].contiguous()
        yk = eng.empty(n)
        eng.check(eng.L.qg_apply(eng.ctx, H.handle(), b.h, b.h, api._ptr(xk), api._ptr(yk), 1))
        assert torch.equal(Y[:, k], yk[:, 0])  # same rows, same order of summation


def test_autotuned_chunk_gives_the_same_bits(api):
    """The autotuner picks the vectors per kernel pass; every choice sums in the same order."""
    import ctypes
    import torch
    rng = np.random.default_rng(6)
    nf = 30
    H = _random_operator(api, nf, 60, 60, rng)
    seed = api.dets_to_bytes(["1" * 8 + "0" * 22], nf)
    eng = api.engine()
    b1 = api.closure(H, seed, nf, None, 2)
    b2 = api.closure(H, seed, nf, None, 2)
    n = b1.n
    X = torch.from_numpy(rng.normal(size=(n, 13)) + 1j * rng.normal(size=(n, 13))).cuda()
    Y1, Y2 = eng.empty(n, 13), eng.empty(n, 13)
    ch = ctypes.c_int32()
    try:
        eng.check(eng.L.qg_apply(eng.ctx, H.handle(), b1.h, b1.h, api._ptr(X), api._ptr(Y1), 13))
        eng.check(eng.L.qg_apply_chunk(eng.ctx, H.handle(), b1.h, 13, ctypes.byref(ch)))
        assert ch.value in (1, 2, 3, 4, 8)
        eng.check(eng.L.qg_set_autotune(eng.ctx, 0))
        eng.check(eng.L.qg_apply(eng.ctx, H.handle(), b2.h, b2.h, api._ptr(X), api._ptr(Y2), 13))
        eng.check(eng.L.qg_apply_chunk(eng.ctx, H.handle(), b2.h, 13, ctypes.byref(ch)))
        assert ch.value == 0  # untuned: passes of 8 vectors
    finally:
        eng.check(eng.L.qg_set_autotune(eng.ctx, 1))
    assert torch.equal(Y1, Y2)


@pytest.mark.parametrize("model", ["random", "anderson"])
def test_every_vector_layout_gives_the_same_bits(api, model):
    """Thread-per-row passes of 1/2/3/8 vectors and warp-per-row passes of 32/64 vectors
    (lanes over vectors) sum every vector's connections in the same order."""
    import ctypes
    import torch
    from quanty_gb300 import workloads
    eng = api.engine()
    rng = np.random.default_rng(8)
    if model == "random":
        nf = 30
        H = _random_operator(api, nf, 60, 60, rng)
        seed = api.dets_to_bytes(["1" * 8 + "0" * 22], nf)
        R = None
    else:
        H, R, s0, info = workloads.anderson_impurity(nshell=2, hole_max=2, particle_max=2)
        nf = H.nf
        seed = api.dets_to_bytes([s0], nf)
    nvec = 40
    out = {}
    for chunk in (1, 2, 3, 8, -32, -64):
        b = api.closure(H, seed, nf, R, 3 if model == "random" else -1)
        if chunk == 1:
            X = torch.from_numpy(rng.normal(size=(b.n, nvec)) + 1j * rng.normal(size=(b.n, nvec))).cuda()
        Y = eng.empty(b.n, nvec)
        eng.check(eng.L.qg_apply_set_chunk(eng.ctx, H.handle(), b.h, nvec, chunk))
        eng.check(eng.L.qg_apply(eng.ctx, H.handle(), b.h, b.h, api._ptr(X), api._ptr(Y), nvec))
        ch = ctypes.c_int32()
        eng.check(eng.L.qg_apply_chunk(eng.ctx, H.handle(), b.h, nvec, ctypes.byref(ch)))
        assert ch.value == chunk
        out[chunk] = Y
    for chunk, Y in out.items():
        assert torch.equal(Y, out[1]), chunk


def test_batched_lanczos_with_warp_layout_matches_single(api):
    import torch
    from quanty_gb300 import workloads
    eng = api.engine()
    H, R, s0, info = workloads.anderson_impurity(nshell=2, hole_max=2, particle_max=2)
    b = api.closure(H, api.dets_to_bytes([s0], H.nf), H.nf, R)
    rng = np.random.default_rng(9)
    nvec = 36
    X = torch.from_numpy(rng.normal(size=(b.n, nvec)) + 1j * rng.normal(size=(b.n, nvec))).cuda()
    eng.check(eng.L.qg_apply_set_chunk(eng.ctx, H.handle(), b.h, nvec, -64))
    A, B = api.lanczos_block(H, b, X.clone(), 20, 0.0, 0.0, eng)
    for k in (0, 17, 35):
        a, bb = api.lanczos_block(H, b, X[:, k:k + 1].contiguous(), 20, 0.0, 0.0, eng)
        # the block's inner products are reduced in another order; without reorthogonalisation
        # such last-bit differences grow about tenfold per step once orthogonality is lost
        # (here after ~20 steps on a basis of a few thousand determinants), so the chains are
        # compared over their first 20 steps
        assert np.max(np.abs(A[k] - a[0])) < 1e-10 * np.max(np.abs(a[0]))
        assert np.max(np.abs(B[k] - bb[0])) < 1e-10 * np.max(np.abs(bb[0]))
        g1 = api.TriDiagonalMatrixToSpectrum(0.0, A[k], B[k], -20.0, 20.0, 400, 0.5, eng)
        g0 = api.TriDiagonalMatrixToSpectrum(0.0, a[0], bb[0], -20.0, 20.0, 400, 0.5, eng)
        assert np.max(np.abs(g1 - g0)) < 1e-8 * np.max(np.abs(g0))


def test_edge_cases(api):
    H = api.NewOperator(4, 0, [[0, -1, 0.5], [1, -0.0, 0.5]])
    empty = api.Wavefunction(4, np.zeros((0, 1), np.uint8), [])
    out = api.OperatorPsi(H, empty)
    assert out.N == 0
    none = api.Operator(4, [])
    psi = api.NewWavefunction(4, 0, [["1100", 1.0], ["1010", 0.5j]])
    assert api.OperatorPsi(none, psi).N == 0
    # duplicate determinants merge (the reference adds into the existing element)
    dup = api.NewWavefunction(4, 0, [["1010", 1.0], ["1010", 2.0]])
    out = api.OperatorPsi(H, dup)
    d = dict(zip(out.dets(), out.val))
    assert abs(d["0110"] - 1.5) < 1e-15
    # one orbital, and the widest supported determinant
    one = api.NewOperator(1, 0, [[0, -0.0, 2.0]])
    r = api.OperatorPsi(one, api.NewWavefunction(1, 0, [["1", 1.0]]))
    assert r.dets() == ["1"] and abs(r.val[0] - 2.0) < 1e-15
    wide = api.NewOperator(127, 0, [[126, -0.0, 1.0]])
    r = api.OperatorPsi(wide, api.NewWavefunction(127, 0, [["1" + "0" * 126, 1.0]]))
    assert r.dets() == ["0" * 126 + "1"]
    # more orbitals than supported: a clear argument error
    with pytest.raises(api.qgpu.QGError):
        api.OperatorPsi(api.NewOperator(128, 0, [[127, -0.0, 1.0]]), api.NewWavefunction(128, 0, [["1" + "0" * 127, 1.0]]))


def test_closure_counts_and_table_growth(api):
    """Hopping on 30 orbitals with 7 electrons reaches all C(30,7) = 2,035,800 determinants;
    this passes the 2^20 initial table capacity, so the grow-and-retry path runs."""
    nf, nel = 30, 7
    terms = []
    for i in range(nf - 1):
        terms.append(([i + 1, i | api.CREATION], 1.0))
        terms.append(([i, (i + 1) | api.CREATION], 1.0))
    H = api.Operator(nf, terms)
    b = api.closure(H, api.dets_to_bytes(["1" * nel + "0" * (nf - nel)], nf), nf)
    assert b.n == math.comb(nf, nel)
    # restricted: at most 2 electrons in the last 10 orbitals
    R = [("0" * 20 + "1" * 10, 0, 2)]
    br = api.closure(H, api.dets_to_bytes(["1" * nel + "0" * (nf - nel)], nf), nf, R)
    want = sum(math.comb(10, k) * math.comb(20, nel - k) for k in range(0, 3))
    assert br.n == want
    # sorted, unique, and every determinant finds itself
    d = b.dets_bytes()
    idx = b.find(d[:5000])
    assert np.array_equal(idx, np.arange(5000))


@pytest.mark.parametrize("nshell,hmax,pmax", [(2, 2, 2), (3, 2, 1)])
def test_anderson_impurity_apply_matches_oracle(api, oracle_mod, nshell, hmax, pmax):
    """The benchmark Hamiltonian's structure at a size the oracle handles: impurity terms take
    the local-block path, hybridisation the scanned path with window bits, the diagonal is
    cached; every amplitude equals the oracle's push-form H*psi on the same basis."""
    from quanty_gb300 import workloads
    O = oracle_mod
    H, R, seed, info = workloads.anderson_impurity(nshell=nshell, hole_max=hmax, particle_max=pmax)
    b = api.closure(H, api.dets_to_bytes([seed], H.nf), H.nf, R)
    assert b.n == info["sector_determinants"]
    dets = b.dets_bytes()
    rng = np.random.default_rng(nshell)
    x = rng.normal(size=len(dets)) + 1j * rng.normal(size=len(dets))
    y = api.OperatorPsiConserveBasis(H, api.Wavefunction(H.nf, dets, x))
    op = O.Op({"nf": H.nf, "terms": [[list(t[0]), t[1].real, t[1].imag] for t in H.terms]})
    want = O.apply_conserve(op, O.WF(H.nf, dets, x))
    assert rel_err(y.val, want) < TOL
    # the same on a basis given as plain determinants (no windows, no closure): full checks
    y2 = api.OperatorPsiConserveBasis(H, api.Wavefunction(H.nf, dets[::-1].copy(), x[::-1].copy()))
    assert rel_err(y2.val[::-1], want) < TOL


@pytest.mark.parametrize("model", ["random", "anderson"])
def test_connection_lists_give_the_same_bits(api, model):
    """The apply over per-row connection lists (sources resolved once per operator and basis)
    sums every row's connections in the hash path's order: outputs are bitwise equal, for one
    vector, several vectors and a Lanczos chain."""
    import ctypes
    import torch
    from quanty_gb300 import workloads
    eng = api.engine()
    rng = np.random.default_rng(12)
    if model == "random":
        nf = 30
        H = _random_operator(api, nf, 60, 60, rng)
        seed, R, depth = api.dets_to_bytes(["1" * 8 + "0" * 22], nf), None, 3
    else:
        H, R, s0, info = workloads.anderson_impurity(nshell=2, hole_max=2, particle_max=2)
        nf, seed, depth = H.nf, api.dets_to_bytes([s0], H.nf), -1
    out = {}
    try:
        for on in (0, 1):
            eng.check(eng.L.qg_set_connection_lists(eng.ctx, on))
            b = api.closure(H, seed, nf, R, depth)
            if on == 0:
                X = torch.from_numpy(rng.normal(size=(b.n, 5)) + 1j * rng.normal(size=(b.n, 5))).cuda()
            x1 = X[:, :1].contiguous()
            y1, y5 = eng.empty(b.n), eng.empty(b.n, 5)
            eng.check(eng.L.qg_apply(eng.ctx, H.handle(), b.h, b.h, api._ptr(x1), api._ptr(y1), 1))
            eng.check(eng.L.qg_apply_set_chunk(eng.ctx, H.handle(), b.h, 5, 4))
            eng.check(eng.L.qg_apply(eng.ctx, H.handle(), b.h, b.h, api._ptr(X), api._ptr(y5), 5))
            built, nconn = ctypes.c_int32(), ctypes.c_int64()
            eng.check(eng.L.qg_apply_list_info(eng.ctx, H.handle(), b.h, ctypes.byref(built), ctypes.byref(nconn)))
            assert built.value == on
            if on:
                assert nconn.value > 0
            a, bb = api.lanczos_block(H, b, x1.clone(), 30, 0.0, 0.0, eng)
            out[on] = (y1, y5, a, bb)
    finally:
        eng.check(eng.L.qg_set_connection_lists(eng.ctx, 1))
    assert torch.equal(out[0][0], out[1][0])
    assert torch.equal(out[0][1], out[1][1])
    assert np.array_equal(out[0][2], out[1][2]) and np.array_equal(out[0][3], out[1][3])


def test_host_buffer_entry_point_matches_device_apply(api):
    """qg_apply_host (the reference's calling convention, psi and Opsi in host memory) gives
    the device apply's bits: page-locked buffers used in place, pageable ones staged; one and
    several vectors; on one basis and between bases; an empty source basis gives zeros."""
    import torch
    rng = np.random.default_rng(21)
    nf = 30
    H = _random_operator(api, nf, 60, 60, rng)
    T = api.Operator(nf, [([i, (i + 7) % nf | api.CREATION], 0.5 + 0.1j * i) for i in range(nf)])
    eng = api.engine()
    b = api.closure(H, api.dets_to_bytes(["1" * 8 + "0" * 22], nf), nf, None, 2)
    bt = api.OperatorPsiBasis(T, b)
    for dst, src, op in ((b, b, H), (bt, b, T)):
        for nvec in (1, 3):
            X = torch.from_numpy(rng.normal(size=(src.n, nvec)) + 1j * rng.normal(size=(src.n, nvec)))
            Yd = eng.empty(dst.n, nvec)
            Xd = X.cuda()
            eng.check(eng.L.qg_apply(eng.ctx, op.handle(), dst.h, src.h, api._ptr(Xd), api._ptr(Yd), nvec))
            torch.cuda.synchronize()
            want = Yd.cpu()
            for pinned in (True, False):
                xh = X.clone().pin_memory() if pinned else X.clone()
                yh = torch.zeros((dst.n, nvec), dtype=torch.complex128)
                if pinned:
                    yh = yh.pin_memory()
                for _ in range(2):  # twice: the staging buffers are reused
                    eng.check(eng.L.qg_apply_host(eng.ctx, op.handle(), dst.h, src.h, api._ptr(xh), api._ptr(yh),
                                                  nvec))
                    assert torch.equal(yh, want), (pinned, nvec, dst is b)
    empty = api.Basis.from_bytes(nf, np.zeros((0, api.nword(nf)), np.uint8), eng)[0]
    yh = torch.ones((b.n, 1), dtype=torch.complex128)
    xh = torch.zeros((1, 1), dtype=torch.complex128)
    eng.check(eng.L.qg_apply_host(eng.ctx, T.handle(), b.h, empty.h, api._ptr(xh), api._ptr(yh), 1))
    assert torch.count_nonzero(yh) == 0


@pytest.mark.parametrize("complex_values", [False, True])
def test_fp64_operation_count(api, complex_values):
    """qg_apply_fp64_ops counts what the list kernel issues: 2 multiplies per row for a real
    diagonal, 2 FMAs per real connection, 4 per complex one (distinct random actions, no
    local block decomposition, so connections and list entries coincide)."""
    import ctypes
    rng = np.random.default_rng(31)
    nf = 30
    H = _random_operator(api, nf, 60, 60, rng, complex_values=complex_values)
    b = api.closure(H, api.dets_to_bytes(["1" * 8 + "0" * 22], nf), nf, None, 2)
    eng = api.engine()
    ops = ctypes.c_int64()
    eng.check(eng.L.qg_apply_fp64_ops(eng.ctx, H.handle(), b.h, ctypes.byref(ops)))
    nnz_off = api.count_nnz(H, b, offdiag=True)
    assert ops.value == 2 * b.n + (4 if complex_values else 2) * nnz_off
