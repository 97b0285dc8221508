"""Parity at the sizes the benchmarks run, against the CPU oracle.

* The H*psi benchmark's own configuration: the 86-spin-orbital Anderson impurity (7 bath
  shells, 47,481,880 determinants in 128-bit keys), the same closure, operator and apply
  call the benchmark times (connection lists, certain-offset local moves, block classes).  The
  oracle cannot afford all 31 G (determinant, term) pairs in a test, so x is zero except on a
  spread sample of rows (every STRIDE-th): push from those sources is exactly the pull
  result for that x, so every one of the 47.5 M outputs is compared (the reference's
  OperatorPsiConserveBasisPreAllocated, Core/OperatorWaveFunction.cpp:784-838).
* The batched XAS form at its own basis sizes: 6 bath shells, 1,701,795 ground and
  3,899,040 core-excited determinants, 16 states x 3 polarisations = 48 chains in one
  multi-vector Lanczos (and 8 real states, whose 24 real chains run two per complex vector),
  against the reference's three-term recursion (Core/Lanczos.cpp:1905-2830, restated below at
  Epsilon 0 on the closed basis) with the oracle's multi-vector push.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STRIDE = 32
TOL = 1e-12


def rel_err(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.fixture(scope="module")
def api():
    from quanty_gb300 import build
    build.build()
    from quanty_gb300 import api
    return api


def _oracle_op(O, H):
    return O.Op({"nf": H.nf, "terms": [[list(t[0]), t[1].real, t[1].imag] for t in H.terms]})


def test_hpsi_at_the_benchmark_configuration(api, oracle_mod):
    import torch
    from quanty_gb300 import workloads
    O = oracle_mod
    eng = api.engine()
    H, R, seed, info = workloads.anderson_impurity()
    b = api.closure(H, api.dets_to_bytes([seed], H.nf), H.nf, R, -1, eng)
    n = b.n
    assert n == info["sector_determinants"] == 47481880
    ops = H.info()
    # every string keeps its own action (no two merge on the device) and the list is closed
    # under conjugation, so counts of pull connections into rows equal the oracle's counts of
    # push connections out of them
    assert ops["nterms"] == len(H.terms) and ops["hermitian"] == 1
    rows = np.arange(0, n, STRIDE)
    rng = np.random.default_rng(2024)
    x = np.zeros(n, dtype=np.complex128)
    x[rows] = rng.normal(size=len(rows)) + 1j * rng.normal(size=len(rows))
    xd = torch.from_numpy(x.reshape(n, 1)).cuda()
    yd = eng.empty(n)
    eng.check(eng.L.qg_apply(eng.ctx, H.handle(), b.h, b.h, api._ptr(xd), api._ptr(yd), 1))
    built, nconn = C.c_int32(0), C.c_int64(0)
    eng.check(eng.L.qg_apply_list_info(eng.ctx, H.handle(), b.h, C.byref(built), C.byref(nconn)))
    assert built.value == 1  # the benchmark's path: connection lists
    y = eng.to_host(yd[:, 0])
    cnt = C.c_int64(0)
    eng.check(eng.L.qg_count_nnz_rows(eng.ctx, H.handle(), b.h, 0, STRIDE, 0, C.byref(cnt)))
    dets = b.dets_bytes()
    op = _oracle_op(O, H)
    h = O.WF(H.nf, dets, x).handle()
    try:
        want = O.apply_sampled(op, h, n, STRIDE)
        cnt_o = O.count_nnz_sampled(op, h, n, STRIDE)
    finally:
        O.lib().qo_wf_free(h)
    assert np.array_equal(y != 0, want != 0)  # the same rows are reached
    assert rel_err(y, want) < TOL
    assert cnt.value == cnt_o


def _lanczos_oracle(O, op, h, n, Y, ntri):
    """The reference's three-term Lanczos (LanczosTriDiagonalizeCC, Core/Lanczos.cpp:1905-2830,
    as qo_lanczos_tridiag restates it) for every column of Y at once, on the closed basis at
    Epsilon 0 (nothing is truncated): a[0] = 0, b[0] = |v0|."""
    m = Y.shape[1]
    A, B = np.zeros((m, ntri + 1)), np.zeros((m, ntri))
    B[:, 0] = np.sqrt((np.abs(Y) ** 2).sum(0))
    V = Y / B[:, 0]
    W = O.apply_multi(op, h, h, n, n, V)
    A[:, 1] = np.einsum("ik,ik->k", W.conj(), V).real
    Vp = V
    for i in range(1, ntri):
        W -= A[:, i] * Vp
        B[:, i] = np.sqrt((np.abs(W) ** 2).sum(0))
        V = W / B[:, i]
        W = O.apply_multi(op, h, h, n, n, V)
        A[:, i + 1] = np.einsum("ik,ik->k", W.conj(), V).real
        W -= B[:, i] * Vp
        Vp = V
    return A, B


@pytest.mark.parametrize("states", ["complex", "real"])
def test_batched_xas_at_its_basis_sizes(api, oracle_mod, states):
    """Complex states run as complex multi-vector chains; real states (those of this real
    Hamiltonian) give real Tx/Tz and purely imaginary Ty chains, which run two per complex
    vector."""
    import torch
    from quanty_gb300 import workloads
    O = oracle_mod
    eng = api.engine()
    H, R, seed, info = workloads.anderson_impurity(nshell=6, hole_max=1, particle_max=2)
    _, Rx, _, _ = workloads.anderson_impurity(nshell=6, hole_max=1, particle_max=2, core_holes=1)
    at = workloads.atomic()
    Ts = [api.Operator(H.nf, at[k].terms, name=k) for k in ("Tx", "Ty", "Tz")]
    g = api.closure(H, api.dets_to_bytes([seed], H.nf), H.nf, R, -1, eng)
    assert g.n == 1701795
    nstate, ntri = (16, 3) if states == "complex" else (8, 3)
    rng = np.random.default_rng(16)
    X = rng.normal(size=(g.n, nstate)) + (1j * rng.normal(size=(g.n, nstate)) if states == "complex" else 0j)
    o = {"NTri": ntri, "NE": 512, "Emin": -20.0, "Emax": 20.0, "Gamma": 0.5, "Epsilon": 0.0, "Restrictions": Rx}
    S, A, B = api.CreateSpectraResident(H, Ts, g, torch.from_numpy(X).cuda(), np.zeros(nstate), o, eng)
    # the final basis: the closure under H of every T's targets, within the core-hole windows
    Rp = api.parse_restrictions(Rx)
    bt = None
    for t in Ts:
        tb = api.OperatorPsiBasis(t, g, Rp, eng)
        bt = tb if bt is None else api.basis_union(bt, tb, eng)
    f = api.closure_of(H, bt, Rp, -1, eng)
    assert f.n == 3899040
    gd, fd = g.dets_bytes(), f.dets_bytes()
    hg = O.WF(H.nf, gd, np.zeros(g.n)).handle()
    hf = O.WF(H.nf, fd, np.zeros(f.n)).handle()
    try:
        Y = np.concatenate([O.apply_multi(_oracle_op(O, t), hg, hf, g.n, f.n, X) for t in Ts], axis=1)
        Ao, Bo = _lanczos_oracle(O, _oracle_op(O, H), hf, f.n, Y, ntri)
    finally:
        O.lib().qo_wf_free(hg)
        O.lib().qo_wf_free(hf)
    assert rel_err(B, Bo) < 1e-10 and rel_err(A[:, 1:], Ao[:, 1:]) < 1e-10
    de = (o["Emax"] - o["Emin"]) / o["NE"]
    for s in range(3 * nstate):
        want = O.cf_spectrum(Ao[s], Bo[s], 0.0, o["Emin"], de, o["NE"], o["Gamma"])
        assert rel_err(S.G[s], want) < 1e-8
