"""The persistent Lanczos kernel of small bases (one block per chain, every step in one launch)
against the general path: each chain's coefficients are bitwise those of the general path run
with that vector alone, with truncation and broadening active, with stored Krylov vectors, on a
real and on a complex operator; and it really is one launch."""
import ctypes

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


def _cases(api):
    g = golden("c1_lf.json")  # the 26-orbital ligand-field ion: 120 final-state determinants
    HX = api.Operator.from_fixture(g["HX"])
    Ts = [api.Operator.from_fixture(g[t]) for t in ("Tx", "Ty", "Tz")]
    psis = [api.Wavefunction.from_fixture(p) for p in g["psi"]]
    yield "ligand_field", HX, Ts, psis
    rng = np.random.default_rng(3)
    # complex Hermitian hopping inside the 3d shell (orbitals 6-15) added to HX: every term and
    # its conjugate; the closure keeps the same 120 determinants
    terms = []
    for _ in range(40):
        i, j = rng.choice(np.arange(6, 16), 2, replace=False)
        v = complex(rng.normal(), rng.normal())
        terms += [([0x8000 | int(i), int(j)], v), ([0x8000 | int(j), int(i)], v.conjugate())]
    yield "complex", api.Operator(HX.nf, list(HX.terms) + terms), Ts, psis


@pytest.mark.parametrize("eps,gamma", [(0.0, 0.0), (1e-6, 0.3)])
def test_small_basis_chains_match_the_general_path(api, eps, gamma):
    import torch
    eng = api.engine()
    for name, H, Ts, psis in _cases(api):
        tpsi = [api.OperatorPsi(T, p) for T in Ts for p in psis]
        tpsi = [t for t in tpsi if t.N]
        seed = np.concatenate([t.det for t in tpsi])
        b = api.closure(H, seed, H.nf, None, -1, eng)
        assert 0 < b.n <= 2048
        X = np.zeros((b.n, len(tpsi)), dtype=np.complex128)
        for s, t in enumerate(tpsi):
            np.add.at(X[:, s], b.find(t.det), t.val)
        x = torch.from_numpy(X).cuda()
        ntri = 60
        try:
            eng.check(eng.L.qg_set_small_basis_lanczos(eng.ctx, 0))
            alone = [api.lanczos_block(H, b, x[:, s:s + 1].contiguous(), ntri, eps, gamma, eng)
                     for s in range(X.shape[1])]
            eng.check(eng.L.qg_set_small_basis_lanczos(eng.ctx, 1))
            l0 = eng.L.qg_launch_count(eng.ctx)
            A, B = api.lanczos_block(H, b, x.contiguous(), ntri, eps, gamma, eng)
            launches = eng.L.qg_launch_count(eng.ctx) - l0
        finally:
            eng.check(eng.L.qg_set_small_basis_lanczos(eng.ctx, 1))
        for s, (a1, b1) in enumerate(alone):
            assert np.array_equal(A[s], a1[0]) and np.array_equal(B[s], b1[0]), (name, s)
        assert launches <= 4, (name, launches)  # the rows (two) and one persistent launch


def test_small_basis_krylov_vectors(api):
    import torch
    eng = api.engine()
    name, H, Ts, psis = next(_cases(api))
    t = api.OperatorPsi(Ts[0], psis[0])
    b = api.closure(H, t.det, H.nf, None, -1, eng)
    X = np.zeros((b.n, 1), dtype=np.complex128)
    np.add.at(X[:, 0], b.find(t.det), t.val)
    x = torch.from_numpy(X).cuda()
    ntri = 30
    K = {}
    try:
        for on in (0, 1):
            eng.check(eng.L.qg_set_small_basis_lanczos(eng.ctx, on))
            K[on] = torch.zeros((ntri, b.n), dtype=torch.complex128, device="cuda")
            K[on] = (api.lanczos_block(H, b, x.clone(), ntri, 0.0, 0.0, eng, krylov=K[on]), K[on])
    finally:
        eng.check(eng.L.qg_set_small_basis_lanczos(eng.ctx, 1))
    (a0, b0), K0 = K[0]
    (a1, b1), K1 = K[1]
    assert np.array_equal(a0, a1) and np.array_equal(b0, b1)
    assert torch.equal(K0, K1)
