"""Real Lanczos chains two per complex vector (a real operator; start vectors with a zero
imaginary or zero real part): one pair gives coefficients bitwise those of each chain run alone;
several pairs, an odd chain out, a complex and an empty chain beside them agree with the runs
alone to rounding; with truncation and broadening on."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def api():
    from quanty_gb300 import build
    build.build()
    from quanty_gb300 import api
    return api


@pytest.mark.parametrize("eps,gamma", [(0.0, 0.0), (1e-5, 0.4)])
def test_paired_real_chains_match_their_runs_alone(api, eps, gamma):
    import torch
    from quanty_gb300 import workloads
    eng = api.engine()
    H, R, s0, info = workloads.anderson_impurity(nshell=2, hole_max=2, particle_max=2)
    b = api.closure(H, api.dets_to_bytes([s0], H.nf), H.nf, R)
    assert H.info()["nterms"] > 0
    n = b.n
    rng = np.random.default_rng(9)
    cols = [rng.normal(size=n) + 0j,                        # real
            1j * rng.normal(size=n),                        # imaginary
            rng.normal(size=n) + 1j * rng.normal(size=n),   # complex
            rng.normal(size=n) + 0j,                        # real
            np.zeros(n, dtype=np.complex128),               # empty
            rng.normal(size=n) * np.where(rng.random(n) < 0.5, 0.0, 1.0) + 0j]  # sparse real
    X = torch.from_numpy(np.stack(cols, axis=1)).cuda()
    ntri = 40
    try:
        eng.check(eng.L.qg_set_small_basis_lanczos(eng.ctx, 0))  # the general path on any size
        alone = [api.lanczos_block(H, b, X[:, k:k + 1].contiguous(), ntri, eps, gamma, eng) for k in range(len(cols))]
        l0 = eng.launches()
        A, B = api.lanczos_block(H, b, X.contiguous(), ntri, eps, gamma, eng)
        paired = eng.launches() - l0
        eng.check(eng.L.qg_set_split_chains(eng.ctx, 0))
        l0 = eng.launches()
        Ac, Bc = api.lanczos_block(H, b, X.contiguous(), ntri, eps, gamma, eng)
        unpaired = eng.launches() - l0
    finally:
        eng.check(eng.L.qg_set_split_chains(eng.ctx, 1))
        eng.check(eng.L.qg_set_small_basis_lanczos(eng.ctx, 1))
    # rounding differences grow along an unreorthogonalised recursion, so compare the first
    # steps tightly and the whole chain loosely
    for k, (a1, b1) in enumerate(alone):
        sc_a, sc_b = max(np.max(np.abs(a1[0])), 1e-300), max(np.max(np.abs(b1[0])), 1e-300)
        assert np.max(np.abs(A[k, :12] - a1[0, :12])) <= 1e-12 * sc_a, k
        assert np.max(np.abs(B[k, :12] - b1[0, :12])) <= 1e-12 * sc_b, k
        assert np.max(np.abs(A[k] - a1[0])) <= 1e-5 * sc_a, k
        assert np.max(np.abs(B[k] - b1[0])) <= 1e-5 * sc_b, k
    # the complex multi-vector path agrees over the first steps (further on, truncation
    # decisions near the threshold follow the rounding of either path)
    assert np.max(np.abs(Ac[:, :12] - A[:, :12])) < 1e-12 * np.max(np.abs(A))
    assert paired > 0 and unpaired > 0
    # one pair (a real and an imaginary chain): the same reductions, the same bits
    try:
        eng.check(eng.L.qg_set_small_basis_lanczos(eng.ctx, 0))
        A2, B2 = api.lanczos_block(H, b, X[:, :2].contiguous(), ntri, eps, gamma, eng)
    finally:
        eng.check(eng.L.qg_set_small_basis_lanczos(eng.ctx, 1))
    for k in range(2):
        assert np.array_equal(A2[k], alone[k][0][0]) and np.array_equal(B2[k], alone[k][1][0]), k


@pytest.mark.parametrize("eps,gamma", [(0.0, 0.0), (1e-5, 0.4)])
def test_single_real_chain_on_real_vectors(api, eps, gamma):
    """One real (or purely imaginary) chain runs on real vectors: coefficients bitwise those of the
    same chain run as a complex vector."""
    import torch
    from quanty_gb300 import workloads
    eng = api.engine()
    H, R, s0, info = workloads.anderson_impurity(nshell=2, hole_max=2, particle_max=2)
    b = api.closure(H, api.dets_to_bytes([s0], H.nf), H.nf, R)
    rng = np.random.default_rng(11)
    for col in (rng.normal(size=b.n) + 0j, 1j * rng.normal(size=b.n)):
        x = torch.from_numpy(col.reshape(-1, 1)).cuda()
        out = {}
        try:
            eng.check(eng.L.qg_set_small_basis_lanczos(eng.ctx, 0))
            for on in (0, 1):
                eng.check(eng.L.qg_set_split_chains(eng.ctx, on))
                out[on] = api.lanczos_block(H, b, x.clone(), 40, eps, gamma, eng)
        finally:
            eng.check(eng.L.qg_set_split_chains(eng.ctx, 1))
            eng.check(eng.L.qg_set_small_basis_lanczos(eng.ctx, 1))
        assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
