"""Parameter scans: H = sum_k p_k O_k kept on the device (OperatorSum) against operators built
directly from the summed ladder strings, before and after rescaling, on fresh bases and on a
basis whose caches were built under the old coefficients."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12


def rel_err(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.fixture(scope="module")
def api():
    from quanty_gb300 import build
    build.build()
    from quanty_gb300 import api
    return api


def _components(api):
    """The 2-shell Anderson impurity split into four parts: the atomic multiplet and field
    (impurity only), the d-d and p-d Coulomb F0, the hybridisation, the bath energies."""
    from quanty_gb300 import workloads
    H, R, seed, info = workloads.anderson_impurity(nshell=2, hole_max=2, particle_max=2)
    groups = {"local": [], "hyb": [], "bath": []}
    for ops, v in H.terms:
        orbs = [o & 0x7FFF for o in ops]
        if all(o < 16 for o in orbs):
            groups["local"].append((ops, v))
        elif len(ops) == 2 and orbs[0] != orbs[1]:
            groups["hyb"].append((ops, v))
        else:
            groups["bath"].append((ops, v))
    comps = [api.Operator(H.nf, groups[k], name=k) for k in ("local", "hyb", "bath")]
    # a fourth component overlapping the first (same strings): merged in the union
    comps.append(api.Operator(H.nf, groups["local"][: len(groups["local"]) // 3], name="overlap"))
    return H, R, seed, comps


def _direct(api, comps, p):
    return api.Operator(comps[0].nf, [(o, complex(v) * complex(c)) for comp, c in zip(comps, p) for o, v in comp.terms])


def _apply(api, H, b, x):
    import torch
    eng = api.engine()
    y = eng.empty(b.n, x.shape[1])
    eng.check(eng.L.qg_apply(eng.ctx, H.handle(), b.h, b.h, api._ptr(x), api._ptr(y), x.shape[1]))
    torch.cuda.synchronize()
    return y.cpu().numpy()


def test_sum_operator_matches_direct_and_rescales(api, oracle_mod):
    import torch
    H0, R, seed, comps = _components(api)
    nf = H0.nf
    p1 = [1.0, 1.0, 1.0, 0.0]
    S = api.OperatorSum(comps, p1)
    D1 = _direct(api, comps, p1)
    sd = api.dets_to_bytes([seed], nf)
    b = api.closure(S, sd, nf, R)
    assert b.n == api.closure(D1, sd, nf, R).n
    rng = np.random.default_rng(3)
    x = torch.from_numpy(rng.normal(size=(b.n, 3)) + 1j * rng.normal(size=(b.n, 3))).cuda()
    x1 = x[:, :1].contiguous()
    assert rel_err(_apply(api, S, b, x1), _apply(api, D1, b, x1)) < TOL
    assert rel_err(_apply(api, S, b, x), _apply(api, D1, b, x)) < TOL
    assert S.info()["hermitian"]
    # rescale: the same basis object (caches built under p1) and a fresh one
    p2 = [0.8, 1.7, -0.4, 0.35 + 0.0j]
    S.set_coefficients(p2)
    D2 = _direct(api, comps, p2)
    assert rel_err(_apply(api, S, b, x1), _apply(api, D2, b, x1)) < TOL
    assert rel_err(_apply(api, S, b, x), _apply(api, D2, b, x)) < TOL
    # against the oracle's push-form H*psi of the summed strings on the same basis
    O = oracle_mod
    dets = b.dets_bytes()
    xv = x1.cpu().numpy()[:, 0]
    op = O.Op({"nf": nf, "terms": [[list(t[0]), t[1].real, t[1].imag] for t in D2.terms]})
    want = O.apply_conserve(op, O.WF(nf, dets, xv))
    assert rel_err(_apply(api, S, b, x1)[:, 0], want) < TOL
    # Lanczos on the rescaled sum equals Lanczos on the direct operator
    a_s, b_s = api.lanczos_block(S, b, x1.clone(), 40, 0.0, 0.0)
    a_d, b_d = api.lanczos_block(D2, b, x1.clone(), 40, 0.0, 0.0)
    assert np.max(np.abs(a_s[0, :20] - a_d[0, :20])) < 1e-10 * np.max(np.abs(a_d[0, :20]))
    assert np.max(np.abs(b_s[0, :20] - b_d[0, :20])) < 1e-10 * np.max(np.abs(b_d[0, :20]))


def test_zero_coefficient_grows_the_reference_basis(api):
    """A component scaled to zero reaches nothing: closure of the sum equals the closure of
    the operator that leaves those strings out."""
    H0, R, seed, comps = _components(api)
    nf = H0.nf
    sd = api.dets_to_bytes([seed], nf)
    S = api.OperatorSum(comps[:3], [1.0, 1.0, 1.0])
    n_full = api.closure(S, sd, nf, None, 3).n
    S.set_coefficients([1.0, 0.0, 1.0])  # no hybridisation: the impurity keeps its electrons
    b0 = api.closure(S, sd, nf, None, 3)
    Dn = api.Operator(nf, [(o, v) for comp in (comps[0], comps[2]) for o, v in comp.terms])
    bd = api.closure(Dn, sd, nf, None, 3)
    assert b0.n == bd.n < n_full
    assert sorted(map(bytes, b0.dets_bytes())) == sorted(map(bytes, bd.dets_bytes()))


def test_eigensystem_through_a_scan(api):
    """Lowest energies of the 26-orbital ligand-field ion along a scan of its ligand terms
    (hybridisation and ligand energies), each equal to a fresh operator's (1e-10 eV)."""
    from quanty_gb300 import workloads
    ops, R = workloads.ligand_field()
    H = ops["H"]
    local = [(o, v) for o, v in H.terms if all((c & 0x7FFF) < 16 for c in o)]
    ligand = [(o, v) for o, v in H.terms if not all((c & 0x7FFF) < 16 for c in o)]
    comps = [api.Operator(26, local), api.Operator(26, ligand)]
    S = api.OperatorSum(comps, [1.0, 1.0])
    res = [26, 0] + [list(r) for r in R]
    for v in (1.0, 0.6, 1.4):
        S.set_coefficients([1.0, v])
        _, Es = api.Eigensystem(S, res, 3, {"Zero": 1e-12})
        _, Ed = api.Eigensystem(_direct(api, comps, [1.0, v]), res, 3, {"Zero": 1e-12})
        assert np.max(np.abs(np.asarray(Es) - np.asarray(Ed))) < 1e-10
    # the block-Lanczos branch on the rescaled sum (a 190-determinant basis: one restart)
    _, El = api.Eigensystem(S, res, 3, {"Zero": 1e-12, "DenseBorder": 0})
    assert np.max(np.abs(np.asarray(El) - np.asarray(Ed))) < 1e-10


def test_rescaling_a_plain_operator_is_refused(api):
    import ctypes
    H0, R, seed, comps = _components(api)
    eng = api.engine()
    c = np.array([1.0])
    st = eng.L.qg_operator_set_coefficients(comps[0].handle(), api._ptr(c), None)
    assert st == 4
