"""Host logic of CreateResonantSpectra, Eigensystem and CreateSpectra's KrylovBasis option
checked on the CPU against the reference's outputs: branch choice (dense below DenseBorder,
Krylov otherwise), the bases of the dense branch, lists of operators and states, the spectrum
order of every form, energy shifts, automatic energy ranges (including the zero eigenvalue of
the reference's unused blocks in the Krylov tensor form), Eigensystem's basis growth and the
vectors KrylovBasis returns.

Only the orchestration in quanty_gb300/api.py runs here: every device call it makes (bases,
H*psi, dense operator matrices, the Lanczos recursions, the spectrum kernels) is replaced for
the test by the oracle's CPU equivalent.  The device path itself is checked against the same
fixtures by tests/test_gpu_rixs.py and tests/test_gpu_eigen.py."""
import contextlib

import numpy as np
import pytest
import torch

from conftest import golden

TOL = 1e-8


def _oop(O, op):
    return O.Op({"nf": op.nf, "terms": [[list(t[0]), t[1].real, t[1].imag] for t in op.terms]})


class _Basis:
    """A sorted determinant set standing in for a device basis."""

    def __init__(self, O, api, nf, dets):
        dets = np.asarray(dets, dtype=np.uint8).reshape(-1, api.nword(nf))
        self.O, self.nf = O, nf
        self.dets = np.unique(dets, axis=0) if len(dets) else dets
        self.h = self
        self.idx = {bytes(r): i for i, r in enumerate(self.dets)}

    @property
    def n(self):
        return len(self.dets)

    def find(self, d):
        return np.array([self.idx.get(bytes(r), -1) for r in np.asarray(d).reshape(len(d), -1)], dtype=np.int64)

    def dets_bytes(self):
        return self.dets

    def wf(self, v=None):
        return self.O.WF(self.nf, self.dets, np.ones(self.n) if v is None else v)


@pytest.fixture
def host_api(monkeypatch, oracle_mod):
    from quanty_gb300 import api
    O = oracle_mod

    def B(nf, dets):
        return _Basis(O, api, nf, dets)

    def apply_vec(T, dst, src, x):
        out = np.zeros(dst.n, dtype=np.complex128)
        if src.n:
            w = O.operator_psi(_oop(O, T), src.wf(x))
            for r, v in zip(w.det, w.val):
                i = dst.idx.get(bytes(r))
                if i is not None:
                    out[i] += v
        return out

    class L:
        def qg_basis_map(self, ctx, src, xs, dst, x, k):
            X, Xs = x.numpy(), xs.numpy()
            for r, d in enumerate(src.dets):
                X[dst.idx[bytes(d)], :k] = Xs[r, :k]
            return 0

        def qg_lanczos_krylov(self, ctx, H, b, x, ntri, eps, a, bb, K):
            aa, b2, Ks = O.lanczos_krylov(_oop(O, H), b.wf(x.numpy()[:b.n, 0]), ntri, eps)
            a[:], bb[:] = aa, b2
            Kn = K.numpy()
            for i, w in enumerate(Ks):
                for r, v in zip(w.det, w.val):
                    Kn[i, b.idx[bytes(r)]] += v
            return 0

        def qg_expectation(self, ctx, H, b, x, k, out):
            M = O.dense_matrix(_oop(O, H), b.wf())
            X = x.numpy()[:b.n]
            for j in range(k):
                e = np.vdot(X[:, j], M @ X[:, j])
                out[2 * j], out[2 * j + 1] = e.real, e.imag
            return 0

        def qg_apply(self, ctx, T, dst, src, x, y, k):
            X, Y = x.numpy(), y.numpy()
            for c in range(k):
                Y[:dst.n, c] = apply_vec(T, dst, src, X[:src.n, c])
            return 0

        def qg_krylov_combine(self, ctx, K, n, nk, C, npc, out):
            out.numpy()[:n, :npc] = K.numpy()[:nk, :n].T @ np.asarray(C).reshape(nk, npc)
            return 0

        def qg_norm(self, ctx, n, k, x, out):
            out[:k] = np.linalg.norm(x.numpy()[:n, :k], axis=0)
            return 0

        def qg_block_adjoint_product(self, ctx, A, lda, ka, B, ldb, kb, n, C):
            C.numpy()[:ka, :kb] = A.numpy()[:n, :ka].conj().T @ B.numpy()[:n, :kb]
            return 0

        def qg_block_product(self, ctx, A, lda, ka, M, kb, n, alpha, beta, X, ldx):
            Xn = X.numpy()
            Xn[:n, :kb] = beta * Xn[:n, :kb] + alpha * (A.numpy()[:n, :ka] @ M.numpy()[:ka, :kb])
            return 0

    zeros, empty = torch.zeros, torch.empty

    class Eng:
        device, ctx = 0, None

        def __init__(self):
            self.torch, self.L = torch, L()

        def check(self, st, ctx=None):
            assert st == 0

        def empty(self, n, nvec=1):
            return zeros((max(n, 1), nvec), dtype=torch.complex128)

        def on_stream(self):
            return contextlib.nullcontext()

        def to_host(self, t):
            return t.numpy().copy()

    def plain_lanczos(H, b, x, ntri, eps, gamma, eng=None, krylov=None):
        """Three-term recursion without truncation, as the device runs it at Epsilon 0."""
        X = x.numpy()
        M = O.dense_matrix(_oop(O, H), b.wf())
        A, Bv = [], []
        for c in range(X.shape[1]):
            v0 = X[:b.n, c]
            a, bb = np.zeros(ntri + 1), np.zeros(ntri)
            bb[0] = np.linalg.norm(v0)
            v = v0 / bb[0] if bb[0] > 0 else 0 * v0
            vp, bp = 0 * v0, 0.0
            for i in range(ntri):
                if krylov is not None:
                    krylov.numpy()[i, :b.n, c] = v
                w = M @ v
                a[i + 1] = np.vdot(v, w).real
                w = w - a[i + 1] * v - bp * vp
                if i + 1 < ntri:
                    nb = np.linalg.norm(w)
                    bb[i + 1] = nb
                    vp, v, bp = v, (w / nb if nb > 100 * np.finfo(float).tiny else 0 * w), nb
            A.append(a)
            Bv.append(bb)
        return np.array(A), np.array(Bv)

    def lowdin_once(V, reduce, sv):
        S = V.conj().T @ V
        w, U = np.linalg.eigh(0.5 * (S + S.conj().T))
        s = np.sqrt(np.maximum(w, 0.0))
        zero = max(sv, 3 * np.sqrt(np.finfo(float).eps) * (s.max() if len(s) else 0.0))
        keep = [i for i in range(len(s)) if (not reduce and s[i] > 0) or s[i] > zero]
        if len(keep) == len(s):
            return V @ (U / s) @ U.conj().T
        return V @ (U[:, keep] / s[keep])

    def block_lanczos(H, b, x, ntri, eps, sv, eng=None, krylov=None):
        """The block recursion of qg_block_lanczos in numpy on the dense H: Loewdin twice with
        the deflation rule, six projections, entries below eps zeroed."""
        Hm = O.dense_matrix(_oop(O, H), b.wf())
        V0 = x.numpy()[:b.n]
        m = V0.shape[1]
        A = np.zeros((ntri + 1, m, m), dtype=np.complex128)
        Bm = np.zeros((ntri, m, m), dtype=np.complex128)
        sizes = np.zeros(ntri + 1, dtype=np.int32)
        sizes[0] = m

        def lowdin(V):
            Q = lowdin_once(V, True, sv)
            return lowdin_once(Q, False, sv) if Q.shape[1] else Q
        Q = lowdin(V0)
        k = Q.shape[1]
        sizes[1] = k
        Bm[0][:, :k] = (Q.conj().T @ V0).T
        Qp = np.zeros((b.n, 0), dtype=np.complex128)
        for it in range(1, ntri + 1):
            if k == 0:
                break
            if krylov is not None:
                krylov.numpy()[(it - 1) * m:(it - 1) * m + k, :b.n] = Q.T
            W = Hm @ Q
            A[it][:k, :k] = Q.conj().T @ W
            if it > 1:
                Bm[it - 1][:Qp.shape[1], :k] = Qp.conj().T @ W
            if it == ntri:
                break
            for P in (Q, Q, Qp, Qp, Q, Qp):
                W = W - P @ (P.conj().T @ W)
            Qn = lowdin(W)
            if eps > 0:
                Qn = np.where(np.abs(Qn) ** 2 < eps * eps, 0.0, Qn)
            sizes[it + 1] = Qn.shape[1]
            Qp, Q, k = Q, Qn, Qn.shape[1]
        return A, Bm, sizes

    def block_cf(E0, A, Bm, emin, emax, ne, g, eng=None):
        m = A.shape[1]
        out = np.zeros((m * m, ne + 1), dtype=np.complex128)
        for kf in range(ne + 1):
            w = emin + kf * (emax - emin) / ne + E0
            G = np.zeros((m, m), dtype=np.complex128)
            for blk in range(A.shape[0] - 1, 0, -1):
                G = np.linalg.inv((w + 0.5j * g) * np.eye(m) - A[blk] - G)
                Bk = Bm[blk - 1]
                G = (Bk.conj() @ G @ Bk.T) if blk == 1 else (Bk @ G @ Bk.conj().T)
            out[:, kf] = G.reshape(-1)
        return out

    def poles(E0, p, W, emin, emax, ne, g, eng=None):
        W = np.atleast_2d(W)
        P = np.broadcast_to(np.atleast_2d(p), W.shape)
        E = np.broadcast_to(np.asarray(E0, float), (W.shape[0],))
        return np.array([O.poles_spectrum(P[s], W[s], E[s], emin, (emax - emin) / ne, ne, g)
                         for s in range(W.shape[0])])

    def cf(E0, A, Bv, emin, emax, ne, g, eng=None):
        E = np.broadcast_to(np.asarray(E0, float), (len(A),))
        return np.array([O.cf_spectrum(A[s], Bv[s], E[s], emin, (emax - emin) / ne, ne, g) for s in range(len(A))])

    def eigh(M, nv=None, eng=None):
        w, v = np.linalg.eigh(0.5 * (M + M.conj().T))
        return w, v[:, :(len(w) if nv is None else nv)]

    def opsi(T, p, R=None, eng=None):
        w = O.operator_psi(_oop(O, T), O.WF(p.nf, p.det, p.val), api.parse_restrictions(R))
        return api.Wavefunction(p.nf, w.det, w.val)

    def closure_of(H, s, R=None, m=-1, eng=None):
        if not s.n:
            return s
        return B(s.nf, O.closure(_oop(O, H), s.wf(), api.parse_restrictions(R)).det)

    def krylov_one(H1, H2, T, T2s, p, o, eng):
        G = O.resonant_spectra(_oop(O, H1), _oop(O, H2), _oop(O, T), [_oop(O, t) for t in T2s],
                               O.WF(p.nf, p.det, p.val),
                               dict(o, Restrictions1=api.parse_restrictions(o.get("Restrictions1")),
                                    Restrictions2=api.parse_restrictions(o.get("Restrictions2"))))
        return G, {"emin2": o["Emin2"], "emax2": o["Emax2"]}

    monkeypatch.setattr(torch.Tensor, "to", lambda self, *a, **k: self)
    monkeypatch.setattr(torch, "zeros", lambda *a, **k: zeros(*a, **{x: y for x, y in k.items() if x != "device"}))
    monkeypatch.setattr(torch, "empty", lambda *a, **k: empty(*a, **{x: y for x, y in k.items() if x != "device"}))
    monkeypatch.setattr(api, "_engine", Eng())
    monkeypatch.setattr(api, "_ptr", lambda a: a)
    monkeypatch.setattr(api.Operator, "handle", lambda self, eng=None: self)
    def from_bytes(cls, nf, d, eng=None):
        b = B(nf, d)
        return b, b.find(d)

    monkeypatch.setattr(api.Basis, "from_bytes", classmethod(from_bytes))
    def device_targets(T, b, R=None, eng=None):
        # the device growth leaves zero-valued strings out
        nz = api.Operator(T.nf, [(o, v) for o, v in T.terms if v != 0])
        return B(b.nf, opsi(nz, api.Wavefunction(b.nf, b.dets, np.ones(b.n)), R).det)

    monkeypatch.setattr(api, "OperatorPsiBasis", device_targets)
    monkeypatch.setattr(api, "basis_union", lambda a, b, eng=None: B(a.nf, np.concatenate([a.dets, b.dets])))
    monkeypatch.setattr(api, "closure_of", closure_of)
    monkeypatch.setattr(api, "closure", lambda H, d, nf, R=None, m=-1, eng=None: closure_of(H, B(nf, d), R))
    monkeypatch.setattr(api, "OperatorPsi", opsi)
    monkeypatch.setattr(api, "PsiOperatorPsi",
                        lambda H, p, eng=None: O.expectation(_oop(O, H), O.WF(p.nf, p.det, p.val)))
    monkeypatch.setattr(api, "OperatorToDeterminantMatrix", lambda H, b, eng=None: O.dense_matrix(_oop(O, H), b.wf()))
    monkeypatch.setattr(api, "hermitian_eigh", eigh)
    def apply_between(T, dst, src, X, eng, device=False):
        X = X if isinstance(X, np.ndarray) else X.numpy()
        Y = np.stack([apply_vec(T, dst, src, X[:, c]) for c in range(X.shape[1])], 1) if X.shape[1] \
            else np.zeros((dst.n, 0), dtype=np.complex128)
        return torch.from_numpy(np.ascontiguousarray(Y, dtype=np.complex128)) if device else Y

    monkeypatch.setattr(api, "_apply_between", apply_between)
    monkeypatch.setattr(api, "ListOfPolesToSpectrum", poles)
    monkeypatch.setattr(api, "lanczos_block", plain_lanczos)
    monkeypatch.setattr(api, "TriDiagonalMatrixToSpectrum", cf)
    monkeypatch.setattr(api, "_rixs_krylov", krylov_one)
    monkeypatch.setattr(api, "block_lanczos", block_lanczos)
    monkeypatch.setattr(api, "BlockTriDiagonalMatrixToSpectra", block_cf)
    return api


GRID = {"Emin1": -5, "Emax1": 15, "NE1": 4, "Gamma1": 0.8, "Emin2": -2, "Emax2": 8, "NE2": 64, "Gamma2": 0.3}
KRYLOV = {"DenseBorder": 0, "Epsilon": 0.0}
CASES = [
    # key, T1, T2, number of initial states, options, branch
    ("dense_lists", ("Tx", "Ty"), ("Txd", "Tyd", "Tzd"), 2, GRID, "dense"),
    ("dense_auto", ("Tx",), ("Txd", "Tyd"), 1, {"NE1": 4, "Gamma1": 0.8, "NE2": 64, "Gamma2": 0.3}, "dense"),
    ("dense_tensor", ("Tx", "Ty"), ("Txd", "Tyd"), 1, dict(GRID, Tensor=True), "dense"),
    ("dense_tensor_psi", ("Tx",), ("Tyd",), 2, dict(GRID, Tensor=True), "dense"),
    ("dense_shifts", ("Tx", "Ty"), ("Txd",), 2, dict(GRID, E0_1=-37.0, E0_2=-17.0), "dense"),
    ("dense_e0", ("Tx", "Ty"), ("Txd",), 2, dict(GRID, E0=-30.0), "dense"),
    ("krylov_lists", ("Tx", "Ty"), ("Txd", "Tyd"), 2, dict(GRID, **KRYLOV), "krylov"),
    ("krylov_tensor", ("Tx", "Ty"), ("Txd", "Tyd"), 1, dict(GRID, Tensor=True, NTri1=40, NTri2=40, **KRYLOV),
     "krylov_tensor"),
    ("krylov_tensor_auto", ("Tx", "Ty"), ("Txd",), 1,
     dict(KRYLOV, NE1=3, NE2=48, Tensor=True, NTri1=40, NTri2=40), "krylov_tensor"),
    ("krylov_tensor_psi", ("Tx",), ("Tyd",), 2, dict(GRID, Tensor=True, NTri1=40, NTri2=40, **KRYLOV),
     "krylov_tensor"),
    ("dense_res2", ("Tx", "Ty"), ("Txd", "Tyd"), 1, dict(GRID, Restrictions2=[16, 0, ["000000 1010101010", 4, 4]]),
     "dense"),
    ("krylov_res2", ("Tx", "Ty"), ("Txd", "Tyd"), 1,
     dict(GRID, Restrictions2=[16, 0, ["000000 1010101010", 4, 4]], **KRYLOV), "krylov"),
    ("dense_res1", ("Tx", "Ty"), ("Txd", "Tyd"), 1, dict(GRID, Restrictions1=[16, 0, ["000000 1010101010", 5, 5]]),
     "dense"),
    ("krylov_res1", ("Tx", "Ty"), ("Txd", "Tyd"), 1,
     dict(GRID, Restrictions1=[16, 0, ["000000 1010101010", 5, 5]], **KRYLOV), "krylov"),
    ("krylov_tensor_res1", ("Tx", "Ty"), ("Txd", "Tyd"), 1,
     dict(GRID, Restrictions1=[16, 0, ["000000 1010101010", 5, 5]], Tensor=True, **KRYLOV), "krylov_tensor"),
    ("krylov_tensor_short", ("Tx", "Ty"), ("Txd", "Tyd"), 1, dict(GRID, Tensor=True, NTri1=4, NTri2=5, **KRYLOV),
     "krylov_tensor"),
    ("krylov_tensor_short_auto", ("Tx", "Ty"), ("Txd",), 1,
     dict(KRYLOV, NE1=3, NE2=48, Tensor=True, NTri1=6, NTri2=8), "krylov_tensor"),
]


ONEBODY = [("list_dense", "psilist", 10000, "dense"), ("list_krylov", "psilist", 1, "krylov"),
           ("psi0_dense", "psi0", 10000, "dense"), ("psi0_krylov", "psi0", 1, "krylov")]


def test_zero_valued_strings_shape_the_dense_bases(host_api):
    """The zero constant of "OppT = 0 + ..." puts the initial states' sector into the dense
    bases of RIXS and of CreateSpectra, so the automatic energy ranges span it (reference
    outputs of the one-particle model)."""
    api = host_api
    g = golden("rixs_onebody.json")
    H1, H0, T, T2 = (api.Operator.from_fixture(g[k]) for k in ("H1", "H0", "OppT", "T2"))
    p0 = api.Wavefunction.from_fixture(g["psi0"])
    G, st = api.CreateResonantSpectra(H1, H0, T, T2, p0, {"NE1": 5, "Gamma1": 0.1, "NE2": 200, "Gamma2": 0.1})
    ref = g["psi0_dense_auto"]
    R = np.array(ref["re"]) + 1j * np.array(ref["im"])
    assert st["method"] == "dense" and abs(st["emin2"] - ref["emin"]) < 1e-10 and abs(st["emax2"] - ref["emax"]) < 1e-10
    assert np.max(np.abs(G - R)) / np.max(np.abs(R)) < TOL
    S, _ = api.CreateSpectra(H1, T, p0, {"NE": 100})
    ref = g["xas_dense_auto"]
    R = np.array(ref["re"]) + 1j * np.array(ref["im"])
    assert abs(S.Emin - ref["emin"]) < 1e-10 and abs(S.Emax - ref["emax"]) < 1e-10 and abs(S.Gamma - ref["gamma"]) < 1e-10
    assert np.max(np.abs(S.G - R)) / np.max(np.abs(R)) < TOL


@pytest.mark.parametrize("key,which,border,branch", ONEBODY, ids=[c[0] for c in ONEBODY])
def test_one_particle_rixs_of_the_reference_test(host_api, key, which, border, branch):
    """The one-particle model of TestScripts/CreateResonantSpectra.Quanty: DenseBorder 10000
    takes the dense branch, DenseBorder 1 the Krylov branch (one run per state of the list)."""
    api = host_api
    g = golden("rixs_onebody.json")
    H1, H0, T, T2 = (api.Operator.from_fixture(g[k]) for k in ("H1", "H0", "OppT", "T2"))
    psi = ([api.Wavefunction.from_fixture(p) for p in g["psilist"]] if which == "psilist"
           else api.Wavefunction.from_fixture(g["psi0"]))
    G, st = api.CreateResonantSpectra(H1, H0, T, T2, psi, dict(g["opts"], DenseBorder=border))
    R = np.array(g[key]["re"]) + 1j * np.array(g[key]["im"])
    assert st["method"] == branch and G.shape == R.shape
    assert np.max(np.abs(G - R)) / np.max(np.abs(R)) < TOL


@pytest.mark.parametrize("key,t1,t2,npsi,opts,branch", CASES, ids=[c[0] for c in CASES])
def test_resonant_spectra_orchestration_matches_reference(host_api, key, t1, t2, npsi, opts, branch):
    api = host_api
    g = golden("rixs.json")
    op = lambda k: api.Operator.from_fixture(g[k])  # noqa: E731
    psis = [api.Wavefunction.from_fixture(p) for p in g["psi"][:npsi]]
    G, st = api.CreateResonantSpectra(op("HX"), op("H"), [op(t) for t in t1], [op(t) for t in t2],
                                      psis if npsi > 1 else psis[0], dict(opts))
    ref = g[key]
    R = np.array(ref["re"]) + 1j * np.array(ref["im"])
    assert st["method"] == branch
    assert G.shape == R.shape
    assert np.max(np.abs(G - R)) / np.max(np.abs(R)) < TOL
    assert abs(st["emin2"] - ref["emin"]) < 1e-10 and abs(st["emax2"] - ref["emax"]) < 1e-10
    if "gamma2" in st:
        assert abs(st["gamma2"] - ref["gamma"]) < 1e-10


def test_eigensystem_growth_and_call_forms(host_api):
    """Growth beyond the start restrictions without the Restrictions option, confinement with
    it, and the start-state call form, against the reference's energies."""
    api = host_api
    g = golden("eigen_growth.json")
    H = api.Operator.from_fixture(golden("c1_lf.json")["H"])
    Rn = [26, 0] + [list(r) for r in g["start_restrictions"]]
    _, E = api.Eigensystem(H, Rn, 3)
    assert np.max(np.abs(np.array(E) - g["energies_grown"])) < 1e-10
    psis, E = api.Eigensystem(H, Rn, 3, {"Restrictions": Rn})
    assert np.max(np.abs(np.array(E) - g["energies_confined"])) < 1e-10
    out, E = api.Eigensystem(H, psis)
    assert len(out) == 3 and np.max(np.abs(np.array(E) - g["energies_from_states"])) < 1e-10
    # ExpandBasis false: the confined states' own basis, so the confined energies again
    out, E = api.Eigensystem(H, psis, {"ExpandBasis": False})
    assert np.max(np.abs(np.array(E) - g["energies_confined"])) < 1e-10


def _wf_err(api, ref, got):
    R = api.Wavefunction.from_fixture(ref)
    d = {bytes(r): v for r, v in zip(got.det, got.val)}
    assert len(got.val) == len(R.val)
    v = np.array([d[bytes(r)] for r in R.det])
    return np.max(np.abs(v - R.val)) / np.max(np.abs(R.val))


def test_krylov_basis_option(host_api):
    """KrylovBasis: the Lanczos branch returns the reference's Krylov vectors (the count of
    non-empty ones, and the leading ones element by element; later ones depend on rounding
    that the recursion amplifies) with unchanged spectra, a list per pair for several pairs
    (at Epsilon 0 the orthogonality test keeps one vector each); the dense branch returns the
    eigenstates of H."""
    import math
    api = host_api
    g = golden("krylov_basis.json")
    r = golden("rixs.json")
    HX, Tx, Tz = (api.Operator.from_fixture(d) for d in (r["HX"], r["Tx"], g["Tz"]))
    psi1, psi2 = (api.Wavefunction.from_fixture(p) for p in r["psi"])
    o = {"NE": 32, "Emin": -10, "Emax": 20, "Gamma": 0.5}

    def spec(key):
        return np.array(g[key]["re"]) + 1j * np.array(g[key]["im"])

    S, tri, K = api.CreateSpectra(HX, Tz, psi1, dict(o, Method="Lanczos", KrylovBasis=True, NTri=80))
    assert np.max(np.abs(S.G - spec("lanczos_one"))) / np.max(np.abs(spec("lanczos_one"))) < TOL
    assert len(K) == len(g["krylov_one"])
    for ref, got in list(zip(g["krylov_one"], K))[:12]:
        assert _wf_err(api, ref, got) < 1e-10
    S, tri, K = api.CreateSpectra(HX, [Tx, Tz], [psi1, psi2],
                                  dict(o, Method="Lanczos", KrylovBasis=True, NTri=80, Epsilon=0.0))
    assert np.max(np.abs(S.G - spec("lanczos_lists"))) / np.max(np.abs(spec("lanczos_lists"))) < TOL
    assert [len(k) for k in K] == [len(k) for k in g["krylov_lists"]]
    for refs, got in zip(g["krylov_lists"], K):
        for ref, k in zip(refs, got):
            assert _wf_err(api, ref, k) < 1e-12
    S, poles, K = api.CreateSpectra(HX, Tz, psi1, dict(o, Method="Dense", KrylovBasis=True))
    assert np.max(np.abs(S.G - spec("dense_states"))) / np.max(np.abs(spec("dense_states"))) < TOL
    E = [api.PsiOperatorPsi(HX, k).real for k in K]
    assert len(E) == len(g["dense_energies"]) and np.max(np.abs(np.array(E) - g["dense_energies"])) < 1e-10
    assert math.isclose(np.linalg.norm(K[0].val), 1.0, rel_tol=1e-12)


def test_zero_valued_strings_reach_their_targets(oracle_mod, monkeypatch):
    """H*psi inserts the targets of zero-valued strings with amplitude 0, as the reference's
    OperatorPsi does (the "O = 0; O = O + ..." constant, cancelled sums): the host
    enumeration of those targets equals the oracle's, with and without restrictions, and
    OperatorPsi merges them into the device result in sorted order."""
    from quanty_gb300 import api
    O = oracle_mod
    g = golden("rixs.json")
    g1 = golden("rixs_onebody.json")
    HX = api.Operator.from_fixture(g["HX"])
    psi = api.Wavefunction.from_fixture(g["psi"][0])
    Z = api.Operator(HX.nf, [(ops, 0.0) for ops, v in HX.terms])  # every string, value zero
    R = [("1111110000000000", 5, 6), ("0000001111111111", 8, 9)]
    for res in (None, R):
        got = api._zero_term_targets(Z, psi.det, res)
        ref = O.operator_psi(O.Op({"nf": 16, "terms": [[list(t[0]), 0.0, 0.0] for t in HX.terms]}),
                             O.WF(16, psi.det, psi.val), res)
        assert sorted(map(bytes, got)) == sorted(map(bytes, ref.det))
        assert np.all(ref.val == 0)
    # the merge: a device growth without the zero-valued strings, then OperatorPsi's result
    T = api.Operator.from_fixture(g1["OppT"])  # holds the zero constant of "OppT = 0 + ..."
    p0 = api.Wavefunction.from_fixture(g1["psi0"])
    nz = api.Operator(T.nf, [(o, v) for o, v in T.terms if v != 0])
    dev = O.operator_psi(_oop(O, nz), O.WF(T.nf, p0.det, p0.val))
    order = np.lexsort(dev.det.T[::-1])

    class Dst:
        n = len(order)
        h = None

        def dets_bytes(self):
            return dev.det[order]

    class Eng:
        torch = torch

        def check(self, st, ctx=None):
            pass

        def empty(self, n, nvec=1):
            return torch.zeros((max(n, 1), nvec), dtype=torch.complex128)

        def to_host(self, t):
            return np.asarray(dev.val[order])

    eng = Eng()
    monkeypatch.setattr(api.Basis, "from_bytes", classmethod(lambda cls, nf, d, eng=None: (Dst(), np.arange(len(d)))))
    monkeypatch.setattr(api, "_upload", lambda *a, **k: None)
    monkeypatch.setattr(api, "OperatorPsiBasis", lambda *a, **k: Dst())
    monkeypatch.setattr(api, "_ptr", lambda a: a)
    eng.L = type("L", (), {"qg_apply": staticmethod(lambda *a: 0)})()
    eng.ctx = None
    monkeypatch.setattr(api.Operator, "handle", lambda self, eng=None: None)
    out = api.OperatorPsi(T, p0, eng=eng)
    ref = O.operator_psi(_oop(O, T), O.WF(T.nf, p0.det, p0.val))
    assert out.N == len(ref.val) == len(order) + p0.N
    assert [bytes(r) for r in out.det] == sorted(bytes(r) for r in ref.det)
    d = ref.as_dict()
    assert np.allclose([d[bytes(r)] for r in out.det], out.val, rtol=0, atol=1e-15)


def test_operator_restrictions_apply_to_h_psi(monkeypatch):
    """O.Restrictions (OperatorType.Res) makes O * psi the restricted product, as the
    reference's OperatorPsi dispatch does; an explicit restrictions argument wins."""
    from quanty_gb300 import api
    seen = []

    class Dst:
        n, h = 0, None

        def dets_bytes(self):
            return np.zeros((0, 1), dtype=np.uint8)

    class Eng:
        ctx, L = None, type("L", (), {"qg_apply": staticmethod(lambda *a: 0)})()

        def check(self, st, ctx=None):
            pass

        def empty(self, n, nvec=1):
            return torch.zeros((max(n, 1), nvec), dtype=torch.complex128)

        def to_host(self, t):
            return t.numpy()

    monkeypatch.setattr(api.Basis, "from_bytes", classmethod(lambda cls, nf, d, eng=None: (Dst(), np.arange(len(d)))))
    monkeypatch.setattr(api, "_upload", lambda *a, **k: None)
    monkeypatch.setattr(api, "OperatorPsiBasis", lambda O, b, R=None, eng=None: seen.append(R) or Dst())
    monkeypatch.setattr(api, "_ptr", lambda a: a)
    monkeypatch.setattr(api.Operator, "handle", lambda self, eng=None: None)
    O = api.NewOperator(4, 0, [[0, -1, 1.0]])
    psi = api.NewWavefunction(4, 0, [["0100", 1.0]])
    api.OperatorPsi(O, psi, eng=Eng())
    O.Restrictions = [4, 0, ["1100", 1, 1]]
    api.OperatorPsi(O, psi, eng=Eng())
    api.OperatorPsi(O, psi, [4, 0, ["1111", 1, 1]], eng=Eng())
    assert seen == [None, [4, 0, ["1100", 1, 1]], [4, 0, ["1111", 1, 1]]]


TENSOR = {
    "tensor_lanczos": {"Tensor": True, "Method": "Lanczos", "NE": 40, "Emin": -5, "Emax": 15, "Gamma": 0.6,
                       "Epsilon": 0.0},
    "tensor_lanczos_short": {"Tensor": True, "Method": "Lanczos", "NTri": 5, "NE": 40, "Emin": -5, "Emax": 15,
                             "Gamma": 0.6, "Epsilon": 0.0},
    "tensor_lanczos_short_auto": {"Tensor": True, "Method": "Lanczos", "NTri": 8, "NE": 32},
}


@pytest.mark.parametrize("key", list(TENSOR))
def test_tensor_spectra_orchestration_matches_reference(host_api, key):
    """CreateSpectra with Tensor = true, block-Lanczos branch: the block recursion, the pole
    range from the whole block tridiagonal matrix and the block continued fraction (numpy
    restatements of the device calls) against the reference's spectra, complete and incomplete
    Krylov spaces."""
    api = host_api
    g = golden("tensor.json")
    HX = api.Operator.from_fixture(g["HX"])
    Ts = [api.Operator.from_fixture(g[t]) for t in ("Tx", "Ty", "Tz")]
    psi = api.Wavefunction.from_fixture(g["psi"])
    S, _ = api.CreateSpectra(HX, Ts, [psi], TENSOR[key])
    R = api.Spectra.from_text(g[key])
    assert S.G.shape == R.G.shape
    assert abs(S.Emin - R.Emin) < 1e-8 and abs(S.Emax - R.Emax) < 1e-8 and abs(S.Gamma - R.Gamma) < 1e-8
    assert abs(S.EminPole - R.EminPole) < 1e-8 and abs(S.EmaxPole - R.EmaxPole) < 1e-8
    assert np.max(np.abs(S.G - R.G)) < TOL * np.max(np.abs(R.G))


def test_merged_calls_match_separate_calls(host_api):
    """The served form's continuous batching: CreateSpectra calls on one Hamiltonian with the same
    Lanczos settings but their own operators, states, windows and frequencies run as one
    multi-vector Lanczos over exactly their pairs, and each gets the spectra of its call alone."""
    api = host_api
    g = golden("rixs.json")
    HX, Tx, Ty = (api.Operator.from_fixture(g[k]) for k in ("HX", "Tx", "Ty"))
    psi1, psi2 = (api.Wavefunction.from_fixture(p) for p in g["psi"][:2])
    base = {"Method": "Lanczos", "NTri": 40, "Epsilon": 0.0, "Gamma": 0.5}
    jobs = [(Tx, psi1, dict(base, NE=32, Emin=-10, Emax=20)),
            ([Tx, Ty], [psi1, psi2], dict(base, NE=16)),
            (Ty, psi2, dict(base, NE=24, Emin=-5, Emax=15))]
    assert len({api.lanczos_merge_key(HX, *j) for j in jobs}) == 1
    assert api.lanczos_merge_key(HX, Tx, psi1, dict(base, NTri=41)) != api.lanczos_merge_key(HX, *jobs[0])
    merged = api.CreateSpectraMerged(HX, jobs)
    for (T, psi, o), (S, tri) in zip(jobs, merged):
        S1, tri1 = api.CreateSpectra(HX, T, psi, o)
        assert S.G.shape == S1.G.shape
        assert np.max(np.abs(S.G - S1.G)) <= 1e-10 * np.max(np.abs(S1.G))
        assert abs(S.Emin - S1.Emin) < 1e-10 and abs(S.Emax - S1.Emax) < 1e-10
