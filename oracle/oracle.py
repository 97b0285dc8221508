"""CPU oracle for the H*psi / Lanczos / continued-fraction path -- TEST INFRASTRUCTURE ONLY.

This module is the checker: tests/ compare the CUDA library against it, and bench.py's
CPU-baseline leg times it.  It loads ``oracle/_build/libqoracle.so`` (built by
``oracle/Makefile`` from ``qoracle.c``, a plain-C restatement of the reference) and adds small
numpy drivers.  The product under ``quanty_gb300/`` never imports it.

Determinants are handled in the reference's byte layout (``Core/OperatorWaveFunction.cpp:7-43``):
``nword = ceil(nf/8)`` bytes, orbital ``i`` in byte ``i>>3`` under mask ``128>>(i&7)``.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libqoracle.so")
CREATION = 0x8000

_lib = None


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        P, I64, D, I = C.c_void_p, C.c_int64, C.c_double, C.c_int
        L.qo_wf_from.restype = P
        L.qo_wf_from.argtypes = [I, I64, P, P, P]
        L.qo_wf_free.argtypes = [P]
        L.qo_wf_size.restype = I64
        L.qo_wf_size.argtypes = [P]
        L.qo_wf_get.argtypes = [P, P, P, P]
        L.qo_operator_psi.restype = P
        L.qo_operator_psi.argtypes = [I, P, P, P, P, P, P, I, P, P, P]
        L.qo_apply_conserve.argtypes = [I, P, P, P, P, P, P, I64, I64, P]
        L.qo_apply_conserve_strided.argtypes = [I, P, P, P, P, P, P, I64, I64, I64, P]
        L.qo_count_nnz.restype = I64
        L.qo_count_nnz.argtypes = [I, P, P, P, P, I64, I64]
        L.qo_count_nnz_strided.restype = I64
        L.qo_apply_multi.argtypes = [I, P, P, P, P, P, P, P, I, P, P]
        L.qo_count_nnz_strided.argtypes = [I, P, P, P, P, I64, I64, I64]
        L.qo_lanczos_tridiag.argtypes = [I, P, P, P, P, P, P, I, D, D, I, P, P, P, P, P]
        L.qo_cf_spectrum.argtypes = [I, P, P, D, D, D, I, D, P, P]
        L.qo_lanczos_krylov.argtypes = [I, P, P, P, P, P, P, I, D, I, P, P, P, P, P, P]
        L.qo_ladder.restype = I
        L.qo_ladder.argtypes = [P, P, I]
        L.qo_num_threads.restype = I
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


# ----------------------------------------------------------------------------- data helpers

def nword(nf):
    return (nf + 7) // 8


def dets_to_bytes(dets, nf):
    """'0101...' strings (orbital 0 first) -> uint8 array (n, nword), MSB-first bytes."""
    nw = nword(nf)
    out = np.zeros((len(dets), nw), dtype=np.uint8)
    for r, s in enumerate(dets):
        for i, ch in enumerate(s[:nf]):
            if ch == "1":
                out[r, i >> 3] |= 128 >> (i & 7)
    return out


def bytes_to_dets(b, nf):
    out = []
    for row in b:
        out.append("".join("1" if row[i >> 3] & (128 >> (i & 7)) else "0" for i in range(nf)))
    return out


class Op:
    """Flat term table: ladder strings concatenated, o[0] acting first, bit 15 = creation."""

    def __init__(self, fixture_op):
        self.nf = fixture_op["nf"]
        terms = fixture_op["terms"]
        self.len = np.array([len(t[0]) for t in terms], dtype=np.int32)
        self.off = np.zeros(len(terms), dtype=np.int64)
        if len(terms):
            self.off[1:] = np.cumsum(self.len)[:-1]
        flat = [o for t in terms for o in t[0]]
        self.ops = np.array(flat if flat else [0], dtype=np.uint16)
        self.vre = np.array([t[1] for t in terms], dtype=np.float64)
        self.vim = np.array([t[2] for t in terms], dtype=np.float64)
        self.nterms = len(terms)

    def args(self):
        return [self.nterms, _p(self.len), _p(self.off), _p(self.ops), _p(self.vre), _p(self.vim)]


class Restr:
    def __init__(self, nf, restrictions):
        self.n = len(restrictions or [])
        nw = nword(nf)
        self.masks = np.zeros((max(self.n, 1), nw), dtype=np.uint8)
        self.mn = np.zeros(max(self.n, 1), dtype=np.int32)
        self.mx = np.zeros(max(self.n, 1), dtype=np.int32)
        for r, (mask, lo, hi) in enumerate(restrictions or []):
            self.masks[r] = dets_to_bytes([mask.replace(" ", "")], nf)[0]
            self.mn[r] = lo
            self.mx[r] = hi

    def args(self):
        return [self.n, _p(self.masks), _p(self.mn), _p(self.mx)]


class WF:
    """Wavefunction in the oracle's own representation (insertion-ordered determinants)."""

    def __init__(self, nf, det_bytes, values):
        self.nf = nf
        self.det = np.ascontiguousarray(det_bytes, dtype=np.uint8).reshape(-1, nword(nf))
        self.val = np.ascontiguousarray(values, dtype=np.complex128).reshape(-1)

    @classmethod
    def from_fixture(cls, f):
        return cls(f["nf"], dets_to_bytes(f["dets"], f["nf"]), np.array(f["re"]) + 1j * np.array(f["im"]))

    def handle(self):
        re = np.ascontiguousarray(self.val.real)
        im = np.ascontiguousarray(self.val.imag)
        return lib().qo_wf_from(self.nf, len(self.val), _p(self.det), _p(re), _p(im))

    @classmethod
    def from_handle(cls, nf, h):
        L = lib()
        n = L.qo_wf_size(h)
        det = np.zeros((n, nword(nf)), dtype=np.uint8)
        re = np.zeros(n)
        im = np.zeros(n)
        if n:
            L.qo_wf_get(h, _p(det), _p(re), _p(im))
        L.qo_wf_free(h)
        return cls(nf, det, re + 1j * im)

    def as_dict(self):
        return {bytes(r): v for r, v in zip(self.det, self.val)}


# ----------------------------------------------------------------------------- algorithms

def operator_psi(op, psi, restrictions=None):
    """Growing-basis H*psi (reference OperatorPsi / OperatorPsiRestricted)."""
    r = Restr(psi.nf, restrictions)
    h = psi.handle()
    out = lib().qo_operator_psi(*op.args(), h, *r.args())
    lib().qo_wf_free(h)
    return WF.from_handle(psi.nf, out)


def apply_conserve(op, psi, row0=0, row1=None):
    """Fixed-basis H*psi, push form (reference OperatorPsiConserveBasisPreAllocated)."""
    row1 = len(psi.val) if row1 is None else row1
    h = psi.handle()
    y = np.zeros(2 * len(psi.val))
    lib().qo_apply_conserve(*op.args(), h, row0, row1, _p(y))
    lib().qo_wf_free(h)
    return y[0::2] + 1j * y[1::2]


def count_nnz(op, psi, row0=0, row1=None):
    row1 = len(psi.val) if row1 is None else row1
    h = psi.handle()
    n = lib().qo_count_nnz(op.nterms, _p(op.len), _p(op.off), _p(op.ops), h, row0, row1)
    lib().qo_wf_free(h)
    return n


def apply_sampled(op, handle, n, stride, row0=0):
    """Fixed-basis H*psi from the source rows row0, row0 + stride, ... only (push form, the
    full basis of the handle as the lookup target): equal to H applied to x with every other
    row zeroed.  `handle` is a WF.handle() the caller frees."""
    y = np.zeros(2 * n)
    lib().qo_apply_conserve_strided(*op.args(), handle, row0, n, stride, _p(y))
    return y[0::2] + 1j * y[1::2]


def apply_multi(op, src_handle, dst_handle, n_src, n_dst, X):
    """Push-form op X for the columns of X (n_src x nvec complex, rows in the order of the
    src handle's determinants) into the basis of dst (the same handle: the fixed-basis
    apply); returns n_dst x nvec."""
    X = np.ascontiguousarray(X, dtype=np.complex128)
    nvec = X.shape[1]
    Y = np.zeros((n_dst, nvec), dtype=np.complex128)
    lib().qo_apply_multi(*op.args(), src_handle, dst_handle, nvec, _p(X), _p(Y))
    return Y


def count_nnz_sampled(op, handle, n, stride, row0=0):
    """Pairs (source row, term) with a non-zero sign and the target in the basis, over the
    source rows row0, row0 + stride, ... (the pairs the push loop visits from them)."""
    return lib().qo_count_nnz_strided(op.nterms, _p(op.len), _p(op.off), _p(op.ops), handle, row0, n, stride)


def lanczos_tridiag(op, psi, ntri, eps, gamma, restrictions=None):
    """Reference LanczosTriDiagonalize on a growing basis; returns a (ntri+1), b (ntri)."""
    r = Restr(psi.nf, restrictions)
    a = np.zeros(ntri + 1)
    b = np.zeros(ntri)
    h = psi.handle()
    lib().qo_lanczos_tridiag(*op.args(), h, ntri, eps, gamma, *r.args(), _p(a), _p(b))
    lib().qo_wf_free(h)
    return a, b


def lanczos_krylov(op, psi, ntri, eps, restrictions=None):
    """Reference LanczosTriDiagonalizeKrylov (full reorthogonalisation, keeps the vectors):
    returns a (ntri+1), b (ntri) and the list of Krylov vectors (WF)."""
    r = Restr(psi.nf, restrictions)
    a = np.zeros(ntri + 1)
    b = np.zeros(ntri)
    handles = (C.c_void_p * ntri)()
    h = psi.handle()
    lib().qo_lanczos_krylov(*op.args(), h, ntri, eps, *r.args(), _p(a), _p(b), C.cast(handles, C.c_void_p))
    lib().qo_wf_free(h)
    K = [WF.from_handle(psi.nf, handles[i]) for i in range(ntri)]
    return a, b, K


def expectation(op, psi):
    """<psi|O|psi> with the growing-basis H*psi and the hashed dot (PsiOperatorPsi)."""
    d = operator_psi(op, psi).as_dict()
    return complex(sum(np.conj(v) * d.get(bytes(r), 0.0) for r, v in zip(psi.det, psi.val)))


def linear_combination(nf, vecs, coef):
    """sum_i coef_i vecs_i on the union basis (WaveFunctionAddComplexMultipliedUnionBasis)."""
    acc = {}
    order = []
    for v, c in zip(vecs, coef):
        for r, x in zip(v.det, v.val):
            k = bytes(r)
            if k not in acc:
                acc[k] = 0j
                order.append(r)
            acc[k] += c * x
    if not order:
        return WF(nf, np.zeros((0, nword(nf)), np.uint8), [])
    return WF(nf, np.array(order), [acc[bytes(r)] for r in order])


def resonant_spectra(H1, H2, T1, T2s, psi, o):
    """Reference ResonantSpectra (Core/ResonantSpectra.cpp:6-283): Krylov-projected resolvent of
    H1 on T1|psi>, then for every incident energy and every T2 a Lanczos of H2.  o holds
    NTri1, NTri2, Epsilon, Emin1, Emax1, NE1, Gamma1, Emin2, Emax2, NE2, Gamma2,
    Restrictions1/2.  Returns (G [NT2*(NE1+1), NE2+1], emin2, emax2, gamma2); spectrum index
    i*(NE1+1) + p."""
    eps = o["Epsilon"]
    n2 = float(np.real(np.vdot(psi.val, psi.val)))
    e1 = expectation(H1, psi).real / (n2 if n2 > np.finfo(float).eps else 1.0)
    e2 = expectation(H2, psi).real / (n2 if n2 > np.finfo(float).eps else 1.0)
    Tpsi = operator_psi(T1, psi, o.get("Restrictions1"))
    N1 = o["NTri1"]
    a, b, K = lanczos_krylov(H1, Tpsi, N1, eps, o.get("Restrictions1"))
    M = np.diag(a[1:N1 + 1]) + np.diag(b[1:N1], 1) + np.diag(b[1:N1], -1)
    ev, Z = np.linalg.eigh(M)
    emin1, emax1, ne1, g1 = o["Emin1"], o["Emax1"], o["NE1"], o["Gamma1"]
    res = []
    for p in range(ne1 + 1):
        w = emin1 + (emax1 - emin1) * p / ne1 + e1
        inv = 1.0 / (w - ev + 0.5j * g1)
        c = b[0] * (Z * (inv * Z[0, :])[None, :]).sum(axis=1)
        res.append(linear_combination(psi.nf, K, c))
    tri = []
    for T2 in T2s:
        for p in range(ne1 + 1):
            TG = operator_psi(T2, res[p], o.get("Restrictions2"))
            tri.append(lanczos_tridiag(H2, TG, o["NTri2"], eps, np.sqrt(np.finfo(float).eps) + o["Gamma2"],
                                       o.get("Restrictions2")))
    emin2, emax2, ne2, g2 = o["Emin2"], o["Emax2"], o["NE2"], o["Gamma2"]
    G = np.array([cf_spectrum(a2, b2, e2, emin2, (emax2 - emin2) / ne2, ne2, g2) for a2, b2 in tri])
    return G


def _auto_range(emin, emax, ne, gamma, lo_ev, hi_ev, e_lo, e_hi):
    """Energy-range defaults of the dense RIXS branch (Core/ResonantSpectra.cpp:472-535):
    unset Emin/Emax (None) from the extreme eigenvalues, then NE and Gamma."""
    if emin is None and emax is None:
        emin = 1.1 * lo_ev - 0.1 * hi_ev - e_hi
        emax = 1.1 * hi_ev - 0.1 * lo_ev - e_lo
    if emin is None:
        emin = 1.1 * lo_ev - 0.1 * emax - e_hi
    if emax is None:
        emax = 1.1 * hi_ev - 0.1 * emin - e_lo
    if gamma == 0 and ne == 0:
        ne = 1000
        gamma = 5 * (emax - emin) / ne
    if ne == 0:
        ne = int(5 * (emax - emin) / gamma)
    if gamma == 0:
        gamma = 5 * (emax - emin) / ne
    return emin, emax, ne, gamma


def _on_basis(wf, index, n):
    v = np.zeros(n, dtype=np.complex128)
    for r, x in zip(wf.det, wf.val):
        v[index[bytes(r)]] += x
    return v


def resonant_spectra_dense(H1, H2, T1s, T2s, psis, o, tensor=False, krylov_layout=False):
    """Reference dense RIXS, ResonantSpectraDense and ResonantSpectraDenseTensor
    (Core/ResonantSpectra.cpp:290-663, :665-1073), on the bases LuaCreateResonantSpectra builds
    for them (LuaInterface/ssp.cpp:3300-3371): the union of the initial states, the targets of
    every T1, their closure under H1; the targets of every T2 from there, their closure under H2.

    Intermediate eigenpairs (E_m, |m>), final (E_f, |f>), A[m, j] = <m|T1 psi_j> with
    j = iT1 + NT1 ipsi, B_k[f, m] = <f|T2_k|m>; per incident energy w_l the amplitudes
    D_k = B_k (A / (w_l - E_m + E1_psi + i Gamma1/2)).  Non-tensor spectrum l + (NE1+1)(k + NT2 j):
    sum_f |D_k[f, j]|^2 / (w - E_f + E2_psi + i Gamma2/2).  Tensor spectrum
    l + (NE1+1)(j2 + NT2(i1 + NT1(n2 + NT2(m1 + NT1(r + Npsi s))))):
    sum_f conj(D_n2[f, m1 + NT1 s]) D_j2[f, i1 + NT1 r] / (w - E_f + E2_psi0 + i Gamma2/2).
    krylov_layout gives the index order and energy shifts of the Krylov tensor branch
    (ResonantSpectraTensor, Core/ResonantSpectra.cpp:1204-1686: the left vector carries psi r,
    the right psi s, both shifts from psi 0), which it equals once its Krylov spaces are complete.
    o holds Emin1..Gamma2 (None / 0 for automatic), E0_1, E0_2 (None: <psi|H|psi>/<psi|psi>),
    Restrictions1/2.  Returns (G [nspec, NE2+1], settings)."""
    nf = psis[0].nf
    R1, R2 = o.get("Restrictions1"), o.get("Restrictions2")
    npsi, nt1, nt2 = len(psis), len(T1s), len(T2s)
    u = linear_combination(nf, psis, [1.0] * npsi)
    seed1 = linear_combination(nf, [operator_psi(T, u, R1) for T in T1s], [1.0] * nt1)
    b1 = closure(H1, seed1, R1)
    n1 = len(b1.val)
    idx1 = {bytes(r): i for i, r in enumerate(b1.det)}
    seed2 = linear_combination(nf, [operator_psi(T, b1, R2) for T in T2s], [1.0] * nt2)
    b2 = closure(H2, seed2, R2)
    n2 = len(b2.val)
    idx2 = {bytes(r): i for i, r in enumerate(b2.det)}

    def energies(H, key):
        if o.get(key) is not None:
            return np.full(npsi, float(o[key]))
        out = []
        for p in psis:
            nn = float(np.real(np.vdot(p.val, p.val)))
            out.append(expectation(H, p).real / (nn if nn > np.finfo(float).eps else 1.0))
        return np.array(out)

    e1, e2 = energies(H1, "E0_1"), energies(H2, "E0_2")
    if krylov_layout:
        e1[:], e2[:] = e1[0], e2[0]
    X = np.zeros((n1, npsi * nt1), dtype=np.complex128)
    for ip, p in enumerate(psis):
        for it, T in enumerate(T1s):
            X[:, it + nt1 * ip] = _on_basis(operator_psi(T, p, R1), idx1, n1)
    w1, V1 = np.linalg.eigh(dense_matrix(H1, b1)) if n1 else (np.zeros(0), np.zeros((0, 0)))
    w2, V2 = np.linalg.eigh(dense_matrix(H2, b2)) if n2 else (np.zeros(0), np.zeros((0, 0)))
    A = V1.conj().T @ X
    B = []
    for T in T2s:
        M = np.zeros((n2, n1), dtype=np.complex128)
        for c in range(n1):
            e = np.zeros(n1)
            e[c] = 1.0
            M[:, c] = _on_basis(operator_psi(T, WF(nf, b1.det, e), R2), idx2, n2)
        B.append(V2.conj().T @ M @ V1)
    emin1, emax1, ne1, g1 = _auto_range(o.get("Emin1"), o.get("Emax1"), o.get("NE1", 1000), o.get("Gamma1", 0.0),
                                        w1[0], w1[-1], e1.min(), e1.max())
    emin2, emax2, ne2, g2 = _auto_range(o.get("Emin2"), o.get("Emax2"), o.get("NE2", 1000), o.get("Gamma2", 0.0),
                                        w2[0] if n2 else 0.0, w2[-1] if n2 else 0.0, e2.min(), e2.max())
    np1 = ne1 + 1
    wl = np.array([emin2 + (m / ne2) * (emax2 - emin2) for m in range(ne2 + 1)])
    M1 = npsi * nt1
    nspec = (M1 * nt2) ** 2 * np1 if tensor else M1 * nt2 * np1
    G = np.zeros((nspec, ne2 + 1), dtype=np.complex128)
    psi_of = np.arange(M1) // nt1
    for l in range(np1):
        wres = emin1 + (emax1 - emin1) * l / ne1
        Cm = A / (wres - w1[:, None] + e1[psi_of][None, :] + 0.5j * g1)
        D = [Bk @ Cm for Bk in B]
        if not tensor:
            for k in range(nt2):
                for j in range(M1):
                    lor = 1.0 / (wl[:, None] - w2[None, :] + e2[psi_of[j]] + 0.5j * g2)
                    G[l + np1 * (k + nt2 * j)] = lor @ (np.abs(D[k][:, j]) ** 2)
            continue
        lor = 1.0 / (wl[:, None] - w2[None, :] + e2[0] + 0.5j * g2)
        for r in range(npsi):
            for s_ in range(npsi):
                for i1 in range(nt1):
                    for j2 in range(nt2):
                        for m1 in range(nt1):
                            for n2_ in range(nt2):
                                t = l + np1 * (j2 + nt2 * (i1 + nt1 * (n2_ + nt2 * (m1 + nt1 * (r + npsi * s_)))))
                                if krylov_layout:
                                    left, right = D[n2_][:, m1 + nt1 * r], D[j2][:, i1 + nt1 * s_]
                                else:
                                    left, right = D[n2_][:, m1 + nt1 * s_], D[j2][:, i1 + nt1 * r]
                                G[t] = lor @ (np.conj(left) * right)
    st = {"emin1": emin1, "emax1": emax1, "ne1": ne1, "gamma1": g1,
          "emin2": emin2, "emax2": emax2, "ne2": ne2, "gamma2": g2, "n1": n1, "n2": n2}
    return G, st


def cf_spectrum(a, b, e0, emin, de, ne, gamma):
    """Continued fraction on NE+1 points (reference TriDiagonalMatrixToSpectrum)."""
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    gre = np.zeros(ne + 1)
    gim = np.zeros(ne + 1)
    lib().qo_cf_spectrum(len(b), _p(a), _p(b), e0, emin, de, ne, gamma, _p(gre), _p(gim))
    return gre + 1j * gim


def poles_spectrum(a, b, e0, emin, de, ne, gamma):
    """Sum of Lorentzians on NE+1 points (reference ListOfPolesToSpectrum, Core/Spectral.cpp:1516,
    Gamma > 0 branch :1576-1588): G(w) = sum_k b_k (w - a_k - i gamma/2) / ((gamma/2)^2 + (w - a_k)^2)
    at w = emin + k de + e0, summed in pole order."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    out = np.zeros(ne + 1, dtype=np.complex128)
    hg = gamma / 2.0
    for k in range(ne + 1):
        w = k * de + emin + e0
        d = w - a
        den = hg * hg + d * d
        out[k] = complex(np.sum(b * d / den), np.sum(b * (-hg) / den))
    return out


def closure(op, seed, restrictions=None, max_rounds=10000):
    """All determinants reachable from the seed determinants under repeated H (within the
    restrictions); the seed comes first, then targets in discovery order."""
    basis = WF(seed.nf, seed.det, np.ones(len(seed.val)))
    known = {bytes(r) for r in basis.det}
    frontier = basis
    rounds = 0
    while len(frontier.val) and rounds < max_rounds:
        nxt = operator_psi(op, WF(seed.nf, frontier.det, np.ones(len(frontier.val))), restrictions)
        new = [i for i, r in enumerate(nxt.det) if bytes(r) not in known]
        for i in new:
            known.add(bytes(nxt.det[i]))
        frontier = WF(seed.nf, nxt.det[new], np.ones(len(new)))
        basis = WF(seed.nf, np.concatenate([basis.det, frontier.det]), np.ones(len(basis.val) + len(new)))
        rounds += 1
    return basis


def enumerate_restricted(nf, restrictions, nel=None):
    """Every determinant on nf orbitals that satisfies the occupation windows (the complete
    basis the reference builds for small systems, ExtendBasisCompletenessSmallSystems,
    Core/BlockLanczos.cpp:102).  Brute force over 2^nf; meant for nf <= 26."""
    masks = [int(m.replace(" ", "")[::-1], 2) for m, _, _ in restrictions]
    rows = []
    for x in range(1 << nf):
        if nel is not None and bin(x).count("1") != nel:
            continue
        if all(lo <= bin(x & m).count("1") <= hi for m, (_, lo, hi) in zip(masks, restrictions)):
            rows.append(x)
    dets = ["".join("1" if (x >> i) & 1 else "0" for i in range(nf)) for x in rows]
    return WF(nf, dets_to_bytes(dets, nf), np.ones(len(dets)))


def dense_matrix(op, basis):
    """<i|H|j> on a basis (columns from the fixed-basis apply on unit vectors)."""
    n = len(basis.val)
    M = np.zeros((n, n), dtype=np.complex128)
    for j in range(n):
        e = np.zeros(n, dtype=np.complex128)
        e[j] = 1.0
        M[:, j] = apply_conserve(op, WF(basis.nf, basis.det, e))
    return M


def exact_eigensystem(op, basis, k):
    """Lowest k eigenpairs of H on a closed basis, by dense diagonalisation."""
    M = dense_matrix(op, basis)
    w, v = np.linalg.eigh(0.5 * (M + M.conj().T))
    return w[:k], v[:, :k]


def num_threads():
    return lib().qo_num_threads()
