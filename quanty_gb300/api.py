"""Host-side mirror of the reference's operator / wavefunction interface for the H*psi path.

The names follow the reference's Lua and C entry points so code written against them reads the
same: ``NewOperator``, ``NewWavefunction``, ``OperatorPsi`` (``H*psi``,
``Core/OperatorWaveFunction.cpp:5598``), ``OperatorPsiConserveBasis`` (:5507/:5541),
``PsiOperatorPsi`` (:5680), ``LanczosTriDiagonalize`` (``Core/Lanczos.cpp:5274``),
``TriDiagonalMatrixToSpectrum`` (``Core/Spectral.cpp:1433``), ``CreateSpectra``
(``LuaInterface/ssp.cpp:1906``), ``CreateResonantSpectra`` (:3090) and ``Eigensystem``
(``LuaInterface/ssp.cpp:4039``).  Options take the reference's names and defaults
(``InitConvergenceSettings``, ``Core/StructDef.cpp:291-320``).  Operator applications, bases and
closures, the Lanczos recursions, dense operator matrices and spectrum evaluations run in
libqgpu.so on the GPU; this module converts layouts, owns handles and sequences calls, and does
on the host only what is small by construction: products of eigenvector matrices of the dense
branches (bases within DenseBorder), the library's host eigensolver on them, and arithmetic
between wavefunctions the caller holds on the host.  There is no CPU path for any GPU step.
"""
import ctypes as C
import math

import numpy as np

from . import qgpu

CREATION = 0x8000
DBL_EPSILON = np.finfo(float).eps
DEFAULTS = {
    "DenseBorder": 1513, "NKrylovStart": 100, "NKrylovMax": 500, "NKrylovStep": 10, "NTri": 200,
    "NTri1": 100, "NTri2": 100, "Zero": 100 * math.sqrt(DBL_EPSILON), "Epsilon": math.sqrt(DBL_EPSILON) / 100,
    "Emin": None, "Emax": None, "NE": 1000, "Gamma": 0.0, "NBitsKey": 16,
    "SingularValue": math.sqrt(DBL_EPSILON),
}

_engine = None


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("quanty_gb300 needs a CUDA GPU; there is no CPU path")
    return torch


class Engine:
    """One qg_context on one device, running on torch's current CUDA stream."""

    def __init__(self, device=0):
        torch = _torch()
        self.torch = torch
        self.L = qgpu.load()
        self.device = device
        torch.cuda.set_device(device)
        h = C.c_void_p()
        self.check(self.L.qg_init(device, C.byref(h)), ctx=None)
        self.ctx = h
        # one explicit stream shared by torch (buffers, events) and the library; it becomes
        # torch's current stream so tensors and CUDA events are ordered with the kernels
        self.stream = torch.cuda.Stream(device)
        torch.cuda.set_stream(self.stream)
        self.check(self.L.qg_set_stream(self.ctx, C.c_void_p(self.stream.cuda_stream)))

    def check(self, st, ctx="self"):
        if st != 0:
            msg = ""
            if ctx == "self" and getattr(self, "ctx", None):
                msg = self.L.qg_last_error(self.ctx).decode(errors="replace")
            raise qgpu.QGError(st, msg)

    def launches(self):
        return int(self.L.qg_launch_count(self.ctx))

    def empty(self, n, nvec=1):
        with self.torch.cuda.stream(self.stream):
            return self.torch.zeros((max(n, 1), nvec), dtype=self.torch.complex128, device="cuda:%d" % self.device)

    def on_stream(self):
        """Context manager: torch work ordered with this engine's kernels."""
        return self.torch.cuda.stream(self.stream)

    def to_host(self, t):
        """Copy a device tensor to numpy after this engine's queued work."""
        self.stream.synchronize()
        with self.on_stream():
            return t.cpu().numpy()

    def close(self):
        if getattr(self, "ctx", None):
            self.L.qg_finalize(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def engine():
    global _engine
    if _engine is None:
        _engine = Engine(0)
    return _engine


def _ptr(a):
    return C.c_void_p(a.ctypes.data) if isinstance(a, np.ndarray) else C.c_void_p(a.data_ptr())


def nword(nf):
    return (nf + 7) // 8


# ----------------------------------------------------------------------------- determinants

def dets_to_bytes(dets, nf):
    """'0110...' strings (orbital 0 first) -> uint8 (n, ceil(nf/8)), reference byte layout."""
    nw = nword(nf)
    n = len(dets)
    bits = np.zeros((n, nw * 8), dtype=np.uint8)
    if n:
        arr = np.frombuffer("".join(d.replace(" ", "")[:nf].ljust(nf, "0") for d in dets).encode(), dtype=np.uint8)
        bits[:, :nf] = (arr.reshape(n, nf) == ord("1"))
    return np.packbits(bits, axis=1, bitorder="big")


def bytes_to_dets(b, nf):
    bits = np.unpackbits(np.asarray(b, dtype=np.uint8), axis=1, bitorder="big")[:, :nf]
    return ["".join("1" if x else "0" for x in row) for row in bits]


# ----------------------------------------------------------------------------- operators

class Operator:
    """A second-quantized operator: sum of ladder strings with complex values.

    ``terms``: iterable of ``(ops, value)`` where ``ops`` is a sequence of ladder codes with
    ``ops[0]`` acting first and bit 15 set for a creation operator (the reference's
    OperatorFixedLengthType strings, ``Core/StructDef.cpp:223``)."""

    def __init__(self, nf, terms, name="Operator"):
        self.nf = int(nf)
        self.name = name
        self.terms = [(tuple(int(o) for o in ops), complex(v)) for ops, v in terms]
        self._handles = {}
        # occupation windows attached to the operator (the Lua field O.Restrictions,
        # OperatorType.Res, Core/StructDef.cpp:247): O * psi then keeps only targets inside them
        # (OperatorPsi dispatches to OperatorPsiRestricted, Core/OperatorWaveFunction.cpp:5600)
        self.Restrictions = None

    @classmethod
    def from_fixture(cls, d):
        return cls(d["nf"], [(t[0], complex(t[1], t[2])) for t in d["terms"]])

    def handle(self, eng=None):
        eng = eng or engine()
        key = id(eng)
        if key not in self._handles:
            n = len(self.terms)
            lens = np.array([len(t[0]) for t in self.terms], dtype=np.int32)
            flat = np.array([o for t in self.terms for o in t[0]] or [0], dtype=np.uint16)
            vre = np.array([t[1].real for t in self.terms] or [0.0])
            vim = np.array([t[1].imag for t in self.terms] or [0.0])
            h = C.c_void_p()
            eng.check(eng.L.qg_operator_create(eng.ctx, self.nf, n, _ptr(lens), _ptr(flat), _ptr(vre), _ptr(vim),
                                               C.byref(h)))
            self._handles[key] = (eng, h, (lens, flat, vre, vim))
        return self._handles[key][1]

    def info(self, eng=None):
        eng = eng or engine()
        a, b, c = C.c_int32(), C.c_int32(), C.c_int32()
        eng.check(eng.L.qg_operator_info(self.handle(eng), C.byref(a), C.byref(b), C.byref(c)))
        return {"nterms": a.value, "ngroups": b.value, "hermitian": bool(c.value)}

    def __add__(self, other):
        return Operator(self.nf, self.terms + other.terms)

    def dagger(self):
        """Conjugate transpose (the reference's ConjugateTranspose): each ladder string reversed
        with creation and annihilation exchanged, each value conjugated."""
        return Operator(self.nf, [(tuple(o ^ CREATION for o in reversed(ops)), complex(v).conjugate())
                                  for ops, v in self.terms], name=self.name + "^dag")

    def __mul__(self, other):
        if isinstance(other, Wavefunction):
            return OperatorPsi(self, other)
        return Operator(self.nf, [(o, v * other) for o, v in self.terms])

    __rmul__ = __mul__

    def __del__(self):
        for eng, h, _ in self._handles.values():
            try:
                if eng.ctx:
                    eng.L.qg_operator_destroy(h)
            except Exception:
                pass


class OperatorSum(Operator):
    """H = sum_k p_k O_k kept on the device for parameter scans.  A Quanty scan rebuilds H with
    OperatorAdd (Core/OperatorArithmetic.cpp:5674) for every parameter set; here the union of
    the components' terms is uploaded once and ``set_coefficients`` rewrites only the values,
    so every basis keeps its local blocks and connection lists and refreshes only the values.
    ``terms`` always holds the current sum as plain ladder strings."""

    def __init__(self, components, coefficients, name="OperatorSum"):
        self.components = list(components)
        if not self.components or any(c.nf != self.components[0].nf for c in self.components):
            raise ValueError("OperatorSum: components must exist and share nf")
        self.coefficients = np.asarray(coefficients, dtype=np.complex128).reshape(-1)
        if len(self.coefficients) != len(self.components):
            raise ValueError("OperatorSum: one coefficient per component")
        super().__init__(self.components[0].nf, self._sum_terms(), name)

    def _sum_terms(self):
        return [(o, complex(v) * complex(p)) for comp, p in zip(self.components, self.coefficients)
                for o, v in comp.terms]

    def _coef_arrays(self):
        return (np.ascontiguousarray(self.coefficients.real), np.ascontiguousarray(self.coefficients.imag))

    def handle(self, eng=None):
        eng = eng or engine()
        key = id(eng)
        if key not in self._handles:
            hs = np.array([c.handle(eng).value for c in self.components], dtype=np.uint64)
            re, im = self._coef_arrays()
            h = C.c_void_p()
            eng.check(eng.L.qg_operator_create_sum(eng.ctx, len(self.components), _ptr(hs), _ptr(re), _ptr(im),
                                                   C.byref(h)))
            self._handles[key] = (eng, h, (hs, re, im))
        return self._handles[key][1]

    def set_coefficients(self, coefficients):
        c = np.asarray(coefficients, dtype=np.complex128).reshape(-1)
        if len(c) != len(self.components):
            raise ValueError("OperatorSum: one coefficient per component")
        self.coefficients = c
        self.terms = [(tuple(int(o) for o in ops), complex(v)) for ops, v in self._sum_terms()]
        re, im = self._coef_arrays()
        for eng, h, _ in self._handles.values():
            eng.check(eng.L.qg_operator_set_coefficients(h, _ptr(re), _ptr(im)))
        return self


def NewOperator(nf, nb, terms):
    """Lua-style constructor: each term is ``[i1, i2, ..., value]`` with a non-negative index
    for a creation and a negative index (or -0.0) for an annihilation operator, leftmost factor
    first as in ``NewOperator(NF, 0, {{0, -0, 1, -1, U}})``."""
    if nb:
        raise ValueError("bosons are not supported")
    out = []
    for t in terms:
        *idx, v = t
        ops = []
        for i in idx:
            neg = (i < 0) or (isinstance(i, float) and math.copysign(1.0, i) < 0)
            ops.append(int(abs(i)) if neg else (int(i) | CREATION))
        ops.reverse()  # the rightmost factor acts first
        out.append((ops, v))
    return Operator(nf, out)


# ----------------------------------------------------------------------------- wavefunctions

class Wavefunction:
    """Determinants (reference byte layout) with complex FP64 amplitudes."""

    __array_ufunc__ = None  # numpy scalars defer to the arithmetic below

    def __init__(self, nf, det_bytes, values):
        self.nf = int(nf)
        self.det = np.ascontiguousarray(det_bytes, dtype=np.uint8).reshape(-1, nword(nf))
        self.val = np.ascontiguousarray(values, dtype=np.complex128).reshape(-1)
        assert len(self.det) == len(self.val)

    @classmethod
    def from_fixture(cls, d):
        return cls(d["nf"], dets_to_bytes(d["dets"], d["nf"]), np.array(d["re"]) + 1j * np.array(d["im"]))

    @property
    def N(self):
        return len(self.val)

    def dets(self):
        return bytes_to_dets(self.det, self.nf)

    def as_dict(self):
        return {bytes(r): v for r, v in zip(self.det, self.val)}

    def put(self, var=None, complex_values=None, name="Wave Function", nbitskey=16):
        """The reference's io.put text of this wavefunction (get_put.cpp:588-634)."""
        from .quanty_text import format_wavefunction
        wf = {"nf": self.nf, "nb": 0, "dets": self.dets(), "re": list(self.val.real), "im": list(self.val.imag),
              "name": name, "nbitskey": nbitskey}
        if complex_values is not None:
            wf["complex"] = bool(complex_values)
        return format_wavefunction(wf, var)

    @classmethod
    def from_put(cls, text):
        from .quanty_text import parse_wavefunction
        d = parse_wavefunction(text)
        return cls(d["nf"], dets_to_bytes(d["dets"], d["nf"]), np.array(d["re"]) + 1j * np.array(d["im"]))

    def norm(self):
        return float(np.linalg.norm(self.val))

    # The Lua methods that change a wavefunction in place (LuaInterface/Wavefunction.cpp:507-556).

    def Chop(self, border=10 * DBL_EPSILON):
        """psi.Chop(): drop determinants with |a|^2 <= border^2 (WaveFunctionTruncateBasis)."""
        keep = self.val.real ** 2 + self.val.imag ** 2 > border * border
        self.det, self.val = np.ascontiguousarray(self.det[keep]), np.ascontiguousarray(self.val[keep])

    def Conjugate(self):
        """psi.Conjugate(): complex-conjugate every amplitude."""
        self.val = np.conj(self.val)

    def Norm(self):
        """psi.Norm(): normalise to unit length (WaveFunctionNormalize; the Lua name)."""
        n = self.norm()
        if n > 0:
            self.val = self.val / n

    # ------------------------------------------------------------- arithmetic (host side)
    # The reference's Lua metamethods (LuaInterface/Wavefunction.cpp:1-440): sums on the union
    # basis, scaling by numbers, <a|b> for two wavefunctions, O|psi> and <psi|O = O^dag|psi>.

    def _keys(self):
        return np.ascontiguousarray(self.det).view(np.dtype((np.void, self.det.shape[1]))).ravel()

    def _union_add(self, other, c):
        """self + c * other on the union basis, self's determinants first, then the new ones of
        other in their order (WaveFunctionAddUnionBasis)."""
        if not isinstance(other, Wavefunction):
            return NotImplemented
        if other.nf != self.nf:
            raise ValueError("adding wavefunctions with %d and %d fermions" % (self.nf, other.nf))
        dets = np.concatenate([self.det, other.det])
        keys = np.ascontiguousarray(dets).view(np.dtype((np.void, dets.shape[1]))).ravel()
        _, first, inv = np.unique(keys, return_index=True, return_inverse=True)
        order = np.argsort(first, kind="stable")
        rank = np.empty_like(order)
        rank[order] = np.arange(len(order))
        vals = np.zeros(len(order), dtype=np.complex128)
        np.add.at(vals, rank[inv.ravel()], np.concatenate([self.val, c * other.val]))
        return Wavefunction(self.nf, dets[first[order]], vals)

    def dot(self, other):
        """<self|other>, the left side conjugated (WaveFunctionDotProduct); a real number when
        the imaginary part is below 10 (DBL_EPSILON |Re| + DBL_MIN), as the reference returns."""
        if other.nf != self.nf:
            raise ValueError("dot product of wavefunctions with %d and %d fermions" % (self.nf, other.nf))
        _, ia, ib = np.intersect1d(self._keys(), other._keys(), assume_unique=True, return_indices=True)
        d = complex(np.sum(np.conj(self.val[ia]) * other.val[ib]))
        if abs(d.imag) < 10 * (DBL_EPSILON * abs(d.real) + np.finfo(float).tiny):
            return d.real
        return d

    def __add__(self, other):
        if isinstance(other, (list, tuple)):
            return [self + o for o in other]
        return self._union_add(other, 1.0)

    def __sub__(self, other):
        if isinstance(other, (list, tuple)):
            return [self - o for o in other]
        return self._union_add(other, -1.0)

    def __neg__(self):
        return Wavefunction(self.nf, self.det, -self.val)

    def __mul__(self, other):
        if isinstance(other, (list, tuple)):
            return [self * o for o in other]
        if isinstance(other, Wavefunction):
            return self.dot(other)
        if isinstance(other, Operator):
            return OperatorPsi(other.dagger(), self)  # <psi|O as the ket O^dag|psi>
        if isinstance(other, (int, float, complex, np.number)):
            return Wavefunction(self.nf, self.det, self.val * other)
        return NotImplemented

    def __rmul__(self, other):
        if isinstance(other, (list, tuple)):
            return [o * self for o in other]
        if isinstance(other, (int, float, complex, np.number)):
            return Wavefunction(self.nf, self.det, other * self.val)
        return NotImplemented

    def __truediv__(self, other):
        if isinstance(other, (int, float, complex, np.number)):
            return Wavefunction(self.nf, self.det, self.val / other)
        return NotImplemented


def NewWavefunction(nf, nb, entries):
    if nb:
        raise ValueError("bosons are not supported")
    dets = [e[0] for e in entries]
    vals = [complex(e[1]) for e in entries]
    return Wavefunction(nf, dets_to_bytes(dets, nf), vals)


class Basis:
    """A device basis (sorted determinants + lookup hash)."""

    def __init__(self, eng, handle, nf):
        self.eng, self.h, self.nf = eng, handle, nf

    @classmethod
    def from_bytes(cls, nf, det_bytes, eng=None):
        eng = eng or engine()
        det_bytes = np.ascontiguousarray(det_bytes, dtype=np.uint8)
        n = len(det_bytes)
        perm = np.zeros(max(n, 1), dtype=np.int64)
        h = C.c_void_p()
        eng.check(eng.L.qg_basis_create(eng.ctx, nf, n, _ptr(det_bytes), C.byref(h), _ptr(perm)))
        b = cls(eng, h, nf)
        return b, perm[:n]

    @property
    def n(self):
        return int(self.eng.L.qg_basis_size(self.h))

    def dets_bytes(self):
        out = np.zeros((max(self.n, 1), nword(self.nf)), dtype=np.uint8)
        self.eng.check(self.eng.L.qg_basis_get_dets(self.h, _ptr(out)))
        return out[:self.n]

    def find(self, det_bytes):
        det_bytes = np.ascontiguousarray(det_bytes, dtype=np.uint8)
        out = np.zeros(max(len(det_bytes), 1), dtype=np.int64)
        self.eng.check(self.eng.L.qg_basis_find(self.h, len(det_bytes), _ptr(det_bytes), _ptr(out)))
        return out[:len(det_bytes)]

    def __del__(self):
        try:
            if self.eng.ctx and self.h:
                self.eng.L.qg_basis_destroy(self.h)
        except Exception:
            pass


class _Res:
    """qg_restrictions built from [(mask string, min, max), ...]."""

    def __init__(self, nf, restrictions):
        self.r = qgpu.Restrictions()
        rs = list(restrictions or [])
        self.masks = dets_to_bytes([m for m, _, _ in rs], nf) if rs else np.zeros((1, nword(nf)), np.uint8)
        self.mn = np.array([lo for _, lo, _ in rs] or [0], dtype=np.int32)
        self.mx = np.array([hi for _, _, hi in rs] or [0], dtype=np.int32)
        self.r.n = len(rs)
        self.r.masks = self.masks.ctypes.data
        self.r.min = self.mn.ctypes.data
        self.r.max = self.mx.ctypes.data

    def ptr(self):
        return C.byref(self.r) if self.r.n else None


def parse_restrictions(R):
    """Accept the Lua form {NF, NB, {"mask", min, max}, ...} or a list of (mask, min, max)."""
    if R is None:
        return None
    R = list(R)
    if R and isinstance(R[0], (int, np.integer)):
        R = R[2:]
    return [(str(m).replace(" ", ""), int(lo), int(hi)) for m, lo, hi in R]


def _upload(eng, basis, perm, values, nvec=1):
    """Host amplitudes in input order -> device block in basis order (n x nvec)."""
    torch = eng.torch
    n = basis.n
    v = np.zeros((max(n, 1), nvec), dtype=np.complex128)
    vals = np.asarray(values).reshape(len(perm), nvec)
    np.add.at(v, perm, vals)
    with eng.on_stream():
        return torch.from_numpy(v).to("cuda:%d" % eng.device)


# ----------------------------------------------------------------------------- H * psi

def OperatorPsiBasis(O, basis, restrictions=None, eng=None):
    eng = eng or engine()
    res = _Res(O.nf, parse_restrictions(restrictions))
    h = C.c_void_p()
    eng.check(eng.L.qg_operator_psi_basis(eng.ctx, O.handle(eng), basis.h, res.ptr(), C.byref(h)))
    return Basis(eng, h, O.nf)


def OperatorPsi(O, psi, restrictions=None, eng=None):
    """O|psi> with basis growth (reference OperatorPsi / OperatorPsiRestricted).  The output
    determinants are the targets of all applicable (determinant, string) pairs, in sorted
    order.  Strings whose value is zero (the constant of the common "O = 0; O = O + ..." or a
    cancelled sum) reach their targets too, with amplitude 0, as in the reference, which
    inserts every applicable target whatever the value; the device growth leaves them out and
    they are added here on the host."""
    eng = eng or engine()
    if O.nf != psi.nf:
        raise ValueError("operator and wavefunction have different numbers of fermions")
    if restrictions is None:
        restrictions = getattr(O, "Restrictions", None)
    src, perm = Basis.from_bytes(psi.nf, psi.det, eng)
    x = _upload(eng, src, perm, psi.val)
    dst = OperatorPsiBasis(O, src, restrictions, eng)
    y = eng.empty(dst.n)
    eng.check(eng.L.qg_apply(eng.ctx, O.handle(eng), dst.h, src.h, _ptr(x), _ptr(y), 1))
    dets, vals = dst.dets_bytes(), eng.to_host(y[:dst.n, 0])
    extra = _zero_term_targets(O, psi.det, parse_restrictions(restrictions))
    if len(extra):
        both = np.concatenate([np.asarray(dets, dtype=np.uint8).reshape(-1, nword(psi.nf)), extra])
        dets, first, inv = np.unique(both, axis=0, return_index=True, return_inverse=True)
        v = np.zeros(len(dets), dtype=np.complex128)
        v[inv.ravel()[:len(vals)]] = vals
        vals = v
    return Wavefunction(psi.nf, dets, vals)


def _targets_basis(O, src, restrictions=None, eng=None):
    """The targets of O from a device basis as the reference's OperatorPsi reaches them: the
    device growth, plus the targets of O's zero-valued strings (host enumeration)."""
    tb = OperatorPsiBasis(O, src, restrictions, eng)
    if src.n and any(v == 0 for _, v in O.terms):
        extra = _zero_term_targets(O, src.dets_bytes(), parse_restrictions(restrictions))
        if len(extra):
            tb = basis_union(tb, Basis.from_bytes(O.nf, extra, eng)[0], eng)
    return tb


def _zero_term_targets(O, dets, restrictions=None):
    """The determinants that O's zero-valued strings reach from `dets` (host ladder
    application in the reference's byte layout, Core/OperatorWaveFunction.cpp:7-115: orbital i
    in byte i>>3 under mask 128>>(i&7), the first code acts first, an annihilator needs the
    orbital occupied and a creator empty), kept when they satisfy the restrictions."""
    zero = [ops for ops, v in O.terms if v == 0]
    dets = np.asarray(dets, dtype=np.uint8).reshape(-1, nword(O.nf))
    if not zero or not len(dets):
        return np.zeros((0, nword(O.nf)), dtype=np.uint8)
    out = []
    for ops in zero:
        d = dets.copy()
        ok = np.ones(len(d), dtype=bool)
        for code in ops:
            i = code & 0x7FFF
            byte, mask = i >> 3, np.uint8(128 >> (i & 7))
            occ = (d[:, byte] & mask) != 0
            ok &= ~occ if code & CREATION else occ
            d[:, byte] ^= mask
        out.append(d[ok])
    t = np.concatenate(out)
    for m, lo, hi in restrictions or []:
        mb = dets_to_bytes([m], O.nf)[0]
        cnt = np.unpackbits(t & mb[None, :], axis=1).sum(axis=1)
        t = t[(cnt >= lo) & (cnt <= hi)]
    return np.unique(t, axis=0) if len(t) else t


def OperatorPsiConserveBasis(O, psi, eng=None):
    """O|psi> kept on the basis of psi (reference OperatorPsiConserveBasis[PreAllocated])."""
    eng = eng or engine()
    b, perm = Basis.from_bytes(psi.nf, psi.det, eng)
    x = _upload(eng, b, perm, psi.val)
    y = eng.empty(b.n)
    eng.check(eng.L.qg_apply(eng.ctx, O.handle(eng), b.h, b.h, _ptr(x), _ptr(y), 1))
    yh = eng.to_host(y[:b.n, 0])
    return Wavefunction(psi.nf, psi.det, yh[perm])


def PsiOperatorPsi(O, psi, eng=None):
    eng = eng or engine()
    b, perm = Basis.from_bytes(psi.nf, psi.det, eng)
    x = _upload(eng, b, perm, psi.val)
    out = np.zeros(2)
    eng.check(eng.L.qg_expectation(eng.ctx, O.handle(eng), b.h, _ptr(x), 1, _ptr(out)))
    return complex(out[0], out[1])


def count_nnz(O, basis, eng=None, offdiag=False):
    """Non-zero (row, term) connections of O on a basis (sources inside the basis); with
    offdiag=True only those that change the determinant."""
    eng = eng or engine()
    n = C.c_int64()
    f = eng.L.qg_count_nnz_offdiag if offdiag else eng.L.qg_count_nnz
    eng.check(f(eng.ctx, O.handle(eng), basis.h, C.byref(n)))
    return n.value


def closure(O, seed_bytes, nf, restrictions=None, max_rounds=-1, eng=None):
    eng = eng or engine()
    seed, _ = Basis.from_bytes(nf, seed_bytes, eng)
    return closure_of(O, seed, restrictions, max_rounds, eng)


def basis_union(a, b, eng=None):
    eng = eng or engine()
    h = C.c_void_p()
    eng.check(eng.L.qg_basis_union(eng.ctx, a.h, b.h, C.byref(h)))
    return Basis(eng, h, a.nf)


def closure_of(O, seed, restrictions=None, max_rounds=-1, eng=None):
    """Closure of a device basis under O (within the restrictions)."""
    eng = eng or engine()
    nf = seed.nf
    res = _Res(nf, parse_restrictions(restrictions))
    h = C.c_void_p()
    rounds = C.c_int32()
    eng.check(eng.L.qg_basis_closure(eng.ctx, O.handle(eng), seed.h, res.ptr(), max_rounds, C.byref(h),
                                     C.byref(rounds)))
    return Basis(eng, h, nf)


# ----------------------------------------------------------------------------- Lanczos + spectra

def lanczos_block(H, basis, x, ntri, eps, gamma, eng=None, krylov=None):
    """Batched Lanczos on a device basis: x is an (n, nvec) complex CUDA tensor."""
    eng = eng or engine()
    nvec = x.shape[1]
    a = np.zeros(nvec * (ntri + 1))
    b = np.zeros(nvec * ntri)
    kp = _ptr(krylov) if krylov is not None else None
    eng.check(eng.L.qg_lanczos_tridiag(eng.ctx, H.handle(eng), basis.h, _ptr(x), nvec, ntri, eps, gamma, _ptr(a),
                                       _ptr(b), kp))
    return a.reshape(nvec, ntri + 1), b.reshape(nvec, ntri)


def LanczosTriDiagonalize(H, psi, NTri=200, epsilon=DEFAULTS["Epsilon"], Gamma=None, restrictions=None, eng=None):
    """Reference LanczosTriDiagonalize[Restricted] (Core/Lanczos.cpp:5228/:5274): returns (a, b)
    with a[0] = 0 and b[0] = |psi|.  The Krylov space lives on the closure of psi's
    determinants under H (within the restrictions)."""
    eng = eng or engine()
    gamma = epsilon if Gamma is None else Gamma
    basis = closure(H, psi.det, psi.nf, restrictions, -1, eng)
    src, perm = Basis.from_bytes(psi.nf, psi.det, eng)
    xs = _upload(eng, src, perm, psi.val)
    x = eng.empty(basis.n)
    eng.check(eng.L.qg_basis_map(eng.ctx, src.h, _ptr(xs), basis.h, _ptr(x), 1))
    a, b = lanczos_block(H, basis, x, NTri, epsilon, gamma, eng)
    return a[0], b[0]


def TriDiagonalMatrixToSpectrum(E0, a, b, Emin, Emax, NE, Gamma, eng=None):
    """G(w) for w = Emin + k dE + E0, k = 0..NE (Core/Spectral.cpp:1433); a, b may hold several
    spectra as rows."""
    eng = eng or engine()
    a = np.ascontiguousarray(np.atleast_2d(a), dtype=np.float64)
    b = np.ascontiguousarray(np.atleast_2d(b), dtype=np.float64)
    ns, ntri = b.shape
    e0 = np.ascontiguousarray(np.broadcast_to(np.asarray(E0, dtype=np.float64), (ns,)))
    g = np.zeros(2 * ns * (NE + 1))
    de = (Emax - Emin) / NE
    eng.check(eng.L.qg_cf_spectra(eng.ctx, ns, ntri, _ptr(a), _ptr(b), _ptr(e0), Emin, de, NE, Gamma, _ptr(g)))
    G = g[0::2] + 1j * g[1::2]
    return G.reshape(ns, NE + 1)


def _opts(options):
    o = dict(DEFAULTS)
    if options:
        items = options.items() if isinstance(options, dict) else options
        for k, v in items:
            k = {"epsilon": "Epsilon", "restrictions": "Restrictions", "zero": "Zero",
                 "restrictions1": "Restrictions1", "restrictions2": "Restrictions2"}.get(k, k)
            o[k] = v
    return o


class Spectra:
    """CreateSpectra's result: G_s(w) on NE+1 points per spectrum (SpectraType, Core/StructDef.cpp:986),
    with the pole range the energy window defaults were taken from."""

    def __init__(self, G, Emin, Emax, NE, Gamma, EminPole=float("nan"), EmaxPole=float("nan")):
        self.G, self.Emin, self.Emax, self.NE, self.Gamma = np.atleast_2d(G), Emin, Emax, NE, Gamma
        self.EminPole, self.EmaxPole = EminPole, EmaxPole

    @property
    def energies(self):
        return self.Emin + np.arange(self.NE + 1) * (self.Emax - self.Emin) / self.NE

    def Print(self, file=None):
        """The reference's spectra file (Spectra.Print, StreamPrintSpectra IO/StreamPrint.cpp:4):
        three header lines of window, pole range and (dE, Gamma) per spectrum, a column header,
        then one line per frequency.  Returns the text; writes it to `file` when given."""
        ns = self.G.shape[0]
        de = (self.Emax - self.Emin) / self.NE
        out = ["#Spectra: %i\n" % ns]
        out.append("Emin______Emax     " + "".join(" %22.15E %22.15E" % (self.Emin, self.Emax) for _ in range(ns)) + "\n")
        out.append("EminPole__EmaxPole " + "".join(" %22.15E %22.15E" % (self.EminPole, self.EmaxPole)
                                                   for _ in range(ns)) + "\n")
        out.append("dE________Gamma    " + "".join(" %22.15E %22.15E" % (de, self.Gamma) for _ in range(ns)) + "\n")
        hdr = "Energy             "
        for i in range(ns):
            w = len(str(i))
            hdr += "  Re[%s]%s Im[%s]%s" % (i, " " * (18 - w), i, " " * (17 - w))
        out.append(hdr + "\n")
        for j in range(self.NE + 1):
            row = "%19.12E" % (de * j + self.Emin)
            row += "".join(" %22.15E %22.15E" % (self.G[i, j].real, self.G[i, j].imag) for i in range(ns))
            out.append(row + "\n")
        text = "".join(out)
        if file is not None:
            with open(file, "w") as f:
                f.write(text)
        return text

    @classmethod
    def from_text(cls, text):
        """Read a spectra file written by Print (or by the reference)."""
        lines = text.splitlines()
        ns = int(lines[0].split(":")[1])
        emin, emax = (float(t) for t in lines[1].split()[1:3])
        pmin, pmax = (float(t) for t in lines[2].split()[1:3])
        de, gamma = (float(t) for t in lines[3].split()[1:3])
        rows = [[float(t) for t in ln.split()] for ln in lines[5:] if ln.strip()]
        G = np.array([[r[1 + 2 * i] + 1j * r[2 + 2 * i] for r in rows] for i in range(ns)])
        return cls(G, emin, emax, len(rows) - 1, gamma, pmin, pmax)


# ----------------------------------------------------------------------------- dense path

def OperatorToDeterminantMatrix(O, basis, eng=None):
    """O as a dense matrix on a device basis (Core/MatrixOperator.cpp:1149): M[r, c] = <r|O|c>."""
    eng = eng or engine()
    n = basis.n
    m = np.zeros((max(n, 1), max(n, 1)), dtype=np.complex128)
    eng.check(eng.L.qg_operator_dense(eng.ctx, O.handle(eng), basis.h, _ptr(m)))
    return m[:n, :n]


def hermitian_eigh(M, nvec=None, eng=None):
    """All eigenvalues (ascending) and the lowest nvec eigenvectors (columns) of a Hermitian
    matrix, by the library's device eigensolver (cyclic Jacobi up to order 40; above, Householder
    reduction to a tridiagonal matrix, multisection and inverse iteration)."""
    eng = eng or engine()
    k = M.shape[0]
    nv = k if nvec is None else int(nvec)
    a = np.ascontiguousarray(M, dtype=np.complex128)
    w = np.zeros(k)
    v = np.zeros((k, max(nv, 1)), dtype=np.complex128)
    eng.check(eng.L.qg_hermitian_eigh(eng.ctx, k, _ptr(a), _ptr(w), _ptr(v), nv))
    return w, v[:, :nv]


def ListOfPolesToSpectrum(E0, poles, weights, Emin, Emax, NE, Gamma, eng=None):
    """G(w) = sum_k b_k / (w - a_k + i Gamma/2) at w = Emin + k dE + E0 (Core/Spectral.cpp:1516);
    poles and weights may hold several spectra as rows."""
    eng = eng or engine()
    b = np.ascontiguousarray(np.atleast_2d(weights), dtype=np.float64)
    ns, npole = b.shape
    a = np.ascontiguousarray(np.broadcast_to(np.atleast_2d(np.asarray(poles, dtype=np.float64)), (ns, npole)))
    e0 = np.ascontiguousarray(np.broadcast_to(np.asarray(E0, dtype=np.float64), (ns,)))
    g = np.zeros(2 * ns * (NE + 1))
    eng.check(eng.L.qg_poles_spectra(eng.ctx, ns, npole, _ptr(a), _ptr(b), _ptr(e0), float(Emin),
                                     (Emax - Emin) / NE, int(NE), float(Gamma), _ptr(g)))
    return (g[0::2] + 1j * g[1::2]).reshape(ns, NE + 1)


def _spectra_dense(H, Tpsi, e0, o, basis, eng, states=False):
    """CreateSpectra's dense branch (LuaInterface/ssp.cpp:2347-2460): the eigensystem of H on
    the union basis, poles at its eigenvalues with weights |<E_k|T psi>|^2.  With states=True
    (the KrylovBasis option, :2538-2580) the eigenstates come back as a third result."""
    n = basis.n
    w, V = hermitian_eigh(OperatorToDeterminantMatrix(H, basis, eng), n, eng)
    X = np.zeros((n, len(Tpsi)), dtype=np.complex128)
    for s, t in enumerate(Tpsi):
        if t.N:
            rows = basis.find(t.det)
            np.add.at(X[:, s], rows, t.val)
    Wt = np.abs(V.conj().T @ X) ** 2  # (pole, spectrum)
    lo = min(w[0] - e for e in e0)
    hi = max(w[-1] - e for e in e0)
    NE = int(o["NE"])
    emin, emax, gamma = _default_window(lo, hi, o["Emin"], o["Emax"], float(o["Gamma"]), NE)
    G = ListOfPolesToSpectrum(np.asarray(e0), np.tile(w, (len(Tpsi), 1)), Wt.T, emin, emax, NE, gamma, eng)
    poles = [(w - e0[s], Wt[:, s].copy()) for s in range(len(Tpsi))]
    if states:
        db = basis.dets_bytes()
        return Spectra(G, emin, emax, NE, gamma, lo, hi), poles, [Wavefunction(H.nf, db, V[:, k]) for k in range(n)]
    return Spectra(G, emin, emax, NE, gamma, lo, hi), poles


def block_lanczos(H, basis, X, ntri, eps, singular_value, eng=None, krylov=None):
    """Block Lanczos on a device basis (LanczosBlockTriDiagonalize, Core/BlockLanczos.cpp:2131):
    X is an (n, m) complex CUDA tensor of start vectors.  Returns A ((ntri+1), m, m), B (ntri, m,
    m) complex and the block sizes (ntri + 1); krylov (a complex CUDA tensor of ntri * m * n
    entries) receives the orthonormal blocks as Krylov vectors, vector-major."""
    eng = eng or engine()
    m = X.shape[1]
    a = np.zeros((ntri + 1, m, m), dtype=np.complex128)
    b = np.zeros((ntri, m, m), dtype=np.complex128)
    sizes = np.zeros(ntri + 1, dtype=np.int32)
    Xc = X.contiguous()
    kp = _ptr(krylov) if krylov is not None else None
    eng.check(eng.L.qg_block_lanczos(eng.ctx, H.handle(eng), basis.h, _ptr(Xc), m, ntri, float(eps),
                                     float(singular_value), _ptr(a), _ptr(b), _ptr(sizes), kp))
    return a, b, sizes


def block_chop(A, eps):
    """Components below eps set to zero, real and imaginary parts separately
    (BlockTridiagonalMatrixChop, Core/BasicMathBlock/BasicMath_BlockTridiagonalMatrix.cpp:137)."""
    re = np.where(np.abs(A.real) < eps, 0.0, A.real)
    im = np.where(np.abs(A.imag) < eps, 0.0, A.imag)
    return re + 1j * im


def block_tridiagonal_dense(A, B):
    """The Hermitian (N m) x (N m) matrix of the blocks A_1..A_N on the diagonal and B_1..B_{N-1}
    beside it, zero rows and columns for deflated directions included, as the reference's
    BlockTriDiagonalMatrixEigenValues sees it (Core/BasicMathBlock/BasicMath_BlockTypeConversion.cpp:1731)."""
    N, m = A.shape[0] - 1, A.shape[1]
    T = np.zeros((N * m, N * m), dtype=np.complex128)
    for k in range(1, N + 1):
        T[(k - 1) * m:k * m, (k - 1) * m:k * m] = A[k]
        if k < N:
            T[(k - 1) * m:k * m, k * m:(k + 1) * m] = B[k]
            T[k * m:(k + 1) * m, (k - 1) * m:k * m] = B[k].conj().T
    return (T + T.conj().T) / 2


def BlockTriDiagonalMatrixToSpectra(E0, A, B, Emin, Emax, NE, Gamma, eng=None):
    """G_ij(w) = <v0_i| (w - H + i Gamma/2)^-1 |v0_j> at w = Emin + k dE + E0 from a block
    tridiagonal matrix by the block continued fraction (BlockTriDiagonalMatrixToSpectraWithBroadening,
    Core/BasicMathBlock/BasicMath_BlockTypeConversion.cpp:1636): (m*m, NE+1), spectrum i*m + j."""
    eng = eng or engine()
    m, ntri = A.shape[1], B.shape[0]
    a = np.ascontiguousarray(A, dtype=np.complex128)
    b = np.ascontiguousarray(B, dtype=np.complex128)
    g = np.zeros((m * m, NE + 1), dtype=np.complex128)
    eng.check(eng.L.qg_block_cf_spectra(eng.ctx, m, ntri, _ptr(a), _ptr(b), float(E0), float(Emin),
                                        (Emax - Emin) / NE, int(NE), float(Gamma), _ptr(g)))
    return g


def _spectra_tensor(H, Tpsi, E0, o, R, method, eng):
    """CreateSpectra with Tensor = true (ssp.cpp:2480-2530, :2753-2800): the m x m matrix
    G_ij(w) = <T_i psi| (w + E0 - H + i Gamma/2)^-1 |T_j psi>, spectrum i*m + j, one energy
    shift E0 (the first state's).  Dense branch: poles of H on the union basis with weights
    conj(c_ki) c_kj, c_ki = <E_k|T_i psi> (BasicMath_CompactMatrixVector.cpp:4064,
    BasicMath_BlockTypeConversion.cpp:588).  Lanczos branch: the reference's block Lanczos on the
    device from the m vectors T_i psi on their common basis (qg_block_lanczos, NTri blocks), the
    pole range from the eigenvalues of the whole block tridiagonal matrix, and the spectra by the
    block continued fraction (qg_block_cf_spectra)."""
    m = len(Tpsi)
    NE, gamma, ntri, eps = int(o["NE"]), float(o["Gamma"]), int(o["NTri"]), float(o["Epsilon"])
    seed = np.concatenate([t.det for t in Tpsi if t.N] or [np.zeros((0, nword(H.nf)), np.uint8)])
    if not len(seed):
        raise ValueError("CreateSpectra: every T psi is empty")
    ub = closure(H, seed, H.nf, R, -1, eng)
    n = ub.n
    X = np.zeros((n, m), dtype=np.complex128)
    for s, t in enumerate(Tpsi):
        if t.N:
            np.add.at(X[:, s], ub.find(t.det), t.val)
    if method == "dense" or (method != "lanczos" and n <= int(o["DenseBorder"])):
        w, V = hermitian_eigh(OperatorToDeterminantMatrix(H, ub, eng), n, eng)
        Cm = V.conj().T @ X  # (pole, vector)
        lo, hi = w[0] - E0, w[-1] - E0
        emin, emax, gamma = _default_window(lo, hi, o["Emin"], o["Emax"], gamma, NE)
        Wt = (Cm.conj()[:, :, None] * Cm[:, None, :]).reshape(n, m * m).T  # (i*m + j, pole)
        poles = w - E0
        G = (ListOfPolesToSpectrum(0.0, poles, Wt.real.copy(), emin, emax, NE, gamma, eng)
             + 1j * ListOfPolesToSpectrum(0.0, poles, Wt.imag.copy(), emin, emax, NE, gamma, eng))
        return Spectra(G, emin, emax, NE, gamma, lo, hi), {"poles": poles, "weights": Wt}
    with eng.on_stream():
        x = eng.torch.from_numpy(X).to("cuda:%d" % eng.device).contiguous()
    sv = float(o.get("SingularValue", DEFAULTS["SingularValue"]))
    A, B, sizes = block_lanczos(H, ub, x, ntri, eps, sv, eng)
    val, _ = hermitian_eigh(block_tridiagonal_dense(A, B), 0, eng)
    lo, hi = val[0] - E0, val[-1] - E0
    emin, emax, gamma = _default_window(lo, hi, o["Emin"], o["Emax"], gamma, NE)
    G = BlockTriDiagonalMatrixToSpectra(E0, A, B, emin, emax, NE, gamma, eng)
    return Spectra(G, emin, emax, NE, gamma, lo, hi), {"a": A, "b": B, "block_sizes": sizes}


def CreateSpectraResident(H, T, basis, X, E0, options=None, eng=None, batched=True, max_vectors=None):
    """The batched form of CreateSpectra for initial states held on the device: X is an
    (n, npsi) complex CUDA tensor on `basis`, E0 their energies.  The final-state basis is the
    closure under H of the targets of every T (within the Restrictions option); all (T, psi)
    pairs, ordered iT*npsi + ipsi, then run as one multi-vector Lanczos (batched=True, or
    groups of `max_vectors`) or one Lanczos per pair (batched=False, the plain path).
    Returns (Spectra, A, B) with the raw Lanczos coefficients A (a_0..a_NTri) and B."""
    eng = eng or engine()
    o = _opts(options)
    Ts = T if isinstance(T, (list, tuple)) else [T]
    R = parse_restrictions(o.get("Restrictions"))
    ntri, eps, gamma = int(o["NTri"]), float(o["Epsilon"]), float(o["Gamma"])
    npsi = X.shape[1]
    bt = None
    for t in Ts:
        tb = OperatorPsiBasis(t, basis, R, eng)
        bt = tb if bt is None else basis_union(bt, tb, eng)
    bf = closure_of(H, bt, R, -1, eng)
    nvec = len(Ts) * npsi
    Y = eng.empty(bf.n, nvec)
    Xc = X.contiguous()
    for j, t in enumerate(Ts):
        yj = eng.empty(bf.n, npsi)
        eng.check(eng.L.qg_apply(eng.ctx, t.handle(eng), bf.h, basis.h, _ptr(Xc), _ptr(yj), npsi))
        with eng.on_stream():
            Y[:, j * npsi:(j + 1) * npsi] = yj
    step = nvec if batched else 1
    if batched and max_vectors:
        step = int(max_vectors)
    A = np.zeros((nvec, ntri + 1))
    B = np.zeros((nvec, ntri))
    for c0 in range(0, nvec, step):
        c1 = min(nvec, c0 + step)
        with eng.on_stream():
            x = Y[:, c0:c1].contiguous()
        a, b = lanczos_block(H, bf, x, ntri, eps, max(gamma, eps), eng)
        A[c0:c1] = a
        B[c0:c1] = b
    e0 = np.array([E0[i % npsi] for i in range(nvec)], dtype=np.float64)
    NE = int(o["NE"])
    G = TriDiagonalMatrixToSpectrum(e0, A, B, o["Emin"], o["Emax"], NE, gamma, eng)
    return Spectra(G, o["Emin"], o["Emax"], NE, gamma), A, B


def _spectra_method(o):
    """CreateSpectra's Method and ForceDenseMethod options (LuaInterface/ssp.cpp:2029-2058):
    "dense" (Method "Dense" or ForceDenseMethod), "lanczos" (Method "Lanczos", any size) or ""
    (Method "Auto": dense within DenseBorder).  Contradicting or unknown choices raise, as the
    reference's luaL_error; Method "Mesh" (the hybridisation on an energy mesh, a self-energy
    feature) is not part of this library."""
    m = str(o.get("Method") or "Auto")
    force = bool(o.get("ForceDenseMethod"))
    key = m.lower()
    if key not in ("auto", "dense", "lanczos", "mesh"):
        raise ValueError('CreateSpectra: unknown Method "%s", possible are "Auto", "Dense", "Lanczos" and "Mesh"' % m)
    if key in ("lanczos", "mesh") and force:
        raise ValueError('CreateSpectra: Method "%s" and ForceDenseMethod true contradict each other' % m)
    if key == "mesh":
        raise NotImplementedError('CreateSpectra: Method "Mesh" (hybridisation on an energy mesh) is not supported')
    # the self-energy options (ssp.cpp:1973-1977, used with a self-energy argument, :1992-2070)
    if (o.get("GridPoints") is not None or o.get("NTriFull") is not None or o.get("NonCrossing")
            or int(o.get("NBathExcitations", 1)) != 1):
        raise NotImplementedError("CreateSpectra: self-energy options (GridPoints, NTriFull, NBathExcitations, "
                                  "NonCrossing) are not supported")
    if force or key == "dense":
        return "dense"
    return "lanczos" if key == "lanczos" else ""


def CreateSpectra(H, T, psi, options=None, eng=None, batched=True):
    """Reference CreateSpectra (LuaInterface/ssp.cpp:1906): spectra of all (T, psi) pairs,
    ordered iT*Npsi + ipsi.  Lanczos branch (:2586-2720): returns (Spectra, [(a, b) shifted by
    -E0]); batched=True runs all pairs as one multi-vector Lanczos with every step on the
    device.  Dense branch (:2347-2460; Method "Dense", or a union basis within DenseBorder
    unless Method is "Lanczos"): returns (Spectra, [(poles - E0, weights)]).  KrylovBasis adds a
    third result: the Lanczos branch's Krylov vectors of every pair (the reference's Krylov-basis
    Lanczos, LanczosTriDiagonalizeKrylov, Core/Lanczos.cpp:5405; empty vectors left out; one list
    for one pair, else a list per pair, :2729-2745), or the dense branch's eigenstates of H."""
    o = _opts(options)
    method = _spectra_method(o)
    krylov = bool(o.get("KrylovBasis"))
    if krylov and o.get("Tensor"):
        raise NotImplementedError("CreateSpectra: KrylovBasis with Tensor (a block Krylov basis) is not supported")
    eng = eng or engine()
    Ts = T if isinstance(T, (list, tuple)) else [T]
    psis = psi if isinstance(psi, (list, tuple)) else [psi]
    ntri, eps = int(o["NTri"]), float(o["Epsilon"])
    R = parse_restrictions(o.get("Restrictions"))
    gamma = float(o["Gamma"])
    if batched and not o.get("Tensor") and method != "dense" and not krylov:
        got = _batched_lanczos_device(H, Ts, psis, o, R, eng)
        if got is not None:
            A, B, E0 = got
            e0 = np.array([E0[i % len(psis)] for i in range(len(Ts) * len(psis))])
            return _lanczos_spectra(A, B, e0, o, gamma, ntri, eng)
    E0 = [PsiOperatorPsi(H, p, eng).real for p in psis] if o.get("E0") is None else [float(o["E0"])] * len(psis)
    Tpsi = []
    for t in Ts:
        for p in psis:
            Tpsi.append(OperatorPsi(t, p, R, eng))
    e0 = np.array([E0[i % len(psis)] for i in range(len(Tpsi))])
    # dense branch (ssp.cpp:2262-2319): Method "Dense", or the union basis of all T psi closed
    # under H within DenseBorder determinants (unless Method is "Lanczos")
    if o.get("Tensor"):
        return _spectra_tensor(H, Tpsi, float(E0[0]), o, R, method, eng)
    if method != "lanczos":
        seed = np.concatenate([t.det for t in Tpsi if t.N] or [np.zeros((0, nword(H.nf)), np.uint8)])
        ub = closure(H, seed, H.nf, R, -1, eng) if len(seed) else None
        if ub is not None and (method == "dense" or ub.n <= int(o["DenseBorder"])):
            return _spectra_dense(H, Tpsi, e0, o, ub, eng, states=krylov)
    # the plain path: one Lanczos per pair on the closure of its own T psi, as the reference
    # runs them; an empty T psi has a zero spectrum (all coefficients zero)
    A = np.zeros((len(Tpsi), ntri + 1))
    B = np.zeros((len(Tpsi), ntri))
    vectors = [[] for _ in Tpsi]
    for i in range(len(Tpsi)):
        if Tpsi[i].N == 0:
            continue
        basis = closure(H, Tpsi[i].det, H.nf, R, -1, eng)
        src, perm = Basis.from_bytes(H.nf, Tpsi[i].det, eng)
        xs = _upload(eng, src, perm, Tpsi[i].val)
        x = eng.empty(basis.n)
        eng.check(eng.L.qg_basis_map(eng.ctx, src.h, _ptr(xs), basis.h, _ptr(x), 1))
        if krylov:
            vectors[i], A[i], B[i] = _krylov_vectors(H, basis, x, ntri, eps, eng)
            continue
        a, b = lanczos_block(H, basis, x, ntri, eps, max(gamma, eps), eng)
        A[i] = a[0]
        B[i] = b[0]
    out = _lanczos_spectra(A, B, e0, o, gamma, ntri, eng)
    if krylov:
        return out + (vectors[0] if len(vectors) == 1 else vectors,)
    return out


def _krylov_vectors(H, basis, x, ntri, eps, eng):
    """The reference's Krylov-basis Lanczos on the device (qg_lanczos_krylov: full
    reorthogonalisation, orthogonality test, truncation): its non-empty vectors as
    wavefunctions (zero amplitudes left out, as the reference's truncated vectors), a and b."""
    with eng.on_stream():
        K = eng.torch.zeros((ntri, basis.n), dtype=eng.torch.complex128, device="cuda:%d" % eng.device)
    a = np.zeros(ntri + 1)
    b = np.zeros(ntri)
    eng.check(eng.L.qg_lanczos_krylov(eng.ctx, H.handle(eng), basis.h, _ptr(x), ntri, eps, _ptr(a), _ptr(b), _ptr(K)))
    Kh = eng.to_host(K)
    db = basis.dets_bytes()
    out = []
    for k in range(ntri):
        nz = np.flatnonzero(Kh[k])
        if len(nz):
            out.append(Wavefunction(H.nf, db[nz], Kh[k][nz]))
    return out, a, b


def _batched_lanczos_device(H, Ts, psis, o, R, eng, pairs=None):
    """The batched Lanczos branch with every step on the device: the initial states on one
    basis, their energies as one multi-vector expectation value, each T applied to all of them
    at once straight into the final basis (the closure under H of every T's targets, within
    the restrictions), the empty (T, psi) pairs left out, one multi-vector Lanczos for the
    rest.  pairs: the (iT, ipsi) to run, in the order of the result rows (default every pair,
    iT*Npsi + ipsi).  Returns (A, B, E0), or None when the dense branch applies (a final basis
    within DenseBorder and Method not "Lanczos")."""
    torch = eng.torch
    nf, npsi = H.nf, len(psis)
    ntri, eps, gamma = int(o["NTri"]), float(o["Epsilon"]), float(o["Gamma"])
    method = _spectra_method(o)
    dets = np.concatenate([p.det for p in psis])
    b0, perm = Basis.from_bytes(nf, dets, eng)
    X = np.zeros((max(b0.n, 1), npsi), dtype=np.complex128)
    off = 0
    for j, p in enumerate(psis):
        np.add.at(X[:, j], perm[off:off + p.N], np.asarray(p.val, dtype=np.complex128))
        off += p.N
    with eng.on_stream():
        Xd = torch.from_numpy(X).to("cuda:%d" % eng.device)
    if o.get("E0") is None:
        out = np.zeros(2 * npsi)
        eng.check(eng.L.qg_expectation(eng.ctx, H.handle(eng), b0.h, _ptr(Xd), npsi, _ptr(out)))
        E0 = [float(out[2 * j]) for j in range(npsi)]
    else:
        E0 = [float(o["E0"])] * npsi
    bt = None
    for t in Ts:
        tb = _targets_basis(t, b0, R, eng)
        bt = tb if bt is None else basis_union(bt, tb, eng)
    bf = closure_of(H, bt, R, -1, eng)
    if method != "lanczos" and 0 < bf.n <= int(o["DenseBorder"]):
        return None
    if pairs is None:
        pairs = [(j, i) for j in range(len(Ts)) for i in range(npsi)]
    nvec = len(pairs)
    A = np.zeros((nvec, ntri + 1))
    B = np.zeros((nvec, ntri))
    if bf.n == 0:
        return A, B, E0
    Y = eng.empty(bf.n, nvec)
    for j, t in enumerate(Ts):
        cols = [c for c, (jt, _) in enumerate(pairs) if jt == j]
        if not cols:
            continue
        yj = eng.empty(bf.n, npsi)
        eng.check(eng.L.qg_apply(eng.ctx, t.handle(eng), bf.h, b0.h, _ptr(Xd), _ptr(yj), npsi))
        with eng.on_stream():
            Y[:, cols] = yj[:, [pairs[c][1] for c in cols]]
    norms = np.zeros(nvec)
    eng.check(eng.L.qg_norm(eng.ctx, bf.n, nvec, _ptr(Y), _ptr(norms)))
    live = [i for i in range(nvec) if norms[i] > 0.0]
    if live:
        with eng.on_stream():
            x = Y[:, live].contiguous()
        a, b = lanczos_block(H, bf, x, ntri, eps, max(gamma, eps), eng)
        A[live] = a
        B[live] = b
    return A, B, E0


def lanczos_merge_key(H, T, psi, options=None, batched=True):
    """What several CreateSpectra calls must share to run as one multi-vector Lanczos: the
    Hamiltonian and every option the Lanczos coefficients depend on (NTri, Epsilon, Gamma,
    E0, Restrictions, DenseBorder, Method).  None when the call does not take the batched
    Lanczos branch (Tensor, KrylovBasis, the dense method, batched=False)."""
    o = _opts(options)
    if not batched or o.get("Tensor") or o.get("KrylovBasis") or _spectra_method(o) == "dense":
        return None
    return (id(H), int(o["NTri"]), float(o["Epsilon"]), float(o["Gamma"]), o.get("E0"),
            repr(o.get("Restrictions")), int(o["DenseBorder"]), _spectra_method(o))


def CreateSpectraMerged(H, jobs, eng=None):
    """Several CreateSpectra calls on one Hamiltonian as one multi-vector Lanczos (the served
    form's continuous batching): jobs is a list of (T, psi, options) with equal
    lanczos_merge_key.  Every job's (T, psi) pairs, and only those, run side by side on the
    closure of all their targets; each job then takes its own rows, its own energy window,
    broadening and number of frequencies.  A job's coefficients equal those of its call alone
    to rounding (the closed bases differ only by determinants its vectors never reach).
    Returns one (Spectra, tri) per job, or each call's own result when the dense branch
    applies."""
    eng = eng or engine()
    Ts, tidx, psis, pairs, rows = [], {}, [], [], []
    for T, psi, _ in jobs:
        tl = T if isinstance(T, (list, tuple)) else [T]
        pl = psi if isinstance(psi, (list, tuple)) else [psi]
        base = len(psis)
        psis.extend(pl)
        r = []
        for t in tl:
            if id(t) not in tidx:
                tidx[id(t)] = len(Ts)
                Ts.append(t)
            for i in range(len(pl)):
                r.append(len(pairs))
                pairs.append((tidx[id(t)], base + i))
        rows.append(r)
    o = _opts(jobs[0][2])
    got = _batched_lanczos_device(H, Ts, psis, o, parse_restrictions(o.get("Restrictions")), eng, pairs)
    if got is None:
        return [CreateSpectra(H, T, psi, opt, eng=eng) for T, psi, opt in jobs]
    A, B, E0 = got
    out = []
    for (T, psi, opt), r in zip(jobs, rows):
        oj = _opts(opt)
        e0 = np.array([E0[pairs[c][1]] for c in r])
        out.append(_lanczos_spectra(A[r], B[r], e0, oj, float(oj["Gamma"]), int(oj["NTri"]), eng))
    return out


def _lanczos_spectra(A, B, e0, o, gamma, ntri, eng):
    """Spectra of the Lanczos branch from the coefficients: pole range from the extreme
    eigenvalues of every tridiagonal matrix, the default Emin/Emax/Gamma from it
    (ssp.cpp:2651-2684), all spectra at all frequencies in one kernel."""
    lo, hi = np.inf, -np.inf
    for s in range(A.shape[0]):
        m = ntri
        for k in range(1, ntri):  # a chain that ended early (b = 0) is shorter
            if B[s, k] == 0.0:
                m = k
                break
        w0, w1 = _tri_extremes(A[s, 1:m + 1], B[s, 1:m])
        lo, hi = min(lo, w0 - e0[s]), max(hi, w1 - e0[s])
    emin, emax, NE = o["Emin"], o["Emax"], int(o["NE"])
    emin, emax, gamma = _default_window(lo, hi, emin, emax, gamma, NE)
    G = TriDiagonalMatrixToSpectrum(e0, A, B, emin, emax, NE, gamma, eng)
    tri = [(np.r_[0.0, A[s, 1:] - e0[s]], B[s].copy()) for s in range(A.shape[0])]
    return Spectra(G, emin, emax, NE, gamma, lo, hi), tri


def _tri_extremes(a, b):
    """Lowest and highest eigenvalue of the symmetric tridiagonal matrix with diagonal a and
    off-diagonal b, as CreateSpectra takes them for the pole range (LuaInterface/ssp.cpp:2651-2663,
    TriDiagonalMatrixToEigenvalues, Core/BasicMath/BasicMath_MatrixTypeConversion.cpp:1538):
    LAPACK bisection for the two wanted eigenvalues, O(m) each, not a dense eigensolve."""
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    m = len(a)
    if m == 1:
        return float(a[0]), float(a[0])
    try:
        from scipy.linalg import eigvalsh_tridiagonal
        lo = eigvalsh_tridiagonal(a, b, select="i", select_range=(0, 0))[0]
        hi = eigvalsh_tridiagonal(a, b, select="i", select_range=(m - 1, m - 1))[0]
        return float(lo), float(hi)
    except ImportError:
        w = np.linalg.eigvalsh(np.diag(a) + np.diag(b, 1) + np.diag(b, -1))
        return float(w[0]), float(w[-1])


def _default_window(lo, hi, emin, emax, gamma, NE):
    """Emin/Emax/Gamma not given: from the pole range [lo, hi] (ssp.cpp:2664-2684)."""
    if lo == hi:
        if lo == 0:
            emin = -1.0 if emin is None else emin
            emax = 1.0 if emax is None else emax
        elif lo < 0:
            emin = 2.125 * lo if emin is None else emin
            emax = -0.125 * lo if emax is None else emax
        else:
            emin = -0.125 * lo if emin is None else emin
            emax = 2.125 * lo if emax is None else emax
    if emin is None:
        emin = lo - 0.125 * (hi - lo)
    if emax is None:
        emax = hi + 0.125 * (hi - lo)
    if gamma == 0:
        gamma = 10 * (emax - emin) / NE
    return emin, emax, gamma


# ----------------------------------------------------------------------------- eigensystem

def enumerate_restricted(nf, restrictions):
    """All determinants that satisfy occupation windows on disjoint masks (the complete basis
    the reference builds for small systems, Core/BlockLanczos.cpp:102)."""
    import itertools
    masks = [[i for i, ch in enumerate(m) if ch == "1"] for m, _, _ in restrictions]
    covered = set(i for m in masks for i in m)
    free = [i for i in range(nf) if i not in covered]
    seen = set()
    for a in masks:
        if seen & set(a):
            raise ValueError("overlapping restriction masks: enumerate by closure instead")
        seen |= set(a)
    choices = []
    for (m, lo, hi), idx in zip(restrictions, masks):
        opts = []
        for k in range(lo, min(hi, len(idx)) + 1):
            opts.extend(itertools.combinations(idx, k))
        choices.append(opts)
    free_opts = [c for k in range(len(free) + 1) for c in itertools.combinations(free, k)] if free else [()]
    rows = []
    for combo in itertools.product(*choices, free_opts):
        s = np.zeros(nf, dtype=np.uint8)
        for part in combo:
            for i in part:
                s[i] = 1
        rows.append(s)
    bits = np.zeros((len(rows), nword(nf) * 8), dtype=np.uint8)
    if rows:
        bits[:, :nf] = np.array(rows)
    return np.packbits(bits, axis=1, bitorder="big")


def Eigensystem(H, StartRestrictions, Npsi=None, options=None, eng=None, seed=12345):
    """Lowest eigenstates of a Hermitian H (reference Eigensystem -> BlockGroundState,
    LuaInterface/ssp.cpp:4039-4260, Core/BlockLanczos.cpp:5782).  Two call forms, as the
    reference: Eigensystem(H, StartRestrictions, Npsi[, options]) starts from every determinant
    the start restrictions allow; Eigensystem(H, psi or [psi, ...][, options]) starts from the
    given states' determinants and finds as many states as were given.  The basis then grows
    under H within the Restrictions option, or without limit when it is absent (the reference's
    growth loop uses only that option, BlockLanczos.cpp:5843-5884; ExpandBasis false keeps the
    start determinants), and the eigenproblem on that basis is solved densely (at most DenseBorder determinants, raised to Npsi when
    options are given, BlockLanczosGroundStateConserveBasisDense) or by restarted block Lanczos
    on the device.  Returns (list of Wavefunction, energies)."""
    states = None
    if isinstance(StartRestrictions, Wavefunction) or (
            isinstance(StartRestrictions, (list, tuple)) and len(StartRestrictions)
            and isinstance(StartRestrictions[0], Wavefunction)):
        states = _as_list(StartRestrictions)
        if options is None and not isinstance(Npsi, (int, np.integer)):
            options = Npsi
        Npsi = len(states)
    elif Npsi is None:
        raise ValueError("Eigensystem called with start restrictions needs the number of states")
    eng = eng or engine()
    o = _opts(options)
    if options:
        o["DenseBorder"] = max(int(o["DenseBorder"]), int(Npsi))
    if states is None:
        seed_dets = enumerate_restricted(H.nf, parse_restrictions(StartRestrictions))
    else:
        seed_dets = np.concatenate([np.asarray(p.det, dtype=np.uint8).reshape(-1, nword(H.nf)) for p in states])
    basis, _ = Basis.from_bytes(H.nf, seed_dets, eng)
    if o.get("ExpandBasis", True):
        basis = closure_of(H, basis, o.get("Restrictions"), -1, eng)
    # ExpandBasis false: the eigenproblem on the start determinants as they are
    # (BlockLanczosGroundStateConserveBasis, LuaInterface/ssp.cpp:4231-4238)
    if basis.n <= int(o["DenseBorder"]):
        # dense branch (BlockLanczosGroundStateConserveBasisDense, Core/BlockLanczos.cpp:370)
        w, V = hermitian_eigh(OperatorToDeterminantMatrix(H, basis, eng), min(Npsi, basis.n), eng)
        db = basis.dets_bytes()
        return [Wavefunction(H.nf, db, V[:, k]) for k in range(V.shape[1])], w[:V.shape[1]]
    x, en = EigensystemOnBasis(H, basis, Npsi, options, eng, seed)
    X = eng.to_host(x)
    db = basis.dets_bytes()
    out = [Wavefunction(H.nf, db, X[:, k]) for k in range(Npsi)]
    return out, en


def EigensystemOnBasis(H, basis, Npsi, options=None, eng=None, seed=12345, max_restarts=200, status=None):
    """Lowest Npsi eigenpairs of H on a device basis, kept on the device: returns
    ((n, Npsi) complex CUDA tensor, energies).  With a dict `status`, a restart limit reached
    before convergence returns the current Ritz pairs and sets status["converged"] = False
    (otherwise it raises)."""
    eng = eng or engine()
    o = _opts(options)
    n = basis.n
    rng = np.random.default_rng(seed)
    x0 = rng.standard_normal((n, Npsi)).astype(np.complex128)
    if any(v.imag != 0 for _, v in H.terms):
        x0 += 1j * rng.standard_normal((n, Npsi))
    # a real H starts from real vectors and keeps them real, as the reference's real-vector
    # solver does: the eigenstates come out real, and so do the Lanczos chains built on them
    with eng.on_stream():
        x = eng.torch.from_numpy(x0).to("cuda:%d" % eng.device).contiguous()
    en = np.zeros(Npsi)
    it = C.c_int32()
    # Krylov space up to Npsi + NKrylovMax vectors (grown per restart from Npsi + 100), within
    # half of the free device memory
    free = eng.torch.cuda.mem_get_info(eng.device)[0]
    K = int(min(Npsi + int(o["NKrylovMax"]), n, max(2 * Npsi, free // (2 * 16 * max(n, 1)))))
    tol = float(o["Zero"])
    st = eng.L.qg_block_groundstate(eng.ctx, H.handle(eng), basis.h, Npsi, _ptr(x), _ptr(en), tol, K,
                                    int(max_restarts), C.byref(it))
    if status is not None:
        status["converged"] = st == 0
        status["applies"] = it.value
        status["krylov_max"] = K
        if st == qgpu.QG_ERR_TIMEOUT:
            st = 0
    eng.check(st)
    return x, en


# ----------------------------------------------------------------------------- RIXS

def _as_list(x):
    return list(x) if isinstance(x, (list, tuple)) else [x]


def CreateResonantSpectra(H1, H2, T1, T2, psi, options=None, eng=None):
    """Reference CreateResonantSpectra (LuaInterface/ssp.cpp:3090-3447).  T1, T2 and psi are an
    operator / a wavefunction or lists of them.  Returns (G [nspec, NE2+1], settings).

    Branch choice as in the reference (ssp.cpp:3300-3371): the dense branch when the union of
    the initial states, the targets of every T1, their closure under H1, the targets of every T2
    and their closure under H2 all stay within DenseBorder (or ForceDenseMethod), else the
    Krylov branch.  Spectrum order: dense, l + (NE1+1)(k + NT2 (iT1 + NT1 ipsi)); Krylov,
    one block of NT2 (NE1+1) spectra (index k (NE1+1) + l) per (ipsi, iT1) pair, psi outer;
    tensor forms, (NT1 NT2 Npsi)^2 (NE1+1) spectra (see _rixs_dense and _rixs_krylov_tensor)."""
    eng = eng or engine()
    o = _opts(options)
    T1s, T2s, psis = _as_list(T1), _as_list(T2), _as_list(psi)
    if not T1s or not T2s or not psis:
        raise ValueError("CreateResonantSpectra: empty list of operators or wavefunctions")
    for k in ("E0_1", "E0_2"):
        if o.get(k) is None and o.get("E0") is not None:
            o[k] = o["E0"]
    tensor = bool(o.get("Tensor"))
    bases = _rixs_dense_bases(H1, H2, T1s, T2s, psis, o, eng)
    if bases is not None:
        return _rixs_dense(H1, H2, T1s, T2s, psis, o, bases[0], bases[1], tensor, eng)
    if tensor:
        return _rixs_krylov_tensor(H1, H2, T1s, T2s, psis, o, eng)
    blocks, sts = [], []
    for p in psis:
        for T in T1s:
            G, st = _rixs_krylov(H1, H2, T, T2s, p, o, eng)
            blocks.append(G)
            sts.append(st)
    st = dict(sts[0], method="krylov")
    if len(sts) > 1:
        st["blocks"] = sts
    return np.concatenate(blocks), st


def _rixs_krylov(H1, H2, T1, T2s, psi, o, eng):
    """One Krylov RIXS run, ResonantSpectra (Core/ResonantSpectra.cpp:6): spectrum
    iT2 (NE1+1) + p, every incident energy and T2 batched on the device (qg_resonant_spectra)."""
    big = np.finfo(float).max
    st = qgpu.RixsSettings()
    st.ntri1, st.ntri2 = int(o["NTri1"]), int(o["NTri2"])
    st.epsilon = float(o["Epsilon"])
    st.emin1 = float(o.get("Emin1", big)) if o.get("Emin1") is not None else big
    st.emax1 = float(o.get("Emax1", -big)) if o.get("Emax1") is not None else -big
    st.ne1 = int(o.get("NE1", 1000))
    st.gamma1 = float(o.get("Gamma1", 0.0))
    st.emin2 = float(o.get("Emin2", big)) if o.get("Emin2") is not None else big
    st.emax2 = float(o.get("Emax2", -big)) if o.get("Emax2") is not None else -big
    st.ne2 = int(o.get("NE2", 1000))
    st.gamma2 = float(o.get("Gamma2", 0.0))
    st.energy1 = float(o["E0_1"]) if o.get("E0_1") is not None else big
    st.energy2 = float(o["E0_2"]) if o.get("E0_2") is not None else big
    r1 = _Res(H1.nf, parse_restrictions(o.get("Restrictions1")))
    r2 = _Res(H1.nf, parse_restrictions(o.get("Restrictions2")))
    st.res1 = C.cast(C.pointer(r1.r), C.c_void_p) if r1.r.n else None
    st.res2 = C.cast(C.pointer(r2.r), C.c_void_p) if r2.r.n else None
    b, perm = Basis.from_bytes(psi.nf, psi.det, eng)
    x = _upload(eng, b, perm, psi.val)
    t2h = (C.c_void_p * len(T2s))(*[t.handle(eng) for t in T2s])
    g = np.zeros(2 * len(T2s) * (st.ne1 + 1) * (st.ne2 + 1))
    eng.check(eng.L.qg_resonant_spectra(eng.ctx, H1.handle(eng), H2.handle(eng), T1.handle(eng),
                                        C.cast(t2h, C.c_void_p), len(T2s), b.h, _ptr(x), C.byref(st), _ptr(g)))
    G = (g[0::2] + 1j * g[1::2]).reshape(len(T2s) * (st.ne1 + 1), st.ne2 + 1)
    return G, {k: getattr(st, k) for k, _ in st._fields_ if not k.startswith("res")}


def _rixs_dense_bases(H1, H2, T1s, T2s, psis, o, eng):
    """The two bases of the dense branch, or None when one of them outgrows DenseBorder
    (LuaInterface/ssp.cpp:3300-3371): the union of the initial states; the targets of every T1
    from it; their closure under H1 (intermediate states); the targets of every T2 from that;
    their closure under H2 (final states), all within Restrictions1 / Restrictions2."""
    force = bool(o.get("ForceDenseMethod"))
    border = int(o["DenseBorder"])

    def fits(n):
        return force or n <= border

    nf = H1.nf
    if not fits(max(p.N for p in psis)):  # then their union is larger still
        return None
    dets = np.unique(np.concatenate([np.asarray(p.det, dtype=np.uint8).reshape(-1, nword(nf)) for p in psis]), axis=0)
    if not fits(len(dets)):
        return None
    R1, R2 = o.get("Restrictions1"), o.get("Restrictions2")
    u, _ = Basis.from_bytes(nf, dets, eng)
    bases = []
    for H, Ts, R in ((H1, T1s, R1), (H2, T2s, R2)):
        bt = None
        for T in Ts:
            t = _targets_basis(T, u, R, eng)
            bt = t if bt is None else basis_union(bt, t, eng)
            if not fits(bt.n):
                return None
        u = closure_of(H, bt, R, -1, eng)
        if not fits(u.n):
            return None
        bases.append(u)
    return bases


def _rixs_energies(H, psis, key, o, eng, normalise=True):
    """E0_1 / E0_2 when given, else <psi|H|psi> (divided by <psi|psi> when that exceeds
    DBL_EPSILON, Core/ResonantSpectra.cpp:345-373) for every initial state."""
    if o.get(key) is not None:
        return np.full(len(psis), float(o[key]))
    out = []
    for p in psis:
        e = PsiOperatorPsi(H, p, eng).real
        nn = float(np.real(np.vdot(p.val, p.val)))
        out.append(e / nn if normalise and nn > DBL_EPSILON else e)
    return np.array(out)


def _rixs_range(emin, emax, ne, gamma, lo_ev, hi_ev, e_lo, e_hi):
    """Energy-range defaults of the dense branch (Core/ResonantSpectra.cpp:472-535)."""
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
    return float(emin), float(emax), int(ne), float(gamma)


def _apply_between(O, dst, src, X, eng, device=False):
    """O applied to every column of the matrix X (rows on src; host, or a device tensor) into
    dst, one multi-vector pull launch sequence on the device; returns the host matrix
    (dst.n x columns), or the device tensor with device=True."""
    k = X.shape[1]
    if not dst.n or not src.n or not k:
        z = np.zeros((dst.n, k), dtype=np.complex128)
        return _to_dev(eng, z) if device else z
    x = X if not isinstance(X, np.ndarray) else _to_dev(eng, X)
    y = eng.empty(dst.n, k)
    eng.check(eng.L.qg_apply(eng.ctx, O.handle(eng), dst.h, src.h, _ptr(x), _ptr(y), k))
    return y[:dst.n] if device else eng.to_host(y[:dst.n])


def _to_dev(eng, A):
    with eng.on_stream():
        return eng.torch.from_numpy(np.ascontiguousarray(A, dtype=np.complex128)).to("cuda:%d" % eng.device)


def _adjoint_product(eng, A, B):
    """A^H B of device tensors A (n x ka), B (n x kb), by the library's block kernels."""
    n, ka = A.shape
    kb = B.shape[1]
    A, B = A.contiguous(), B.contiguous()
    C = eng.empty(ka, kb)
    if n and ka and kb:
        eng.check(eng.L.qg_block_adjoint_product(eng.ctx, _ptr(A), ka, ka, _ptr(B), kb, kb, n, _ptr(C)))
    return C[:ka]


def _block_product(eng, A, M):
    """A M of device tensors A (n x ka), M (ka x kb), by the library's block kernels."""
    n, ka = A.shape
    kb = M.shape[1]
    A, M = A.contiguous(), M.contiguous()
    X = eng.empty(n, kb)
    if n and ka and kb:
        eng.check(eng.L.qg_block_product(eng.ctx, _ptr(A), ka, ka, _ptr(M), kb, n, 1.0, 0.0, _ptr(X), kb))
    return X[:n]


def _poles_complex(e0, poles, W, emin, emax, ne, gamma, eng):
    """Sum of Lorentzians with complex weights: the poles kernel on the real and imaginary parts."""
    G = ListOfPolesToSpectrum(e0, poles, np.ascontiguousarray(W.real), emin, emax, ne, gamma, eng)
    if np.any(W.imag):
        G = G + 1j * ListOfPolesToSpectrum(e0, poles, np.ascontiguousarray(W.imag), emin, emax, ne, gamma, eng)
    return G


def _rixs_dense(H1, H2, T1s, T2s, psis, o, b1, b2, tensor, eng):
    """Dense RIXS, ResonantSpectraDense / ResonantSpectraDenseTensor (Core/ResonantSpectra.cpp:290,
    :665).  H1 and H2 as dense matrices on their bases (device), their eigensystems (host
    solver), A[m, j] = <m|T1 psi_j> (j = iT1 + NT1 ipsi), B_k[f, m] = <f|T2_k|m> with T2_k
    applied to every intermediate eigenvector on the device; per incident energy w_l the
    amplitudes D_k = B_k (A / (w_l - E_m + E1_psi + i Gamma1/2)) and the spectra as sums of
    Lorentzians at the final eigenvalues (the poles kernel, all spectra and energies at once).
    Non-tensor spectrum l + (NE1+1)(k + NT2 j): weights |D_k[f, j]|^2, shift E2 of psi_j.
    Tensor spectrum l + (NE1+1)(j2 + NT2(i1 + NT1(n2 + NT2(m1 + NT1(r + Npsi s))))): weights
    conj(D_n2[f, m1 + NT1 s]) D_j2[f, i1 + NT1 r], shift E2 of psi 0."""
    npsi, nt1, nt2 = len(psis), len(T1s), len(T2s)
    n1, n2 = b1.n, b2.n
    M1 = npsi * nt1
    R1 = o.get("Restrictions1")
    e1 = _rixs_energies(H1, psis, "E0_1", o, eng)
    e2 = _rixs_energies(H2, psis, "E0_2", o, eng)
    X = np.zeros((n1, M1), dtype=np.complex128)
    for ip, p in enumerate(psis):
        for it, T in enumerate(T1s):
            t = OperatorPsi(T, p, R1, eng)
            if t.N and n1:
                # zero-amplitude targets of zero-valued strings may lie outside the device basis
                rows = b1.find(t.det)
                keep = rows >= 0
                if not np.all(t.val[~keep] == 0):
                    raise RuntimeError("CreateResonantSpectra: T1 psi reaches outside the intermediate basis")
                np.add.at(X[:, it + nt1 * ip], rows[keep], t.val[keep])
    if n1:
        w1, V1 = hermitian_eigh(OperatorToDeterminantMatrix(H1, b1, eng), n1, eng)
    else:
        w1, V1 = np.zeros(1), np.zeros((0, 0), dtype=np.complex128)
    if n2:
        w2, V2 = hermitian_eigh(OperatorToDeterminantMatrix(H2, b2, eng), n2, eng)
    else:
        w2, V2 = np.zeros(1), np.zeros((0, 0), dtype=np.complex128)
    # the eigenvector products on the device (the reference's BLAS products)
    V1d = _to_dev(eng, V1) if n1 else None
    V2d = _to_dev(eng, V2) if n2 else None
    A = eng.to_host(_adjoint_product(eng, V1d, _to_dev(eng, X))) if n1 else np.zeros((0, M1), dtype=np.complex128)
    Bd = [_adjoint_product(eng, V2d, _apply_between(T, b2, b1, V1d, eng, device=True)) for T in T2s] \
        if n1 and n2 else []
    # unset Emin/Emax (None) are derived from the extreme eigenvalues
    emin1, emax1, ne1, g1 = _rixs_range(o.get("Emin1"), o.get("Emax1"), int(o.get("NE1", 1000)),
                                        float(o.get("Gamma1", 0.0)), w1[0], w1[-1], e1.min(), e1.max())
    emin2, emax2, ne2, g2 = _rixs_range(o.get("Emin2"), o.get("Emax2"), int(o.get("NE2", 1000)),
                                        float(o.get("Gamma2", 0.0)), w2[0], w2[-1], e2.min(), e2.max())
    np1 = ne1 + 1
    wres = np.array([emin1 + (emax1 - emin1) * l / ne1 for l in range(np1)])
    psi_of = np.arange(M1) // nt1
    Cm = A[None, :, :] / (wres[:, None, None] - w1[None, :n1, None] + e1[psi_of][None, None, :] + 0.5j * g1)
    if n2 and n1:  # D_k[l] = B_k Cm[l] for every l at once: (n2 x n1) (n1 x np1 M1)
        Md = _to_dev(eng, np.ascontiguousarray(Cm.transpose(1, 0, 2)).reshape(n1, np1 * M1))
        D = np.stack([eng.to_host(_block_product(eng, Bk, Md)).reshape(n2, np1, M1).transpose(1, 0, 2)
                      for Bk in Bd])
    else:
        D = np.zeros((nt2, np1, n2, M1), dtype=np.complex128)
    st = {"method": "dense", "emin1": emin1, "emax1": emax1, "ne1": ne1, "gamma1": g1, "emin2": emin2,
          "emax2": emax2, "ne2": ne2, "gamma2": g2, "energy1": e1.tolist(), "energy2": e2.tolist(),
          "n1": n1, "n2": n2, "resonant_energies": wres.tolist()}
    if not tensor:
        nspec = nt2 * M1 * np1
        if not n2:
            return np.zeros((nspec, ne2 + 1), dtype=np.complex128), st
        W = np.zeros((nspec, n2))
        e0 = np.zeros(nspec)
        for k in range(nt2):
            for j in range(M1):
                rows = np.arange(np1) + np1 * (k + nt2 * j)
                W[rows] = np.abs(D[k][:, :, j]) ** 2
                e0[rows] = e2[psi_of[j]]
        return ListOfPolesToSpectrum(e0, w2, W, emin2, emax2, ne2, g2, eng), st
    M = M1 * nt2
    nspec = M * M * np1
    G = np.zeros((nspec, ne2 + 1), dtype=np.complex128)
    if not n2:
        return G, st
    lk, lc, rk, rc, base = [], [], [], [], []
    for r in range(npsi):
        for s_ in range(npsi):
            for i1 in range(nt1):
                for j2 in range(nt2):
                    for m1 in range(nt1):
                        for n2_ in range(nt2):
                            base.append(np1 * (j2 + nt2 * (i1 + nt1 * (n2_ + nt2 * (m1 + nt1 * (r + npsi * s_))))))
                            lk.append(n2_)
                            lc.append(m1 + nt1 * s_)
                            rk.append(j2)
                            rc.append(i1 + nt1 * r)
    lk, lc, rk, rc, base = (np.array(v) for v in (lk, lc, rk, rc, base))
    step = max(1, int(2 ** 24 // max(1, M * M * n2)))  # bound the host weight block
    for l0 in range(0, np1, step):
        ls = np.arange(l0, min(np1, l0 + step))
        W = np.conj(D[lk[:, None], ls[None, :], :, lc[:, None]]) * D[rk[:, None], ls[None, :], :, rc[:, None]]
        W = W.reshape(-1, n2)  # rows (pair, l)
        rows = (base[:, None] + ls[None, :]).reshape(-1)
        G[rows] = _poles_complex(e2[0], w2, W, emin2, emax2, ne2, g2, eng)
    return G, st


def _rixs_krylov_tensor(H1, H2, T1s, T2s, psis, o, eng):
    """Krylov tensor RIXS (ResonantSpectraTensor, Core/ResonantSpectra.cpp:1204-1700): the matrix
    <v_a| (w + E2 - H2 + i Gamma2/2)^-1 |v_b> of the vectors v_(psi, T1, T2) = T2 G1(w_l) T1 psi
    for every incident energy w_l, both shifts from psi 0, as the reference computes it:
      1. the block of T1 psi (j = iT1 + NT1 ipsi) on one basis, entries below Epsilon dropped;
      2. a block Lanczos of H1 from it that keeps its Krylov blocks (qg_block_lanczos), the block
         tridiagonal matrix chopped at Epsilon and diagonalised on the device; the intermediate
         window from its extreme eigenvalues;
      3. G1(w_l) T1 psi_j = Q (w_l - T + i Gamma1/2)^-1 Q^H T1 psi_j for all l at once: the
         coefficients in the Krylov basis (Q^H T1 psi_j is the first block's b_0) and the
         combination of the stored vectors on the device (qg_krylov_combine);
      4. T2 on all of them in one multi-vector launch per T2;
      5. per incident energy a block Lanczos of H2 from its NT2 NT1 Npsi vectors, chopped, the
         final window from the first energy's block eigenvalues (the reference sets it there and
         keeps it), and the m x m spectra by the block continued fraction.
    The reference's index order is kept: spectrum
    l + (NE1+1)(j2 + NT2(i1 + NT1(n2 + NT2(m1 + NT1(r + Npsi s)))))
    holds the element between v_(r, m1, n2) (left) and v_(s, i1, j2) (right)."""
    torch = eng.torch
    dev = "cuda:%d" % eng.device
    npsi, nt1, nt2 = len(psis), len(T1s), len(T2s)
    M1, nf = npsi * nt1, H1.nf
    eps, ntri1, ntri2 = float(o["Epsilon"]), int(o["NTri1"]), int(o["NTri2"])
    sv = float(o.get("SingularValue", DEFAULTS["SingularValue"]))
    R1, R2 = o.get("Restrictions1"), o.get("Restrictions2")
    e1 = float(_rixs_energies(H1, psis[:1], "E0_1", o, eng, normalise=False)[0])
    e2 = float(_rixs_energies(H2, psis[:1], "E0_2", o, eng, normalise=False)[0])
    ne1, ne2 = int(o.get("NE1", 1000)), int(o.get("NE2", 1000))
    np1 = ne1 + 1
    M = M1 * nt2
    Tpsi = [OperatorPsi(T, p, R1, eng) for p in psis for T in T1s]  # j = iT1 + NT1 ipsi
    seed = [t.det for t in Tpsi if t.N]
    if not seed:
        raise ValueError("CreateResonantSpectra: every T1 psi is empty")
    b1 = closure(H1, np.concatenate(seed), nf, R1, -1, eng)
    n1 = b1.n
    X1 = np.zeros((n1, M1), dtype=np.complex128)
    for j, t in enumerate(Tpsi):
        if t.N:
            # ComplexWaveFunctionTruncateBasis (Core/ComplexWaveFunctionArithmetic.cpp:1073):
            # keep |a|^2 > epsilon^2
            v = np.where(t.val.real ** 2 + t.val.imag ** 2 > eps * eps, t.val, 0.0)
            np.add.at(X1[:, j], b1.find(t.det), v)
    nk = ntri1 * M1
    with eng.on_stream():
        x1 = torch.from_numpy(X1).to(dev)
        K1 = torch.zeros((nk, n1), dtype=torch.complex128, device=dev)
    A1, B1, sizes1 = block_lanczos(H1, b1, x1, ntri1, eps, sv, eng, krylov=K1)
    A1, B1 = block_chop(A1, eps), block_chop(B1, eps)
    T1m = block_tridiagonal_dense(A1, B1)
    ev, Z = hermitian_eigh(T1m, nk, eng)
    # the intermediate window from the Krylov directions the recursion kept: the rows of
    # deflated directions are zero and their eigenvalue 0 stays out of it (they carry no weight
    # of T1 psi either)
    live = [k * M1 + c for k in range(ntri1) for c in range(int(sizes1[k + 1]))]
    evl = hermitian_eigh(T1m[np.ix_(live, live)], 0, eng)[0] if live else np.zeros(1)
    emin1, emax1, g1 = _default_window(evl[0] - e1, evl[-1] - e1, o.get("Emin1"), o.get("Emax1"),
                                       float(o.get("Gamma1", 0.0)), ne1)
    wres = np.array([emin1 + (emax1 - emin1) * p / ne1 + e1 for p in range(np1)])
    # coefficients of G1(w_l) T1 psi_j in the Krylov basis, column l * M1 + j:
    # Z diag(1 / (w_l - ev + i g1/2)) Z^H[:, first block] b_0^T
    first = Z[:M1, :].conj().T @ B1[0].T
    Cc = np.zeros((nk, np1 * M1), dtype=np.complex128)
    for p in range(np1):
        Cc[:, p * M1:(p + 1) * M1] = Z @ (first / (wres[p] - ev + 0.5j * g1)[:, None])
    GT = eng.empty(n1, np1 * M1)
    Cc = np.ascontiguousarray(Cc)
    eng.check(eng.L.qg_krylov_combine(eng.ctx, _ptr(K1), n1, nk, _ptr(Cc), np1 * M1, _ptr(GT)))
    del K1
    # final-state basis: targets of every T2, closure under H2
    bt = None
    for T in T2s:
        t = _targets_basis(T, b1, R2, eng)
        bt = t if bt is None else basis_union(bt, t, eng)
    b2 = closure_of(H2, bt, R2, -1, eng)
    n2 = b2.n
    G = np.zeros((M * M * np1, ne2 + 1), dtype=np.complex128)
    st = {"method": "krylov_tensor", "emin1": emin1, "emax1": emax1, "ne1": ne1, "gamma1": g1,
          "energy1": e1, "energy2": e2, "n1": n1, "n2": n2, "resonant_energies": (wres - e1).tolist()}
    if not n2:
        st.update(emin2=o.get("Emin2"), emax2=o.get("Emax2"), ne2=ne2, gamma2=float(o.get("Gamma2", 0.0)))
        return G, st
    # T2_s G1(w_l) T1 psi_j: Y[s] column l * M1 + j
    Y = []
    for T in T2s:
        yv = eng.empty(n2, np1 * M1)
        eng.check(eng.L.qg_apply(eng.ctx, T.handle(eng), b2.h, b1.h, _ptr(GT), _ptr(yv), np1 * M1))
        Y.append(yv[:n2])
    emin2 = emax2 = g2 = None
    Gm = np.zeros((np1, M, M, ne2 + 1), dtype=np.complex128)  # vectors in the order s * M1 + j
    for p in range(np1):
        with eng.on_stream():
            Zp = torch.cat([y[:, p * M1:(p + 1) * M1] for y in Y], dim=1).contiguous()
        A2, B2, _ = block_lanczos(H2, b2, Zp, ntri2, eps, sv, eng)
        A2, B2 = block_chop(A2, eps), block_chop(B2, eps)
        if emin2 is None:
            val, _ = hermitian_eigh(block_tridiagonal_dense(A2, B2), 0, eng)
            emin2, emax2, g2 = _default_window(val[0] - e2, val[-1] - e2, o.get("Emin2"), o.get("Emax2"),
                                               float(o.get("Gamma2", 0.0)), ne2)
            st.update(emin2=emin2, emax2=emax2, ne2=ne2, gamma2=g2)
        Gm[p] = BlockTriDiagonalMatrixToSpectra(e2, A2, B2, emin2, emax2, ne2, g2, eng).reshape(M, M, ne2 + 1)
    for r in range(npsi):
        for s_ in range(npsi):
            for i1 in range(nt1):
                for j2 in range(nt2):
                    for m1 in range(nt1):
                        for n2_ in range(nt2):
                            idx = j2 + nt2 * (i1 + nt1 * (n2_ + nt2 * (m1 + nt1 * (r + npsi * s_))))
                            row = n2_ * M1 + (m1 + nt1 * r)
                            col = j2 * M1 + (i1 + nt1 * s_)
                            G[np1 * idx:np1 * (idx + 1)] = Gm[:, row, col]
    return G, st
