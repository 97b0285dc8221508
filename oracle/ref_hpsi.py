"""Driver of oracle/_ref/ref_hpsi (TEST AND MEASUREMENT INFRASTRUCTURE ONLY): the reference's
own fixed-basis H*psi (OperatorPsiConserveBasisPreAllocated, Core/OperatorWaveFunction.cpp:5541)
compiled from its unmodified sources by ``oracle/build_ref.sh <ref> hpsi``, fed a basis, an
operator and the amplitudes of a set of source rows through a file.  Used by tests/ to pin the
oracle and the GPU path to the reference itself, and by bench.py's reference arm."""
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BINARY = os.path.join(HERE, "_ref", "ref_hpsi")


def available():
    return os.path.exists(BINARY)


def write_input(path, nf, terms, dets, src_rows, x_src):
    """terms: [(ladder codes, complex value)]; dets: (n, nword) uint8 in basis order;
    src_rows: int64 rows of the sources; x_src: their complex amplitudes."""
    dets = np.ascontiguousarray(dets, dtype=np.uint8)
    src_rows = np.ascontiguousarray(src_rows, dtype=np.int64)
    x_src = np.ascontiguousarray(x_src, dtype=np.complex128)
    with open(path, "wb") as f:
        np.array([nf, len(terms)], dtype=np.int32).tofile(f)
        np.array([len(dets), len(src_rows)], dtype=np.int64).tofile(f)
        np.array([len(t[0]) for t in terms], dtype=np.int32).tofile(f)
        np.array([o for t in terms for o in t[0]], dtype=np.uint16).tofile(f)
        np.array([complex(t[1]).real for t in terms], dtype=np.float64).tofile(f)
        np.array([complex(t[1]).imag for t in terms], dtype=np.float64).tofile(f)
        dets.tofile(f)
        src_rows.tofile(f)
        x_src.view(np.float64).tofile(f)


def run(path, threads, repeats, want_y=False, n=None, timeout=3600):
    """Returns (basis build seconds, [seconds per call], (determinant, term) pairs per call,
    y or None).  y is the result on the whole basis (n complex values) when want_y."""
    out = tempfile.mktemp(prefix="ref_hpsi_y_") if want_y else None
    cmd = [BINARY, path, str(int(threads)), str(int(repeats))] + ([out] if out else [])
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=timeout)
    if r.returncode != 0:
        raise RuntimeError("ref_hpsi failed (%d): %s %s" % (r.returncode, r.stdout[-2000:], r.stderr[-2000:]))
    line = [ln for ln in r.stdout.splitlines() if ln.startswith("basis_s=")][-1]
    f = dict(kv.split("=", 1) for kv in line.replace("call_s=", "call_s=|").split(" ") if "=" in kv)
    calls = [float(v) for v in line.split("call_s=")[1].split(" pairs=")[0].split()]
    y = None
    if out:
        y = np.fromfile(out, dtype=np.complex128)
        os.unlink(out)
    return float(f["basis_s"]), calls, int(f["pairs"]), y
