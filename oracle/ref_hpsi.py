"""Driver of oracle/_ref/ref_hpsi (TEST AND MEASUREMENT INFRASTRUCTURE ONLY): the reference's
own fixed-basis H*psi (OperatorPsiConserveBasisPreAllocated, Core/OperatorWaveFunction.cpp:5541)
compiled from its unmodified sources by ``oracle/build_ref.sh <ref> hpsi``, fed a basis, an
operator and amplitudes through a file.  Used by tests/ to pin the oracle and the GPU path to
the reference itself, and by bench.py's reference arm."""
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BINARY = os.path.join(HERE, "_ref", "ref_hpsi")


def available():
    return os.path.exists(BINARY)


def write_input(path, nf, terms, dets, x):
    """terms: [(ladder codes, complex value)]; dets: (n, nword) uint8 in basis order; x: the
    n complex amplitudes."""
    dets = np.ascontiguousarray(dets, dtype=np.uint8)
    x = np.ascontiguousarray(x, dtype=np.complex128)
    with open(path, "wb") as f:
        np.array([nf, len(terms)], dtype=np.int32).tofile(f)
        np.array([len(dets)], dtype=np.int64).tofile(f)
        np.array([len(t[0]) for t in terms], dtype=np.int32).tofile(f)
        np.array([o for t in terms for o in t[0]], dtype=np.uint16).tofile(f)
        np.array([complex(t[1]).real for t in terms], dtype=np.float64).tofile(f)
        np.array([complex(t[1]).imag for t in terms], dtype=np.float64).tofile(f)
        dets.tofile(f)
        x.view(np.float64).tofile(f)


def run(path, runs, want_y=False, timeout=3600):
    """Runs the reference's H*psi on the basis of the input file.  runs: [(threads, spec,
    calls)] with spec "s<stride>" (sources every stride-th row) or "t<seconds>" (a stride
    picked for about that many seconds per call).  Returns ([{threads, stride, sources, pairs,
    basis_s, calls}], y): y is the first run's result on the whole basis when want_y."""
    out = tempfile.mktemp(prefix="ref_hpsi_y_") if want_y else None
    arg = ",".join("%d:%s:%d" % (int(t), sp, int(c)) for t, sp, c in runs)
    r = subprocess.run([BINARY, path, arg] + ([out] if out else []), capture_output=True, text=True, timeout=timeout)
    if r.returncode != 0:
        raise RuntimeError("ref_hpsi failed (%d): %s %s" % (r.returncode, r.stdout[-2000:], r.stderr[-2000:]))
    res = []
    for ln in r.stdout.splitlines():
        if not ln.startswith("threads="):
            continue
        head, calls = ln.split(" call_s=")
        d = dict(kv.split("=") for kv in head.split())
        res.append({"threads": int(d["threads"]), "stride": int(d["stride"]), "sources": int(d["sources"]),
                    "pairs": int(d["pairs"]), "basis_s": float(d["basis_s"]),
                    "calls": [float(v) for v in calls.split()]})
    y = None
    if out:
        y = np.fromfile(out, dtype=np.complex128)
        os.unlink(out)
    return res, y
