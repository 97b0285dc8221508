"""Driver of the reference Quanty binary (oracle/_ref/Quanty, built from the reference's
unmodified sources by ``oracle/build_ref.sh <ref> quanty``) for timing a whole calculation on
the host cores.  TEST AND MEASUREMENT INFRASTRUCTURE ONLY: bench.py runs it beside the GPU path;
nothing in the product links or runs it.

The calculation is the 26-orbital ligand-field XAS: the operators of
tests/golden/gen/c1_lf.lua (the script the fixtures come from, read here up to its operator
dump), then per repetition Eigensystem for the lowest 3 states (LuaEigensystem,
LuaInterface/ssp.cpp:4039) and CreateSpectra of the three dipole operators on them
(LuaCreateSpectra, ssp.cpp:1906; Lanczos, 200 steps, 2049 frequencies).  The script prints a
marker, flushed, before and after each call; the wall clock between markers is read here, so
the figures hold the calls alone (no process start, no operator construction).  The last
repetition's spectra are written with Spectra.Print for a parity check."""
import os
import shutil
import subprocess
import tempfile
import threading
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
BINARY = os.path.join(HERE, "_ref", "Quanty")
GEN = os.path.join(ROOT, "tests", "golden", "gen")

LF_CALL = {"eigensystem": 'psiList = Eigensystem(H, R, 3)',
           "spectra": 'S = CreateSpectra(HX, {Tx, Ty, Tz}, psiList, {{"Emin", -10}, {"Emax", 20}, {"NE", 2048}, '
                      '{"Gamma", 0.5}, {"NTri", 200}, {"Method", "Lanczos"}, {"Epsilon", 0}})'}


def available():
    return os.access(BINARY, os.X_OK)


def lf_script(reps):
    """The timing script: c1_lf.lua's operator construction, then `reps` repetitions of the
    Eigensystem and CreateSpectra calls between flushed markers."""
    head = []
    for ln in open(os.path.join(GEN, "c1_lf.lua")).read().splitlines():
        if ln.startswith("for _, n in ipairs"):  # the operator dump: the construction ends here
            break
        head.append(ln)
    body = ['R = {NF, 0, {"111111 0000000000 0000000000", 6, 6}, {"000000 1111111111 1111111111", 18, 18}}',
            'function mark(s) print("QTMARK " .. s); io.stdout:flush() end',
            'mark("start")',
            "for rep = 1, %d do" % reps,
            "  " + LF_CALL["eigensystem"],
            '  mark("E" .. rep)',
            "  " + LF_CALL["spectra"],
            '  mark("S" .. rep)',
            "end",
            'S.Print({{"file", "spectra.dat"}})',
            'E = {}',
            'for i = 1, 3 do E[i] = Complex.Re(psiList[i] * H * psiList[i]) end',
            'print(string.format("QTENERGY %.17g %.17g %.17g", E[1], E[2], E[3]))']
    return "\n".join(head + body) + "\n"


def time_lf(reps=3, threads=None, timeout=900):
    """Runs the calculation `reps` times under the reference binary with `threads` OpenMP
    threads (all host cores by default).  Returns {"threads", "eigensystem_s": [...],
    "spectra_s": [...], "energies": [3], "spectra_text": Spectra.Print of the last repetition}."""
    threads = int(threads or os.cpu_count() or 1)
    work = tempfile.mkdtemp(prefix="qref_lf_")
    try:
        return _run_lf(work, reps, threads, timeout)
    finally:
        shutil.rmtree(work, ignore_errors=True)


def _run_lf(work, reps, threads, timeout):
    with open(os.path.join(GEN, "common.lua")) as f, open(os.path.join(work, "common.lua"), "w") as g:
        g.write(f.read())
    with open(os.path.join(work, "lf_time.lua"), "w") as f:
        f.write(lf_script(reps))
    env = dict(os.environ, OMP_NUM_THREADS=str(threads))
    p = subprocess.Popen([BINARY, "lf_time.lua"], cwd=work, env=env, stdout=subprocess.PIPE,
                         stderr=subprocess.STDOUT, text=True)
    marks, energies, tail = {}, None, []
    watchdog = threading.Timer(timeout, p.kill)  # a run that stops printing still ends
    watchdog.start()
    try:
        for ln in p.stdout:
            now = time.perf_counter()
            s = ln.split()
            if len(s) == 2 and s[0] == "QTMARK":
                marks[s[1]] = now
            elif s and s[0] == "QTENERGY":
                energies = [float(v) for v in s[1:4]]
            else:
                tail = (tail + [ln])[-20:]
        rc = p.wait()
    finally:
        watchdog.cancel()
    if rc != 0 or energies is None or any(("E%d" % r) not in marks or ("S%d" % r) not in marks
                                          for r in range(1, reps + 1)):
        raise RuntimeError("reference run failed (%s): %s" % (rc, "".join(tail)[-600:]))
    prev = marks["start"]
    eig, spec = [], []
    for r in range(1, reps + 1):
        eig.append(marks["E%d" % r] - prev)
        spec.append(marks["S%d" % r] - marks["E%d" % r])
        prev = marks["S%d" % r]
    with open(os.path.join(work, "spectra.dat")) as f:
        text = f.read()
    return {"threads": threads, "eigensystem_s": eig, "spectra_s": spec, "energies": energies,
            "spectra_text": text}
