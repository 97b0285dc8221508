"""Benchmark: fixed-basis H*psi on the large discretised-bath Anderson impurity.

Workload (the largest single-GPU configuration of the reference's benchmark set): 86
spin-orbitals (2p + 3d + 7 bath shells of 10), 47,481,880 determinants in 128-bit words,
complex FP64 amplitudes; see quanty_gb300/workloads.py.  One step = one H*psi over the whole
basis (OperatorPsiConserveBasisPreAllocated semantics).  Metric: determinant x term
applications per second (N_det * N_terms / t), the work unit the reference's loop evaluates.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the reference's own fixed-basis H*psi on the host cores: its unmodified
sources (staged in baseline/_ref) built by oracle/build_ref.sh into oracle/_ref/ref_hpsi, under
OpenMP with all host threads, on a bounded sample of source rows of the same basis each step;
the oracle's C restatement stands in only when that build fails.  The default line also carries
`secondary` entries: the ligand-field XAS batched against plain, the whole ligand-field
calculation against the reference binary, the batched impurity XAS and two served streams
(bench_forms.py).  With N > 1 every rank runs an independent replica (the path does not
shard); rank 0 prints the line.
"""
import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--shells", type=int, default=7)
    p.add_argument("--hole-max", type=int, default=3)
    p.add_argument("--particle-max", type=int, default=2)
    p.add_argument("--cpu-seconds", type=float, default=15.0)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-secondary", action="store_true")
    p.add_argument("--mode", default="hpsi", choices=["hpsi", "batched", "served", "layouts", "chains", "eigh"])
    p.add_argument("--k", type=int, default=190, help="eigh mode: order of the matrix")
    p.add_argument("--layout", type=int, default=None)
    p.add_argument("--jobs", type=int, default=24)
    p.add_argument("--states", type=int, default=16)
    p.add_argument("--ntri", type=int, default=200)
    p.add_argument("--no-rixs", action="store_true")
    p.add_argument("--max-det", type=float, default=2e6)
    p.add_argument("--rate", type=float, default=50.0)
    p.add_argument("--slots", type=int, default=4)
    p.add_argument("--restarts", type=int, default=20)
    p.add_argument("--policy", default="sjf", choices=["fifo", "sjf"])
    p.add_argument("--materials", type=int, default=0,
                   help="served mode: jobs share this many Hamiltonians (0: every job its own)")
    return p.parse_args()


class Clocks:
    """nvidia-smi sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def probe_fp64_peak(eng):
    """The device's FP64 issue ceiling in G lane-operations/s (bench_probe.cu, built beside this
    file by __graft_entry__.build(); independent FMA chains on every lane of 8 blocks per SM)."""
    lib = os.path.join(ROOT, "bench_probe.so")
    if not os.path.exists(lib):
        import __graft_entry__
        __graft_entry__.build()
    L = C.CDLL(lib)
    L.bench_fp64_peak.argtypes = [C.c_void_p, C.c_void_p]
    out = C.c_double(0.0)
    if L.bench_fp64_peak(eng.L.qg_get_stream(eng.ctx), C.byref(out)) != 0:
        raise RuntimeError("bench_fp64_peak failed")
    return out.value


def profiled_traffic(workload):
    """DRAM bytes (read + write) per launch of the H*psi kernel on this workload, from one ncu
    capture recorded in profiles/traffic.json (None when none was recorded)."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(p) as f:
            return float(json.load(f)[workload]["dram_bytes_per_launch"])
    except Exception:
        return None


def build_workload(api, args):
    from quanty_gb300 import workloads
    H, R, seed, info = workloads.anderson_impurity(nshell=args.shells, hole_max=args.hole_max,
                                                   particle_max=args.particle_max)
    eng = api.engine()
    t0 = time.perf_counter()
    basis = api.closure(H, api.dets_to_bytes([seed], H.nf), H.nf, R, -1, eng)
    eng.stream.synchronize()
    info["closure_s"] = time.perf_counter() - t0
    return H, R, basis, info


def timed_sample(O, op, wf_handle, n, seconds):
    """Time the oracle's push-form H*psi over a spread sample of source rows (every stride-th
    row of the basis, the full basis as lookup target), grown until one pass takes at least
    half of `seconds` (or covers the basis)."""
    L = O.lib()
    y = np.zeros(2 * n)
    target = min(n, 2000)
    while True:
        stride = max(1, n // target)
        rows = (n + stride - 1) // stride
        t0 = time.perf_counter()
        L.qo_apply_conserve_strided(*op.args(), wf_handle, 0, n, stride, O._p(y))
        dt = time.perf_counter() - t0
        if dt >= 0.5 * seconds or rows >= n:
            return rows, stride, dt
        target = int(min(n, max(2 * rows, rows * seconds / max(dt, 1e-6))))


PARITY_STRIDE = 32


def cpu_baseline(api, H, basis, seconds, eng):
    """The CPU side of the default bench line, on the GPU machine's host cores.

    Timing: the reference's own fixed-basis H*psi (oracle/_ref/ref_hpsi, when it has been built
    from the staged reference sources) on a spread sample of source rows with the whole basis as
    the lookup target, on all host threads and on one; beside it, as a calibration, the
    oracle's restatement of the same loop (OpenMP, all host threads) on a sample sized for about
    `seconds`.  Without the reference program the oracle's figure is the baseline ("port").

    Parity of the timed GPU call at this configuration: x zero except on every
    PARITY_STRIDE-th row, the device apply against the oracle's push from those rows and, with
    the reference program, against the reference's own result; all rows compared (amplitudes
    to 1e-12 relative, the set of rows reached exactly), and the connection count of the
    sampled rows.  Returns (baseline, parity)."""
    import torch
    from oracle import oracle as O
    from oracle import ref_hpsi
    O.build()
    dets = basis.dets_bytes()
    n = len(dets)
    rng = np.random.default_rng(0)
    x = rng.normal(size=n) + 1j * rng.normal(size=n)
    op = O.Op({"nf": H.nf, "terms": [[list(t[0]), t[1].real, t[1].imag] for t in H.terms]})
    h = O.WF(H.nf, dets, x).handle()
    try:
        rows, stride, dt = timed_sample(O, op, h, n, seconds)
        port = {"value": rows * op.nterms / dt / 1e9, "unit": "Gdet·terms/s", "cores": O.num_threads(),
                "kind": "port",
                "sample": "every %d-th of %d source determinants (%d rows), full basis as lookup target, %d terms, "
                          "%.1f s" % (stride, n, rows, op.nterms, dt)}
        xm = np.zeros(n, dtype=np.complex128)
        xm[::PARITY_STRIDE] = x[::PARITY_STRIDE]
        xd = torch.from_numpy(xm.reshape(n, 1)).cuda()
        yd = eng.empty(n)
        eng.check(eng.L.qg_apply(eng.ctx, H.handle(), basis.h, basis.h, api._ptr(xd), api._ptr(yd), 1))
        y = eng.to_host(yd[:, 0])
        del xd, yd
        cnt = C.c_int64(0)
        eng.check(eng.L.qg_count_nnz_rows(eng.ctx, H.handle(), basis.h, 0, PARITY_STRIDE, 0, C.byref(cnt)))
        want = O.apply_sampled(op, h, n, PARITY_STRIDE)
        cnt_o = O.count_nnz_sampled(op, h, n, PARITY_STRIDE)
    finally:
        O.lib().qo_wf_free(h)
    max_rel = float(np.max(np.abs(y - want)) / np.max(np.abs(want)))
    reached = bool(np.array_equal(y != 0, want != 0))
    parity = {"rows": int((n + PARITY_STRIDE - 1) // PARITY_STRIDE), "stride": PARITY_STRIDE, "outputs_compared": n,
              "max_rel": max_rel, "tolerance": 1e-12, "rows_reached_equal": reached,
              "nnz_sample": int(cnt.value), "nnz_sample_oracle": int(cnt_o),
              "ok": bool(max_rel < 1e-12 and reached and cnt.value == cnt_o),
              "checker": "oracle push-form H*psi from the sampled source rows (OpenMP C restatement)"}
    del want
    base = dict(port)
    if ref_hpsi.available():
        threads = os.cpu_count() or 1
        res, yref, why = reference_runs(H, dets, x, [(threads, "s%d" % PARITY_STRIDE, 1), (threads, "t%g" % seconds, 2),
                                                     (1, "t%g" % min(seconds, 10.0), 1)], want_y=True)
        if res:
            r1, r2 = res[1], res[2]
            base = {"value": r1["pairs"] / min(r1["calls"]) / 1e9, "unit": "Gdet·terms/s", "cores": threads,
                    "kind": "reference",
                    "sample": "reference OperatorPsiConserveBasisPreAllocated from every %d-th of %d source "
                              "determinants (%d rows, %d terms) into the whole basis" % (r1["stride"], n, r1["sources"],
                                                                                         op.nterms),
                    "one_thread_value": r2["pairs"] / r2["calls"][0] / 1e9, "port": port}
            base["port_over_reference"] = port["value"] / base["value"]
            rel = float(np.max(np.abs(y - yref)) / np.max(np.abs(yref)))
            same = bool(np.array_equal(y != 0, yref != 0))
            parity["reference"] = {"max_rel": rel, "rows_reached_equal": same, "ok": bool(rel < 1e-12 and same),
                                   "checker": "the reference's own OperatorPsiConserveBasisPreAllocated (unmodified "
                                              "sources) from the same sampled rows"}
            parity["ok"] = parity["ok"] and parity["reference"]["ok"]
        else:
            base["reference_unavailable"] = why
    return base, parity


def xas_spectra_rate(api):
    """Spectra/s of the 26-orbital ligand-field XAS (3 states x 3 polarisations, 200 Lanczos
    steps, 2049 frequencies), batched (one 9-vector Lanczos) and plain (one per spectrum)."""
    from quanty_gb300 import workloads
    ops, R = workloads.ligand_field()
    eng = api.engine()
    psis, E = api.Eigensystem(ops["H"], [26, 0] + [list(r) for r in R], 3, {"Zero": 1e-12}, eng=eng)
    o = {"Emin": -10, "Emax": 20, "NE": 2048, "Gamma": 0.5, "NTri": 200, "Epsilon": 0.0, "Method": "Lanczos"}
    Ts = [ops["Tx"], ops["Ty"], ops["Tz"]]
    out = {}
    for mode in (True, False):
        api.CreateSpectra(ops["HX"], Ts, psis, o, eng=eng, batched=mode)  # warm
        eng.stream.synchronize()
        t0 = time.perf_counter()
        reps = 3
        for _ in range(reps):
            S, _ = api.CreateSpectra(ops["HX"], Ts, psis, o, eng=eng, batched=mode)
        eng.stream.synchronize()
        dt = (time.perf_counter() - t0) / reps
        out["batched" if mode else "plain"] = 9 / dt
    return {"workload": "ligand_field_26so_xas_3x3_ntri200_ne2048", "unit": "spectra/s",
            "batched": out["batched"], "plain": out["plain"], "speedup": out["batched"] / out["plain"]}


def lf_calc_vs_reference(api, reps=3):
    """The whole 26-orbital ligand-field XAS calculation -- Eigensystem for the lowest 3 states,
    then CreateSpectra of the three dipole operators on them (Lanczos, 200 steps, 2049
    frequencies) -- through this library on the GPU (plain: one Lanczos per spectrum; batched:
    one multi-vector Lanczos), and through the reference binary on the host cores with all
    threads and with one.  Seconds per calculation; the reference's figures are its calls alone
    (between markers its script prints).  Parity: the ground energies and the spectra summed
    over the three states (the states span a degenerate manifold, so single spectra depend on
    the basis chosen within it and only their sum is fixed) against the reference's."""
    from quanty_gb300 import workloads
    ops, R = workloads.ligand_field()
    eng = api.engine()
    Rr = [26, 0] + [list(r) for r in R]
    o = {"Emin": -10, "Emax": 20, "NE": 2048, "Gamma": 0.5, "NTri": 200, "Epsilon": 0.0, "Method": "Lanczos"}
    Ts = [ops["Tx"], ops["Ty"], ops["Tz"]]

    def calc(batched):
        eng.stream.synchronize()
        t0 = time.perf_counter()
        psis, E = api.Eigensystem(ops["H"], Rr, 3, eng=eng)
        eng.stream.synchronize()
        t1 = time.perf_counter()
        S, _ = api.CreateSpectra(ops["HX"], Ts, psis, o, eng=eng, batched=batched)
        eng.stream.synchronize()
        return t1 - t0, time.perf_counter() - t1, np.asarray(E, dtype=float), S

    out = {"workload": "ligand_field_26so_eigensystem3_xas3pol_ntri200_ne2048", "unit": "s per calculation"}
    gpu_S = None
    for batched in (False, True):
        calc(batched)  # warm
        runs = [calc(batched) for _ in range(reps)]
        e_s, s_s = float(np.median([r[0] for r in runs])), float(np.median([r[1] for r in runs]))
        out["gpu_batched" if batched else "gpu_plain"] = {"eigensystem_s": e_s, "spectra_s": s_s,
                                                          "total_s": e_s + s_s}
        if not batched:
            gpu_E, gpu_S = runs[-1][2], runs[-1][3]
    ref, why = reference_quanty()
    if ref is None:
        out["reference"] = {"unavailable": why}
        return out
    from quanty_gb300.api import Spectra
    e_best = s_best = ref_S = None
    for threads in dict.fromkeys((os.cpu_count() or 1, 1)):
        r = ref.time_lf(reps=reps, threads=threads)
        e_s, s_s = float(np.median(r["eigensystem_s"])), float(np.median(r["spectra_s"]))
        out["reference_%dt" % threads] = {"eigensystem_s": e_s, "spectra_s": s_s, "total_s": e_s + s_s,
                                          "threads": threads}
        e_best = e_s if e_best is None else min(e_best, e_s)
        s_best = s_s if s_best is None else min(s_best, s_s)
        if ref_S is None:
            ref_S = Spectra.from_text(r["spectra_text"])
            ref_E = np.sort(np.asarray(r["energies"]))
    # the reference's faster thread count for each call (its Eigensystem on this small basis is
    # faster on one thread, its CreateSpectra on all)
    best = e_best + s_best
    out["reference_best_s"] = best
    out["reference_kind"] = "the reference binary (unmodified sources) running the calculation as a Lua script"
    out["speedup_plain_vs_reference"] = best / out["gpu_plain"]["total_s"]
    out["speedup_batched_vs_reference"] = best / out["gpu_batched"]["total_s"]
    g = np.asarray(gpu_S.G).reshape(3, 3, -1).sum(axis=1)
    rg = np.asarray(ref_S.G).reshape(3, 3, -1).sum(axis=1)
    out["parity"] = {"energy_max_abs_eV": float(np.max(np.abs(np.sort(gpu_E) - ref_E))),
                     "state_summed_spectra_max_rel": float(np.max(np.abs(g - rg)) / np.max(np.abs(rg))),
                     "window_equal": bool(abs(gpu_S.Emin - ref_S.Emin) < 1e-10 and abs(gpu_S.Emax - ref_S.Emax) < 1e-10)}
    return out


def reference_quanty():
    """The reference binary (oracle/_ref/Quanty), built from the reference sources staged in
    baseline/_ref when it is missing.  Returns (module, None) or (None, why)."""
    from oracle import ref_quanty
    if ref_quanty.available():
        return ref_quanty, None
    src = os.path.join(ROOT, "baseline", "_ref")
    if not os.path.isfile(os.path.join(src, "LuaInterface", "main.cpp")):
        return None, "reference sources not staged in baseline/_ref"
    r = subprocess.run([os.path.join(ROOT, "oracle", "build_ref.sh"), src, "quanty"], capture_output=True, text=True)
    if r.returncode != 0 or not ref_quanty.available():
        return None, "reference build failed: " + (r.stderr or r.stdout)[-300:].replace("\n", " ")
    return ref_quanty, None


def reference_program():
    """The reference's own fixed-basis H*psi program (oracle/_ref/ref_hpsi), built from the
    reference sources staged in baseline/_ref when it is missing.  Returns (module, None) or
    (None, why it is unavailable)."""
    from oracle import ref_hpsi
    if ref_hpsi.available():
        return ref_hpsi, None
    src = os.path.join(ROOT, "baseline", "_ref")
    if not os.path.isfile(os.path.join(src, "LuaInterface", "main.cpp")):
        return None, "reference sources not staged in baseline/_ref"
    # the reference binary (the whole-calculation comparison) builds beside it, in parallel
    from oracle import ref_quanty
    targets = ["hpsi"] + ([] if ref_quanty.available() else ["quanty"])
    r = subprocess.run([os.path.join(ROOT, "oracle", "build_ref.sh"), src] + targets, capture_output=True, text=True)
    if r.returncode != 0 or not ref_hpsi.available():
        return None, "reference build failed: " + (r.stderr or r.stdout)[-300:].replace("\n", " ")
    return ref_hpsi, None


def reference_runs(H, dets, x, runs, want_y=False):
    """The reference's OperatorPsiConserveBasisPreAllocated with the whole basis as the lookup
    target and sources every stride-th row, for each (threads, spec, calls) of `runs` (spec
    "t<seconds>": a stride for about that many seconds per call; "s<stride>").  Returns
    (harness runs, y or None, None) or (None, None, why it is unavailable)."""
    ref, why = reference_program()
    if ref is None:
        return None, None, why
    import tempfile
    fd, path = tempfile.mkstemp(prefix="ref_hpsi_in_")
    os.close(fd)
    try:
        ref.write_input(path, H.nf, H.terms, dets, x)
        res, y = ref.run(path, runs, want_y=want_y)
        return res, y, None
    except Exception as e:  # reported by the caller
        return None, None, str(e)[-300:]
    finally:
        os.unlink(path)


def run_reference(args):
    """The reference arm: the reference's own fixed-basis H*psi (its unmodified sources, built
    here) on the host cores, on the same basis and operator, each step a spread sample of
    source rows.  Falls back to the oracle's restatement when the reference cannot be built."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    from quanty_gb300 import workloads
    # the basis comes from the same closure rules, enumerated on the host without a GPU
    H, R, seed, info = workloads.anderson_impurity(nshell=args.shells, hole_max=args.hole_max,
                                                   particle_max=args.particle_max)
    dets = workloads.anderson_sector_bytes(info, H.nf, hole_max=args.hole_max, particle_max=args.particle_max)
    n = len(dets)
    rng = np.random.default_rng(0)
    x = rng.normal(size=n) + 1j * rng.normal(size=n)
    threads = os.cpu_count() or 1
    per_step = max(2.0, min(10.0, 40.0 / max(args.steps + args.warmup, 1)))
    runs, _, why = reference_runs(H, dets, x, [(threads, "t%g" % per_step, args.steps + args.warmup),
                                              (1, "t%g" % per_step, 1)])
    workload = "anderson_impurity_%dso_hpsi" % H.nf
    if runs:
        r0 = runs[0]
        times = r0["calls"][args.warmup:] or r0["calls"]
        t = sum(times) / len(times)
        val = r0["pairs"] / t / 1e9
        base = {"value": val, "unit": "Gdet·terms/s", "cores": threads, "kind": "reference",
                "sample": "reference OperatorPsiConserveBasisPreAllocated from every %d-th of %d source determinants "
                          "(%d rows, %d terms) into the whole basis, per step" % (r0["stride"], n, r0["sources"],
                                                                                 len(H.terms)),
                "basis_build_s": r0["basis_s"]}
        if len(runs) > 1:
            r1 = runs[1]
            base["one_thread_value"] = r1["pairs"] / r1["calls"][0] / 1e9
    else:
        # the oracle's restatement of the same loop, when the reference cannot be built here
        from oracle import oracle as O
        O.build()
        op = O.Op({"nf": H.nf, "terms": [[list(t_[0]), t_[1].real, t_[1].imag] for t_ in H.terms]})
        h = O.WF(H.nf, dets, x).handle()
        L = O.lib()
        y = np.zeros(2 * n)
        rows, stride, _ = timed_sample(O, op, h, n, per_step)
        for _ in range(args.warmup):
            L.qo_apply_conserve_strided(*op.args(), h, 0, n, max(stride, n // 1000), O._p(y))
        times = []
        for _ in range(args.steps):
            t0 = time.perf_counter()
            L.qo_apply_conserve_strided(*op.args(), h, 0, n, stride, O._p(y))
            times.append(time.perf_counter() - t0)
        L.qo_wf_free(h)
        t = sum(times) / len(times)
        val = rows * op.nterms / t / 1e9
        base = {"value": val, "unit": "Gdet·terms/s", "cores": O.num_threads(), "kind": "port",
                "sample": "every %d-th of %d source determinants (%d rows) per step" % (stride, n, rows),
                "reference_unavailable": why}
    line = {"impl": "reference", "metric": "H·ψ det·terms/s", "value": val, "unit": "Gdet·terms/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128",
            "data": "synthetic", "config": {"workload": workload, "n_det": n, "n_terms": len(H.terms)},
            "cpu_baseline": base,
            "e2e": {"value": val, "unit": "Gdet·terms/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.mode != "hpsi":
        import bench_forms
        return bench_forms.main(args)
    import torch
    from quanty_gb300 import replicas
    world, rank, local = replicas.init("nccl")
    torch.cuda.set_device(local)
    from quanty_gb300 import build
    build.build()
    from quanty_gb300 import api
    api._engine = api.Engine(local)
    eng = api.engine()
    t_setup = time.perf_counter()
    H, R, basis, info = build_workload(api, args)
    n = basis.n
    t_setup = time.perf_counter() - t_setup
    nterms = H.info()["nterms"]
    nnz = api.count_nnz(H, basis)
    nnz_off = api.count_nnz(H, basis, offdiag=True)
    rng = np.random.default_rng(1)
    x = torch.from_numpy(rng.normal(size=(n, 1)) + 1j * rng.normal(size=(n, 1))).cuda()
    y = eng.empty(n)
    stream = torch.cuda.current_stream()

    def step():
        eng.check(eng.L.qg_apply(eng.ctx, H.handle(), basis.h, basis.h, api._ptr(x), api._ptr(y), 1))

    # the first apply builds the per-(operator, basis) data the later ones reuse (diagonal,
    # local blocks and their classes, connection lists): timed once, for the amortised figure
    torch.cuda.synchronize()
    t_first = time.perf_counter()
    step()
    torch.cuda.synchronize()
    t_first = time.perf_counter() - t_first
    for _ in range(max(args.warmup, 3) - 1):
        step()
    torch.cuda.synchronize()
    # connections the apply gathers through its per-row lists (the rest are local moves at a
    # certain offset in another block of the sorted basis)
    built, nconn = C.c_int32(0), C.c_int64(0)
    eng.check(eng.L.qg_apply_list_info(eng.ctx, H.handle(), basis.h, C.byref(built), C.byref(nconn)))
    clocks = Clocks(local)
    clocks.start()
    replicas.barrier()
    torch.cuda.synchronize()
    l0 = eng.launches()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        step()
    ev1.record(stream)
    torch.cuda.synchronize()
    replicas.barrier()
    ms = ev0.elapsed_time(ev1) / args.steps
    launches = eng.launches() - l0
    # e2e: the host-buffer entry point, pinned host memory, copies inside the timed region
    xh = torch.empty((n, 1), dtype=torch.complex128).pin_memory()
    xh.copy_(x.cpu())
    yh = torch.empty((n, 1), dtype=torch.complex128).pin_memory()
    for _ in range(2):
        eng.check(eng.L.qg_apply_host(eng.ctx, H.handle(), basis.h, basis.h, api._ptr(xh), api._ptr(yh), 1))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        eng.check(eng.L.qg_apply_host(eng.ctx, H.handle(), basis.h, basis.h, api._ptr(xh), api._ptr(yh), 1))
    e2e_s = (time.perf_counter() - t0) / args.steps
    clk = clocks.stop()
    ms, e2e_ms = replicas.max_over_ranks([ms, e2e_s * 1e3], device="cuda")
    if rank != 0:
        return 0
    # CPU baseline after the GPU timing (its threads would compete with the host-buffer copies)
    cpu, parity = {}, None
    if not args.no_cpu_baseline:
        try:
            cpu, parity = cpu_baseline(api, H, basis, args.cpu_seconds, eng)
        except Exception as e:  # reported, never fatal to the GPU number
            cpu = {"value": None, "error": str(e)}
    secondary = {}
    if not args.no_secondary:
        import bench_forms
        for key, fn in (("xas_spectra", lambda: xas_spectra_rate(api)),
                        ("lf_calc_vs_reference", lambda: lf_calc_vs_reference(api)),
                        ("batched_xas_c3", bench_forms.batched_secondary),
                        ("served_c4", bench_forms.served_secondary),
                        ("served_shared_h", lambda: bench_forms.served_secondary(materials=4))):
            try:
                secondary[key] = fn()
            except Exception as e:  # reported, never fatal to the headline number
                secondary[key] = {"error": str(e)}
    value = replicas.aggregate_rate(n * nterms, world, ms * 1e-3) / 1e9
    e2e_val = replicas.aggregate_rate(n * nterms, world, e2e_ms * 1e-3) / 1e9
    # algorithmic bytes of one H*psi, per unit of work: one key, one source
    # amplitude and one result per row, one 16-byte amplitude gather per non-zero connection
    # (no cache reuse credited), the term table once.  The diagonal connection of a row reads
    # the row's own amplitude, already counted once per row, so nnz counts the connections that
    # change the determinant; the literal count with the diagonal pairs is reported beside it.
    W = 16
    term_bytes = nterms * 64
    alg_bytes = n * (W + 16 + 16) + nnz_off * 16 + term_bytes
    peak, peak_kind = measured_peak()
    achieved = alg_bytes / (ms * 1e-3) / 1e9
    workload = "anderson_impurity_%dso_hpsi" % H.nf
    # FP64 ceiling: the exact FP64 operations of the launch (2 per real connection, 4 per
    # complex one, 2-4 for the diagonal) against 2 FP64 lanes per SM per clock at the clock
    # sampled under load
    ops = C.c_int64(0)
    eng.check(eng.L.qg_apply_fp64_ops(eng.ctx, H.handle(), basis.h, C.byref(ops)))
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    mhz = clk.get("sm_mhz") or clk.get("sm_max_mhz") or 2070.0
    fp64_nominal = 2.0 * sms * mhz * 1e6 / 1e9  # G FP64 lane-operations per second
    fp64_peak = probe_fp64_peak(eng)
    fp64_achieved = ops.value / (ms * 1e-3) / 1e9
    hbm_floor_ms = alg_bytes / (peak * 1e9) * 1e3
    fp64_floor_ms = ops.value / (fp64_peak * 1e9) * 1e3
    line = {
        "metric": "H·ψ det·terms/s", "value": value, "unit": "Gdet·terms/s", "n_gpus": world, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "c128", "data": "synthetic",
        "config": {"workload": workload, "n_det": n, "n_terms": nterms, "nnz": nnz,
                   "nnz_offdiag": nnz_off, "connection_lists": bool(built.value), "nnz_listed": nconn.value,
                   "det_words_bits": 128, "l2": "inputs larger than L2 (x, y %d MB each)" % (n * 16 // 2**20),
                   "values": "real (every term of this Hamiltonian is real-valued)" if all(
                       t[1].imag == 0 for t in H.terms) else "complex",
                   "closure_s": round(info["closure_s"], 3), "setup_s": round(t_setup, 2),
                   "parallelism": "replicas" if world > 1 else "single"},
        # what the timed kernel evaluates: one FP64 complex multiply-add per non-zero connection
        # (diagonal included; the (determinant, term) pairs of the headline unit that vanish are
        # never visited), and the per-step time of a 200-step Lanczos that pays the one-off
        # per-(operator, basis) build of the first apply (diagonal, local blocks, connection lists)
        "rates": {"connections_per_s": replicas.aggregate_rate(nnz, world, ms * 1e-3),
                  "offdiag_connections_per_s": replicas.aggregate_rate(nnz_off, world, ms * 1e-3),
                  "first_apply_s": round(t_first, 4),
                  "amortised_ms_per_step_200": (t_first * 1e3 + 199 * ms) / 200},
        "e2e": {"value": e2e_val, "unit": "Gdet·terms/s", "h2d_bytes_per_step": n * 16, "d2h_bytes_per_step": n * 16,
                "ms_per_step": e2e_ms},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": profiled_traffic(workload), "peak_source": peak_kind,
                     "algorithmic_bytes_per_launch": alg_bytes,
                     "fp64": {"ops_per_launch": ops.value, "achieved_gops": fp64_achieved,
                              "peak_gops": fp64_peak, "frac": fp64_achieved / fp64_peak,
                              "peak_source": "measured (independent FMA chains on every lane, bench_probe.cu)",
                              "nominal_gops": fp64_nominal, "frac_of_nominal": fp64_achieved / fp64_nominal,
                              "nominal_source": "2 FP64 lanes per SM per clock x %d SMs x %.0f MHz sampled" % (sms, mhz)},
                     "floors_ms": {"hbm": hbm_floor_ms, "fp64": fp64_floor_ms,
                                   "frac_of_larger": max(hbm_floor_ms, fp64_floor_ms) / ms},
                     "limiter": "fp64" if fp64_floor_ms > hbm_floor_ms else "hbm"},
        "cpu_baseline": cpu or None,
        "parity": parity,
        "clocks": clk,
        "gpu_launches": launches,
        "secondary": secondary or None,
    }
    print(json.dumps(line))
    return 0


if __name__ == "__main__":
    sys.exit(main())
