"""Serving form: a request loop for CreateSpectra / Eigensystem jobs.

Jobs of mixed Hilbert-space sizes arrive over time.  The server keeps ``slots`` workers, each
with its own context and CUDA stream (``api.Engine``) and its own host thread, so the kernels
of different jobs overlap on the device.  A job is admitted when a slot is free and its
estimated device footprint fits into the HBM budget next to the jobs already running; it
keeps its Krylov state on the device until it finishes.  Continuous batching: when a slot
takes a CreateSpectra job, the waiting CreateSpectra jobs on the same Hamiltonian with the same
Lanczos settings (``api.lanczos_merge_key``) join it, and all their (T, psi) pairs run as one
multi-vector Lanczos (``api.CreateSpectraMerged``); each job still gets its own window and
frequencies.  Results in the mix equal results alone (to rounding for merged jobs).

    srv = Server(slots=4, hbm_budget=200e9)
    fut = srv.submit(SpectraJob(H, [T], [psi], {"NTri": 200, "NE": 2048, ...}))
    result = fut.result()
    srv.close()
"""
import threading
import time
from collections import deque
from concurrent.futures import Future

import numpy as np

from . import api


def _footprint(n_det, nvec, ntri=0, krylov=False):
    """Device bytes a job holds at its peak (basis, lookup table, connection lists with up to
    12 hashed connections per row, Lanczos state)."""
    keys = 16 * n_det
    table = 32 * 2 * n_det + 8 * 2 * n_det
    lists = 8 * n_det + 8 * 12 * n_det
    vectors = 16 * n_det * nvec * 7
    kry = 16 * n_det * ntri if krylov else 0
    return int(keys + table + lists + vectors + kry + (64 << 20))


def _final_basis_size(H, Ts, psis, options):
    """Determinants of CreateSpectra's final-state basis: the closure under H (within the
    Restrictions option) of the targets of every T on every initial state."""
    R = api.parse_restrictions((options or {}).get("Restrictions"))
    eng = api.engine()
    dets = np.concatenate([p.det for p in psis])
    b0, _ = api.Basis.from_bytes(H.nf, dets, eng)
    bt = None
    for t in Ts:
        tb = api.OperatorPsiBasis(t, b0, R, eng)
        bt = tb if bt is None else api.basis_union(bt, tb, eng)
    return max(int(api.closure_of(H, bt, R, -1, eng).n), 1)


class SpectraJob:
    """CreateSpectra(H, T, psi, options) (LuaInterface/ssp.cpp:1906)."""

    def __init__(self, H, T, psi, options=None, n_det_hint=None, batched=True):
        self.H, self.T, self.psi, self.options, self.batched = H, T, psi, options or {}, batched
        self.n_det_hint = n_det_hint
        self.nspec = len(T) * len(psi)

    def footprint(self):
        # without a hint the final basis is measured: the closure under H of the targets of
        # every T (what CreateSpectra builds), so admission never counts on a guessed size
        if self.n_det_hint is None:
            self.n_det_hint = _final_basis_size(self.H, self.T, self.psi, self.options)
        return _footprint(self.n_det_hint, self.nspec)

    def merge_key(self):
        return api.lanczos_merge_key(self.H, self.T, self.psi, self.options, self.batched)

    def run(self, eng):
        S, tri = api.CreateSpectra(self.H, self.T, self.psi, self.options, eng=eng, batched=self.batched)
        return _spectra_result(S, tri)


def _spectra_result(S, tri):
    return {"G": S.G, "tri": tri, "Emin": S.Emin, "Emax": S.Emax, "Gamma": S.Gamma}


def run_merged(jobs, eng):
    """SpectraJobs with equal merge keys as one CreateSpectraMerged call; one result each."""
    got = api.CreateSpectraMerged(jobs[0].H, [(j.T, j.psi, j.options) for j in jobs], eng)
    return [_spectra_result(S, tri) for S, tri in got]


class EigenJob:
    """Eigensystem(H, restrictions, Npsi, options) (LuaInterface/ssp.cpp:4039)."""

    def __init__(self, H, restrictions, npsi, options=None, n_det_hint=None, seed_dets=None):
        self.H, self.R, self.npsi, self.options = H, restrictions, npsi, options or {}
        self.n_det_hint = n_det_hint
        self.seed_dets = seed_dets  # basis = closure of these determinants (overlapping masks)
        self.nspec = 0

    def footprint(self):
        n = self.n_det_hint or 10000
        return _footprint(n, self.npsi, ntri=max(8 * self.npsi, 128), krylov=True)

    def run(self, eng):
        if self.seed_dets is None:
            psis, E = api.Eigensystem(self.H, self.R, self.npsi, self.options, eng=eng)
            return {"energies": E, "psi": psis}
        basis = api.closure(self.H, self.seed_dets, self.H.nf, self.R, -1, eng)
        x, E = api.EigensystemOnBasis(self.H, basis, self.npsi, self.options, eng)
        return {"energies": E, "n": basis.n}


class Server:
    """Continuous batching over a fixed set of device slots with HBM-budget admission."""

    def __init__(self, slots=4, hbm_budget=None, device=0, policy="fifo", merge=True, max_merge=16, paused=False):
        import torch
        self.torch = torch
        if policy not in ("fifo", "sjf"):
            raise ValueError("policy is 'fifo' or 'sjf'")
        self.policy = policy
        self.merge, self.max_merge = bool(merge), int(max_merge)
        self.paused = bool(paused)  # workers admit nothing until resume()
        if hbm_budget is None:
            free, total = torch.cuda.mem_get_info(device)
            hbm_budget = int(0.8 * free)
        self.budget = int(hbm_budget)
        self.in_use = 0
        self.queue = deque()
        self.cv = threading.Condition()
        self.closed = False
        prev = torch.cuda.current_stream(device)
        # device clock origin: every job's start and end are also recorded as CUDA events on its
        # slot's stream and measured from this event, so overlap is checked on the device
        self.t_ref = torch.cuda.Event(enable_timing=True)
        self.t_ref.record(prev)
        self.t_ref.synchronize()
        self.engines = [api.Engine(device) for _ in range(slots)]
        torch.cuda.set_stream(prev)  # the engines' streams are used only by their workers
        self.records = []
        self.threads = [threading.Thread(target=self._worker, args=(e,), daemon=True) for e in self.engines]
        for t in self.threads:
            t.start()

    def submit(self, job, arrival=None):
        fut = Future()
        rec = {"arrival": arrival if arrival is not None else time.perf_counter(), "job": job, "future": fut}
        with self.cv:
            self.queue.append(rec)
            self.cv.notify_all()
        return fut

    def _admit(self):
        """fifo: the oldest job, when its footprint fits.  sjf: the waiting job with the smallest
        footprint (the oldest among equals), when it fits.  A job larger than the whole budget
        runs alone."""
        if not self.queue:
            return None
        if getattr(self, "policy", "fifo") == "sjf":
            i = min(range(len(self.queue)), key=lambda k: (self.queue[k]["job"].footprint(), k))
        else:
            i = 0  # first-come first-served: do not overtake a waiting job
        rec = self.queue[i]
        need = rec["job"].footprint()
        if self.in_use + need <= self.budget or (self.in_use == 0 and need > self.budget):
            del self.queue[i]
            group = [rec]
            merge = getattr(self, "merge", True) and isinstance(rec["job"], SpectraJob)
            key = rec["job"].merge_key() if merge else None
            if key is not None:  # waiting jobs that can share this one's Lanczos run join it
                for other in list(self.queue):
                    if len(group) >= getattr(self, "max_merge", 16):
                        break
                    oj = other["job"]
                    if isinstance(oj, SpectraJob) and oj.merge_key() == key:
                        extra = oj.footprint()
                        if self.in_use + need + extra > self.budget:
                            break
                        self.queue.remove(other)
                        need += extra
                        group.append(other)
            self.in_use += need
            rec["need"] = need
            rec["group"] = group
            return rec
        return None

    def resume(self):
        with self.cv:
            self.paused = False
            self.cv.notify_all()

    def _worker(self, eng):
        self.torch.cuda.set_stream(eng.stream)
        while True:
            with self.cv:
                rec = None
                while not self.closed:
                    rec = None if self.paused else self._admit()
                    if rec is not None:
                        break
                    self.cv.wait(0.05)
                if rec is None:
                    return
            group = rec["group"]
            t_start = time.perf_counter()
            ev0 = self.torch.cuda.Event(enable_timing=True)
            ev1 = self.torch.cuda.Event(enable_timing=True)
            ev0.record(eng.stream)
            try:
                if len(group) > 1:
                    outs = run_merged([g["job"] for g in group], eng)
                else:
                    outs = [rec["job"].run(eng)]
                ev1.record(eng.stream)
                ev1.synchronize()
                t_end = time.perf_counter()
                for g, out in zip(group, outs):
                    g["start"], g["end"], g["merged"] = t_start, t_end, len(group)
                    # the job's window on the device: its stream reached the first event before
                    # its first kernel and the second after its last
                    g["dev_start"] = self.t_ref.elapsed_time(ev0) * 1e-3
                    g["dev_end"] = self.t_ref.elapsed_time(ev1) * 1e-3
                    g["future"].set_result(out)
            except Exception as exc:  # reported through the futures
                t_end = time.perf_counter()
                for g in group:
                    g["start"], g["end"], g["merged"] = t_start, t_end, len(group)
                    g["future"].set_exception(exc)
            with self.cv:
                self.in_use -= rec["need"]
                self.records.extend(group)
                self.cv.notify_all()

    def close(self):
        with self.cv:
            self.closed = True
            self.cv.notify_all()
        for t in self.threads:
            t.join()
        for e in self.engines:
            e.close()

    def latencies(self):
        return np.array([r["end"] - r["arrival"] for r in self.records])


def run_stream(jobs, rate, slots=4, hbm_budget=None, seed=0, server=None, policy="fifo", stats=None):
    """Submit jobs at Poisson arrival times (mean `rate` per second); wait for all.
    Returns (results in submission order, latencies, wall seconds); `stats` (a dict), when
    given, receives how many jobs ran merged with others."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, len(jobs))
    srv = server or Server(slots=slots, hbm_budget=hbm_budget, policy=policy)
    t0 = time.perf_counter()
    futs = []
    for gap, job in zip(gaps, jobs):
        target = time.perf_counter() + gap
        while time.perf_counter() < target:
            time.sleep(min(0.001, max(0.0, target - time.perf_counter())))
        futs.append(srv.submit(job, arrival=time.perf_counter()))
    results = [f.result() for f in futs]
    wall = time.perf_counter() - t0
    lat = np.array([r["end"] - r["arrival"] for r in sorted(srv.records, key=lambda r: r["arrival"])])
    if stats is not None:
        stats["merged_jobs"] = sum(1 for r in srv.records if r.get("merged", 1) > 1)
    if server is None:
        srv.close()
    return results, lat, wall


def run_plain(jobs, rate, seed=0, eng=None):
    """The same stream served one job at a time on one context with one Lanczos per spectrum
    (the plain GPU path).  Returns (results, latencies, wall seconds)."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, len(jobs))
    arrivals = np.cumsum(gaps)
    eng = eng or api.engine()
    t0 = time.perf_counter()
    results, lat = [], []
    for a, job in zip(arrivals, jobs):
        now = time.perf_counter() - t0
        if now < a:
            time.sleep(a - now)
        if isinstance(job, SpectraJob):
            plain = SpectraJob(job.H, job.T, job.psi, job.options, job.n_det_hint, batched=False)
            results.append(plain.run(eng))
        else:
            results.append(job.run(eng))
        eng.torch.cuda.current_stream().synchronize()
        lat.append(time.perf_counter() - t0 - a)
    return results, np.array(lat), time.perf_counter() - t0
