"""The two added forms of the spectra path, measured beside the H*psi headline.

* ``batched``: a 6-shell discretised-bath impurity (76 spin-orbitals, 2p + 3d + 6 bath shells
  of 10; at most 1 hole in the filled bath shells, at most 2 particles in the empty ones:
  1,701,795 ground-sector determinants).  The 16 lowest states (restarted block Lanczos),
  Boltzmann weights at 300 K, then the XAS of all 16 states x 3 dipole polarisations
  (Tx, Ty, Tz; 2p -> 3d) as ONE 48-vector Lanczos on the common core-excited basis, against
  the plain path (one closure + one single-vector Lanczos per spectrum, as a one-job-at-a-time
  caller runs it), timed on a sample of the 48 spectra.  Then the RIXS of the lowest state:
  64 incident energies over 16 eV (Gamma1 = 0.4 eV) x 3 emission polarisations, all 192
  second-stage recursions in one batched Lanczos.
* ``served``: a Poisson stream of Eigensystem and CreateSpectra jobs on discretised-bath
  impurities with seeded random charge-transfer energy (1-6 eV), hybridisation (0.5-3 eV) and
  1-6 bath shells, sizes log-uniform up to ``--max-det`` determinants, 150-1000 Lanczos steps
  and 1024-4096 frequencies; served by ``serve.Server`` (4 slots, HBM-budget admission,
  3-polarisation batched Lanczos) against ``serve.run_plain`` (one job at a time, one
  Lanczos per spectrum) on the same stream.  p50/p99 latencies and spectra/s for both.

Both print one JSON line.
"""
import json
import math
import time

import numpy as np

KT_300K = 8.617333262e-5 * 300.0  # eV


def _xas_ops(api, workloads, nf):
    at = workloads.atomic()
    return [api.Operator(nf, at[k].terms, name=k) for k in ("Tx", "Ty", "Tz")]


def _sync(eng):
    eng.stream.synchronize()


def _log(msg):
    import sys
    print("[bench] " + msg, file=sys.stderr, flush=True)


def batched(args):
    from quanty_gb300 import api, workloads
    eng = api.engine()
    nshell, hm, pm = 6, 1, 2
    H, R, seed, info = workloads.anderson_impurity(nshell=nshell, hole_max=hm, particle_max=pm)
    _, Rx, _, _ = workloads.anderson_impurity(nshell=nshell, hole_max=hm, particle_max=pm, core_holes=1)
    Ts = _xas_ops(api, workloads, H.nf)
    nstates = int(args.states)
    t0 = time.perf_counter()
    basis = api.closure(H, api.dets_to_bytes([seed], H.nf), H.nf, R, -1, eng)
    est = {}
    # the reference's default Zero; a bounded number of restarts (the spectra timing below
    # does not depend on how far the initial states converged, which is reported)
    X, E = api.EigensystemOnBasis(H, basis, nstates, {"NKrylovMax": 8 * nstates}, eng,
                                  max_restarts=int(args.restarts), status=est)
    _sync(eng)
    t_eigen = time.perf_counter() - t0
    with eng.on_stream():
        HX = eng.empty(basis.n, nstates)
    eng.check(eng.L.qg_apply(eng.ctx, H.handle(eng), basis.h, basis.h, api._ptr(X), api._ptr(HX), nstates))
    with eng.on_stream():
        Et = eng.torch.from_numpy(E).to(X.device)
        res = float((HX - X * Et[None, :]).abs().pow(2).sum(0).max().item())
    del HX
    _log("eigensystem: %d states, %.1f s, converged=%s, max variance %.2e" % (nstates, t_eigen, est["converged"], res))
    w = np.exp(-(E - E.min()) / KT_300K)
    w /= w.sum()
    ntri = int(args.ntri)
    o = {"NTri": ntri, "NE": 2048, "Emin": -20.0, "Emax": 20.0, "Gamma": 0.5, "Restrictions": Rx}
    nspec = len(Ts) * nstates

    def run_batched():
        return api.CreateSpectraResident(H, Ts, basis, X, E, o, eng, batched=True)

    S, A, B = run_batched()  # warm-up: graphs, caches
    _sync(eng)
    reps = max(1, int(args.steps))
    t0 = time.perf_counter()
    for _ in range(reps):
        S, A, B = run_batched()
    _sync(eng)
    t_batched = (time.perf_counter() - t0) / reps
    _log("batched: %d spectra in %.2f s" % (nspec, t_batched))
    xas = np.array([(w[:, None] * S.G[j * nstates:(j + 1) * nstates]).sum(0) for j in range(len(Ts))])

    # plain path on a sample of the pairs: closure + T psi + one Lanczos + CF per spectrum
    sample = [(j, i) for i in range(min(2, nstates)) for j in range(len(Ts))]
    with eng.on_stream():
        cols = [X[:, i:i + 1].contiguous() for i in range(nstates)]
    api.CreateSpectraResident(H, [Ts[0]], basis, cols[0], [E[0]], o, eng, batched=False)  # warm
    _sync(eng)
    t0 = time.perf_counter()
    diff = 0.0
    for j, i in sample:
        Sp, _, _ = api.CreateSpectraResident(H, [Ts[j]], basis, cols[i], [E[i]], o, eng, batched=False)
        g = S.G[j * nstates + i]
        diff = max(diff, float(np.max(np.abs(Sp.G[0] - g)) / np.max(np.abs(g))))
    _sync(eng)
    t_plain = (time.perf_counter() - t0) / len(sample)
    _log("plain: %.2f s per spectrum" % t_plain)

    # the Lanczos stage alone: one 48-vector recursion against single-vector recursions
    eps = float(api.DEFAULTS["Epsilon"])
    bf, Y = _final_vectors(api, H, Ts, basis, X, Rx, eng)
    t_lz_b = _lanczos_seconds(api, H, bf, Y, ntri, eps, eng)
    with eng.on_stream():
        y1 = [Y[:, c:c + 1].contiguous() for c in (0, nstates)]
    t_lz_p = sum(_lanczos_seconds(api, H, bf, y, ntri, eps, eng) for y in y1) / len(y1)
    _log("lanczos only: batched %.2f s, plain %.3f s per vector" % (t_lz_b, t_lz_p))
    n_final = bf.n
    # every vector layout of the multi-vector apply, timed on the 48-vector block
    import ctypes
    ch = ctypes.c_int32()
    eng.check(eng.L.qg_apply_chunk(eng.ctx, H.handle(eng), bf.h, nspec, ctypes.byref(ch)))
    tuned = ch.value
    layouts = {}
    Z = eng.empty(bf.n, nspec)
    torch = eng.torch
    for c in (1, 2, 4, 8, -32, -64):
        eng.check(eng.L.qg_apply_set_chunk(eng.ctx, H.handle(eng), bf.h, nspec, c))
        eng.check(eng.L.qg_apply(eng.ctx, H.handle(eng), bf.h, bf.h, api._ptr(Y), api._ptr(Z), nspec))
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(eng.stream)
        for _ in range(3):
            eng.check(eng.L.qg_apply(eng.ctx, H.handle(eng), bf.h, bf.h, api._ptr(Y), api._ptr(Z), nspec))
        e1.record(eng.stream)
        e1.synchronize()
        layouts[str(c)] = e0.elapsed_time(e1) / 3
    eng.check(eng.L.qg_apply_set_chunk(eng.ctx, H.handle(eng), bf.h, nspec, tuned if tuned else 8))
    z1 = eng.empty(bf.n, 1)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    eng.check(eng.L.qg_apply(eng.ctx, H.handle(eng), bf.h, bf.h, api._ptr(y1[0]), api._ptr(z1), 1))
    e0.record(eng.stream)
    for _ in range(3):
        eng.check(eng.L.qg_apply(eng.ctx, H.handle(eng), bf.h, bf.h, api._ptr(y1[0]), api._ptr(z1), 1))
    e1.record(eng.stream)
    e1.synchronize()
    single_ms = e0.elapsed_time(e1) / 3
    _log("apply ms for 48 vectors by layout %s (autotuned %d); one vector %.3f ms" % (layouts, tuned, single_ms))
    del Y, y1, bf, Z, z1

    rixs = None
    if not args.no_rixs:
        psi0 = api.Wavefunction(H.nf, basis.dets_bytes(), eng.to_host(X[:, 0]))
        ro = {"NTri1": ntri // 2, "NTri2": ntri // 2, "Epsilon": o.get("Epsilon", api.DEFAULTS["Epsilon"]),
              "Emin1": -8.0, "Emax1": 8.0, "NE1": 63, "Gamma1": 0.4,
              "Emin2": -2.0, "Emax2": 10.0, "NE2": 1024, "Gamma2": 0.1,
              "Restrictions1": Rx, "Restrictions2": R}
        Te = [t.dagger() for t in Ts]  # emission: 3d -> 2p
        G, _ = api.CreateResonantSpectra(H, H, Ts[2], Te, psi0, ro, eng)  # warm
        _sync(eng)
        t0 = time.perf_counter()
        G, st = api.CreateResonantSpectra(H, H, Ts[2], Te, psi0, ro, eng)
        _sync(eng)
        t_rixs = time.perf_counter() - t0
        _log("rixs: %d spectra in %.2f s" % (G.shape[0], t_rixs))
        rixs = {"incident_energies": 64, "emission_polarisations": 3, "spectra": int(G.shape[0]),
                "ntri1": ro["NTri1"], "ntri2": ro["NTri2"], "ne2": 1024, "seconds": t_rixs,
                "spectra_per_s": G.shape[0] / t_rixs, "finite": bool(np.all(np.isfinite(G)))}

    line = {
        "metric": "batched CreateSpectra spectra/s",
        "value": nspec / t_batched,
        "unit": "spectra/s",
        "mode": "batched",
        "n_gpus": 1,
        "steps": reps,
        "higher_is_better": True,
        "dtype": "c128",
        "data": "synthetic (seeded impurity Hamiltonian)",
        "config": {"workload": "impurity_76so_6shell_xas_16states_x3pol", "ground_determinants": basis.n,
                   "core_excited_determinants": int(n_final),
                   "ntri": ntri, "ne": 2048, "vectors_per_launch": nspec, "temperature_K": 300},
        "batched": {"seconds": t_batched, "spectra": nspec, "spectra_per_s": nspec / t_batched},
        "plain": {"seconds_per_spectrum": t_plain, "spectra_per_s": 1.0 / t_plain, "sample": len(sample)},
        "speedup_vs_plain": (nspec / t_batched) * t_plain,
        "max_rel_diff_batched_vs_plain": diff,
        "lanczos_only": {"batched_seconds": t_lz_b, "plain_seconds_per_vector": t_lz_p,
                         "speedup": nspec * t_lz_p / t_lz_b},
        "apply_ms_by_layout": layouts, "apply_ms_one_vector": single_ms, "autotuned_layout": tuned,
        "eigensystem": {"seconds": t_eigen, "converged": est["converged"], "max_variance": res,
                        "block_applies": est["applies"], "krylov_max": est["krylov_max"]},
        "energies_eV": [float(e) for e in E],
        "boltzmann_weights": [float(x) for x in w],
        "xas_peak": float(np.max(-xas.imag)),
        "rixs": rixs,
    }
    print(json.dumps(line), flush=True)
    return 0


def _final_vectors(api, H, Ts, basis, X, R, eng):
    """Common core-excited basis and the (n, len(Ts) * npsi) block of T psi on it."""
    bt = None
    for t in Ts:
        tb = api.OperatorPsiBasis(t, basis, R, eng)
        bt = tb if bt is None else api.basis_union(bt, tb, eng)
    bf = api.closure_of(H, bt, R, -1, eng)
    npsi = X.shape[1]
    Y = eng.empty(bf.n, len(Ts) * npsi)
    for j, t in enumerate(Ts):
        yj = eng.empty(bf.n, npsi)
        eng.check(eng.L.qg_apply(eng.ctx, t.handle(eng), bf.h, basis.h, api._ptr(X), api._ptr(yj), npsi))
        with eng.on_stream():
            Y[:, j * npsi:(j + 1) * npsi] = yj
    return bf, Y


def _lanczos_seconds(api, H, bf, Y, ntri, eps, eng, reps=1):
    api.lanczos_block(H, bf, Y, ntri, eps, eps, eng)  # warm (graph capture)
    _sync(eng)
    t0 = time.perf_counter()
    for _ in range(reps):
        api.lanczos_block(H, bf, Y, ntri, eps, eps, eng)
    _sync(eng)
    return (time.perf_counter() - t0) / reps


# ----------------------------------------------------------------------------- served

def make_stream(njobs, seed=0, max_det=2e6, min_det=1e3, eigen_frac=0.25):
    """Seeded mixed jobs: (kind, params) with target sizes log-uniform in [min_det, max_det]."""
    from quanty_gb300 import workloads
    rng = np.random.default_rng(seed)
    out = []
    for j in range(njobs):
        target = math.exp(rng.uniform(math.log(min_det), math.log(max_det)))
        nshell = int(rng.integers(1, 7))
        delta = float(rng.uniform(1.0, 6.0))
        v = float(rng.uniform(0.5, 3.0))
        bath_seed = int(rng.integers(0, 1 << 30))
        eps = np.sort(np.random.default_rng(bath_seed).uniform(-5.0, 5.0, nshell))
        nfill = int((eps < 0).sum())
        best = None
        for hm in range(0, 4):
            for pm in range(0, 4):
                n = workloads.sector_size(nfill, nshell - nfill, hole_max=hm, particle_max=pm)
                d = abs(math.log(n) - math.log(target))
                if best is None or d < best[0]:
                    best = (d, hm, pm, n)
        kind = "eigen" if rng.random() < eigen_frac else "spectra"
        out.append({"kind": kind, "nshell": nshell, "delta": delta, "v": v, "seed": bath_seed,
                    "hole_max": best[1], "particle_max": best[2], "sector": best[3],
                    "ntri": int(rng.integers(150, 1001)), "ne": int(rng.integers(1024, 4097))})
    return out


def make_shared_stream(njobs, materials=4, seed=5, max_det=2e6, min_det=1e3):
    """Seeded CreateSpectra jobs on a few materials: `materials` impurity Hamiltonians drawn as in
    make_stream (one Lanczos length each), every job on one of them with its own initial state
    and its own number of frequencies -- the case the served form merges."""
    rng = np.random.default_rng(seed)
    mats = make_stream(materials, seed=seed, max_det=max_det, min_det=min_det, eigen_frac=0.0)
    out = []
    for j in range(njobs):
        m = int(rng.integers(0, materials))
        p = dict(mats[m], kind="spectra", material=m, ne=int(rng.integers(1024, 4097)),
                 state_seed=int(rng.integers(0, 1 << 30)))
        out.append(p)
    return out


def build_shared_job(api, serve, workloads, p, cache):
    """A job of make_shared_stream: the material's Hamiltonian and operators are built once and
    shared (one object per material); the initial state is the material's seed determinant plus
    0.3 times a seeded neighbour determinant (a target of H on the seed) with a seeded phase."""
    m = p["material"]
    if m not in cache:
        H, R, seed, info = workloads.anderson_impurity(nshell=p["nshell"], seed=p["seed"], delta=p["delta"],
                                                       v2_total=p["v"] ** 2, hole_max=p["hole_max"],
                                                       particle_max=p["particle_max"])
        _, Rx, _, _ = workloads.anderson_impurity(nshell=p["nshell"], seed=p["seed"], delta=p["delta"],
                                                  v2_total=p["v"] ** 2, hole_max=p["hole_max"],
                                                  particle_max=p["particle_max"], core_holes=1)
        seed_b = api.dets_to_bytes([seed], H.nf)
        nb = api.OperatorPsi(H, api.Wavefunction(H.nf, seed_b, np.ones(1, dtype=np.complex128)), R)
        cache[m] = (H, Rx, seed_b, nb.det, _xas_ops(api, workloads, H.nf))
    H, Rx, seed_b, neigh, Ts = cache[m]
    rng = np.random.default_rng(p["state_seed"])
    k = int(rng.integers(0, len(neigh)))
    dets = np.concatenate([seed_b.reshape(1, -1), neigh[k:k + 1]])
    if np.array_equal(dets[0], dets[1]):
        dets = dets[:1]
    vals = np.array([1.0, 0.3 * np.exp(2j * np.pi * rng.random())])[:len(dets)]
    psi = api.Wavefunction(H.nf, dets, vals)
    o = {"NTri": p["ntri"], "NE": p["ne"], "Emin": -20.0, "Emax": 20.0, "Gamma": 0.5, "Restrictions": Rx}
    return serve.SpectraJob(H, Ts, [psi], o, n_det_hint=6 * p["sector"])


def build_job(api, serve, workloads, p):
    H, R, seed, info = workloads.anderson_impurity(nshell=p["nshell"], seed=p["seed"], delta=p["delta"],
                                                   v2_total=p["v"] ** 2, hole_max=p["hole_max"],
                                                   particle_max=p["particle_max"])
    seed_b = api.dets_to_bytes([seed], H.nf)
    if p["kind"] == "eigen":
        return serve.EigenJob(H, R, 2, None, n_det_hint=p["sector"], seed_dets=seed_b)
    _, Rx, _, _ = workloads.anderson_impurity(nshell=p["nshell"], seed=p["seed"], delta=p["delta"],
                                              v2_total=p["v"] ** 2, hole_max=p["hole_max"],
                                              particle_max=p["particle_max"], core_holes=1)
    Ts = _xas_ops(api, workloads, H.nf)
    psi = api.Wavefunction(H.nf, seed_b, np.ones(1, dtype=np.complex128))
    o = {"NTri": p["ntri"], "NE": p["ne"], "Emin": -20.0, "Emax": 20.0, "Gamma": 0.5, "Restrictions": Rx}
    return serve.SpectraJob(H, Ts, [psi], o, n_det_hint=6 * p["sector"])


def served(args):
    print(json.dumps(served_line(args)), flush=True)
    return 0


def served_line(args):
    """The served stream against the plain one-job-at-a-time path (the JSON line's fields)."""
    from quanty_gb300 import api, serve, workloads
    shared = int(getattr(args, "materials", 0) or 0)
    if shared:
        params = make_shared_stream(int(args.jobs), materials=shared, max_det=float(args.max_det))
        cache = {}
        jobs = [build_shared_job(api, serve, workloads, p, cache) for p in params]
    else:
        params = make_stream(int(args.jobs), seed=0, max_det=float(args.max_det))
        jobs = [build_job(api, serve, workloads, p) for p in params]
    nspec = sum(j.nspec for j in jobs)
    rate = float(args.rate)
    # warm-up: one small job of each kind through both paths (builds, graphs)
    warm = sorted(range(len(jobs)), key=lambda k: params[k]["sector"])[:2]
    eng = api.engine()
    for k in warm:
        jobs[k].run(eng)
    _sync(eng)
    st = {}
    res_s, lat_s, wall_s = serve.run_stream(jobs, rate, slots=int(args.slots), seed=1, policy=args.policy,
                                            stats=st)
    res_p, lat_p, wall_p = serve.run_plain(jobs, rate, seed=1, eng=eng)
    diff = 0.0
    for a, b in zip(res_s, res_p):
        if "G" in a:
            diff = max(diff, float(np.max(np.abs(a["G"] - b["G"])) / np.max(np.abs(b["G"]))))
        else:
            diff = max(diff, float(np.max(np.abs(a["energies"] - b["energies"]))))
    sizes = [p["sector"] * (6 if p["kind"] == "spectra" else 1) for p in params]
    line = {
        "metric": "served CreateSpectra/Eigensystem spectra/s",
        "value": nspec / wall_s,
        "unit": "spectra/s",
        "mode": "served",
        "n_gpus": 1,
        "higher_is_better": True,
        "dtype": "c128",
        "data": "synthetic (seeded impurity Hamiltonians, Poisson arrivals)",
        "config": {"workload": ("poisson_stream_impurity_jobs_%d_materials" % shared) if shared else
                   "poisson_stream_mixed_impurity_jobs", "jobs": len(jobs), "rate_per_s": rate,
                   "slots": int(args.slots), "policy": args.policy, "spectra": nspec,
                   "eigen_jobs": sum(p["kind"] == "eigen" for p in params),
                   "max_det": float(args.max_det), "determinants_min": int(min(sizes)),
                   "determinants_max": int(max(sizes))},
        "served": {"wall_s": wall_s, "spectra_per_s": nspec / wall_s, "jobs_per_s": len(jobs) / wall_s,
                   "p50_s": float(np.percentile(lat_s, 50)), "p99_s": float(np.percentile(lat_s, 99)),
                   "merged_jobs": st.get("merged_jobs", 0)},
        "plain": {"wall_s": wall_p, "spectra_per_s": nspec / wall_p, "jobs_per_s": len(jobs) / wall_p,
                  "p50_s": float(np.percentile(lat_p, 50)), "p99_s": float(np.percentile(lat_p, 99))},
        "speedup_vs_plain": wall_p / wall_s,
        "max_diff_served_vs_plain": diff,
    }
    return line


def batched_secondary(ntri=200, ne=2048, nstates=16, plain_sample=3):
    """The batched XAS form at its own basis sizes for the default bench line: 6 bath shells,
    1,701,795 ground and 3,899,040 core-excited determinants, 16 initial states x 3 polarisations
    = 48 spectra as one multi-vector Lanczos (CreateSpectraResident), against the plain path
    (closure, T psi, one Lanczos and continued fraction per spectrum) on a sample of the pairs.
    The initial states are seeded random real vectors on the ground basis (the eigenstates of this
    real Hamiltonian are real, as the eigensolver returns them): the timing of the spectra depends
    only on that, not on the vectors (the eigensolver itself is timed by --mode batched)."""
    from quanty_gb300 import api, workloads
    eng = api.engine()
    H, R, seed, info = workloads.anderson_impurity(nshell=6, hole_max=1, particle_max=2)
    _, Rx, _, _ = workloads.anderson_impurity(nshell=6, hole_max=1, particle_max=2, core_holes=1)
    Ts = _xas_ops(api, workloads, H.nf)
    basis = api.closure(H, api.dets_to_bytes([seed], H.nf), H.nf, R, -1, eng)
    rng = np.random.default_rng(300)
    Xh = rng.normal(size=(basis.n, nstates)) + 0j  # states of a real Hamiltonian are real
    Xh /= np.linalg.norm(Xh, axis=0)
    E = np.zeros(nstates)
    with eng.on_stream():
        X = eng.torch.from_numpy(Xh).to("cuda:%d" % eng.device)
    o = {"NTri": ntri, "NE": ne, "Emin": -20.0, "Emax": 20.0, "Gamma": 0.5, "Restrictions": Rx}
    S, _, _ = api.CreateSpectraResident(H, Ts, basis, X, E, o, eng, batched=True)  # warm-up
    _sync(eng)
    t0 = time.perf_counter()
    S, _, _ = api.CreateSpectraResident(H, Ts, basis, X, E, o, eng, batched=True)
    _sync(eng)
    t_b = time.perf_counter() - t0
    with eng.on_stream():
        cols = [X[:, i:i + 1].contiguous() for i in range(nstates)]
    api.CreateSpectraResident(H, [Ts[0]], basis, cols[0], [0.0], o, eng, batched=False)  # warm-up
    _sync(eng)
    sample = [(j % 3, j) for j in range(plain_sample)]
    diff = 0.0
    t0 = time.perf_counter()
    for j, i in sample:
        Sp, _, _ = api.CreateSpectraResident(H, [Ts[j]], basis, cols[i], [0.0], o, eng, batched=False)
        g = S.G[j * nstates + i]
        diff = max(diff, float(np.max(np.abs(Sp.G[0] - g)) / np.max(np.abs(g))))
    _sync(eng)
    t_p = (time.perf_counter() - t0) / len(sample)
    nspec = 3 * nstates
    return {"workload": "impurity_76so_6shell_xas_16states_x3pol_ntri%d_ne%d" % (ntri, ne), "unit": "spectra/s",
            "ground_determinants": basis.n, "spectra": nspec, "batched": nspec / t_b, "plain": 1.0 / t_p,
            "speedup": nspec / t_b * t_p, "plain_sample": len(sample), "max_rel_diff_batched_vs_plain": diff}


def served_secondary(jobs=24, rate=50.0, slots=4, max_det=2e6, materials=0):
    """The served stream for the default bench line (the --mode served configuration); with
    materials > 0 the jobs share that many Hamiltonians and the server merges them."""
    import types
    line = served_line(types.SimpleNamespace(jobs=jobs, rate=rate, slots=slots, max_det=max_det, policy="sjf",
                                             materials=materials))
    return {"workload": line["config"]["workload"], "unit": "spectra/s", "jobs": line["config"]["jobs"],
            "merged_jobs": line["served"]["merged_jobs"],
            "spectra": line["config"]["spectra"], "determinants_min": line["config"]["determinants_min"],
            "determinants_max": line["config"]["determinants_max"],
            "served": line["served"]["spectra_per_s"], "plain": line["plain"]["spectra_per_s"],
            "speedup": line["speedup_vs_plain"], "served_p50_s": line["served"]["p50_s"],
            "served_p99_s": line["served"]["p99_s"], "plain_p50_s": line["plain"]["p50_s"],
            "plain_p99_s": line["plain"]["p99_s"], "max_diff_served_vs_plain": line["max_diff_served_vs_plain"]}


def layouts(args):
    """The multi-vector apply alone: 48 random vectors on the core-excited basis of the
    impurity with `--shells` bath shells (at most 1 hole, 2 particles); every vector layout
    timed with CUDA events, or (with --layout) only that one, twice (a profiling target)."""
    import ctypes
    from quanty_gb300 import api, workloads
    eng = api.engine()
    torch = eng.torch
    nshell = int(args.shells)
    H, R, seed, info = workloads.anderson_impurity(nshell=nshell, hole_max=1, particle_max=2)
    _, Rx, _, _ = workloads.anderson_impurity(nshell=nshell, hole_max=1, particle_max=2, core_holes=1)
    T = _xas_ops(api, workloads, H.nf)[2]
    b0 = api.closure(H, api.dets_to_bytes([seed], H.nf), H.nf, R, -1, eng)
    bf = api.closure_of(H, api.OperatorPsiBasis(T, b0, Rx, eng), Rx, -1, eng)
    n, nvec = bf.n, 48
    rng = np.random.default_rng(0)
    with eng.on_stream():
        X = torch.from_numpy(rng.normal(size=(n, nvec)) + 1j * rng.normal(size=(n, nvec))).to(
            "cuda:%d" % eng.device)
    Y = eng.empty(n, nvec)
    eng.check(eng.L.qg_set_autotune(eng.ctx, 0))

    def run(c, reps):
        eng.check(eng.L.qg_apply_set_chunk(eng.ctx, H.handle(eng), bf.h, nvec, c))
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(eng.stream)
        for _ in range(reps):
            eng.check(eng.L.qg_apply(eng.ctx, H.handle(eng), bf.h, bf.h, api._ptr(X), api._ptr(Y), nvec))
        e1.record(eng.stream)
        e1.synchronize()
        return e0.elapsed_time(e1) / reps

    if args.layout is not None:
        run(int(args.layout), 2)
        print(json.dumps({"mode": "layouts", "layout": int(args.layout), "n": n}))
        return 0
    out = {}
    for c in (1, 2, 4, 8, -32, -64):
        run(c, 1)
        out[str(c)] = run(c, 3)
    x1 = X[:, :1].contiguous()
    y1 = eng.empty(n, 1)
    eng.check(eng.L.qg_apply(eng.ctx, H.handle(eng), bf.h, bf.h, api._ptr(x1), api._ptr(y1), 1))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(eng.stream)
    for _ in range(3):
        eng.check(eng.L.qg_apply(eng.ctx, H.handle(eng), bf.h, bf.h, api._ptr(x1), api._ptr(y1), 1))
    e1.record(eng.stream)
    e1.synchronize()
    nnz_off = api.count_nnz(H, bf, offdiag=True)
    print(json.dumps({"mode": "layouts", "n": n, "nvec": nvec, "nnz_offdiag": nnz_off, "apply_ms": out,
                      "one_vector_ms": e0.elapsed_time(e1) / 3}))
    return 0


def chains(args):
    """Real Lanczos chains on the XAS final-state basis of the 76-spin-orbital impurity (6 bath
    shells): Tx psi (real) and Ty psi (purely imaginary) of a real psi, as one complex chain, as
    one chain on real vectors, and as a pair in one complex vector; the coefficients of each form
    against the others (bitwise) and the time per chain and step (CUDA events over --ntri steps).
    Three short runs of each form come first (the ncu target: -k regex:k_apply_list)."""
    from quanty_gb300 import api, workloads
    eng = api.engine()
    torch = eng.torch
    H, R, seed, info = workloads.anderson_impurity(nshell=6, hole_max=1, particle_max=2)
    _, Rx, _, _ = workloads.anderson_impurity(nshell=6, hole_max=1, particle_max=2, core_holes=1)
    Ts = _xas_ops(api, workloads, H.nf)
    g = api.closure(H, api.dets_to_bytes([seed], H.nf), H.nf, R, -1, eng)
    rng = np.random.default_rng(1)
    X = torch.from_numpy(rng.normal(size=(g.n, 1)) + 0j).cuda()
    bf, Y = _final_vectors(api, H, Ts[:2], g, X, Rx, eng)
    pair, one = Y.contiguous(), Y[:, :1].contiguous()

    def run(x, ntri, split):
        eng.check(eng.L.qg_set_split_chains(eng.ctx, split))
        try:
            return api.lanczos_block(H, bf, x, ntri, 0.0, 0.0, eng)
        finally:
            eng.check(eng.L.qg_set_split_chains(eng.ctx, 1))

    short = {"pair": run(pair, 3, 1), "real": run(one, 3, 1), "complex": run(one, 3, 0)}
    same = bool(np.array_equal(short["pair"][0][0], short["real"][0][0]) and
                np.array_equal(short["real"][0], short["complex"][0]))
    ntri = int(args.ntri)
    out = {}
    for name, x, split, nch in (("complex", one, 0, 1), ("real", one, 1, 1), ("pair", pair, 1, 2)):
        run(x, 4, split)  # warm (graphs)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(eng.stream)
        run(x, ntri, split)
        e1.record(eng.stream)
        e1.synchronize()
        out[name] = e0.elapsed_time(e1) / ntri / nch
    line = {"mode": "chains", "n": bf.n, "ntri": ntri, "ms_per_chain_step": out, "bitwise_equal_forms": same}
    print(json.dumps(line), flush=True)
    return 0


def eigh(args):
    """The dense Hermitian eigensolver (qg_hermitian_eigh) on a seeded random Hermitian matrix of
    order --k: three calls with the lowest three eigenvectors, then two with all of them, each
    timed on the host around the call (host matrix in, eigenpairs out), and the eigenvalues
    against LAPACK (numpy)."""
    from quanty_gb300 import api
    eng = api.engine()
    k = int(args.k)
    rng = np.random.default_rng(0)
    A = rng.normal(size=(k, k)) + 1j * rng.normal(size=(k, k))
    A = A + A.conj().T
    out = {}
    for name, nv, reps in (("three_vectors", 3, 3), ("all_vectors", k, 2)):
        ts = []
        for _ in range(reps):
            eng.stream.synchronize()
            t0 = time.perf_counter()
            w, V = api.hermitian_eigh(A, nv, eng)
            eng.stream.synchronize()
            ts.append(time.perf_counter() - t0)
        out[name + "_ms"] = 1e3 * min(ts)
    ref = np.linalg.eigvalsh(A)
    out["eigenvalues_max_rel_vs_lapack"] = float(np.max(np.abs(w - ref)) / np.max(np.abs(ref)))
    print(json.dumps({"mode": "eigh", "k": k, **out}), flush=True)
    return 0


def main(args):
    if args.mode == "eigh":
        return eigh(args)
    if args.mode == "batched":
        return batched(args)
    if args.mode == "layouts":
        return layouts(args)
    if args.mode == "chains":
        return chains(args)
    return served(args)
