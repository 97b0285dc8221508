"""Serving form on the GPU: jobs arriving while others run overlap on the device (one context
and stream per slot; checked with CUDA events on the slots' streams), waiting CreateSpectra jobs
on one Hamiltonian run merged as one multi-vector Lanczos, and every job's result equals its
result alone."""
import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mods():
    from quanty_gb300 import build
    build.build()
    from quanty_gb300 import api, serve, workloads
    return api, serve, workloads


def _jobs(api, serve, workloads):
    g0, g1 = golden("c0_xas.json"), golden("c1_lf.json")
    jobs = []
    for g, ne in ((g0, 1024), (g1, 2048)):
        HX = api.Operator.from_fixture(g["HX"])
        Ts = [api.Operator.from_fixture(g[t]) for t in ("Tx", "Ty", "Tz")]
        psis = [api.Wavefunction.from_fixture(p) for p in g["psi"]]
        o = {"Emin": -10, "Emax": 20, "NE": ne, "Gamma": 0.5, "NTri": 200, "Epsilon": 0.0}
        jobs.append(serve.SpectraJob(HX, Ts, psis, o, n_det_hint=200))
    H, R, seed, info = workloads.anderson_impurity(nshell=2, hole_max=2, particle_max=2)
    b = api.closure(H, api.dets_to_bytes([seed], H.nf), H.nf, R)
    dets = b.dets_bytes()
    rng = np.random.default_rng(7)
    for k in range(3):
        psi = api.Wavefunction(H.nf, dets, rng.normal(size=len(dets)) + 1j * rng.normal(size=len(dets)))
        T = api.Operator(H.nf, [([6 + k], 1.0), ([7 + k], 0.5)])
        o = {"Emin": -15, "Emax": 15, "NE": 1024, "Gamma": 0.4, "NTri": 150, "Restrictions": R,
             "Method": "Lanczos"}
        jobs.append(serve.SpectraJob(H, [T], [psi], o, n_det_hint=info["sector_determinants"]))
    jobs.append(serve.EigenJob(api.Operator.from_fixture(g1["H"]),
                               [26, 0] + [list(r) for r in g1["restrictions"]], 3, {"Zero": 1e-14},
                               n_det_hint=200))
    return jobs


def test_results_in_the_mix_equal_results_alone(mods):
    api, serve, workloads = mods
    jobs = _jobs(api, serve, workloads)
    eng = api.Engine(0)
    alone = [j.run(eng) for j in jobs]
    results, lat, wall = serve.run_stream(jobs, rate=500.0, slots=3)
    assert len(results) == len(jobs)
    for a, r in zip(alone, results):
        if "G" in a:
            assert np.max(np.abs(a["G"] - r["G"])) <= 1e-12 * np.max(np.abs(a["G"]))
        else:
            assert np.max(np.abs(a["energies"] - r["energies"])) < 1e-10
    assert np.all(lat > 0)


def test_jobs_overlap_when_admitted_together(mods):
    api, serve, workloads = mods
    jobs = _jobs(api, serve, workloads)[2:5]
    srv = serve.Server(slots=3)
    futs = [srv.submit(j) for j in jobs]
    [f.result() for f in futs]
    recs = sorted(srv.records, key=lambda r: r["dev_start"])
    srv.close()
    # on the device clock (CUDA events on each slot's stream): the second job's stream began
    # its work before the first job's last kernel finished
    assert recs[1]["dev_start"] < recs[0]["dev_end"]
    assert all(r["dev_end"] > r["dev_start"] >= 0.0 for r in recs)


def test_budget_serialises_jobs(mods):
    api, serve, workloads = mods
    jobs = _jobs(api, serve, workloads)[2:4]
    need = max(j.footprint() for j in jobs)
    srv = serve.Server(slots=2, hbm_budget=need + 1)  # room for one job at a time
    futs = [srv.submit(j) for j in jobs]
    [f.result() for f in futs]
    recs = sorted(srv.records, key=lambda r: r["start"])
    srv.close()
    assert recs[1]["start"] >= recs[0]["end"]


def test_waiting_jobs_on_one_hamiltonian_run_merged(mods):
    """Three CreateSpectra jobs on one impurity Hamiltonian, queued before the only slot starts,
    run as one multi-vector Lanczos; each gets the spectra (and window) of its call alone."""
    api, serve, workloads = mods
    jobs = _jobs(api, serve, workloads)[2:5]
    assert len({j.merge_key() for j in jobs}) == 1
    eng = api.Engine(0)
    alone = [j.run(eng) for j in jobs]
    srv = serve.Server(slots=1, paused=True)
    futs = [srv.submit(j) for j in jobs]
    srv.resume()
    res = [f.result() for f in futs]
    recs = list(srv.records)
    srv.close()
    assert len(recs) == 3 and all(r["merged"] == 3 for r in recs)
    for a, r in zip(alone, res):
        assert np.max(np.abs(a["G"] - r["G"])) <= 1e-12 * np.max(np.abs(a["G"]))
        assert abs(a["Emin"] - r["Emin"]) < 1e-10 and abs(a["Emax"] - r["Emax"]) < 1e-10
