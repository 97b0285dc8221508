"""The multi-GPU form of the bench is replicas (the H*psi path does not shard on one-GPU
boxes): the process-group plumbing -- joining, barriers, the max-over-ranks timing and the
whole-job rate -- checked with two gloo ranks on the CPU, and the reference arm's other ranks
exiting without work."""
import os
import socket
import subprocess
import sys

from conftest import ROOT


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    from quanty_gb300 import replicas
    w, r, local = replicas.init("gloo")
    replicas.barrier()
    # rank r "took" 1 + r seconds for the step and 10 * (world - r) for the e2e call
    mx = replicas.max_over_ranks([1.0 + r, 10.0 * (w - r)])
    rate = replicas.aggregate_rate(100.0, w, mx[0])
    replicas.barrier()
    replicas.finalize()
    q.put((r, w, local, mx, rate))


def test_replicas_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r, (rank, w, local, mx, rate) in enumerate(out):
        assert (rank, w, local) == (r, 2, r)
        assert mx == [2.0, 20.0]          # the slowest rank's times, on every rank
        assert rate == 100.0 * 2 / 2.0    # units of all ranks over the slowest time


def test_single_process_needs_no_group():
    from quanty_gb300 import replicas
    env = {k: os.environ.pop(k) for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK") if k in os.environ}
    try:
        assert replicas.init("gloo") == (1, 0, 0)
        assert replicas.max_over_ranks([3.0, 4.0]) == [3.0, 4.0]
        replicas.barrier()
    finally:
        os.environ.update(env)


def test_reference_arm_other_ranks_exit_without_work():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference"], env=env,
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0
    assert r.stdout.strip() == ""
