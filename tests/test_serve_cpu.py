"""Admission logic of the serving loop, without a GPU: first come first served, a job waits
while the HBM budget is taken, a job larger than the whole budget runs alone."""
import collections
import threading

from quanty_gb300 import serve


class FakeJob:
    def __init__(self, need):
        self.need = need

    def footprint(self):
        return self.need


def server(budget, policy="fifo"):
    s = serve.Server.__new__(serve.Server)
    s.policy = policy
    s.budget = budget
    s.in_use = 0
    s.queue = collections.deque()
    s.cv = threading.Condition()
    return s


def test_fifo_and_budget():
    s = server(100)
    for need in (40, 50, 30, 10):
        s.queue.append({"job": FakeJob(need)})
    a = s._admit()
    b = s._admit()
    assert (a["need"], b["need"]) == (40, 50) and s.in_use == 90
    assert s._admit() is None          # 30 does not fit next to 90, and 10 may not overtake it
    s.in_use -= 40
    assert s._admit()["need"] == 30
    assert s._admit()["need"] == 10


def test_oversized_job_runs_alone():
    s = server(100)
    s.queue.append({"job": FakeJob(500)})
    s.in_use = 10
    assert s._admit() is None
    s.in_use = 0
    assert s._admit()["need"] == 500


def test_footprint_grows_with_size():
    assert serve._footprint(10 ** 6, 4) > serve._footprint(10 ** 5, 4) > 0


def test_shortest_job_first():
    s = server(100, "sjf")
    for need in (60, 30, 50, 10):
        s.queue.append({"job": FakeJob(need)})
    assert s._admit()["need"] == 10
    assert s._admit()["need"] == 30
    assert s._admit()["need"] == 50   # 90 in use
    assert s._admit() is None          # 60 does not fit
    s.in_use = 0
    assert s._admit()["need"] == 60


class FakeSpectra(serve.SpectraJob):
    def __init__(self, need, key):
        self.need, self.key = need, key

    def footprint(self):
        return self.need

    def merge_key(self):
        return self.key


def test_waiting_jobs_with_one_merge_key_join_the_admitted_one():
    s = server(100)
    for need, key in ((20, "h1"), (20, "h2"), (30, "h1"), (60, "h1"), (5, None)):
        s.queue.append({"job": FakeSpectra(need, key)})
    a = s._admit()
    # the waiting h1 job that fits joins; the one that would exceed the budget waits
    assert [g["job"].need for g in a["group"]] == [20, 30] and a["need"] == 50 and s.in_use == 50
    b = s._admit()
    assert [g["job"].need for g in b["group"]] == [20] and s.in_use == 70
    assert s._admit() is None  # 60 does not fit next to 70
    s.in_use = 0
    c = s._admit()
    assert [g["job"].need for g in c["group"]] == [60]
    d = s._admit()
    assert [g["job"].need for g in d["group"]] == [5]  # no key: runs on its own
