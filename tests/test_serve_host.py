"""The job server's host logic on the CPU, with a stand-in engine.

Admission in arrival order under the reserved capacity (back-pressure on
HMD_ERR_NOMEM), retirement when a job's step count is reached, the
reservation arithmetic, and the errors the server passes on.  The device
side of the same server is tested in test_gpu_serve.py.
"""
import os

import numpy as np
import pytest

from halmd_gb300 import _lib, serve
from halmd_gb300._lib import HmdError


@pytest.fixture(autouse=True, scope="module")
def built():
    # system descriptions come from the C library (no GPU needed)
    if not os.path.exists(_lib.LIB_PATH):
        from halmd_gb300 import build
        build.build()


class FakeEngine:
    """Holds systems by slot count; step(n) advances every held system."""

    def __init__(self, precision, fail_code=None):
        self.slots = 0
        self.used = 0
        self.systems = {}
        self.max_running = 0
        self.fail_code = fail_code
        self.closed = False

    def reserve(self, slots, systems, neighbour_capacity):
        self.slots, self.table = slots, systems

    def set_option(self, name, value):
        pass

    def commit(self):
        pass

    def add(self, desc):
        if self.fail_code is not None:
            raise HmdError(self.fail_code, "bad system")
        n = desc.nparticle
        if self.used + n > self.slots or len(self.systems) >= self.table:
            raise HmdError(serve.HMD_ERR_NOMEM, "capacity")
        k = min(set(range(self.table)) - set(self.systems))
        self.systems[k] = dict(n=n, step=0, left=None, data={})
        self.used += n
        self.max_running = max(self.max_running, len(self.systems))
        return k

    def set(self, name, array, k):
        self.systems[k]["data"][name] = np.array(array)

    def set_steps_left(self, steps, k):
        self.systems[k]["left"] = steps

    def step(self, n):
        for s in self.systems.values():
            adv = min(n, s["left"])
            s["step"] += adv
            s["left"] -= adv

    def progress(self, table):
        step = np.zeros(table, dtype=np.uint64)
        left = np.full(table, 0xFFFFFFFF, dtype=np.uint64)
        for k, s in self.systems.items():
            step[k], left[k] = s["step"], s["left"]
        return step, left

    def get(self, name, k):
        return self.systems[k]["data"].get(name if name != "image" else "position")

    def remove(self, k):
        self.used -= self.systems.pop(k)["n"]

    def close(self):
        self.closed = True


def job(jid, n, steps, arrival=0.0):
    r = np.zeros((n, 3))
    return serve.Job(jid, n, [10.0] * 3, dict(r_cut=2.5, truncation="shifted"), r, r, np.zeros(n, np.uint32),
                     steps, arrival)


def make_server(slots, **kw):
    engines = []

    def factory(precision):
        engines.append(FakeEngine(precision, kw.pop("fail_code", None)))
        return engines[-1]

    # per_slot = 360 + 4 * 288 bytes; total_bytes sized for `slots` at fraction 1
    srv = serve.Server(budget_fraction=1.0, total_bytes=slots * (360 + 4 * 288), max_jobs=8, chunk=10,
                       engine_factory=factory)
    return srv, engines[0]


def test_admission_respects_capacity_and_every_job_finishes():
    srv, eng = make_server(4096)
    jobs = [job(j, 1500, steps) for j, steps in enumerate([30, 10, 50, 20, 40])]
    out = srv.run(jobs, realtime=False)
    assert sorted(j.jid for j in srv.done) == list(range(5))
    assert eng.max_running == 2          # 1500-particle jobs: two fit in 4096 slots
    assert not srv.running and not srv.queue and eng.used == 0
    for j in jobs:
        assert j.result["step"] == j.steps and j.completed >= j.admitted
    # admission in arrival order: a later job is never admitted before an earlier one
    adm = [j.admitted for j in sorted(jobs, key=lambda j: j.jid)]
    assert adm == sorted(adm)
    assert out["chunks"] >= max(j.steps for j in jobs) // 10
    lat = serve.latency_stats(jobs)
    assert lat["p50"] <= lat["p99"]


def test_reservation_follows_the_memory_budget():
    srv, eng = make_server(10000)
    assert eng.slots == 10000 and srv.budget["slots"] == 10000
    srv, eng = make_server(100)          # never below one sort tile of slots
    assert eng.slots == 2048


def test_job_larger_than_the_reservation_is_reported():
    srv, eng = make_server(2048)
    with pytest.raises(RuntimeError, match="does not fit"):
        srv.run([job(0, 5000, 10)], realtime=False)


def test_other_engine_errors_pass_through():
    srv, eng = make_server(4096, fail_code=-1)
    with pytest.raises(HmdError):
        srv.run([job(0, 100, 10)], realtime=False)
