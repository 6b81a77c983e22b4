"""Continuous batching: jobs that join and leave a running engine give the
same result as each job run alone (bit-identical phase space), and admission
waits for capacity instead of failing."""
import numpy as np
import pytest

import halmd_gb300 as hg
from halmd_gb300.serve import Job, Server, latency_stats, run_fifo
from _systems import KA_EPS, KA_SIGMA, fcc, maxwell_boltzmann

pytestmark = pytest.mark.gpu


def make_jobs():
    jobs = []
    specs = [(5, 0.85, False, 180), (6, 1.2, True, 120), (4, 0.9, False, 260), (7, 0.8, False, 90),
             (5, 1.1, True, 200), (6, 0.95, False, 150), (4, 1.0, True, 70)]
    for k, (nc, rho, ka, steps) in enumerate(specs):
        r, L = fcc(nc, rho, 0.05, seed=40 + k)
        n = len(r)
        sp = np.zeros(n, dtype=np.uint32)
        if ka:
            sp[np.random.default_rng(k).permutation(n)[: n // 5]] = 1
            desc = dict(epsilon=KA_EPS, sigma=KA_SIGMA, r_cut=2.5, truncation="smooth_r4", smoothing=0.005,
                        skin=0.3, timestep=0.002, integrator="andersen", temperature=0.7, collision_rate=2.0,
                        seed=77 + k)
        else:
            desc = dict(r_cut=2.5, truncation="shifted", skin=0.3, timestep=0.004)
        v = maxwell_boltzmann(n, 1.0, seed=90 + k)
        jobs.append(Job(k, n, L, desc, r, v, sp, steps, arrival=0.0))
    return jobs


def test_results_identical_alone_and_in_the_mix():
    jobs = make_jobs()
    # room for about three jobs at a time: later jobs wait, then join running ones
    srv = Server(max_slots=3 * 2048 + 2048, max_jobs=8, neighbour_capacity=288, chunk=50, force_lanes=4,
                 total_bytes=1 << 40)
    stats = srv.run(jobs, realtime=False)
    assert len(srv.done) == len(jobs) and stats["chunks"] > 3
    admitted = sorted(j.admitted for j in jobs)
    assert admitted[-1] > admitted[0]          # some jobs had to wait for capacity
    mixed = {j.jid: j.result for j in jobs}
    srv.close()
    alone = make_jobs()
    run_fifo(alone, force_lanes=4)
    for j in alone:
        m = mixed[j.jid]
        assert m["step"] == j.steps == j.result["step"]
        for key in ("position", "velocity", "image"):
            assert np.array_equal(m[key], j.result[key]), (j.jid, key)
    assert latency_stats(jobs)["p99"] >= latency_stats(jobs)["p50"]


def test_job_larger_than_capacity_is_reported():
    jobs = make_jobs()[:2]
    big_r, L = fcc(12, 0.8, 0.05, seed=1)
    jobs.append(Job(99, len(big_r), L, dict(r_cut=2.5, truncation="shifted", skin=0.3, timestep=0.004), big_r,
                    maxwell_boltzmann(len(big_r), 1.0), np.zeros(len(big_r), dtype=np.uint32), 10))
    srv = Server(max_slots=4096, max_jobs=4, neighbour_capacity=288, chunk=20, total_bytes=1 << 40)
    with pytest.raises(RuntimeError, match="does not fit"):
        srv.run(jobs, realtime=False)
    # the jobs that fit were served
    assert {j.jid for j in srv.done} == {0, 1}
    srv.close()


def test_capacity_bookkeeping():
    eng = hg.Engine("dsfloat")
    eng.reserve(8 * 2048, 4, 288)
    eng.commit()
    cap = eng.capacity()
    assert cap["slots"] == 8 * 2048 and cap["systems"] == 0
    r, L = fcc(5, 0.9, 0.05)
    ks = [eng.add(hg.system_desc(len(r), L, r_cut=2.5, skin=0.3, timestep=0.004)) for _ in range(3)]
    assert eng.capacity()["systems"] == 3
    eng.remove(ks[1])
    assert eng.capacity()["systems"] == 2
    k = eng.add(hg.system_desc(len(r), L, r_cut=2.5, skin=0.3, timestep=0.004))
    assert k == ks[1]                           # the freed table entry and slot range are reused
    for s in (ks[0], k, ks[2]):
        eng.set("position", r, s)
    eng.step(10)
    assert all(eng.info(s).step == 10 for s in (ks[0], k, ks[2]))
    with pytest.raises(hg.HmdError):
        eng.remove(3)                           # never added
    eng.close()
