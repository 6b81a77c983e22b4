"""The seeded synthetic workloads of bench.py follow their stated distributions.

ENS-256: N log-uniform in [500, 32000], density uniform in [0.7, 1.2], T
uniform in [0.5, 2.0], LJ or KA by a coin flip.  SERVE: Poisson arrivals at
50 per second, N log-uniform in [1e3, 2e5], density uniform in [0.8, 1.2], T
uniform in [0.5, 1.5], steps log-uniform in [1e3, 1e5] (scaled).  Statistical
checks use 4.5 standard errors, the bar of the reference's statistical tests.
"""
import numpy as np

import bench


def _log_uniform_mean_ok(x, lo, hi):
    # ln x is uniform on [ln lo, ln hi]: mean and standard error of the mean
    a, b = np.log(lo), np.log(hi)
    mean, sd = 0.5 * (a + b), (b - a) / np.sqrt(12)
    return abs(np.mean(np.log(x)) - mean) < 4.5 * sd / np.sqrt(len(x))


def test_ensemble_replicas_follow_the_specification():
    specs = bench.ensemble_specs()
    assert len(specs) == 256
    n = np.array([s["n"] for s in specs])
    assert n.min() >= 500 and n.max() < 32000
    assert _log_uniform_mean_ok(n + 0.5, 500, 32000)
    rho = np.array([s["n"] / s["L"] ** 3 for s in specs])
    assert rho.min() >= 0.7 - 1e-9 and rho.max() <= 1.2 + 1e-9
    ka = np.array([s["desc"].get("truncation") == "smooth_r4" for s in specs])
    assert abs(ka.mean() - 0.5) < 4.5 * 0.5 / np.sqrt(len(specs))
    for s in specs[:16]:
        assert s["r"].shape == (s["n"], 3) and np.all(np.abs(s["r"]) <= 0.5 * s["L"])
        assert np.allclose(s["v"].mean(axis=0), 0.0, atol=1e-12)
        if s["desc"].get("truncation") == "smooth_r4":
            assert np.sum(s["sp"] == 1) == s["n"] // 5
            assert 0.5 <= s["desc"]["temperature"] <= 2.0
    # seeded: the same draw every time
    again = bench.ensemble_specs(count=4)
    assert [s["n"] for s in again] == [s["n"] for s in specs[:4]]
    assert np.array_equal(again[0]["r"], specs[0]["r"])


def test_served_jobs_follow_the_specification():
    jobs = bench.serve_jobs(200, 1.0)
    t = np.array([j.arrival for j in jobs])
    gaps = np.diff(np.concatenate([[0.0], t]))
    assert np.all(gaps > 0)
    # exponential gaps at rate 50: mean 0.02, standard deviation 0.02
    assert abs(gaps.mean() - 0.02) < 4.5 * 0.02 / np.sqrt(len(gaps))
    n = np.array([j.n for j in jobs])
    assert n.min() >= 1000 and n.max() < 200000
    assert _log_uniform_mean_ok(n + 0.5, 1e3, 2e5)
    steps = np.array([j.steps for j in jobs])
    assert steps.min() >= 1000 and steps.max() <= 100000
    assert _log_uniform_mean_ok(steps + 0.5, 1e3, 1e5)
    rho = np.array([j.n / j.box ** 3 for j in jobs])
    assert rho.min() >= 0.8 - 1e-9 and rho.max() <= 1.2 + 1e-9
    # the same seed scales the same draws
    scaled = bench.serve_jobs(5, 0.1)
    assert all(abs(s.steps - 0.1 * j.steps) <= 1 for s, j in zip(scaled, jobs[:5]))
    assert [s.n for s in scaled] == [j.n for j in jobs[:5]]
