"""The oracle's untruncated pair force (pair_full), on the CPU.

The untruncated Lennard-Jones potential equals the sharp truncation's pair
values (no energy shift), so the reference's own sharp tables
(test/unit/mdsim/potentials/pair/lennard_jones.cpp:77-211) pin it.  The all-pairs sum (host/forces/pair_full.hpp:229-270)
is checked against a direct numpy double loop.
"""
import numpy as np
import pytest

import oracle
from _systems import KA_EPS, KA_SIGMA

EPS64 = np.finfo(np.float64).eps


def test_untruncated_lj_equals_sharp_tables(golden):
    # the reference's sharp tables hold the bare values at every listed r (the
    # range test is separate from the evaluation), so every row pins the
    # untruncated potential
    g = golden("lj_tables.json")
    none = oracle.Potential(g["epsilon"], g["sigma"], g["r_cut_sigma"], "none")
    tol = g["tolerance_eps_double"] * EPS64
    for pair, (a, b) in {"aa": (0, 0), "ab": (0, 1), "bb": (1, 1)}.items():
        for r, fval, en in g["tables"]["sharp"][pair]:
            f, e = none(r * r, a, b)
            assert abs(f - fval) <= tol * abs(fval) or (fval == 0 and abs(f) < 1e-30), (pair, r, f, fval)
            assert abs(e - en) <= tol * abs(en) or (en == 0 and abs(e) < 1e-12), (pair, r, e, en)


def brute_force(r, sp, L, eps, sigma):
    n = r.shape[0]
    f = np.zeros((n, 3))
    en = np.zeros(n)
    for i in range(n):
        d = r[i] - r
        d -= np.rint(d / L) * L
        rr = np.sum(d * d, axis=1)
        rr[i] = np.inf
        s2 = sigma[sp[i], sp] ** 2 / rr
        s6 = s2 ** 3
        e = eps[sp[i], sp]
        fval = 48 * e * s2 * s6 * (s6 - 0.5) / sigma[sp[i], sp] ** 2
        f[i] = np.sum(fval[:, None] * d, axis=0)
        en[i] = 0.5 * np.sum(4 * e * s6 * (s6 - 1))
    return f, en


def test_all_pairs_force_matches_direct_sum():
    rng = np.random.default_rng(11)
    n, L = 80, 6.0
    r = rng.uniform(-L / 2, L / 2, size=(n, 3))
    sp = (rng.uniform(size=n) < 0.2).astype(np.uint32)
    pot = oracle.Potential(KA_EPS, KA_SIGMA, 1.0, "none")
    got = oracle.forces(r, sp, np.array([L] * 3), pot)
    f, en = brute_force(r, sp, L, np.asarray(KA_EPS), np.asarray(KA_SIGMA))
    assert got["npairs"] == n * (n - 1) // 2
    scale = np.max(np.abs(f))
    assert np.max(np.abs(got["force"] - f)) < 1e-11 * scale
    np.testing.assert_allclose(got["en_pot"], en, rtol=1e-10, atol=1e-12 * np.max(np.abs(en)))
