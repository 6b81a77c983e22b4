"""The GPU pair force at the reference's golden-table distances.

test/unit/mdsim/potentials/pair/lennard_jones.cpp checks the GPU force
kernel with a fake neighbour list (gpu/neighbour_chain.hpp: each particle's
only neighbour is the next) against the host functor at 10 float epsilons,
with the energy halved for the full list (:262, :430).  Here every table
row of the LJ tables (AA, AB, BB at r_c = 5 sigma) becomes an isolated
particle pair on the x axis, far from every other pair, so each particle's
list holds its partner alone; the force and energy the engine computes are
compared with the FP64 host functor of the oracle (pinned to the same
tables on the CPU, test_oracle_golden.py) at the pair's separation.  The
positions are floats, so the lo words of the double-single state are zero,
as the reference's test places its particles.
"""
import json
import os

import numpy as np
import pytest

import halmd_gb300 as hg
import oracle

pytestmark = pytest.mark.gpu

EPS_F = float(np.finfo(np.float32).eps)
TOL = 10 * EPS_F
GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "lj_tables.json")


@pytest.mark.parametrize("trunc", ["sharp", "shifted", "smooth_r4", "force_shifted"])
def test_isolated_pairs_match_host_functor(trunc):
    g = json.load(open(GOLDEN))
    eps, sigma, rcs = g["epsilon"], g["sigma"], float(g["r_cut_sigma"])
    skin = 0.3
    rc = rcs * np.asarray(sigma, dtype=float)
    pairs = []   # (species a, species b, r)
    for name, (a, b) in {"aa": (0, 0), "ab": (0, 1), "bb": (1, 1)}.items():
        for r, fval, en in g["tables"][trunc][name]:
            if r < rc[a, b]:
                pairs.append((a, b, r))
    spacing = 2 * (rc.max() + skin) + 5.0
    # pairs at positive x with x0 >= r, positions rounded to float: the lo
    # words are zero and the float difference of the two hi words is exact
    # (Sterbenz), so the kernel sees the separation d computed below
    L = np.array([2 * spacing * (len(pairs) + 1), 2 * rc.max() + 10.0, 2 * rc.max() + 10.0])
    n = 2 * len(pairs)
    pos = np.zeros((n, 3))
    sp = np.zeros(n, dtype=np.uint32)
    for k, (a, b, r) in enumerate(pairs):
        x0 = (k + 1) * spacing
        pos[2 * k] = (x0, 0.0, 0.0)
        pos[2 * k + 1] = (x0 + r, 0.0, 0.0)
        sp[2 * k], sp[2 * k + 1] = a, b
    eng = hg.Engine("dsfloat")
    eng.add_system(hg.system_desc(n, L, epsilon=eps, sigma=sigma, r_cut=rcs, truncation=trunc,
                                  smoothing=g["h"], skin=skin, timestep=0.001))
    eng.commit()
    eng.set("species", sp)
    eng.set("position", pos.astype(np.float32).astype(np.float64))
    eng.set("velocity", np.zeros((n, 3)))
    eng.force(aux=True)
    f = eng.get("force")
    en = eng.get("potential_energy")
    x = eng.get_raw("position_hi")[eng.get("reverse_id")][:, 0].astype(np.float64)
    counts, _ = eng.neighbour_lists()
    assert np.all(counts == 1)           # every list holds the partner alone
    pot = oracle.Potential(eps, sigma, rcs, trunc, h=g["h"])
    for k, (a, b, r) in enumerate(pairs):
        d = x[2 * k] - x[2 * k + 1]       # the float separation the kernel sees (exact difference)
        fval, u = pot(d * d, a, b)
        assert abs(f[2 * k, 0] - fval * d) <= TOL * abs(fval * d), (trunc, a, b, r, f[2 * k, 0], fval * d)
        assert abs(f[2 * k + 1, 0] + fval * d) <= TOL * abs(fval * d), (trunc, a, b, r)
        assert f[2 * k, 1] == 0 and f[2 * k, 2] == 0
        # energy: half per particle (full list); the shifted forms subtract
        # U(r_c), so the float error scales with |U| + |U(r_c)|
        _, u_bare = oracle.Potential(eps, sigma, rcs, "sharp")(d * d, a, b)
        scale = abs(u) + abs(u_bare - u) + 1e-30
        assert abs(2 * en[2 * k] - u) <= TOL * scale, (trunc, a, b, r, 2 * en[2 * k], u)
        assert abs(2 * en[2 * k + 1] - u) <= TOL * scale, (trunc, a, b, r)
    eng.close()


def test_smooth_r4_near_cutoff_pairs_match_host_functor():
    # test/unit/mdsim/forces/trunc/smooth_r4.cpp: r_c = 2.5, 2, 2^(1/6) sigma,
    # h = 1/256, rows close to r_c; the GPU bar there (:88-91) is
    # tol = 8 eps (1 + r_c / (r_c - r)) + 10 eps, forces within
    # 2 tol max(|F|, 1), energies within 2 tol relative
    g = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "smooth_r4_tables.json")))
    eps, sigma, rcs, h = g["epsilon"], g["sigma"], np.asarray(g["r_cut_sigma"], dtype=float), g["h"]
    skin = 0.3
    rc = rcs * np.asarray(sigma, dtype=float)
    pairs = []
    for name, (a, b) in {"aa": (0, 0), "ab": (0, 1), "bb": (1, 1)}.items():
        for row in g["tables"][name]:
            if row[0] < rc[a, b]:
                pairs.append((a, b, row[0]))
    assert len(pairs) >= 10
    spacing = 2 * (rc.max() + skin) + 5.0
    L = np.array([2 * spacing * (len(pairs) + 1), 2 * rc.max() + 10.0, 2 * rc.max() + 10.0])
    n = 2 * len(pairs)
    pos = np.zeros((n, 3))
    sp = np.zeros(n, dtype=np.uint32)
    for k, (a, b, r) in enumerate(pairs):
        x0 = (k + 1) * spacing         # x0 >= r: the float difference is exact
        pos[2 * k] = (x0, 0.0, 0.0)
        pos[2 * k + 1] = (x0 + r, 0.0, 0.0)
        sp[2 * k], sp[2 * k + 1] = a, b
    eng = hg.Engine("dsfloat")
    eng.add_system(hg.system_desc(n, L, epsilon=eps, sigma=sigma, r_cut=rcs, truncation="smooth_r4",
                                  smoothing=h, skin=skin, timestep=0.001))
    eng.commit()
    eng.set("species", sp)
    eng.set("position", pos.astype(np.float32).astype(np.float64))
    eng.set("velocity", np.zeros((n, 3)))
    eng.force(aux=True)
    f = eng.get("force")
    en = eng.get("potential_energy")
    x = eng.get_raw("position_hi")[eng.get("reverse_id")][:, 0].astype(np.float64)
    pot = oracle.Potential(eps, sigma, rcs, "smooth_r4", h=h)
    worst = 0.0
    for k, (a, b, r) in enumerate(pairs):
        d = x[2 * k] - x[2 * k + 1]
        fval, u = pot(d * d, a, b)
        tol = 8 * EPS_F * (1 + rc[a, b] / (rc[a, b] - abs(d))) + 10 * EPS_F
        for q in (2 * k, 2 * k + 1):
            fref = fval * d if q == 2 * k else -fval * d
            err = abs(f[q, 0] - fref) / (2 * tol * max(abs(fref), 1.0))
            worst = max(worst, err)
            assert err <= 1.0, (a, b, r, f[q, 0], fref)
            assert abs(2 * en[q] - u) <= 2 * tol * abs(u), (a, b, r, 2 * en[q], u)
    print("largest force error / bound: %.3g" % worst)
    eng.close()
