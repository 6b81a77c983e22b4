"""Independent systems advanced together in one engine (one launch per phase)
give bit-identical results to each system advanced alone.

Covers uneven sizes, a box with fewer than three cells per dimension (the
all-pairs regime of the reference's from_particle module), two species,
Andersen and Verlet integrators and sorting on / off side by side.
"""
import numpy as np
import pytest

import halmd_gb300 as hg
from _systems import KA_EPS, KA_SIGMA, fcc, maxwell_boltzmann

pytestmark = pytest.mark.gpu


def specs():
    out = []
    r, L = fcc(3, 0.9, 0.1, seed=11)                   # N = 108, L = 4.93: 1 cell per dimension
    out.append(dict(r=r, L=L, desc=dict(r_cut=2.4, truncation="shifted", skin=0.3, timestep=0.004), T=1.0))
    r, L = fcc(5, 1.2, 0.05, seed=12)                  # KA, N = 500, L = 7.47: 2 cells per dimension
    sp = np.zeros(len(r), dtype=np.uint32)
    sp[np.random.default_rng(3).permutation(len(r))[:100]] = 1
    out.append(dict(r=r, L=L, sp=sp, T=0.8,
                    desc=dict(epsilon=KA_EPS, sigma=KA_SIGMA, r_cut=2.5, truncation="smooth_r4", smoothing=0.005,
                              skin=0.3, timestep=0.002, integrator="andersen", temperature=0.8,
                              collision_rate=5.0, seed=99)))
    r, L = fcc(8, 0.8442, 0.1, seed=13)                # N = 2048
    out.append(dict(r=r, L=L, T=1.5, desc=dict(r_cut=2.5, truncation="shifted", skin=0.3, timestep=0.005)))
    r, L = fcc(6, 0.7, 0.1, seed=14)                   # N = 864, sorting off
    out.append(dict(r=r, L=L, T=2.0, desc=dict(r_cut=2.5, truncation="force_shifted", skin=0.4, timestep=0.003,
                                               sort=False)))
    return out


def load(eng, k, sp):
    n = len(sp["r"])
    if "sp" in sp:
        eng.set("species", sp["sp"], k)
    eng.set("position", sp["r"], k)
    eng.set("velocity", maxwell_boltzmann(n, sp["T"], seed=100 + n), k)


def test_batched_equals_alone():
    S = specs()
    batch = hg.Engine("dsfloat")
    for sp in S:
        batch.add_system(hg.system_desc(len(sp["r"]), sp["L"], **sp["desc"]))
    batch.set_option("force_lanes", 4)
    batch.commit()
    for k, sp in enumerate(S):
        load(batch, k, sp)
    batch.step(40, aux_last=True)
    for k, sp in enumerate(S):
        alone = hg.Engine("dsfloat")
        alone.add_system(hg.system_desc(len(sp["r"]), sp["L"], **sp["desc"]))
        alone.set_option("force_lanes", 4)
        alone.commit()
        load(alone, 0, sp)
        alone.step(40, aux_last=True)
        for name in ("position", "velocity", "image", "force", "potential_energy"):
            a, b = alone.get(name), batch.get(name, k)
            assert np.array_equal(a, b), (k, name)
        assert alone.info().rebuilds == batch.info(k).rebuilds
        ta, tb = alone.thermo(), batch.thermo(k)
        assert ta["mv2"] == tb["mv2"] and ta["epot"] == tb["epot"]
        alone.close()
    # the small boxes: every pair inside the cutoff is found with < 3 cells per dimension
    assert batch.info(0).ncell[0] == 1 and batch.info(1).ncell[0] == 2
    batch.close()


def test_small_box_lists_match_all_pairs():
    import oracle
    S = specs()
    for k in (0, 1):
        sp = S[k]
        eng = hg.Engine("dsfloat")
        eng.add_system(hg.system_desc(len(sp["r"]), sp["L"], **sp["desc"]))
        eng.commit()
        load(eng, 0, sp)
        eng.force()
        inf = eng.info()
        ns = inf.nspecies
        pos4 = eng.get_raw("r0")[eng.get("reverse_id")]
        counts, lists = eng.neighbour_lists(inf.neighbour_capacity)
        rc, rl, _ = oracle.neighbour_full_f32(pos4, np.array(inf.box_f32), np.array(inf.rr_cut_skin[:ns * ns],
                                              dtype=np.float32), inf.neighbour_capacity)
        assert np.array_equal(counts, rc) and np.array_equal(lists, rl)
        eng.close()


@pytest.mark.parametrize("scan", [1, 2])
def test_batched_lists_match_oracle_with_either_scan(scan):
    # a many-system engine builds its lists in one looped launch over the
    # rebuilding systems' virtual blocks, with either scan
    import oracle
    S = specs()
    batch = hg.Engine("dsfloat")
    for sp in S:
        batch.add_system(hg.system_desc(len(sp["r"]), sp["L"], **sp["desc"]))
    batch.commit()
    batch.set_option("neighbour_scan", scan)
    for k, sp in enumerate(S):
        load(batch, k, sp)
    batch.step(30)
    for k in range(len(S)):
        batch.request_rebuild(k)
    batch.force()
    for k in range(len(S)):
        inf = batch.info(k)
        ns = inf.nspecies
        pos4 = batch.get_raw("r0", k)[batch.get("reverse_id", k)]
        counts, lists = batch.neighbour_lists(inf.neighbour_capacity, k)
        rc, rl, mx = oracle.neighbour_full_f32(pos4, np.array(inf.box_f32),
                                               np.array(inf.rr_cut_skin[:ns * ns], dtype=np.float32),
                                               inf.neighbour_capacity)
        assert np.array_equal(counts, rc) and np.array_equal(lists, rl), k
    batch.close()


def test_tiny_systems_one_and_two_particles():
    # the smallest inputs: one particle has an empty list and no force, so it
    # moves in a straight line; two particles interact as a pair (equal and
    # opposite forces); both advance beside each other in one engine
    eng = hg.Engine("dsfloat")
    eng.add_system(hg.system_desc(1, 10.0, r_cut=2.5, truncation="shifted", skin=0.3, timestep=0.001))
    eng.add_system(hg.system_desc(2, 10.0, r_cut=2.5, truncation="shifted", skin=0.3, timestep=0.001))
    eng.commit()
    eng.set("position", np.array([[0.5, -0.25, 1.0]]), 0)
    eng.set("velocity", np.array([[0.3, -0.2, 0.1]]), 0)
    eng.set("position", np.array([[0.0, 0.0, 0.0], [1.2, 0.0, 0.0]]), 1)
    eng.set("velocity", np.zeros((2, 3)), 1)
    eng.force()
    assert np.all(eng.get("force", 0) == 0)
    counts, _ = eng.neighbour_lists(s=0)
    assert counts[0] == 0
    f = eng.get("force", 1)
    assert f[0, 0] != 0 and f[0, 0] == -f[1, 0]
    eng.step(100)
    np.testing.assert_allclose(eng.get("unwrapped_position", 0), [[0.53, -0.27, 1.01]], atol=1e-6)
    np.testing.assert_allclose(eng.get("velocity", 0), [[0.3, -0.2, 0.1]], atol=1e-12)
    v = eng.get("velocity", 1)
    assert abs(v[0, 0] + v[1, 0]) < 1e-6      # momentum conserved
    eng.close()
