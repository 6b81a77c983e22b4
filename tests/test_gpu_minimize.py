"""Steepest-descent minimisation on the device against the FP64 oracle."""
import numpy as np
import pytest

import halmd_gb300 as hg
import oracle
from _systems import KA_EPS, KA_SIGMA, lj_system

pytestmark = pytest.mark.gpu


def test_descent_matches_fp64_oracle_from_lattice():
    r, v, L = lj_system(ncell=6, jitter=0.12)
    n = r.shape[0]
    eng = hg.Engine("dsfloat")
    eng.add_system(hg.system_desc(n, L, r_cut=2.5, truncation="shifted", skin=0.3, timestep=0.005))
    eng.commit()
    eng.set("position", r)
    eng.set("velocity", v)
    v0 = eng.get("velocity")
    eng.minimize(steps=40, step_size=1e-3, max_move=0.05)
    got = eng.get("unwrapped_position")
    Lf = np.array(eng.info().box_f32, dtype=np.float64)
    pot = oracle.Potential(1.0, 1.0, 2.5, "shifted")
    ro, img, st = oracle.minimize(r, np.zeros(n), Lf, pot, skin=0.3, nsteps=40, step=1e-3, max_move=0.05)
    err = np.abs(got - (ro + img * Lf)).max()
    print("descent position error after 40 steps: %.3g" % err)
    assert err < 1e-5
    # velocities and the step counter are left alone
    assert eng.info().step == 0
    np.testing.assert_array_equal(eng.get("velocity"), v0)
    # forces are those of the relaxed positions: the next MD steps run
    eng.step(10)
    assert eng.info().step == 10
    eng.close()


def test_descent_relaxes_random_mixture_like_the_oracle():
    n, rho = 2000, 1.2
    L = (n / rho) ** (1 / 3)
    rng = np.random.default_rng(5)
    r = rng.uniform(-L / 2, L / 2, size=(n, 3))
    sp = np.zeros(n, dtype=np.uint32)
    sp[rng.permutation(n)[: n // 5]] = 1
    eng = hg.Engine("dsfloat")
    eng.add_system(hg.system_desc(n, L, epsilon=KA_EPS, sigma=KA_SIGMA, r_cut=2.5, truncation="smooth_r4",
                                  smoothing=0.005, skin=0.3, timestep=0.002))
    eng.commit()
    eng.set("species", sp)
    eng.set("position", r)
    eng.minimize(steps=300, step_size=1e-3, max_move=0.05)
    eng.force(aux=True)
    e_gpu = eng.thermo()["epot"]
    Lf = np.array(eng.info().box_f32, dtype=np.float64)
    pot = oracle.Potential(KA_EPS, KA_SIGMA, 2.5 * np.ones((2, 2)), "smooth_r4", h=0.005)
    ro, img, st = oracle.minimize(r, sp, Lf, pot, skin=0.3, nsteps=300, step=1e-3, max_move=0.05)
    print("epot/n gpu %.6f oracle %.6f" % (e_gpu / n, st["epot"] / n))
    assert e_gpu / n < -6.0 and st["epot"] / n < -6.0   # relaxed, no overlaps left
    assert abs(e_gpu - st["epot"]) < 1e-3 * abs(st["epot"])
    eng.close()


def test_descent_holds_other_systems():
    r, v, L = lj_system(ncell=5, jitter=0.1)
    n = r.shape[0]
    eng = hg.Engine("dsfloat")
    for _ in range(2):
        eng.add_system(hg.system_desc(n, L, r_cut=2.5, truncation="shifted", skin=0.3, timestep=0.005))
    eng.commit()
    for s in range(2):
        eng.set("position", r, s)
        eng.set("velocity", v, s)
    eng.step(5)
    before = eng.get("position", 1)
    eng.minimize(steps=20, s=0)
    np.testing.assert_array_equal(eng.get("position", 1), before)
    assert eng.info(0).step == 5 and eng.info(1).step == 5
    eng.step(5)
    assert eng.info(0).step == 10 and eng.info(1).step == 10
    with pytest.raises(hg.HmdError):
        eng.minimize(steps=10, step_size=-1.0)
    eng.close()
