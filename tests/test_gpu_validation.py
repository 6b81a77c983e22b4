"""Thermodynamic validation of the MD step against the reference's own
known answers (test/integration/validation/thermodynamics.cpp, run as
thermodynamics.cmake.in describes): a Lennard-Jones fluid at rho = 0.3,
T = 3, r_c = 4 with the smooth_r4 cut-off (h = 0.005) in a 1 : 2 : 1.01 box
of 4000 particles (the GPU case).

Protocol of thermodynamics.cmake.in: thermalise with Andersen collisions
(rate 1, dt 0.005) for 30 time units; NVE (dt 0.001) for 30 time units after
rescaling the velocities to the internal energy 2.8282 per particle; then 60
time units of NVE production, sampled every 320 steps.  Checks of
thermodynamics.cpp:150-190 (tolerances 4.5 sigma of the reference's
empirical standard deviations for N = 4000 on the GPU):
  P = 1.023 +- 4.5 x 0.003 (Johnson et al.), U/N = -1.673 +- 4.5 x 0.002,
  <T> = 3 +- 4.5 x 0.004, c_V = 1.648 +- 4.5 x 0.02,
  energy drift below 3e-5 + steps x 10 x 3e-14.
"""
import math

import numpy as np
import pytest

import halmd_gb300 as hg
from _systems import maxwell_boltzmann

pytestmark = pytest.mark.gpu


def heat_capacity_nve(mean_temp, var_temp, n):
    # thermodynamics.cpp:63-66 (Lebowitz, Percus and Verlet 1967): called
    # there with the mean and variance of the temperature
    return 1.0 / (2.0 / 3.0 - n * var_temp / (mean_temp * mean_temp))


def desc(n, box, dt, **kw):
    return hg.system_desc(n, box, r_cut=4.0, truncation="smooth_r4", smoothing=0.005, skin=0.5, timestep=dt, **kw)


def sample(eng, n, volume):
    th = eng.thermo()
    temp = th["mv2"] / (3 * n)
    press = (th["mv2"] + th["virial"]) / (3 * volume)
    return temp, press, th["epot"] / n, (0.5 * th["mv2"] + th["epot"]) / n


def test_lennard_jones_equation_of_state():
    n, rho, T = 4000, 0.3, 3.0
    ratios = np.array([1.0, 2.0, 1.01])
    volume = n / rho
    box = ratios * (volume / np.prod(ratios)) ** (1 / 3)
    # start: distinct sites of a simple cubic grid of spacing >= 1.1 (no overlaps)
    rng = np.random.default_rng(4000)
    m = np.floor(box / 1.1).astype(int)
    axes = [(np.arange(k) + 0.5) * (b / k) - 0.5 * b for k, b in zip(m, box)]
    sites = np.stack(np.meshgrid(*axes, indexing="ij"), -1).reshape(-1, 3)
    r = sites[rng.permutation(sites.shape[0])[:n]]
    v = maxwell_boltzmann(n, T, seed=4001)

    # thermalisation (lennard_jones_equilibration.lua): Andersen, rate 1, dt 0.005, 30 time units
    eng = hg.Engine("dsfloat")
    eng.add_system(desc(n, box, 0.005, integrator="andersen", temperature=T, collision_rate=1.0, seed=17))
    eng.commit()
    eng.set("position", r)
    eng.set("velocity", v)
    eng.step(6000)
    r, v = eng.get("position"), eng.get("velocity")
    eng.close()

    # equilibration: NVE, dt 0.001, 30 time units, rescaled to E = 2.8282 per particle
    eng = hg.Engine("dsfloat")
    eng.add_system(desc(n, box, 0.001))
    eng.commit()
    eng.set("position", r)
    eng.set("velocity", v - v.mean(axis=0))
    eng.force(aux=True)
    th = eng.thermo()
    ekin = n * 2.8282 - th["epot"]
    eng.set("velocity", eng.get("velocity") * math.sqrt(ekin / (0.5 * th["mv2"])))
    eng.step(30000)

    # production: 60 time units, state variables every 320 steps
    interval, steps = 320, 60000
    eng.force(aux=True)
    data = [sample(eng, n, volume)]
    for _ in range(steps // interval):
        eng.step(interval, aux_last=True)
        data.append(sample(eng, n, volume))
    eng.close()
    temp, press, en_pot, en_tot = (np.array(x) for x in zip(*data))
    drift = np.max(np.abs(en_tot - en_tot[0])) / abs(en_tot[0])
    cv = heat_capacity_nve(temp.mean(), temp.var(ddof=1), n)
    print("T %.4f  P %.4f  U/N %.4f  c_V %.3f  drift %.2e  (%d samples)"
          % (temp.mean(), press.mean(), en_pot.mean(), cv, drift, len(temp)))
    assert drift < 3e-5 + steps * 10 * 3e-14
    assert abs(temp.mean() - T) / T < 4.5 * 0.004 / T
    assert abs(press.mean() - 1.023) / 1.023 < 4.5 * 0.003 / 1.023
    assert abs(en_pot.mean() + 1.673) / 1.673 < 4.5 * 0.002 / 1.673
    assert abs(cv - 1.648) / 1.648 < 4.5 * 0.02 / 1.648
