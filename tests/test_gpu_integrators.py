"""GPU parity and statistics of the verlet_nvt_hoover, verlet_nvt_boltzmann
and euler integrators (through the C ABI), against the FP64 oracle's
restatement of the host integrators and the checks of the reference's own
test/unit/mdsim/integrators/verlet_nvt_hoover.cpp.
"""
import numpy as np
import pytest

import halmd_gb300 as hg
import oracle
from _systems import lj_system, maxwell_boltzmann

pytestmark = pytest.mark.gpu


def engine(integrator, r, v, L, dt, **kw):
    n = r.shape[0]
    eng = hg.Engine("dsfloat")
    eng.add_system(hg.system_desc(n, L, r_cut=2.5, truncation="shifted", skin=0.3, timestep=dt,
                                  integrator=integrator, **kw))
    eng.commit()
    eng.set("position", r)
    eng.set("velocity", v)
    return eng


def oracle_run(integrator, r, v, L, dt, nsteps, **kw):
    n = r.shape[0]
    pot = oracle.Potential(1.0, 1.0, 2.5, "shifted")
    return oracle.md_run(r, v, np.zeros(n), np.ones(n), [L] * 3, pot, 0.3, dt, nsteps, integrator=integrator, **kw)


def unwrapped(eng):
    return eng.get("unwrapped_position")


def test_hoover_trajectory_against_fp64():
    r, v, L = lj_system(ncell=5, T=1.5)
    dt, nsteps = 0.002, 200
    eng = engine("verlet_nvt_hoover", r, v, L, dt, temperature=1.0, resonance_frequency=5.0)
    eng.step(nsteps)
    st = eng.integrator_state()
    ro, vo, io, info = oracle_run("hoover", r, v, L, dt, nsteps, temperature=1.0, resonance_frequency=5.0)
    assert np.max(np.abs(unwrapped(eng) - (ro + io * L))) < 1e-4
    assert np.max(np.abs(eng.get("velocity") - vo)) < 1e-4
    np.testing.assert_allclose(st["xi"], info["xi"], rtol=1e-4, atol=1e-7)
    np.testing.assert_allclose(st["v_xi"], info["v_xi"], rtol=1e-4, atol=1e-6)
    np.testing.assert_allclose(st["internal_energy"], info["en_nhc"], rtol=1e-4, atol=1e-7)
    eng.close()


def test_hoover_conserves_the_extended_energy_and_thermostats():
    # test/unit/mdsim/integrators/verlet_nvt_hoover.cpp:236-290, shortened: LJ
    # at rho = 0.1 from T = 3 to T = 1, dt = 0.002, resonance frequency 5
    npart, rho, T, dt, f = 1500, 0.1, 1.0, 0.002, 5.0
    L = (npart / rho) ** (1 / 3)
    rng = np.random.default_rng(11)
    # a lattice start (no overlaps): fcc of 8^3 cells holds 2048 sites
    ncell = 8
    sites = oracle.fcc_lattice(ncell, L)
    r = sites[rng.permutation(sites.shape[0])[:npart]]
    v = maxwell_boltzmann(npart, 3.0, seed=12)
    eng = engine("verlet_nvt_hoover", r, v, L, dt, temperature=T, resonance_frequency=f)
    period = int(round(3 / (f * dt)))        # verlet_nvt_hoover.cpp:144
    # equilibrate over 25 time units before the reference energy is taken,
    # as the reference's test does (steps / 20 of its 500 time units)
    eng.step(int(round(25 / dt)))
    nblocks = 200
    temps, vcm, h = [], [], []
    for b in range(nblocks):
        eng.step(period, aux_last=True)
        th = eng.thermo()
        ekin = 0.5 * th["mv2"]
        h.append(ekin + th["epot"] + npart * eng.integrator_state()["internal_energy"])
        vcm.append(th["momentum"] / th["mass"])
        temps.append(th["mv2"] / (3 * npart))
    h = np.array(h)
    drift = np.max(np.abs(h - h[0])) / abs(h[0])
    print("hoover: extended-energy drift %.3g, <T> %.5f over %d samples" % (drift, np.mean(temps), len(temps)))
    # gpu_en_tolerance<dsfloat> of verlet_nvt_hoover.cpp:396-400
    assert drift < 5e-5
    # 4.5 sigma on the mean temperature (verlet_nvt_hoover.cpp:245-250)
    tol = 4.5 * np.sqrt(2.0 / (3 * npart * (len(temps) - 1))) / T
    assert abs(np.mean(temps) - T) / T < tol
    assert np.max(np.abs(vcm)) < 4.5 * np.sqrt(T / (npart * len(vcm) - 1)) + 1e-6
    eng.close()


def test_boltzmann_draws_against_fp64():
    r, v, L = lj_system(ncell=5, T=1.5)
    dt, rate, T = 0.002, 50.0, 0.8              # interval round(1 / (50 * 0.002)) = 10 steps
    eng = engine("verlet_nvt_boltzmann", r, v, L, dt, temperature=T, collision_rate=rate, seed=7)
    eng.step(9)
    v9 = eng.get("velocity")
    eng.step(1)                                  # step 10 draws
    vd = eng.get("velocity")
    st = eng.integrator_state()
    ro, vo, io, _ = oracle_run("boltzmann", r, v, L, dt, 10, temperature=T, coll_rate=rate, seed=7)
    assert np.max(np.abs(vd - vo)) < 2e-5      # same Philox stream; float Box-Muller against double
    assert np.max(np.abs(np.mean(vd, axis=0))) < 1e-6   # centre-of-mass velocity removed
    assert np.max(np.abs(vd - v9)) > 0.1        # the velocities were redrawn
    # the removed centre-of-mass velocity of n Gaussian draws: of order sqrt(T / n)
    assert 0 < np.max(np.abs(st["vcm"])) < 5 * np.sqrt(T / r.shape[0])
    # the remaining steps are plain Verlet until the next draw
    eng.step(5)
    ro2, vo2, io2, _ = oracle_run("boltzmann", r, v, L, dt, 15, temperature=T, coll_rate=rate, seed=7)
    assert np.max(np.abs(eng.get("velocity") - vo2)) < 1e-4
    eng.close()


def test_boltzmann_temperature_statistics():
    r, v, L = lj_system(ncell=8, T=1.5)
    n = r.shape[0]
    dt, rate, T = 0.002, 50.0, 0.8
    eng = engine("verlet_nvt_boltzmann", r, v, L, dt, temperature=T, collision_rate=rate, seed=3)
    temps = []
    for k in range(40):
        eng.step(10)                            # right after a draw
        th = eng.thermo()
        temps.append(th["mv2"] / (3 * n))
    tol = 4.5 * np.sqrt(2.0 / (3 * n * len(temps)))
    assert abs(np.mean(temps) - T) / T < tol + 3.0 / n   # the removed momentum takes 3 degrees of freedom
    eng.close()


def test_euler_drift():
    r, v, L = lj_system(ncell=4, T=1.0)
    dt, nsteps = 0.001, 10
    eng = engine("euler", r, v, L, dt)
    v0 = eng.get("velocity")
    eng.step(nsteps)
    ro, vo, io, _ = oracle_run("euler", r, v, L, dt, nsteps)
    np.testing.assert_array_equal(eng.get("velocity"), v0)      # velocities never change
    # the time step is a float on the device, as in the reference's kernel
    # (euler_kernel.cu: float timestep): 10 v (dt - float(dt)) ~ 1.5e-9
    assert np.max(np.abs(unwrapped(eng) - (ro + io * L))) < 1e-8
    eng.close()


def test_thermostat_arguments_are_checked():
    eng = hg.Engine("dsfloat")
    with pytest.raises(hg.HmdError):
        eng.add_system(hg.system_desc(100, 10.0, integrator="verlet_nvt_hoover", temperature=1.0))  # no frequency
    with pytest.raises(hg.HmdError):
        eng.add_system(hg.system_desc(100, 10.0, integrator="verlet_nvt_boltzmann", temperature=1.0))  # no rate
    eng.close()
    eng = hg.Engine("dsfloat")
    eng.reserve(1 << 14, 4)
    with pytest.raises(hg.HmdError):
        eng.add_system(hg.system_desc(100, 10.0, integrator="euler"))
    eng.close()


def ideal_gas(n, rho, ratios, T, seed):
    """Force-free particles (epsilon = 0) on distinct sites of a simple cubic
    grid in a box of the given aspect ratios; Maxwell-Boltzmann velocities."""
    box = np.asarray(ratios) * (n / rho / np.prod(ratios)) ** (1 / 3)
    m = np.ceil(box * (n / np.prod(box)) ** (1 / 3) * 1.0001).astype(int)
    axes = [(np.arange(k) + 0.5) * (b / k) - 0.5 * b for k, b in zip(m, box)]
    sites = np.stack(np.meshgrid(*axes, indexing="ij"), -1).reshape(-1, 3)
    r = sites[np.random.default_rng(seed).permutation(sites.shape[0])[:n]]
    return r, maxwell_boltzmann(n, T, seed=seed + 1), box


def test_ideal_gas_verlet():
    # test/unit/mdsim/integrators/verlet.cpp:110-170: 1000 free particles,
    # rho = 1, T = 1, dt = 0.001, 1000 NVE steps in a 1 : 2 : 1.01 box
    n, rho, T = 1000, 1.0, 1.0
    r, v, box = ideal_gas(n, rho, [1.0, 2.0, 1.01], T, seed=31)
    eng = hg.Engine("dsfloat")
    # epsilon = 0 and a tiny sigma: no force, and no pair ever close enough
    # for the (zero-weighted) r^-12 term to overflow
    eng.add_system(hg.system_desc(n, box, epsilon=0.0, sigma=0.01, r_cut=2.5, skin=0.5, timestep=0.001))
    eng.commit()
    eng.set("position", r)
    eng.set("velocity", v)
    th0 = eng.thermo()
    eng.step(1000, aux_last=True)
    th = eng.thermo()
    vcm = th["momentum"] / th["mass"]
    assert np.max(np.abs(vcm)) < 1e-12
    assert abs(th["mv2"] - th0["mv2"]) <= 10 * np.finfo(np.float64).eps * th0["mv2"]   # no force: no change
    temp = th["mv2"] / (3 * n)
    volume = np.prod(box)
    press = (th["mv2"] + th["virial"]) / (3 * volume)
    tol = 5 / np.sqrt(n)
    assert abs(temp - T) / T < tol
    assert abs(press / temp / rho - 1.0) < tol
    # ballistic motion: r(t) = r(0) + v t
    np.testing.assert_allclose(eng.get("unwrapped_position"), r + v * 1000 * np.float32(0.001), atol=1e-5)
    eng.close()


def test_andersen_statistics():
    # test/unit/mdsim/integrators/verlet_nvt_andersen.cpp:100-200 (GPU case):
    # 5000 free particles, rho = 0.3, T = 1, collision rate 10, dt = 0.01,
    # 500 time units sampled every round(3 / (rate dt)) = 30 steps
    n, rho, T, rate, dt = 5000, 0.3, 1.0, 10.0, 0.01
    r, v, box = ideal_gas(n, rho, [1.0, 2.0, 1.01], 2.0, seed=41)
    eng = hg.Engine("dsfloat")
    eng.add_system(hg.system_desc(n, box, epsilon=0.0, sigma=0.01, r_cut=2.5, skin=0.5, timestep=dt,
                                  integrator="andersen",
                                  temperature=T, collision_rate=rate, seed=42))
    eng.commit()
    eng.set("position", r)
    eng.set("velocity", v)
    period = int(round(3 / (rate * dt)))
    steps = int(np.ceil(500 / dt))
    eng.step(period * 10)                     # a few periods to thermalise from T = 2
    temps, vcms = [], []
    for _ in range(steps // period):
        eng.step(period)
        th = eng.thermo()
        temps.append(th["mv2"] / (3 * n))
        vcms.append(th["momentum"] / th["mass"])
    temps, vcms = np.array(temps), np.array(vcms)
    c = len(temps)
    # instantaneous values at the end (4.5 sigma)
    assert np.max(np.abs(vcms[-1])) < 4.5 * np.sqrt(T / (n - 1))
    assert abs(temps[-1] - T) / T < 4.5 * np.sqrt(2.0 / (3 * n)) / T
    # averages over the run
    assert np.max(np.abs(vcms.mean(axis=0))) < 4.5 * np.sqrt(T / (n * c - 1))
    assert abs(temps.mean() - T) / T < 4.5 * np.sqrt(2.0 / (3 * n * (c - 1))) / T
    # kinetic specific heat from temperature fluctuations: 3/2
    cv = 1.5 ** 2 * n * temps.var(ddof=1)
    cv_tol = 4.5 * np.sqrt(1.5 * (3 + 6.0 / n) / c) / 1.5
    print("andersen: <T> %.5f, c_V %.4f (tol %.3f), %d samples" % (temps.mean(), cv, cv_tol, c))
    assert abs(cv - 1.5) / 1.5 < cv_tol
    eng.close()
