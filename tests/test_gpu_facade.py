"""A script written against the module-style front end (Lua names) runs the
same kernels as the engine API: identical trajectories and observables."""
import numpy as np
import pytest

import halmd_gb300 as hg
from halmd_gb300 import halmd
import oracle
from _systems import lj_system

pytestmark = pytest.mark.gpu


def test_facade_script_equals_engine_calls():
    r, v, L = lj_system(ncell=6)
    n = r.shape[0]
    halmd.reset()
    box = halmd.mdsim.box(length=[L, L, L])
    particle = halmd.mdsim.particle(dimension=3, particles=n, species=1)
    particle.data["position"] = r
    particle.data["velocity"] = v
    pot = halmd.mdsim.potentials.pair.lennard_jones(epsilon=1, sigma=1).truncate("shifted", cutoff=2.5)
    halmd.mdsim.forces.pair(box=box, particle=particle, potential=pot, neighbour={"skin": 0.3})
    halmd.mdsim.integrators.verlet(box=box, particle=particle, timestep=0.005)
    thermo = halmd.observables.thermodynamics(box=box, group=particle)
    msd = halmd.observables.dynamics.mean_square_displacement(particle=particle)
    blocking = halmd.observables.dynamics.blocking_scheme(max_lag=1.0, every=10, size=4, correlations=[msd])
    seen = []
    halmd.observables.sampler.on_sample(lambda: seen.append((thermo.potential_energy(), thermo.kinetic_energy(),
                                                             thermo.pressure())), every=50)
    halmd.observables.sampler.run(200)
    blocking.finalise()
    got_r = particle.data["position"]
    got_msd = blocking.result(0)

    # the same work through the engine API: the front end steps from sample to sample
    eng = hg.Engine("dsfloat")
    eng.add_system(hg.system_desc(n, L, r_cut=2.5, truncation="shifted", skin=0.3, timestep=0.005))
    eng.commit()
    eng.set("position", r)
    eng.set("velocity", v)
    dyn = hg.Dynamics(eng, 1.0, 10 * 0.005, block_size=4, shift=2, separation=4)
    k = dyn.add_msd(0, n)
    dyn.sample()
    eng.force(aux=True)
    ref = []

    def record():
        t = eng.thermo()
        ref.append((t["epot"] / n, 0.5 * t["mv2"] / n,
                    n / L ** 3 * (t["mv2"] / n / 3 + t["virial"] / n / 3)))
    record()
    for _ in range(20):
        eng.step(10, aux_last=True)
        dyn.sample()
        if eng.info().step % 50 == 0:
            record()
    dyn.finalise()
    assert np.array_equal(got_r, eng.get("position"))
    assert len(seen) == len(ref) == 5
    np.testing.assert_allclose(np.array(seen), np.array(ref), rtol=1e-14)
    mean, err, cnt = dyn.result(k)
    np.testing.assert_array_equal(got_msd[0], mean)
    np.testing.assert_array_equal(got_msd[2], cnt)
    # the per-particle thermodynamic formulas of the reference
    t = eng.thermo()
    vv = eng.get("velocity")
    assert abs(thermo.kinetic_energy() - 0.5 * np.sum(vv * vv) / n) < 1e-12
    assert abs(thermo.temperature() - 2 * thermo.kinetic_energy() / 3) < 1e-15
    assert abs(thermo.potential_energy() - t["epot"] / n) < 1e-15
    dyn.close()
    eng.close()
    halmd.reset()


def test_lattice_and_boltzmann_set_up():
    # positions.lattice and velocities.boltzmann on the device against the oracle
    import halmd_gb300 as hg
    n, box = 3000, np.array([12.0, 20.0, 12.5])
    eng = hg.Engine("dsfloat")
    eng.add_system(hg.system_desc(n, box, r_cut=2.5, skin=0.3, timestep=0.001))
    eng.commit()
    eng.set("position", np.zeros((n, 3)) + 0.1)
    eng.lattice(slab=[1.0, 0.8, 1.0])
    ref, sites = oracle.lattice(n, box, [1.0, 0.8, 1.0])
    np.testing.assert_allclose(eng.get("position"), ref, rtol=0, atol=1e-12)
    assert np.all(eng.get("image") == 0)
    mass = np.linspace(0.5, 2.0, n).astype(np.float32).astype(np.float64)   # the engine keeps floats
    eng.set("mass", mass)
    eng.boltzmann(1.3, seed=11)
    v = eng.get("velocity")
    np.testing.assert_allclose(v, oracle.boltzmann(mass, 1.3, 11), rtol=0, atol=1e-12)
    assert np.max(np.abs((mass[:, None] * v).sum(axis=0))) < 1e-9
    temp = np.sum(mass[:, None] * v * v) / (3 * n)
    assert abs(temp - 1.3) / 1.3 < 4.5 * np.sqrt(2.0 / (3 * n))
    eng.step(20)
    assert np.all(np.isfinite(eng.get("position")))
    eng.close()


def test_facade_lattice_boltzmann_script():
    from halmd_gb300 import halmd
    halmd.reset()
    box = halmd.mdsim.box(length=[16.796, 16.796, 16.796])
    p = halmd.mdsim.particle(particles=4000)
    halmd.mdsim.positions.lattice(box=box, particle=p).set()
    halmd.mdsim.velocities.boltzmann(particle=p, temperature=1.5).set()
    pot = halmd.mdsim.potentials.pair.lennard_jones().truncate(cutoff=2.5)
    halmd.mdsim.forces.pair(box=box, particle=p, potential=pot, neighbour={"skin": 0.3})
    halmd.mdsim.integrators.verlet(box=box, particle=p, timestep=0.005)
    r = p.get("position")
    ref, _ = oracle.lattice(4000, [16.796] * 3)
    np.testing.assert_allclose(r, ref, atol=1e-12)
    thermo = halmd.observables.thermodynamics(box=box, group=p)
    assert abs(thermo.temperature() - 1.5) < 4.5 * 1.5 * np.sqrt(2.0 / 12000)
    halmd.observables.sampler.run(10)
    assert abs(thermo.center_of_mass_velocity()).max() < 1e-9
    halmd.reset()


def test_phase_space_acquire_and_set():
    from halmd_gb300 import halmd
    halmd.reset()
    box = halmd.mdsim.box(length=[12.0, 12.0, 12.0])
    p = halmd.mdsim.particle(particles=500, species=2)
    halmd.mdsim.positions.lattice(box=box, particle=p).set()
    halmd.mdsim.velocities.boltzmann(particle=p, temperature=1.0, seed=3).set()
    pot = halmd.mdsim.potentials.pair.lennard_jones(epsilon=[[1, 1.5], [1.5, 0.5]]).truncate(cutoff=2.5)
    halmd.mdsim.forces.pair(box=box, particle=p, potential=pot)
    halmd.mdsim.integrators.verlet(box=box, particle=p, timestep=0.002)
    ps = halmd.observables.phase_space(box=box, group=p)
    s0 = ps.acquire()
    halmd.observables.sampler.run(50)
    s1 = ps.acquire()
    assert not np.array_equal(s0["position"], s1["position"])
    ps.set(s0)                                   # back to the first sample
    s2 = ps.acquire()
    for name in ("position", "velocity", "species", "mass"):
        np.testing.assert_array_equal(s2[name], s0[name])
    halmd.reset()


def test_non_finite_positions_are_rejected_unchanged():
    # the check runs on the device copy before anything is stored
    import halmd_gb300 as hg
    r, v, L = lj_system(ncell=4)
    eng = hg.Engine("dsfloat")
    eng.add_system(hg.system_desc(r.shape[0], L, r_cut=2.5, skin=0.3, timestep=0.001))
    eng.commit()
    eng.set("position", r)
    before = eng.get("position")
    bad = r.copy()
    bad[17, 1] = np.nan
    with pytest.raises(hg.HmdError):
        eng.set("position", bad)
    bad[17, 1] = np.inf
    with pytest.raises(hg.HmdError):
        eng.set("position", bad)
    np.testing.assert_array_equal(eng.get("position"), before)
    out = np.empty_like(before)
    assert eng.get("position", out=out) is out and np.array_equal(out, before)
    eng.close()


def _ka_two_instance_script(r, v, sp, L, coupled):
    """The KA mixture either as one instance of two species or as two
    instances A and B wired by forces for every ordered pair
    (test/integration/modularity/two_particles.lua)."""
    halmd.reset()
    box = halmd.mdsim.box(length=[L, L, L])
    pot = halmd.mdsim.potentials.pair.lennard_jones(epsilon=[[1, 1.5], [1.5, 0.5]], sigma=[[1, 0.8], [0.8, 0.88]])
    pot = pot.truncate("smooth_r4", cutoff=2.5, h=0.005)
    if not coupled:
        p = halmd.mdsim.particle(particles=r.shape[0], species=2)
        p.data["species"], p.data["position"], p.data["velocity"] = sp, r, v
        halmd.mdsim.forces.pair(box=box, particle=p, potential=pot, neighbour={"skin": 0.3})
        halmd.mdsim.integrators.verlet(box=box, particle=p, timestep=0.002)
        return [p], box
    parts = []
    for label, sel in (("A", sp == 0), ("B", sp == 1)):
        p = halmd.mdsim.particle(particles=int(sel.sum()), species=2, label=label)
        p.data["species"], p.data["position"], p.data["velocity"] = sp[sel], r[sel], v[sel]
        parts.append(p)
    for p1 in parts:
        for p2 in parts:
            halmd.mdsim.forces.pair(box=box, particle=[p1, p2], potential=pot, neighbour={"skin": 0.3})
    for p in parts:
        halmd.mdsim.integrators.verlet(box=box, particle=p, timestep=0.002)
    return parts, box


def test_two_coupled_instances_equal_one_instance_of_two_species():
    from _systems import ka_system
    r, v, sp, L = ka_system(ncell=6)
    order = np.argsort(sp, kind="stable")          # A particles first, then B
    r, v, sp = r[order], v[order], sp[order]
    (one,), box = _ka_two_instance_script(r, v, sp, L, coupled=False)
    t1 = halmd.observables.thermodynamics(box=box, group=one)
    halmd.observables.sampler.run(150)
    ref_r, ref_v, ref_epot = one.data["position"], one.data["velocity"], t1.potential_energy() * r.shape[0]
    parts, box = _ka_two_instance_script(r, v, sp, L, coupled=True)
    thermos = [halmd.observables.thermodynamics(box=box, group=p) for p in parts]
    halmd.observables.sampler.run(150)
    got_r = np.concatenate([p.data["position"] for p in parts])
    got_v = np.concatenate([p.data["velocity"] for p in parts])
    assert np.array_equal(got_r, ref_r) and np.array_equal(got_v, ref_v)
    epot = sum(t.potential_energy() * p.nparticle for t, p in zip(thermos, parts))
    assert abs(epot - ref_epot) < 1e-9 * abs(ref_epot)
    halmd.reset()
