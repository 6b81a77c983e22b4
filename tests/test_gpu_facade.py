"""A script written against the module-style front end (Lua names) runs the
same kernels as the engine API: identical trajectories and observables."""
import numpy as np
import pytest

import halmd_gb300 as hg
from halmd_gb300 import halmd
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
