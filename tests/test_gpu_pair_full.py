"""GPU parity of the untruncated pair force (pair_full) against the FP64 oracle.

mdsim/gpu/forces/pair_full_kernel.cuh: every pair of the system with the
minimum image, no cutoff, no neighbour list; the aux weight is halved
(pair_full.hpp:249-252).  The reference's force constructor picks this
module when the potential has no r_cut (forces/pair.lua.in:78-83).  The
oracle's all-pairs sum is host/forces/pair_full.hpp:229-270 in FP64.
"""
import numpy as np
import pytest

import halmd_gb300 as hg
from halmd_gb300 import halmd
import oracle
from _systems import KA_EPS, KA_SIGMA, ka_system, lj_system, rel_force_error, state_forces

pytestmark = pytest.mark.gpu

# per-particle force error, max_i |F_i - F64_i| / max(|F64_i|, F_rms): the
# Lennard-Jones pair arithmetic is compensated as in the list kernels; the
# other potentials evaluate their pair values in plain FP32
LJ_TOL = 1e-6
POT_TOL = 2e-5

PARAMS = {
    "lennard_jones": {},
    "mie": dict(index_repulsion=[[12, 10], [10, 14]], index_attraction=[[6, 6], [6, 8]]),
    "morse": dict(r_min=[[1.1, 0.9], [0.9, 1.0]], distortion=[[1.0, 1.41], [1.41, 1.5]]),
    "power_law": dict(index=[[12, 9], [9, 6]]),
}


def full_desc(n, L, potential="lennard_jones", dt=0.001):
    return hg.system_desc(n, L, epsilon=KA_EPS, sigma=KA_SIGMA, r_cut=0.0, truncation="none", timestep=dt,
                          potential=potential, **PARAMS[potential])


def full_engine(potential="lennard_jones", ncell=5, dt=0.001):
    r, v, sp, L = ka_system(ncell=ncell)
    eng = hg.Engine("dsfloat")
    eng.add_system(full_desc(r.shape[0], L, potential, dt))
    eng.commit()
    eng.set("species", sp)
    eng.set("position", r)
    eng.set("velocity", v)
    return eng, r, v, sp, L


def oracle_reference(eng, sp, potential):
    pot = oracle.Potential(KA_EPS, KA_SIGMA, 1.0, "none", potential=potential, **PARAMS[potential])
    return state_forces(eng, sp, pot)


@pytest.mark.parametrize("potential", ["lennard_jones", "mie", "morse", "power_law"])
def test_pair_full_force_parity(potential):
    eng, r, v, sp, L = full_engine(potential)
    n = r.shape[0]
    eng.force(aux=True)
    f = eng.get("force")
    en = eng.get("potential_energy")
    st = eng.get("stress_pot")
    ref = oracle_reference(eng, sp, potential)
    assert ref["npairs"] == n * (n - 1) // 2   # every pair once
    tol = LJ_TOL if potential == "lennard_jones" else POT_TOL
    emax, emed = rel_force_error(f, ref["force"])
    print("%s force rel err max %.3g median %.3g" % (potential, emax, emed))
    assert emax < tol
    erms = np.sqrt(np.mean(ref["en_pot"] ** 2))
    assert np.max(np.abs(en - ref["en_pot"]) / np.maximum(np.abs(ref["en_pot"]), erms)) < tol
    assert abs(en.sum() - ref["epot"]) < tol * abs(ref["epot"])
    srms = np.sqrt(np.mean(ref["stress"] ** 2))
    assert np.max(np.abs(st - ref["stress"])) < 10 * tol * srms
    th = eng.thermo()
    assert abs(th["epot"] - ref["epot"]) < tol * abs(ref["epot"])
    assert abs(th["virial"] - ref["virial"]) < tol * abs(ref["virial"])
    eng.close()


def test_pair_full_trajectory_against_fp64_host_backend():
    eng, r, v, sp, L = full_engine(dt=0.001)
    n = r.shape[0]
    nsteps = 50
    eng.step(nsteps)
    Lf = float(np.float32(L))
    pot = oracle.Potential(KA_EPS, KA_SIGMA, 1.0, "none")
    r_ref, v_ref, img_ref, st = oracle.md_run(r, v, sp, np.ones(n), [Lf] * 3, pot, 0.3, 0.001, nsteps)
    ref = r_ref + img_ref * Lf
    got = eng.get("unwrapped_position")
    assert np.max(np.abs(got - ref)) < 1e-5
    np.testing.assert_allclose(eng.get("velocity"), v_ref, atol=1e-4)
    assert eng.info().rebuilds == 0   # no list, so nothing is ever rebuilt
    eng.close()


def test_pair_full_beside_truncated_system_is_unchanged():
    # an untruncated system and a truncated one in one engine advance exactly
    # as in engines of their own
    r1, v1, sp1, L1 = ka_system(ncell=5)
    r2, v2, L2 = lj_system(ncell=6)
    d1 = full_desc(r1.shape[0], L1)
    d2 = hg.system_desc(r2.shape[0], L2, r_cut=2.5, truncation="shifted", skin=0.3, timestep=0.001)

    def engine(descs):
        eng = hg.Engine("dsfloat")
        for d in descs:
            eng.add_system(d)
        eng.commit()
        return eng

    both, only1, only2 = engine([d1, d2]), engine([d1]), engine([d2])
    for eng, s, (r, v, sp) in ((both, 0, (r1, v1, sp1)), (both, 1, (r2, v2, None)), (only1, 0, (r1, v1, sp1)),
                               (only2, 0, (r2, v2, None))):
        if sp is not None:
            eng.set("species", sp, s)
        eng.set("position", r, s)
        eng.set("velocity", v, s)
    for eng in (both, only1, only2):
        eng.step(40)
    for name in ("position", "velocity", "image"):
        assert np.array_equal(both.get(name, 0), only1.get(name, 0)), name
        assert np.array_equal(both.get(name, 1), only2.get(name, 0)), name
    assert only2.info().rebuilds > 0
    for eng in (both, only1, only2):
        eng.close()


def test_pair_full_has_no_neighbour_list_and_no_capacity_mode():
    eng, *_ = full_engine()
    with pytest.raises(hg.HmdError):
        eng.neighbour_lists()
    eng.close()
    r, v, sp, L = ka_system(ncell=4)
    cap = hg.Engine("dsfloat")
    cap.reserve(1 << 16, 8)
    with pytest.raises(hg.HmdError):
        cap.add_system(full_desc(r.shape[0], L))
    cap.close()


def test_facade_untruncated_potential_selects_pair_full():
    r, v, L = lj_system(ncell=4)
    n = r.shape[0]
    halmd.reset()
    box = halmd.mdsim.box(length=[L, L, L])
    particle = halmd.mdsim.particle(dimension=3, particles=n, species=1)
    particle.data["position"] = r
    particle.data["velocity"] = v
    pot = halmd.mdsim.potentials.pair.lennard_jones(epsilon=1, sigma=1)   # no :truncate
    halmd.mdsim.forces.pair(box=box, particle=particle, potential=pot)
    halmd.mdsim.integrators.verlet(box=box, particle=particle, timestep=0.002)
    halmd.observables.sampler.run(30)
    got = particle.data["position"]
    halmd.reset()

    eng = hg.Engine("dsfloat")
    eng.add_system(hg.system_desc(n, L, r_cut=0.0, truncation="none", timestep=0.002))
    eng.commit()
    eng.set("position", r)
    eng.set("velocity", v)
    eng.step(30)
    assert np.array_equal(got, eng.get("position"))
    eng.close()
