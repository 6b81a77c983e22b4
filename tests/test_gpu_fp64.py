"""The FP64 variant of the step (HMD_PRECISION_DOUBLE, kernels_fp64.cu)
against the FP64 oracle: forces at the engine's state and a short
trajectory of the host backend's Verlet integrator from the same start.  It
is the reference run against which the float and dsfloat engines' energy
drift is measured."""
import numpy as np
import pytest

import halmd_gb300 as hg
import oracle
from _systems import KA_EPS, KA_SIGMA, ka_system, lj_system, rel_force_error

pytestmark = pytest.mark.gpu


def _engine(desc, r, v, sp=None):
    eng = hg.Engine("double")
    eng.add_system(desc)
    eng.commit()
    if sp is not None:
        eng.set("species", sp)
    eng.set("position", r)
    eng.set("velocity", v)
    return eng


@pytest.mark.parametrize("trunc", ["shifted", "smooth_r4", "force_shifted", "sharp"])
def test_fp64_forces_match_oracle(trunc):
    r, v, sp, L = ka_system(ncell=6)
    eng = _engine(hg.system_desc(r.shape[0], L, epsilon=KA_EPS, sigma=KA_SIGMA, r_cut=2.5, truncation=trunc,
                                 smoothing=0.005, skin=0.3, timestep=0.002), r, v, sp)
    eng.step(20)
    eng.force(aux=True)
    Lf = np.array(eng.info().box_f32, dtype=np.float64)
    pot = oracle.Potential(KA_EPS, KA_SIGMA, 2.5, trunc, h=0.005)
    ref = oracle.forces(eng.get("position"), sp, Lf, pot)
    emax, _ = rel_force_error(eng.get("force"), ref["force"])
    # the float copy of the force rounds once; the double force drives the integrator
    assert emax < 1e-6
    th = eng.thermo()
    assert abs(th["epot"] - ref["epot"]) < 1e-7 * abs(ref["epot"])
    eng.close()


def test_fp64_trajectory_matches_host_backend():
    r, v, L = lj_system(ncell=6, T=1.5)
    n = r.shape[0]
    eng = _engine(hg.system_desc(n, L, r_cut=2.5, truncation="shifted", skin=0.3, timestep=0.005), r, v)
    Lf = np.array(eng.info().box_f32, dtype=np.float64)
    r0, v0 = eng.get("position"), eng.get("velocity")
    eng.step(100)
    pot = oracle.Potential(1.0, 1.0, 2.5, "shifted")
    rr, vv, im, _ = oracle.md_run(r0, v0, np.zeros(n, dtype=np.uint32), np.ones(n), Lf, pot, 0.3, 0.005, 100)
    got = eng.get("unwrapped_position")
    ref = rr + im * Lf
    assert np.max(np.abs(got - ref)) < 1e-9
    assert np.max(np.abs(eng.get("velocity") - vv)) < 1e-8
    eng.close()


def test_fp64_takes_lennard_jones_and_verlet_only():
    eng = hg.Engine("double")
    with pytest.raises(hg.HmdError):
        eng.add_system(hg.system_desc(100, 10.0, r_cut=2.5, integrator="andersen", temperature=1.0,
                                      collision_rate=1.0))
    with pytest.raises(hg.HmdError):
        eng.add_system(hg.system_desc(100, 10.0, potential="power_law", r_cut=2.5))
    eng.close()
