"""GPU parity of the mie, morse and power_law pair forces against the FP64 oracle.

The other potentials of mdsim/gpu/potentials/pair/ (mie.cpp, morse.cpp,
power_law.cpp) with the sharp / shifted / smooth_r4 / force_shifted
truncations, through the C ABI.  Their pair values are plain FP32 (as the
reference's GPU kernels), so the bar is looser than for Lennard-Jones.
"""
import numpy as np
import pytest

import halmd_gb300 as hg
import oracle
from _systems import KA_EPS, KA_SIGMA, ka_system, rel_force_error, state_forces

pytestmark = pytest.mark.gpu

# per-particle force error bound, max_i |F_i - F64_i| / max(|F64_i|, F_rms),
# and the same bound for the per-particle potential energy
POT_TOL = 2e-5
# smooth_r4 multiplies the float error of U(r) - U(r_c), about
# eps_f32 |U(r_c)|, by ~4/h near r_c; with h = 0.005 and a Morse well still
# at -0.4 eps at r_c that is ~1e-5 of F_rms (measured 1.7e-5)
SMOOTH_TOL = 5e-5

PARAMS = {
    "mie": dict(index_repulsion=[[12, 10], [10, 14]], index_attraction=[[6, 6], [6, 8]]),
    "morse": dict(r_min=[[1.1, 0.9], [0.9, 1.0]], distortion=[[1.0, 1.41], [1.41, 1.5]]),
    "power_law": dict(index=[[12, 9], [9, 6]]),
}


def pot_engine(potential, truncation, lanes=0, block=0, precision="dsfloat"):
    r, v, sp, L = ka_system(ncell=6)
    n = r.shape[0]
    eng = hg.Engine(precision)
    eng.add_system(hg.system_desc(n, L, epsilon=KA_EPS, sigma=KA_SIGMA, r_cut=2.5, truncation=truncation,
                                  smoothing=0.005, skin=0.3, timestep=0.001, potential=potential,
                                  **PARAMS[potential]))
    eng.commit()
    if lanes:
        eng.set_option("force_lanes", lanes)
        eng.set_option("list_block", block)
    eng.set("species", sp)
    eng.set("position", r)
    eng.set("velocity", v)
    return eng, sp


def oracle_reference(eng, sp, potential, truncation):
    pot = oracle.Potential(KA_EPS, KA_SIGMA, 2.5, truncation, h=0.005, potential=potential, **PARAMS[potential])
    return state_forces(eng, sp, pot)


@pytest.mark.parametrize("truncation", ["sharp", "shifted", "smooth_r4", "force_shifted"])
@pytest.mark.parametrize("potential", ["mie", "morse", "power_law"])
def test_potential_force_parity(potential, truncation):
    eng, sp = pot_engine(potential, truncation)
    eng.force(aux=True)
    f = eng.get("force")
    en = eng.get("potential_energy")
    ref = oracle_reference(eng, sp, potential, truncation)
    emax, emed = rel_force_error(f, ref["force"])
    print("%s/%s force rel err max %.3g median %.3g" % (potential, truncation, emax, emed))
    tol = SMOOTH_TOL if truncation == "smooth_r4" else POT_TOL
    assert emax < tol
    erms = np.sqrt(np.mean(ref["en_pot"] ** 2))
    eerr = np.max(np.abs(en - ref["en_pot"]) / np.maximum(np.abs(ref["en_pot"]), erms))
    assert eerr < tol, eerr
    eng.step(20)
    assert np.all(np.isfinite(eng.get("position")))
    eng.close()


@pytest.mark.parametrize("lanes,block", [(1, 4), (2, 8), (4, 8), (8, 8)])
def test_potential_force_shapes_agree(lanes, block):
    # every force-kernel shape, including one entry per load (paired with a masked entry)
    eng, sp = pot_engine("mie", "shifted", lanes, block)
    eng.force()
    f = eng.get("force")
    ref = oracle_reference(eng, sp, "mie", "shifted")
    emax, _ = rel_force_error(f, ref["force"])
    assert emax < POT_TOL
    eng.close()


def test_mie_rejects_bad_indices():
    # mdsim/host/potentials/pair/mie.cpp:72-83 (std::logic_error)
    eng = hg.Engine("dsfloat")
    for m, n in ((13, 6), (12, 7), (6, 6)):
        with pytest.raises(hg.HmdError):
            eng.add_system(hg.system_desc(100, 10.0, potential="mie", index_repulsion=m, index_attraction=n))
    with pytest.raises(ValueError):
        hg.system_desc(100, 10.0, potential="morse")   # r_min is required
    eng.close()
