"""Force accuracy at the benchmark sizes (LJ-1M, KA-64k) against FP64.

Large boxes matter: across the periodic boundary the float difference of two
positions is of order L, and its rounding error grows with L; and the lo
words of a double-single position carry up to ulp(L/2)/2 of it, which the
float hi words alone would drop.  The FP64 reference is evaluated at the
engine's double-single state (hi + lo) in its float box; the error against
FP64 at the float hi words alone (the convention of the reference's GPU
kernels, which read the hi words only) is printed beside it.
Metric: max_i |F_i - F64_i| / max(|F64_i|, F_rms) <= 1e-6.
"""
import numpy as np
import pytest

import halmd_gb300 as hg
import oracle
from _systems import KA_EPS, KA_SIGMA, fcc, maxwell_boltzmann, rel_force_error, state_forces

pytestmark = pytest.mark.gpu

FORCE_TOL = 1e-6


def explain_worst(eng, f, f64, label):
    """Print the pairs near the cut-off of the particle with the largest error."""
    norm = np.linalg.norm(f64, axis=1)
    e = np.linalg.norm(f - f64, axis=1) / np.maximum(norm, np.sqrt(np.mean(norm ** 2)))
    i = int(np.argmax(e))
    r = eng.get("position")
    L = np.array(eng.info().box_f32, dtype=np.float64)
    d = r - r[i]
    d -= L * np.rint(d / L)
    rr = np.sum(d * d, axis=1)
    print("%s worst particle %d: err %.3g, F %s, F64 %s, dF %s" % (label, i, e[i], f[i], f64[i], f[i] - f64[i]))
    for j in np.where((rr > 6.0) & (rr < 6.5))[0]:
        print("   partner %d: rr %.9f" % (j, rr[j]))


def check(eng, species, pot, label):
    eng.force(aux=True)
    f = eng.get("force")
    ref = state_forces(eng, species, pot)
    emax, emed = rel_force_error(f, ref["force"])
    hi = state_forces(eng, species, pot, state=False, aux=False)
    hmax, hmed = rel_force_error(f, hi["force"])
    epot = eng.thermo()["epot"]
    print("%s: force rel err vs FP64 of the dsfloat state: max %.3g median %.3g; "
          "vs FP64 at the float hi words: max %.3g median %.3g; epot rel err %.3g"
          % (label, emax, emed, hmax, hmed, abs(epot - ref["epot"]) / abs(ref["epot"])))
    if emax >= FORCE_TOL:
        explain_worst(eng, f, ref["force"], label)
    assert emax < FORCE_TOL
    assert abs(epot - ref["epot"]) < 1e-6 * abs(ref["epot"])


def test_lj1m_force_accuracy():
    r, L = fcc(64, 0.8442, jitter=0.05, seed=9)
    n = r.shape[0]
    assert n == 1048576
    eng = hg.Engine("dsfloat")
    eng.add_system(hg.system_desc(n, L, r_cut=2.5, truncation="shifted", skin=0.3, timestep=0.002))
    eng.commit()
    eng.set("position", r)
    eng.set("velocity", maxwell_boltzmann(n, 0.722, seed=10))
    eng.step(300)
    check(eng, np.zeros(n), oracle.Potential(1.0, 1.0, 2.5, "shifted"), "LJ-1M")
    eng.close()


def test_ka64k_force_accuracy():
    n, rho = 64000, 1.2
    L = (n / rho) ** (1 / 3)
    rng = np.random.default_rng(64)
    r = rng.uniform(-L / 2, L / 2, size=(n, 3))
    sp = np.zeros(n, dtype=np.uint32)
    sp[rng.permutation(n)[: n // 5]] = 1
    eng = hg.Engine("dsfloat")
    eng.add_system(hg.system_desc(n, L, epsilon=KA_EPS, sigma=KA_SIGMA, r_cut=2.5, truncation="smooth_r4",
                                  smoothing=0.005, skin=0.3, timestep=0.002, integrator="andersen",
                                  temperature=0.7, collision_rate=1.0, seed=3))
    eng.commit()
    eng.set("species", sp)
    eng.set("position", r)
    eng.minimize(steps=1000, step_size=1e-3, max_move=0.05)
    eng.set("velocity", maxwell_boltzmann(n, 0.7, seed=65))
    eng.step(300)
    pot = oracle.Potential(KA_EPS, KA_SIGMA, 2.5 * np.ones((2, 2)), "smooth_r4", h=0.005)
    check(eng, sp, pot, "KA-64k")
    eng.close()


def test_lj1m_energy_drift():
    """NVE energy drift at LJ-1M over 2*10^4 steps, extrapolated linearly to 10^5 steps."""
    r, L = fcc(64, 0.8442, jitter=0.05, seed=9)
    n = r.shape[0]
    eng = hg.Engine("dsfloat")
    eng.add_system(hg.system_desc(n, L, r_cut=2.5, truncation="shifted", skin=0.3, timestep=0.002))
    eng.commit()
    eng.set("position", r)
    eng.set("velocity", maxwell_boltzmann(n, 0.722, seed=10))
    eng.step(2000)                       # let the lattice melt a little before measuring
    t, e = [], []
    for k in range(21):
        if k:
            eng.step(999)
        eng.step(1, aux_last=True)
        th = eng.thermo()
        t.append(k * 1000)
        e.append(0.5 * th["mv2"] + th["epot"])
    e = np.array(e)
    slope = np.polyfit(np.array(t, dtype=float), e, 1)[0]
    drift = abs(slope) * 1e5 / abs(e[0])
    fluct = np.std(e) / abs(e[0])
    print("LJ-1M NVE: E0/n %.6f, drift %.3g per 1e5 steps, fluctuation %.3g" % (e[0] / n, drift, fluct))
    assert drift < 1e-5
    eng.close()


def test_lj1m_precision_variants_against_fp64():
    """LJ-1M in the three precision variants from one start (the dsfloat
    state after 300 steps): float positions, dsfloat positions and the FP64
    variant.  Each variant's force error against FP64 forces of its own state
    (the FP64 engine with the float cut-off test: the same pair set) and its
    energy drift per 1e5 steps against the FP64 run's, fitted over 3000 steps."""
    from _systems import energy_drift
    r, L = fcc(64, 0.8442, jitter=0.05, seed=9)
    n = r.shape[0]
    desc = hg.system_desc(n, L, r_cut=2.5, truncation="shifted", skin=0.3, timestep=0.002)
    eng = hg.Engine("dsfloat")
    eng.add_system(desc)
    eng.commit()
    eng.set("position", r)
    eng.set("velocity", maxwell_boltzmann(n, 0.722, seed=10))
    eng.step(300)
    r0, v0 = eng.get("position"), eng.get("velocity")
    eng.close()

    def start(precision):
        e = hg.Engine(precision)
        e.add_system(desc)
        e.commit()
        e.set("position", r0)
        e.set("velocity", v0)
        return e

    ref = start("double")
    ref.set_option("float_cutoff", 1)
    drift = {}
    for precision in ("float", "dsfloat", "double"):
        e = start(precision)
        if precision != "double":
            e.force()
            ref.set("position", e.get("position"))
            ref.force()
            emax, emed = rel_force_error(e.get("force"), ref.get("force"))
            print("LJ-1M %s: force rel err vs FP64 of its state max %.3g median %.3g" % (precision, emax, emed))
            assert emax < FORCE_TOL
        drift[precision] = energy_drift(e, 3000, 100)
        print("LJ-1M %s: drift %.3g +- %.2g per 1e5 steps, max |dE|/|E| %.3g" % ((precision,) + drift[precision]))
        e.close()
    ref.close()
    for precision in ("float", "dsfloat"):
        assert abs(drift[precision][0]) < 1e-5
        assert abs(drift[precision][0] - drift["double"][0]) < 1e-5
