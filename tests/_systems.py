"""Seeded synthetic systems shared by the tests (inputs only)."""
import numpy as np

import oracle

KA_EPS = [[1.0, 1.5], [1.5, 0.5]]
KA_SIGMA = [[1.0, 0.8], [0.8, 0.88]]


def fcc(ncell, rho, jitter=0.0, seed=0):
    n = 4 * ncell ** 3
    L = ncell * (4.0 / rho) ** (1.0 / 3.0)
    r = oracle.fcc_lattice(ncell, L)
    if jitter:
        r = r + np.random.default_rng(seed).uniform(-jitter, jitter, size=(n, 3))
    return r, L


def maxwell_boltzmann(n, T, seed=1, mass=None):
    rng = np.random.default_rng(seed)
    v = rng.normal(0.0, np.sqrt(T), size=(n, 3))
    v -= v.mean(axis=0)
    v *= np.sqrt(3 * (n - 1) * T / np.sum(v * v)) if n > 1 else 1.0
    return v


def lj_system(ncell=10, rho=0.8442, T=1.5, jitter=0.12, seed=3):
    r, L = fcc(ncell, rho, jitter, seed)
    v = maxwell_boltzmann(r.shape[0], T, seed + 1)
    return r, v, L


def ka_system(ncell=8, rho=1.2, T=0.7, jitter=0.05, seed=5):
    r, L = fcc(ncell, rho, jitter, seed)
    n = r.shape[0]
    species = np.zeros(n, dtype=np.uint32)
    species[np.random.default_rng(seed).permutation(n)[: n // 5]] = 1
    v = maxwell_boltzmann(n, T, seed + 1)
    return r, v, species, L


def rel_force_error(f, f64):
    """max_i |F_i - F64_i| / max(|F64_i|, F_rms) and its median."""
    norm = np.linalg.norm(f64, axis=1)
    frms = np.sqrt(np.mean(norm ** 2))
    e = np.linalg.norm(f - f64, axis=1) / np.maximum(norm, frms)
    return float(e.max()), float(np.median(e))


def state_forces(eng, species, pot, s=0, state=True, aux=True):
    """FP64 forces of an engine's phase-space state.

    The positions are hi + lo of every slot (the double-single state; with
    state=False the float hi words alone, the convention of the reference's
    GPU kernels), the box is the engine's float box (the integrator wraps
    with it, as box_kernel.cuh does), and the pair set is the one the
    kernels use: r^2 < r_c^2 decided in float on the hi words, the list
    criterion.  Returns the oracle's dict.
    """
    Lf = np.array(eng.info(s).box_f32, dtype=np.float32)
    pos4 = eng.get_raw("position_hi", s)[eng.get("reverse_id", s)]
    r = eng.get("position", s) if state else pos4[:, :3].astype(np.float64)
    return oracle.forces(r, species, Lf.astype(np.float64), pot, pos4=pos4, Lf=Lf, aux=aux)


def energy_drift(eng, steps, every, s=0):
    """Energy E = K + U sampled every `every` steps over `steps` steps:
    returns (drift |E| per 1e5 steps from a linear fit, its standard error,
    max |E(t) - E(0)| / |E(0)|)."""
    t, e = [], []
    for k in range(steps // every + 1):
        if k:
            eng.step(every - 1)
        eng.step(1, aux_last=True)
        th = eng.thermo(s)
        t.append(k * every)
        e.append(0.5 * th["mv2"] + th["epot"])
    t, e = np.asarray(t, dtype=float), np.asarray(e)
    (slope, _), cov = np.polyfit(t, e, 1, cov=True)
    scale = 1e5 / abs(e[0])
    return slope * scale, np.sqrt(cov[0, 0]) * scale, float(np.max(np.abs(e - e[0])) / abs(e[0]))
