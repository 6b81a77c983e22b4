"""The FP64 steepest-descent oracle relaxes random positions (CPU only)."""
import numpy as np

import oracle


def test_descent_relaxes_random_positions():
    n, rho = 500, 0.8
    L = (n / rho) ** (1 / 3)
    r = np.random.default_rng(11).uniform(-L / 2, L / 2, size=(n, 3))
    pot = oracle.Potential(1.0, 1.0, 2.5, "shifted")
    e0 = oracle.forces(r, np.zeros(n), np.full(3, L), pot)["epot"]
    r1, img1, s1 = oracle.minimize(r, np.zeros(n), np.full(3, L), pot, skin=0.3, nsteps=50)
    r2, img2, s2 = oracle.minimize(r1, np.zeros(n), np.full(3, L), pot, skin=0.3, nsteps=250, image=img1)
    assert e0 > s1["epot"] > s2["epot"]
    assert s2["epot"] / n < -4.0          # a relaxed LJ liquid, no overlaps left
    assert s2["fmax"] < s1["fmax"]
    # positions stay in the box; unwrapped positions moved by at most 300 * max_move
    assert np.all(np.abs(r2) <= L / 2 + 1e-12)
    moved = np.linalg.norm(r2 + img2 * L - r, axis=1)
    assert moved.max() <= 300 * 0.05 + 1e-9
