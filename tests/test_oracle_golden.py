"""Pin the CPU oracle against the reference's own golden vectors (no GPU).

Fixtures come from tests/golden/make_golden.py: the (r, fval, U) tables of the
reference's unit tests and outputs of the reference's own header-only
routines (Hilbert map, DSFUN) compiled from its source tree.
"""
import struct

import numpy as np
import pytest

import oracle

EPS64 = np.finfo(np.float64).eps


@pytest.mark.parametrize("trunc", ["sharp", "shifted", "force_shifted", "smooth_r4"])
def test_lj_tables(golden, trunc):
    g = golden("lj_tables.json")
    pot = oracle.Potential(g["epsilon"], g["sigma"], g["r_cut_sigma"], trunc, h=g["h"])
    tol = g["tolerance_eps_double"] * EPS64
    for pair, (a, b) in {"aa": (0, 0), "ab": (0, 1), "bb": (1, 1)}.items():
        for r, fval, en in g["tables"][trunc][pair]:
            f, e = pot(r * r, a, b)
            # BOOST_CHECK_CLOSE_FRACTION semantics: |x-y| <= tol*|y| (exact zeros compare absolutely)
            assert abs(f - fval) <= tol * abs(fval) or (fval == 0 and abs(f) < 1e-30), (trunc, pair, r, f, fval)
            assert abs(e - en) <= tol * abs(en) or (en == 0 and abs(e) < 1e-12), (trunc, pair, r, e, en)


# tolerances of the reference's host tests, in units of double epsilon:
# mie.cpp:126 (6), morse.cpp:142-184 (fval 2x: 4 / 5 / 8; U: 2 / 2.5 / 4),
# power_law.cpp:132-172 (1 + n/2)
def _other_tolerance(pot, pair, g, quantity):
    if pot == "mie":
        return 6
    if pot == "morse":
        k = {"aa": 2, "ab": 2.5, "bb": 4}[pair]
        return 2 * k if quantity == "fval" else k
    a, b = {"aa": (0, 0), "ab": (0, 1), "bb": (1, 1)}[pair]
    return 1 + g["index"][a][b] // 2


@pytest.mark.parametrize("pot", ["mie", "morse", "power_law"])
def test_other_potential_tables(golden, pot):
    g = golden("other_potential_tables.json")[pot]
    kw = {}
    if pot == "mie":
        kw = dict(index_repulsion=g["index_m"], index_attraction=g["index_n"])
    elif pot == "morse":
        kw = dict(r_min=g["r_min"], distortion=g["distortion"])
    else:
        kw = dict(index=g["index"])
    P = oracle.Potential(g["epsilon"], g["sigma"], g["r_cut_sigma"], g["truncation"], potential=pot, **kw)
    for pair, (a, b) in {"aa": (0, 0), "ab": (0, 1), "bb": (1, 1)}.items():
        for r, fval, en in g["tables"][pair]:
            f, e = P(r * r, a, b)
            tf = _other_tolerance(pot, pair, g, "fval") * EPS64
            te = _other_tolerance(pot, pair, g, "en") * EPS64
            # BOOST_CHECK_CLOSE_FRACTION; exact zeros of the tables compare absolutely
            assert abs(f - fval) <= tf * abs(fval) or (fval == 0 and abs(f) < 1e-14), (pot, pair, r, f, fval)
            assert abs(e - en) <= te * abs(en) or (en == 0 and abs(e) < 1e-14), (pot, pair, r, e, en)


def test_mie_rejects_bad_indices():
    # mdsim/host/potentials/pair/mie.cpp:72-83: odd indices, m <= n
    for m, n in ((13, 6), (12, 7), (6, 6), (4, 6)):
        with pytest.raises(ValueError):
            oracle.Potential(1.0, 1.0, 2.5, potential="mie", index_repulsion=m, index_attraction=n)


def test_smooth_r4_near_cutoff(golden):
    g = golden("smooth_r4_tables.json")
    pot = oracle.Potential(g["epsilon"], g["sigma"], g["r_cut_sigma"], "smooth_r4", h=g["h"])
    rcut = pot.r_cut
    for pair, (a, b), k, kf in (("aa", (0, 0), 8, 1), ("ab", (0, 1), 8, 1), ("bb", (1, 1), 9, 2)):
        rc = rcut[a, b]
        for r, fval, en in g["tables"][pair]:
            f, e = pot(r * r, a, b)
            tol = k * EPS64 * (1 + rc / (rc - r))
            assert abs(f - fval) <= kf * tol * abs(fval), (pair, r, f, fval)
            assert abs(e - en) <= tol * abs(en), (pair, r, e, en)


def test_accumulator(golden):
    g = golden("accumulator.json")
    s = oracle.accumulate(g["values"])
    assert s["count"] == g["count"]
    for key in ("mean", "variance", "sigma", "error_of_mean", "sum"):
        assert abs(s[key] - g[key]) <= g["tolerance"] * abs(g[key])


def test_hilbert_map_matches_reference(golden):
    g = golden("hilbert_keys.json")
    for case in g["cases"]:
        pts = np.asarray(case["points"], dtype=np.float32)
        keys = oracle.hilbert_map_unit(pts, case["depth"])
        assert keys.tolist() == case["keys"], case["depth"]


def _f(u):
    return struct.unpack("<f", struct.pack("<I", u))[0]


@pytest.mark.parametrize("op", ["add", "sub", "mul"])
def test_dsfun_matches_reference(golden, op):
    rows = np.asarray(golden("dsfun.json")[op], dtype=np.uint64).astype(np.uint32)
    a = rows[:, 0:2].copy().view(np.float32)
    b = rows[:, 2:4].copy().view(np.float32)
    c = oracle.dsfun(op, a, b)
    assert np.array_equal(c.view(np.uint32), rows[:, 4:6])


def test_philox_known_answers():
    # Random123 known-answer vectors for philox4x32-10
    cases = [
        ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
        ((0xFFFFFFFF,) * 4, (0xFFFFFFFF, 0xFFFFFFFF), (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
        ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
         (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
    ]
    for ctr, key, want in cases:
        assert oracle.philox4x32_10(ctr, key).tolist() == list(want)


def test_lattice_restatement():
    # mdsim/host/positions/lattice.cpp:63-175: n = 4 k^3 in a cube fills k^3
    # cells of edge L / k exactly; other counts leave vacancies spread evenly
    k, L = 6, 10.0
    r, sites = oracle.lattice(4 * k ** 3, [L, L, L])
    assert sites == 4 * k ** 3
    a = L / k
    assert np.allclose(r.min(axis=0), -L / 2 + a / 4) and np.allclose(r.max(axis=0), L / 2 - a / 4)
    d = np.linalg.norm(r[None, :40] - r[:40, None], axis=-1) + np.eye(40) * 1e9
    assert np.isclose(d.min(), a / np.sqrt(2))
    r, sites = oracle.lattice(1000, [7.9, 15.8, 7.99], slab=[1.0, 0.5, 1.0])
    assert sites >= 1000 and np.unique(r, axis=0).shape[0] == 1000
    assert np.all(np.abs(r[:, 1]) <= 15.8 * 0.25)
