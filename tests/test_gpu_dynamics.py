"""GPU parity of the dynamic correlations (MSD, ISF) on the blocking-scheme grid.

The engine samples unwrapped positions and density modes on the device; the
expected values come from the oracle's FP64 MSD / density modes / ISF fed with
the same positions, driven by a plain-Python restatement of the reference's
blocking scheme (oracle/blocking.py).
"""
import numpy as np
import pytest

import halmd_gb300 as hg
import oracle
from oracle.blocking import BlockingScheme
from _systems import lj_system

pytestmark = pytest.mark.gpu


def test_msd_isf_blocking_scheme():
    r, v, L = lj_system(ncell=5, T=1.2)
    n = r.shape[0]
    dt = 0.005
    eng = hg.Engine("dsfloat")
    eng.add_system(hg.system_desc(n, L, r_cut=2.5, truncation="shifted", skin=0.3, timestep=dt))
    eng.commit()
    eng.set("position", r)
    eng.set("velocity", v)
    block, shift, sep = 4, 2, 4
    max_lag, res = 40 * dt, dt
    dyn = hg.Dynamics(eng, max_lag, res, block_size=block, shift=shift, separation=sep)
    msd_all = dyn.add_msd(0, n)
    msd_half = dyn.add_msd(n // 4, n // 2)
    k_isf = dyn.add_isf([7.25, 3.0], tolerance=0.05, max_count=7, first=0, last=n, norm=n)

    inf = eng.info()
    Lf = np.array(inf.box_f32, dtype=np.float64)
    q, shells = oracle.wavevectors([7.25, 3.0], Lf.astype(np.float32).astype(np.float64), 0.05, 7)
    keep = [s for s in range(len(shells)) if shells[s, 1] > shells[s, 0]]
    np.testing.assert_allclose(dyn.wavenumbers(k_isf), np.array([7.25, 3.0])[keep])
    q32 = q.astype(np.float32)

    bs = BlockingScheme(dt, max_lag, res, block, shift, sep)
    assert dyn.levels == len(bs.interval)
    np.testing.assert_allclose(dyn.time(), np.array(bs.time()), rtol=1e-15)

    def msd_fn(first, last):
        def fn(a, b):
            o = oracle.msd(a["r"], b["r"], first, last)
            return [(o["count"], o["mean"], o["variance"] * o["count"])]
        return fn

    def isf_fn(a, b):
        sh = np.array([shells[s] for s in keep], dtype=np.int32)
        o = oracle.isf(sh, a["rho"], b["rho"], n)
        return [(c, m, var * c) for c, m, var in o]

    bs.add(msd_fn(0, n))
    bs.add(msd_fn(n // 4, n // 2))
    bs.add(isf_fn, nshell=len(keep))

    for step in range(0, 61):
        if step > 0:
            eng.step(1)
        dyn.sample()

        def acquire():
            pos4 = eng.get_raw("position_hi")[eng.get("reverse_id")]
            return {"r": eng.get("unwrapped_position"), "rho": oracle.density_modes(pos4, q32)}
        bs.sample(step, acquire)
    dyn.finalise()
    bs.finalise()

    for tcf, k, rtol in ((msd_all, 0, 1e-12), (msd_half, 1, 1e-12)):
        mean, err, cnt = dyn.result(tcf)
        ref = bs.mean_error_count(k)
        for lv in range(dyn.levels):
            for j in range(dyn.block_size):
                m, e, c = ref[lv][j][0]
                assert cnt[lv, j, 0] == c
                if c > 0:
                    assert abs(mean[lv, j, 0] - m) <= rtol * max(abs(m), 1e-300) + 1e-18
    mean, err, cnt = dyn.result(k_isf)
    ref = bs.mean_error_count(2)
    for lv in range(dyn.levels):
        for j in range(dyn.block_size):
            for s in range(len(keep)):
                m, e, c = ref[lv][j][s]
                assert cnt[lv, j, s] == c
                if c > 0:
                    assert abs(mean[lv, j, s] - m) < 1e-5 + 1e-5 * abs(m)
    # MSD grows with lag on the finest level
    msd_mean, _, _ = dyn.result(msd_all)
    assert msd_mean[0, 1, 0] < msd_mean[0, block - 1, 0]
    dyn.close()
    eng.close()


def test_mqd_vacf_blocking_scheme():
    """Mean quartic displacement and velocity autocorrelation against the
    FP64 oracle on the same samples (mean_quartic_displacement.hpp:34-41,
    velocity_autocorrelation.hpp:34-38)."""
    r, v, L = lj_system(ncell=5, T=1.2)
    n = r.shape[0]
    dt = 0.005
    eng = hg.Engine("dsfloat")
    eng.add_system(hg.system_desc(n, L, r_cut=2.5, truncation="shifted", skin=0.3, timestep=dt))
    eng.commit()
    eng.set("position", r)
    eng.set("velocity", v)
    block, shift, sep = 4, 2, 4
    max_lag, res = 40 * dt, dt
    dyn = hg.Dynamics(eng, max_lag, res, block_size=block, shift=shift, separation=sep)
    k_mqd = dyn.add_mqd(0, n)
    k_vacf = dyn.add_vacf(n // 3, n)
    bs = BlockingScheme(dt, max_lag, res, block, shift, sep)

    def tcf_fn(kind, key, first, last):
        def fn(a, b):
            o = oracle.tcf(kind, a[key], b[key], first, last)
            return [(o["count"], o["mean"], o["variance"] * o["count"])]
        return fn

    bs.add(tcf_fn("mqd", "r", 0, n))
    bs.add(tcf_fn("vacf", "v", n // 3, n))
    for step in range(0, 61):
        if step > 0:
            eng.step(1)
        dyn.sample()
        bs.sample(step, lambda: {"r": eng.get("unwrapped_position"), "v": eng.get("velocity")})
    dyn.finalise()
    bs.finalise()
    for tcf, k in ((k_mqd, 0), (k_vacf, 1)):
        mean, err, cnt = dyn.result(tcf)
        ref = bs.mean_error_count(k)
        for lv in range(dyn.levels):
            for j in range(dyn.block_size):
                m, e, c = ref[lv][j][0]
                assert cnt[lv, j, 0] == c
                if c > 0:
                    assert abs(mean[lv, j, 0] - m) <= 1e-12 * max(abs(m), 1e-300) + 1e-18
                    assert abs(err[lv, j, 0] - e) <= 1e-9 * max(abs(e), 1e-300) + 1e-15
    # VACF at lag 0 is the mean v^2 of the group: positive and decaying
    vmean, _, _ = dyn.result(k_vacf)
    assert vmean[0, 0, 0] > 0 and vmean[0, 0, 0] > vmean[0, block - 1, 0]
    dyn.close()
    eng.close()


def test_fcc_static_structure_factor():
    # test/unit/observables/ssf.cpp:100-300: the density modes of a perfect
    # fcc lattice in a rectangular box; S(q) = N for wavevectors whose
    # (h, k, l) are integers of one parity, 0 otherwise.  The intermediate
    # scattering function at lag 0 is S(k) averaged over each shell.
    ncell = np.array([4, 8, 5])
    a = (4 / 0.8) ** (1 / 3)
    box = a * ncell
    n = int(4 * np.prod(ncell))
    basis = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
    cells = np.stack(np.meshgrid(*(np.arange(k) for k in ncell), indexing="ij"), -1).reshape(-1, 1, 3)
    r = ((cells + basis[None] + 0.25) * a - 0.5 * box).reshape(-1, 3)   # lattice.cpp offset of 1/4
    eng = hg.Engine("dsfloat")
    eng.add_system(hg.system_desc(n, box, r_cut=2.5, skin=0.3, timestep=0.001))
    eng.commit()
    eng.set("position", r)
    q_lat = 2 * np.pi / a
    wavenumber = sorted(set([q_lat / k for k in ncell] + [np.sqrt(m) * q_lat for m in (1, 2, 3, 4, 5, 6, 8, 9, 10, 12)]))
    dyn = hg.Dynamics(eng, 0.001, 0.001, block_size=2)
    k_isf = dyn.add_isf(wavenumber, tolerance=1e-3, max_count=6, first=0, last=n, norm=n)
    dyn.sample()
    dyn.finalise()
    mean, err, cnt = dyn.result(k_isf)
    s_gpu = mean[0, 0, :]

    Lf = np.array(eng.info().box_f32, dtype=np.float32).astype(np.float64)
    q, shells = oracle.wavevectors(wavenumber, Lf, 1e-3, 6)
    keep = [s for s in range(len(shells)) if shells[s, 1] > shells[s, 0]]
    np.testing.assert_allclose(dyn.wavenumbers(k_isf), np.array(wavenumber)[keep])
    s_ref = []
    for s in keep:
        qs = q[shells[s, 0]:shells[s, 1]]
        hkl_ncell = np.rint(np.abs(qs) * Lf / (2 * np.pi)).astype(int)
        lattice = np.all(hkl_ncell % ncell == 0, axis=1)
        n_odd = np.sum((hkl_ncell // ncell) % 2, axis=1)
        s_ref.append(n * np.mean(lattice & ((n_odd == 0) | (n_odd == 3))))
    s_ref = np.array(s_ref)
    print("S(k):", np.round(s_gpu, 4), "reference", s_ref)
    assert np.any(s_ref > 0) and np.any(s_ref == 0)
    np.testing.assert_allclose(s_gpu, s_ref, rtol=1e-4, atol=1e-4 * n)
    eng.close()
