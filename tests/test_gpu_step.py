"""GPU parity of the MD step against the CPU oracle (calls through the C ABI).

Bars: bit-exact for integer/index work (cells, neighbour sets, Hilbert keys,
sort permutation) and for the float/dsfloat integrator, which rounds every
operation like the oracle; forces within the stated tolerance of an FP64
evaluation of the same double-single state.
"""
import numpy as np
import pytest

import halmd_gb300 as hg
import oracle
from _systems import KA_EPS, KA_SIGMA, ka_system, lj_system, rel_force_error, state_forces

pytestmark = pytest.mark.gpu

# per-particle force error bound: max_i |F_i - F64_i| / max(|F64_i|, F_rms)
FORCE_TOL = 1e-6


def lj_engine(precision="dsfloat", ncell=6, skin=0.3, dt=0.005, **kw):
    r, v, L = lj_system(ncell=ncell)
    n = r.shape[0]
    eng = hg.Engine(precision)
    eng.add_system(hg.system_desc(n, L, r_cut=2.5, truncation="shifted", skin=skin, timestep=dt, **kw))
    eng.commit()
    eng.set("position", r)
    eng.set("velocity", v)
    return eng, r, v, L


def ka_engine(precision="dsfloat", ncell=6, dt=0.002, **kw):
    r, v, sp, L = ka_system(ncell=ncell)
    n = r.shape[0]
    eng = hg.Engine(precision)
    rc = 2.5 * np.asarray(KA_SIGMA) / np.asarray(KA_SIGMA)  # r_c = 2.5 sigma_ab
    eng.add_system(hg.system_desc(n, L, epsilon=KA_EPS, sigma=KA_SIGMA, r_cut=rc, truncation="smooth_r4",
                                  smoothing=0.005, skin=0.3, timestep=dt, **kw))
    eng.commit()
    eng.set("species", sp)
    eng.set("position", r)
    eng.set("velocity", v)
    return eng, r, v, sp, L


def tag_order(eng, raw):
    rid = eng.get("reverse_id")
    return raw[rid]


def oracle_forces(eng, species, pot):
    # FP64 forces of the engine's state (hi + lo positions)
    pos4 = tag_order(eng, eng.get_raw("position_hi"))
    return state_forces(eng, species, pot), pos4


@pytest.mark.parametrize("precision", ["dsfloat", "float"])
def test_lj_force_parity(precision):
    eng, r, v, L = lj_engine(precision)
    n = r.shape[0]
    eng.force(aux=True)
    f = eng.get("force")
    pot = oracle.Potential(1.0, 1.0, 2.5, "shifted")
    ref, _ = oracle_forces(eng, np.zeros(n), pot)
    emax, emed = rel_force_error(f, ref["force"])
    print("LJ force rel err max %.3g median %.3g" % (emax, emed))
    assert emax < FORCE_TOL
    en = eng.get("potential_energy")
    assert abs(en.sum() - ref["epot"]) < 1e-6 * abs(ref["epot"])
    np.testing.assert_allclose(en, ref["en_pot"], rtol=1e-5, atol=1e-5)
    st = eng.get("stress_pot")
    srms = np.sqrt(np.mean(ref["stress"] ** 2))
    assert np.max(np.abs(st - ref["stress"])) < 1e-5 * srms * 10
    th = eng.thermo()
    assert abs(th["epot"] - ref["epot"]) < 1e-6 * abs(ref["epot"])
    assert abs(th["virial"] - ref["virial"]) < 1e-6 * abs(ref["virial"])
    vv = eng.get("velocity")
    assert abs(th["mv2"] - np.sum(vv * vv)) < 1e-12 * np.sum(vv * vv)
    eng.close()


@pytest.mark.parametrize("trunc", ["sharp", "force_shifted", "smooth_r4"])
def test_truncation_parity(trunc):
    # the truncations of truncations/*_kernel.cuh on one species (shifted: above)
    kw = dict(smoothing=0.005) if trunc == "smooth_r4" else {}
    r, v, L = lj_system(ncell=6)
    n = r.shape[0]
    eng = hg.Engine("dsfloat")
    eng.add_system(hg.system_desc(n, L, r_cut=2.5, truncation=trunc, skin=0.3, timestep=0.005, **kw))
    eng.commit()
    eng.set("position", r)
    eng.set("velocity", v)
    eng.step(20)
    eng.force(aux=True)
    f = eng.get("force")
    pot = oracle.Potential(1.0, 1.0, 2.5, trunc, h=0.005) if trunc == "smooth_r4" else oracle.Potential(1.0, 1.0, 2.5, trunc)
    ref, _ = oracle_forces(eng, np.zeros(n), pot)
    emax, emed = rel_force_error(f, ref["force"])
    print("%s force rel err max %.3g median %.3g" % (trunc, emax, emed))
    assert emax < FORCE_TOL
    en = eng.get("potential_energy")
    assert abs(en.sum() - ref["epot"]) < 1e-6 * abs(ref["epot"])
    np.testing.assert_allclose(en, ref["en_pot"], rtol=1e-5, atol=1e-5)
    eng.close()


@pytest.mark.parametrize("lanes,block", [(1, 4), (2, 4), (2, 8), (4, 4), (4, 8), (8, 8)])
def test_force_lanes_agree(lanes, block):
    eng, r, v, L = lj_engine(ncell=7)
    eng.set_option("force_lanes", lanes)
    eng.set_option("list_block", block)
    assert eng.get_option("list_block") == block
    eng.force()
    assert eng.get_option("force_lanes") == lanes
    f = eng.get("force")
    pot = oracle.Potential(1.0, 1.0, 2.5, "shifted")
    ref, _ = oracle_forces(eng, np.zeros(r.shape[0]), pot)
    emax, _ = rel_force_error(f, ref["force"])
    assert emax < FORCE_TOL
    counts, lists = eng.neighbour_lists()
    inf = eng.info()
    rc, rl, _ = oracle.neighbour_full_f32(tag_order(eng, eng.get_raw("r0")), np.array(inf.box_f32),
                                         np.array(inf.rr_cut_skin[:1], dtype=np.float32), inf.neighbour_capacity)
    assert np.array_equal(counts, rc) and np.array_equal(lists, rl)
    eng.step(5)
    assert np.all(np.isfinite(eng.get("position")))
    eng.close()


def test_ka_smooth_r4_force_parity():
    eng, r, v, sp, L = ka_engine()
    eng.force(aux=True)
    f = eng.get("force")
    pot = oracle.Potential(KA_EPS, KA_SIGMA, 2.5 * np.ones((2, 2)) * 1.0, "smooth_r4", h=0.005)
    # r_cut = 2.5 sigma_ab: in units of sigma the cutoff matrix is 2.5 everywhere
    ref, _ = oracle_forces(eng, sp, pot)
    emax, emed = rel_force_error(f, ref["force"])
    print("KA force rel err max %.3g median %.3g" % (emax, emed))
    assert emax < FORCE_TOL
    en = eng.get("potential_energy")
    assert abs(en.sum() - ref["epot"]) < 1e-6 * abs(ref["epot"])
    eng.close()


@pytest.mark.parametrize("scan", [1, 2])
@pytest.mark.parametrize("make", ["lj", "ka", "lj_large", "ka_large", "lj_unsorted", "lj_large_cells",
                                  "ka_large_cells"])
def test_neighbour_lists_bit_exact(make, scan):
    # both list-build scans (per lane, shared per warp) on small boxes (3 cells
    # per dimension: every warp wraps), large boxes (interior warps scan
    # without minimum image), an unsorted system (warps too spread out for
    # the shared scan: it falls back to the per-lane scan), and cells larger
    # than r_c + skin (cell occupancy 2, a size the cell autotuner offers)
    if make == "lj":
        eng, r, v, L = lj_engine()
    elif make == "lj_large":
        eng, r, v, L = lj_engine(ncell=16)
    elif make == "lj_large_cells":
        eng, r, v, L = lj_engine(ncell=16, cell_occupancy=2.0)
    elif make == "ka_large_cells":
        eng, r, v, sp, L = ka_engine(ncell=14, cell_occupancy=2.0)
    elif make == "lj_unsorted":
        eng, r, v, L = lj_engine(ncell=12, sort=0)
        perm = np.random.default_rng(3).permutation(r.shape[0])   # slots in random spatial order
        eng.set("position", r[perm])
        eng.set("velocity", v[perm])
    elif make == "ka_large":
        eng, r, v, sp, L = ka_engine(ncell=14)
    else:
        eng, r, v, sp, L = ka_engine()
    eng.set_option("neighbour_scan", scan)
    eng.request_rebuild()
    eng.force()
    inf = eng.info()
    ns = inf.nspecies
    rrcs = np.array(inf.rr_cut_skin[: ns * ns], dtype=np.float32)
    pos4 = tag_order(eng, eng.get_raw("r0"))   # positions of the last build
    maxn = inf.neighbour_capacity
    counts, lists = eng.neighbour_lists(maxn)
    rc, rl, mx = oracle.neighbour_full_f32(pos4, np.array(inf.box_f32), rrcs, maxn)
    assert np.array_equal(counts, rc)
    assert np.array_equal(lists, rl)
    assert inf.max_neighbours == mx
    eng.close()



@pytest.mark.parametrize("scan", [1, 2])
def test_neighbour_lists_bit_exact_large_grid(scan):
    # 108,000 particles: the one-system list build takes its large-grid form
    # (8 resident blocks per SM) rather than the small-grid one the smaller
    # tests use; cell occupancy 1 (the size the bench's tuner keeps)
    r, v, L = lj_system(ncell=30)
    n = r.shape[0]
    eng = hg.Engine("dsfloat")
    eng.add_system(hg.system_desc(n, L, r_cut=2.5, truncation="shifted", skin=0.3, timestep=0.005,
                                  cell_occupancy=1.0))
    eng.commit()
    eng.set("position", r)
    eng.set("velocity", v)
    eng.step(40)
    eng.set_option("neighbour_scan", scan)
    eng.request_rebuild()
    eng.force()
    inf = eng.info()
    rrcs = np.array(inf.rr_cut_skin[:1], dtype=np.float32)
    pos4 = tag_order(eng, eng.get_raw("r0"))
    maxn = inf.neighbour_capacity
    counts, lists = eng.neighbour_lists(maxn)
    rc, rl, mx = oracle.neighbour_full_f32(pos4, np.array(inf.box_f32), rrcs, maxn)
    assert np.array_equal(counts, rc)
    assert np.array_equal(lists, rl)
    # the engine keeps the largest list length of every build since commit
    assert counts.max() == mx and inf.max_neighbours >= mx
    eng.close()


def test_binning_bit_exact():
    eng, r, v, L = lj_engine(ncell=8)
    eng.force()
    inf = eng.info()
    ncell = np.array(inf.ncell[:], dtype=np.int32)
    Lf = np.array(inf.box_f32, dtype=np.float32)
    cell_len = Lf / ncell.astype(np.float32)
    pos4 = eng.get_raw("position_hi")
    cells, _, maxocc = oracle.binning_f32(pos4, ncell, cell_len, inf.cell_size)
    assert maxocc == inf.max_cell_occupancy
    assert np.array_equal(eng.get_raw("cells"), cells)
    eng.close()


def test_binning_non_uniform_density():
    # test/unit/mdsim/binning.cpp:120-200 bins non-uniform densities: here
    # the density grows as u^3 along x (4x the mean at the dense end), which
    # overflows cells sized for a uniform fluid; after the capacity recovery
    # every particle is binned exactly once, in the oracle's cell and order
    eng, r, v, L = lj_engine(ncell=8)
    n = r.shape[0]
    rng = np.random.default_rng(21)
    u = rng.uniform(size=n) ** 0.25
    pos = np.column_stack([(u - 0.5) * L, rng.uniform(-0.5 * L, 0.5 * L, size=(n, 2))])
    cs0 = eng.info().cell_size
    eng.set("position", pos)
    eng.force()
    inf = eng.info()
    assert inf.cell_size > cs0            # the dense end overflowed the first sizing
    ncell = np.array(inf.ncell[:], dtype=np.int32)
    Lf = np.array(inf.box_f32, dtype=np.float32)
    cell_len = Lf / ncell.astype(np.float32)
    pos4 = eng.get_raw("position_hi")
    cells, _, maxocc = oracle.binning_f32(pos4, ncell, cell_len, inf.cell_size)
    got = eng.get_raw("cells")
    assert maxocc == inf.max_cell_occupancy
    assert np.array_equal(got, cells)
    real = got[got != 0xFFFFFFFF]
    assert real.size == n and np.unique(real).size == n
    eng.close()


def test_hilbert_keys_and_sort_permutation():
    eng, r, v, L = lj_engine(ncell=8)
    n = r.shape[0]
    inf = eng.info()
    pos4 = eng.get_raw("position_hi")[:n]          # slot order == tag order before the first sort
    keys = oracle.hilbert_keys_f32(pos4, np.array(inf.box_f32), inf.hilbert_depth)
    assert inf.hilbert_depth == oracle.hilbert_depth(float(max(inf.box_f32)))
    assert np.array_equal(eng.hilbert_keys(), keys)
    eng.force()                                    # first list build sorts the particles
    ids = eng.get("id")[:n]
    assert np.array_equal(ids, oracle.stable_argsort_u32(keys))
    # the phase space moved with the particles (tag-order view unchanged)
    np.testing.assert_allclose(eng.get("velocity"), v, rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(eng.get("position"), r, rtol=1e-12, atol=1e-12)
    eng.close()


@pytest.mark.parametrize("precision", ["dsfloat", "float"])
def test_integrate_finalize_bit_exact(precision):
    eng, r, v, L = lj_engine(precision)
    ds = precision == "dsfloat"
    eng.force()
    inf = eng.info()
    Lf = np.array(inf.box_f32, dtype=np.float32)
    r4 = np.concatenate([eng.get_raw("position_hi"), eng.get_raw("position_lo")])
    v4 = np.concatenate([eng.get_raw("velocity_hi"), eng.get_raw("velocity_lo")])
    img = eng.get_raw("image")
    f4 = eng.get_raw("force")
    eng.integrate()
    r_ref, v_ref, img_ref = oracle.integrate_f32(r4, v4, img, f4, 0.005, Lf, ds=ds)
    A = inf.slots
    assert np.array_equal(eng.get_raw("position_hi").view(np.uint32), r_ref[:A].view(np.uint32))
    assert np.array_equal(eng.get_raw("velocity_hi").view(np.uint32), v_ref[:A].view(np.uint32))
    if ds:
        assert np.array_equal(eng.get_raw("position_lo").view(np.uint32), r_ref[A:].view(np.uint32))
        assert np.array_equal(eng.get_raw("velocity_lo").view(np.uint32), v_ref[A:].view(np.uint32))
    assert np.array_equal(eng.get_raw("image"), img_ref)
    eng.force()
    r4 = np.concatenate([eng.get_raw("position_hi"), eng.get_raw("position_lo")])
    v4 = np.concatenate([eng.get_raw("velocity_hi"), eng.get_raw("velocity_lo")])
    f4 = eng.get_raw("force")
    eng.finalize()
    v_ref = oracle.finalize_f32(r4, v4, f4, 0.005, ds=ds)
    assert np.array_equal(eng.get_raw("velocity_hi").view(np.uint32), v_ref[:A].view(np.uint32))
    if ds:
        assert np.array_equal(eng.get_raw("velocity_lo").view(np.uint32), v_ref[A:].view(np.uint32))
    eng.close()


def test_andersen_collisions():
    T, rate, dt, seed = 0.7, 60.0, 0.005, 1234
    eng, r, v, L = lj_engine(integrator="andersen", temperature=T, collision_rate=rate, seed=seed)
    eng.force()
    eng.integrate()
    eng.force()
    A = eng.info().slots
    r4 = np.concatenate([eng.get_raw("position_hi"), eng.get_raw("position_lo")])
    v4 = np.concatenate([eng.get_raw("velocity_hi"), eng.get_raw("velocity_lo")])
    f4 = eng.get_raw("force")
    ids = eng.get("id")
    eng.finalize()
    v_ref, coll = oracle.andersen_finalize_f32(r4, v4, f4, ids, dt, T, rate * dt, seed, step=0)
    got = eng.get_raw("velocity_hi")
    assert 0.2 < coll[:len(ids)].mean() < 0.4       # p = 0.3 per particle and step
    keep = ~coll[:A]
    assert np.array_equal(got[keep].view(np.uint32), v_ref[:A][keep].view(np.uint32))
    np.testing.assert_allclose(got[coll[:A], :3], v_ref[:A][coll[:A], :3], rtol=2e-6, atol=2e-6)
    eng.close()


@pytest.mark.parametrize("steps", [7, 237])
@pytest.mark.parametrize("system", ["lj", "ka_andersen"])
def test_graph_step_equals_module_calls(system, steps):
    # 237 steps: two 100-step chunks, three 10-step chunks and single steps,
    # list rebuilds on the way; the chunks fuse the finalize of step k with
    # the integrate of step k + 1
    def make():
        if system == "lj":
            return lj_engine()[0]
        return ka_engine(integrator="andersen", temperature=0.7, collision_rate=20.0, seed=99)[0]
    a, b = make(), make()
    a.step(steps)
    for _ in range(steps):
        b.integrate()
        b.force()
        b.finalize()
    for name in ("position", "velocity", "image"):
        assert np.array_equal(a.get(name), b.get(name)), name
    assert a.info().step == b.info().step == steps
    assert a.info().rebuilds == b.info().rebuilds
    a.close()
    b.close()


def test_short_trajectory_against_fp64_host_backend():
    eng, r, v, L = lj_engine(ncell=5, dt=0.002)
    n = r.shape[0]
    nsteps = 50
    eng.step(nsteps)
    pot = oracle.Potential(1.0, 1.0, 2.5, "shifted")
    Lf = float(np.float32(L))
    r_ref, v_ref, img_ref, st = oracle.md_run(r, v, np.zeros(n), np.ones(n), [Lf] * 3, pot, 0.3, 0.002, nsteps)
    got = eng.get("unwrapped_position")
    ref = r_ref + img_ref * Lf
    assert np.max(np.abs(got - ref)) < 1e-5
    np.testing.assert_allclose(eng.get("velocity"), v_ref, atol=1e-4)
    eng.close()


@pytest.mark.parametrize("precision", ["dsfloat", "float"])
def test_nve_energy_conservation_lj4k(precision):
    """LJ-4k (rho 0.8442, T 1.5, shifted r_c 2.5, skin 0.3, dt 0.005) over
    5e4 steps against the FP64 variant from the same start.  At this time
    step the energy of every variant, FP64 included, wanders by a few 1e-5 of
    |E| per 1e5 steps (the shifted force jumps at r_c), so the precision's
    own share is bounded by comparing with FP64.  Measured on a GB300: over
    1e5 steps, drift per 1e5 steps FP64 -1.0e-5, dsfloat -5.2e-5, float
    1.3e-4 and max |E - E0| / |E0| 3.8e-5, 4.2e-5, 1.5e-4; over 5e4 steps
    FP64 -1.6e-5, dsfloat 8.6e-5, float 8.5e-5 (fit errors 1.6e-5, which
    understate a random walk) and max |E - E0| / |E0| 1.2e-4, 1.4e-4, 1.3e-4."""
    from _systems import energy_drift
    runs = {}
    for prec in (precision, "double"):
        eng, r, v, L = lj_engine(precision=prec, ncell=10, dt=0.005)
        runs[prec] = energy_drift(eng, 50000, 500)
        if prec == precision:
            th = eng.thermo()
            assert np.max(np.abs(th["momentum"])) < 1e-6 * r.shape[0]
            assert eng.info().rebuilds >= 100
        eng.close()
    d, se, wander = runs[precision]
    d64, se64, wander64 = runs["double"]
    print("LJ-4k %s: drift %.3g +- %.2g per 1e5 steps (FP64 %.3g +- %.2g), max |dE|/|E| %.3g (FP64 %.3g)"
          % (precision, d, se, d64, se64, wander, wander64))
    # the drift and the wander within those of FP64 plus what the variant adds
    bound = 3e-4
    assert abs(d) < bound and abs(d - d64) < bound
    assert wander < 2 * wander64 + 1e-4


@pytest.mark.parametrize("scan", [1, 2])
def test_overflow_recovery_matches_ample_capacity(scan):
    a, r, v, L = lj_engine(neighbour_occupancy=20.0)   # list capacity 32 < ~78 needed
    b, *_ = lj_engine()
    for e in (a, b):
        e.set_option("neighbour_scan", scan)
    a.step(20)
    b.step(20)
    assert a.info().neighbour_capacity > 32
    assert np.array_equal(a.get("position"), b.get("position"))
    assert np.array_equal(a.get("velocity"), b.get("velocity"))
    a.close()
    b.close()

