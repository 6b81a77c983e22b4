"""hmd_msd_pair_noalloc (fixed device scratch, no allocation) against the MSD
of the blocking-scheme entry points on the same two samples.

Collected last on purpose: it must pass both after the other GPU tests and
alone in a fresh process, where its first call does the per-device set-up.
"""
import ctypes

import numpy as np
import pytest

import halmd_gb300 as hg
from halmd_gb300 import _lib
from _systems import lj_system

pytestmark = pytest.mark.gpu

# The two paths run the same per-block Welford arithmetic in the same merge
# order; their inputs can differ in the last bit (the dynamics path forms the
# unwrapped position on the device, where the compiler may fuse image * L + r).
RTOL = 1e-12


def _noalloc(L, origin, position, out, count=None):
    count = origin.shape[0] if count is None else count
    return L.hmd_msd_pair_noalloc(ctypes.c_void_p(origin.data_ptr()), ctypes.c_void_p(position.data_ptr()),
                                  count, ctypes.c_void_p(out.data_ptr()), None)


def test_msd_noalloc_matches_dynamics_path():
    torch = pytest.importorskip("torch")
    r, v, L = lj_system(ncell=13, T=1.5)          # 8788 particles: one full block of 8192 and a ragged one
    n = r.shape[0]
    dt, lag = 0.005, 100
    eng = hg.Engine("dsfloat")
    eng.add_system(hg.system_desc(n, L, r_cut=2.5, truncation="shifted", skin=0.3, timestep=dt))
    eng.commit()
    eng.set("position", r)
    eng.set("velocity", v)

    # existing entry points: blocking scheme with one level and two samples
    dyn = hg.Dynamics(eng, lag * dt, lag * dt, block_size=2, shift=1, separation=2)
    k = dyn.add_msd(0, n)
    first = eng.get("unwrapped_position")
    dyn.sample()
    eng.step(lag)
    second = eng.get("unwrapped_position")
    dyn.sample()
    mean, err, cnt = dyn.result(k)
    ref_mean, ref_err, ref_cnt = mean[0, 1, 0], err[0, 1, 0], int(cnt[0, 1, 0])
    assert ref_cnt == n and ref_mean > 0
    dyn.close()

    Lib = _lib.load()
    dev = torch.device("cuda:0")
    a = torch.from_numpy(first).to(dev).contiguous()
    b = torch.from_numpy(second).to(dev).contiguous()
    outs = [torch.full((3,), float("nan"), dtype=torch.float64, device=dev) for _ in range(2)]
    torch.cuda.synchronize()
    for call in range(2):                          # two calls in a row reuse the scratch
        out = outs[call]
        free0 = torch.cuda.mem_get_info(dev)[0]
        assert _noalloc(Lib, a, b, out) == 0, _lib.last_error()
        torch.cuda.synchronize()
        # the call takes no device memory (nothing else runs here)
        assert torch.cuda.mem_get_info(dev)[0] == free0, call
        c, m, var = out.cpu().numpy()
        assert c == n, call
        np.testing.assert_allclose(m, ref_mean, rtol=RTOL, err_msg="call %d" % call)
        np.testing.assert_allclose(np.sqrt(var / (n - 1)), ref_err, rtol=RTOL, err_msg="call %d" % call)
    eng.close()


def test_msd_noalloc_rejects_bad_arguments():
    torch = pytest.importorskip("torch")
    Lib = _lib.load()
    dev = torch.device("cuda:0")
    a = torch.zeros((16, 3), dtype=torch.float64, device=dev)
    out = torch.zeros(3, dtype=torch.float64, device=dev)
    limit = 1 << 25
    # above the fixed scratch size: refused before anything is launched
    assert _noalloc(Lib, a, a, out, count=limit + 1) == -1
    assert "exceed the limit" in _lib.last_error()
    # host memory and null pointers are refused, not dereferenced
    host = np.zeros((16, 3))
    rc = Lib.hmd_msd_pair_noalloc(host.ctypes.data_as(ctypes.c_void_p), ctypes.c_void_p(a.data_ptr()), 16,
                                  ctypes.c_void_p(out.data_ptr()), None)
    assert rc == -1 and "not device memory" in _lib.last_error()
    assert Lib.hmd_msd_pair_noalloc(None, None, 16, ctypes.c_void_p(out.data_ptr()), None) == -1
    # a buffer that ends before count x 3 doubles is refused before any
    # launch: 8 particles' worth of bytes before the end of the allocation
    # (the caching allocator's segment) that holds `a`, asked for 16
    seg = [g for g in torch.cuda.memory_snapshot()
           if g["address"] <= a.data_ptr() < g["address"] + g["total_size"]][0]
    near_end = seg["address"] + seg["total_size"] - 8 * 3 * 8
    rc = Lib.hmd_msd_pair_noalloc(ctypes.c_void_p(near_end), ctypes.c_void_p(a.data_ptr()), 16,
                                  ctypes.c_void_p(out.data_ptr()), None)
    assert rc == -1 and "bytes, the call needs" in _lib.last_error()
    # zero particles: (0, 0, 0)
    out.fill_(float("nan"))
    assert _noalloc(Lib, a, a, out, count=0) == 0, _lib.last_error()
    assert out.cpu().tolist() == [0.0, 0.0, 0.0]
