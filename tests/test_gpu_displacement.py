"""Maximum displacement and the skin/2 rebuild rule against the oracle.

max_displacement::compute (mdsim/gpu/max_displacement.cpp:77-106) is the
largest minimum-image displacement since the last list build, and
from_binning.cpp:130 rebuilds the lists when it exceeds skin/2.  The engine
takes the maximum inside the integrate kernel of every step and decides
there; hmd_max_displacement runs the same reduction as a module call.  Both
are float arithmetic on the hi position words and the build-time positions,
so they are compared bit for bit with the oracle's float restatement.
"""
import numpy as np
import pytest

import halmd_gb300 as hg
import oracle
from _systems import lj_system

pytestmark = pytest.mark.gpu


def test_max_displacement_matches_oracle():
    r, v, L = lj_system(ncell=6, T=1.5)
    n = r.shape[0]
    eng = hg.Engine("dsfloat")
    eng.add_system(hg.system_desc(n, L, r_cut=2.5, truncation="shifted", skin=0.3, timestep=0.005))
    eng.commit()
    eng.set("position", r)
    eng.set("velocity", v)
    Lf = np.array(eng.info().box_f32, dtype=np.float32)
    for steps in (0, 1, 7, 23):
        if steps:
            eng.step(steps)
        else:
            eng.force()
        m2 = oracle.max_displacement2_f32(eng.get_raw("position_hi"), eng.get_raw("r0"), Lf)
        d = eng.max_displacement()
        assert d == np.sqrt(np.float64(m2)), (steps, d, m2)
    eng.close()


def free_particles(v_x):
    # one particle moving along x, three at rest, all further apart than
    # r_c + skin: no forces, so the moving particle drifts by v_x dt per step
    pos = np.array([[1.0, 1.0, 1.0], [-5.0, -5.0, -5.0], [5.0, -5.0, 5.0], [-5.0, 5.0, 5.0]])
    vel = np.zeros((4, 3))
    vel[0, 0] = v_x
    return pos, vel


def test_rebuild_decision_at_half_skin():
    skin, dt, L = 0.3, 0.01, 20.0
    half = skin / 2
    # system 0 reaches skin/2 (1 - 1e-5) after 5 steps: no rebuild until step 6;
    # system 1 reaches skin/2 (1 + 1e-5) after 5 steps: rebuild at step 5
    speeds = [half * (1 - 1e-5) / (5 * dt), half * (1 + 1e-5) / (5 * dt)]
    eng = hg.Engine("dsfloat")
    for _ in speeds:
        eng.add_system(hg.system_desc(4, [L] * 3, r_cut=2.5, truncation="shifted", skin=skin, timestep=dt))
    eng.commit()
    for s, vx in enumerate(speeds):
        pos, vel = free_particles(vx)
        eng.set("position", pos, s)
        eng.set("velocity", vel, s)
    eng.force()                                   # lists built: r0 = the start
    rr_half = np.float32(0.25 * skin * skin)
    first = [None, None]
    for step in range(1, 9):
        before = []
        for s in range(2):
            rid = eng.get("reverse_id", s)
            before.append((eng.get_raw("r0", s)[rid], eng.info(s).rebuilds))
        eng.step(1)
        for s in range(2):
            Lf = np.array(eng.info(s).box_f32, dtype=np.float32)
            pos4 = eng.get_raw("position_hi", s)[eng.get("reverse_id", s)]
            m2 = oracle.max_displacement2_f32(pos4, before[s][0], Lf)
            expect = bool(m2 > rr_half)
            got = eng.info(s).rebuilds - before[s][1]
            assert got == int(expect), (step, s, m2, rr_half)
            if expect and first[s] is None:
                first[s] = step
    assert first == [6, 5]
    eng.close()
