"""The plain-Python blocking scheme restatement (oracle/blocking.py) on the
reference's documented grid (observables/dynamics/blocking_scheme.cpp:56-79)."""
from oracle.blocking import BlockingScheme


def test_levels_and_time_grid():
    bs = BlockingScheme(0.001, 1.0, 0.001, 10, 3, 10)
    assert bs.interval == [1, 3, 10, 30, 100, 300, 1000]
    t = bs.time()
    assert t[2][1] == 10 * 0.001 and t[6][9] == 1000 * 9 * 0.001


def test_process_and_finalise_counts():
    bs = BlockingScheme(1.0, 8.0, 1.0, 4, 2, 4)
    assert bs.interval == [1, 2, 4, 8]
    k = bs.add(lambda a, b: [(1.0, float(b - a), 0.0)])
    for step in range(20):
        bs.sample(step, lambda s=step: s)
    bs.finalise()
    res = bs.mean_error_count(k)
    # level 0 (interval 1): lag j correlates samples j steps apart
    for j in range(4):
        m, e, c = res[0][j][0]
        assert c > 0 and abs(m - j) < 1e-12
    # level 1 (interval 2): lag j is 2j steps
    assert abs(res[1][3][0][0] - 6.0) < 1e-12
