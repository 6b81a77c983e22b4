"""The autotuner's host logic with a stand-in engine (no GPU): it times
every candidate through the engine's phase profiler, keeps the fastest and
leaves the engine (or returns the cell occupancy) on it."""
import types

from halmd_gb300 import tune


class FakeEngine:
    """Phase timings as a function of the options; rebuild requests counted."""

    def __init__(self, rebuild_ms=None, force_ms=None, occupancy=0.5):
        self.opts = {"force_lanes": 1, "list_block": 4, "neighbour_scan": 0, "neighbour_capacity": 128}
        self.rebuild_ms = rebuild_ms or (lambda o, occ: 1.0)
        self.force_ms = force_ms or (lambda o: 1.0)
        self.occupancy = occupancy
        self.systems = [0, 1]
        self.requested = set()
        self.timers = {}
        self.profiling = False
        self.closed = False

    def set_option(self, name, value):
        self.opts[name] = value

    def get_option(self, name):
        return self.opts[name]

    def info(self, s=0):
        return types.SimpleNamespace(slots=4096)

    def request_rebuild(self, s=0):
        self.requested.add(s)

    def force(self):
        if self.profiling:
            if self.requested:
                self._add("rebuild", self.rebuild_ms(self.opts, self.occupancy))
            self._add("force", self.force_ms(self.opts))
        self.requested.clear()

    def _add(self, phase, ms):
        t = self.timers.setdefault(phase, [0.0, 0])
        t[0] += ms
        t[1] += 1

    def profile(self, on=True):
        self.profiling = on
        if on:
            self.timers = {}

    def profile_get(self, phase):
        t = self.timers.get(phase, [0.0, 0])
        return t[0], t[1]

    def close(self):
        self.closed = True


def test_list_build_tuner_keeps_the_fastest_scan():
    eng = FakeEngine(rebuild_ms=lambda o, occ: {1: 0.30, 2: 0.45}[o["neighbour_scan"]])
    best, ms = tune.autotune_list_build(eng, repeats=3, use_cache=False)
    assert best == 1 and eng.get_option("neighbour_scan") == 1
    assert abs(ms["1"] - 0.30) < 1e-12 and abs(ms["2"] - 0.45) < 1e-12


def test_list_build_tuner_rebuilds_every_system():
    eng = FakeEngine()
    seen = []
    orig = eng.force

    def force():
        seen.append(set(eng.requested))
        orig()

    eng.force = force
    tune.autotune_list_build(eng, repeats=2, use_cache=False)
    assert all(s == {0, 1} for s in seen)


def test_force_shape_tuner_keeps_the_fastest_shape():
    def ms(o):
        return 1.0 - (0.5 if (o["force_lanes"], o["list_block"]) == (4, 8) else 0.0)
    eng = FakeEngine(force_ms=ms)
    lanes, out = tune.autotune_force_lanes(eng, repeats=2, use_cache=False)
    assert lanes == 4 and eng.get_option("list_block") == 8
    assert set(out) == {"%d/%d" % c for c in tune.CHOICES}


def test_cell_occupancy_tuner_closes_every_engine_and_returns_the_fastest():
    built = []

    def build(occ):
        e = FakeEngine(rebuild_ms=lambda o, occ: 0.7 + 0.1 * abs(occ - 1.0), occupancy=occ)
        built.append(e)
        return e

    best, ms = tune.autotune_cell_occupancy(build, repeats=2)
    assert best == 1.0
    assert [e.occupancy for e in built] == list(tune.CELL_CHOICES)
    assert all(e.closed for e in built)
    assert set(ms) == {str(c) for c in tune.CELL_CHOICES}
