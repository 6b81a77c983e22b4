"""Autotuner for the engine's launch shapes.

Picks the force kernel's lanes per particle (1, 2, 4 or 8 threads share one
particle's neighbour list) and the list block width (entries one thread
reads with one load = block / lanes) by timing the force kernel on the engine's own
systems with CUDA events (the engine's per-phase profiler), the list
build's scan (per lane over the 27 cells around a particle, or shared by a
warp of 32 particles over the cells around their bounding box) by timing
the rebuild chain the same way, and the cell size of the binning (through
the cell occupancy the reference's sizing rule takes) by timing the
rebuild chain of engines binned at each candidate.  Results are cached as JSON
keyed by (GPU name, slots bucket, list capacity bucket) so a later engine of
similar size reuses the choice without timing.
"""
import json
import math
import os

CACHE = os.environ.get("HMD_TUNE_CACHE", os.path.join(os.path.expanduser("~"), ".cache", "halmd_gb300_tune.json"))
CHOICES = ((1, 4), (2, 4), (2, 8), (4, 4), (4, 8), (8, 8))   # (lanes, list block)
LIST_CHOICES = (1, 2)   # neighbour_scan: per lane, shared per warp
# cell occupancy of the binning (binning.cpp:81-101): the reference's
# default 0.5, whose cells are often capped at r_c + skin, and three that
# give larger cells (cells never get smaller than r_c + skin)
CELL_CHOICES = (0.5, 1.0, 1.5, 2.0)


def _gpu_name():
    try:
        import torch
        return torch.cuda.get_device_name()
    except Exception:
        return "unknown"


def _key(engine):
    slots = sum(engine.info(s).slots for s in range(len(engine.systems)))
    cap = engine.get_option("neighbour_capacity")
    return "%s|slots2^%d|cap%d" % (_gpu_name(), int(round(math.log2(max(slots, 1)))), cap // 16 * 16)


def _load():
    try:
        with open(CACHE) as fh:
            return json.load(fh)
    except (OSError, ValueError):
        return {}


def _store(db):
    try:
        os.makedirs(os.path.dirname(CACHE), exist_ok=True)
        with open(CACHE, "w") as fh:
            json.dump(db, fh, indent=1)
    except OSError:
        pass


def autotune_force_lanes(engine, repeats=10, use_cache=True):
    """Time the force kernel for every (lanes, list block) shape; keep the fastest.

    Returns (lanes, {"lanes/block": ms per launch}) and leaves the engine on
    the fastest shape.  The engine must be committed and hold a representative
    state (positions set)."""
    key = _key(engine)
    db = _load() if use_cache else {}
    if use_cache and key in db and "block" in db[key]:
        engine.set_option("force_lanes", db[key]["lanes"])
        engine.set_option("list_block", db[key]["block"])
        return db[key]["lanes"], db[key]["ms"]
    timings = {}
    for w, b in CHOICES:
        engine.set_option("force_lanes", w)
        engine.set_option("list_block", b)
        engine.force()            # rebuilds the lists in this layout
        engine.profile(True)
        for _ in range(repeats):
            engine.force()
        ms, n = engine.profile_get("force")
        engine.profile(False)
        timings[(w, b)] = ms / max(n, 1)
    best = min(timings, key=timings.get)
    engine.set_option("force_lanes", best[0])
    engine.set_option("list_block", best[1])
    engine.force()
    out = {"%d/%d" % k: v for k, v in timings.items()}
    if use_cache:
        db[key] = {"lanes": best[0], "block": best[1], "ms": out}
        _store(db)
    return best[0], out


def autotune_list_build(engine, repeats=6, use_cache=True):
    """Time the list rebuild chain for every list-build shape; keep the fastest.

    Both scans build the same pair sets (one float criterion), so the choice
    changes only the time (and the order of a particle's entries).  Returns
    (scan, {"scan": ms per chain}) and leaves the engine on the fastest scan.
    The engine must be committed and hold a representative state; every
    system is flagged for a rebuild before each timed force evaluation."""
    key = _key(engine) + "|list"
    db = _load() if use_cache else {}
    if use_cache and key in db and "scan" in db[key]:
        engine.set_option("neighbour_scan", db[key]["scan"])
        return db[key]["scan"], db[key]["ms"]
    nsys = len(engine.systems)

    def rebuild_all():
        for s in range(nsys):
            engine.request_rebuild(s)
        engine.force()

    timings = {}
    for scan in LIST_CHOICES:
        engine.set_option("neighbour_scan", scan)
        rebuild_all()
        engine.profile(True)
        for _ in range(repeats):
            rebuild_all()
        ms, n = engine.profile_get("rebuild")
        engine.profile(False)
        timings[scan] = ms / max(n, 1)
    best = min(timings, key=timings.get)
    engine.set_option("neighbour_scan", best)
    rebuild_all()
    out = {str(k): v for k, v in timings.items()}
    if use_cache:
        db[key] = {"scan": best, "ms": out}
        _store(db)
    return best, out


def autotune_cell_occupancy(build, candidates=CELL_CHOICES, repeats=5):
    """Time the list rebuild chain of engines binned at each cell occupancy;
    return the fastest.

    build(occupancy) returns a committed engine holding the state to tune
    on (positions set); it is closed here.  Every cell size gives the same
    pair sets (the list criterion does not depend on the binning).  Returns
    (occupancy, {"occupancy": ms per chain})."""
    timings = {}
    for occ in candidates:
        eng = build(occ)
        try:
            nsys = len(eng.systems)

            def rebuild_all():
                for s in range(nsys):
                    eng.request_rebuild(s)
                eng.force()

            rebuild_all()   # first build (and any growth of the cell capacity)
            eng.profile(True)
            for _ in range(repeats):
                rebuild_all()
            ms, n = eng.profile_get("rebuild")
            eng.profile(False)
            timings[occ] = ms / max(n, 1)
        finally:
            eng.close()
    best = min(timings, key=timings.get)
    return best, {str(k): v for k, v in timings.items()}
