#!/usr/bin/env python3
"""Benchmark of the GB300 MD step (particle-steps/s).

Workload (default): the Kob-Andersen binary mixture, N = 64000 at density 1.2
(A:B = 80:20), LJ with smooth_r4 cut-off (h = 0.005, r_c = 2.5 sigma_ab),
skin 0.3, Andersen NVT at T = 0.7 (collision rate 1), dt = 0.002, dsfloat
positions and velocities.  One bench step = one captured graph of
`--md-steps` MD steps (integrate, device-decided list rebuild, force,
finalize); L2 is flushed between bench steps.  `--workload lj1m` runs the
LJ fluid with N = 1,048,576.

Arms:
  default           the CUDA engine through the C ABI (this repository)
  --impl reference  the reference's host backend restated on the CPU
                    (single thread, FP64, half list; the reference itself
                    cannot be built: no Boost / Lua / HDF5 in the image)
"""
import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

MEASURED = os.path.join(REPO, "MEASURED_PEAKS.json")

KA = dict(eps=[[1.0, 1.5], [1.5, 0.5]], sigma=[[1.0, 0.8], [0.8, 0.88]])


def workload(name):
    if name == "ka64k":
        return dict(name="KA-64k", n=64000, rho=1.2, T=0.7, dt=0.002, trunc="smooth_r4", skin=0.3, nspecies=2,
                    rate=1.0)
    if name == "lj1m":
        return dict(name="LJ-1M", n=1048576, rho=0.8442, T=0.722, dt=0.002, trunc="shifted", skin=0.3, nspecies=1,
                    rate=0.0)
    if name == "lj4k":
        return dict(name="LJ-4k", n=4000, rho=0.8442, T=1.5, dt=0.005, trunc="shifted", skin=0.3, nspecies=1,
                    rate=0.0)
    # the reference's own benchmark configurations (examples/benchmarks/*), whose
    # published H100 double-single timings are the baseline of vs_baseline
    # (doc/benchmarks.rst.in:29 and :79): equilibrated at T with Andersen
    # collisions, then NVE
    if name == "ref-lj64k":
        # lennard_jones/{generate_configuration,run_benchmark}.lua: rho 0.4, T 1.2, r_c 3, skin 0.7, dt 0.002
        return dict(name="reference LJ-64k (rho 0.4)", n=64000, rho=0.4, T=1.2, dt=0.002, trunc="shifted", rc=3.0,
                    skin=0.7, nspecies=1, rate=0.0, equilibrate=dict(steps=4000, rate=2.0, dt=0.002),
                    published=1.0 / 3.4e-9)
    if name == "ref-ka256k":
        # kob_andersen/{generate_configuration,run_benchmark}.lua: 256000, rho 1.2, T 0.7, shifted r_c 2.5 sigma,
        # skin 0.3, list occupancy 0.7, dt 0.001
        return dict(name="reference KA-256k (rho 1.2)", n=256000, rho=1.2, T=0.7, dt=0.001, trunc="shifted",
                    rc=2.5, skin=0.3, occupancy=0.7, nspecies=2, rate=0.0,
                    equilibrate=dict(steps=4000, rate=2.0, dt=0.002), published=1.0 / 1.79e-9)
    raise SystemExit("unknown workload " + name)


RELAX_STEPS = 1000        # steepest-descent steps that relax the random KA start
RELAX_STEP_SIZE = 1e-3    # move = step_size * F (LJ units) ...
RELAX_MAX_MOVE = 0.05     # ... at most this far per step


def initial_state(w, seed=2024):
    """Seeded synthetic input: fcc lattice (LJ; simple cubic where n is not
    4 k^3) or uniform random positions
    with random 80:20 species (KA; relaxed afterwards by steepest descent),
    Maxwell-Boltzmann velocities with zero momentum."""
    n = w["n"]
    rng = np.random.default_rng(seed)
    ncell = int(round((n / 4) ** (1 / 3)))
    if w["nspecies"] == 2:
        L = (n / w["rho"]) ** (1 / 3)
        r = rng.uniform(-0.5 * L, 0.5 * L, size=(n, 3))
    elif 4 * ncell ** 3 == n:
        L = ncell * (4 / w["rho"]) ** (1 / 3)
        a = L / ncell
        basis = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
        c = np.stack(np.meshgrid(*(np.arange(ncell),) * 3, indexing="ij"), -1).reshape(-1, 1, 3)
        r = ((c + basis[None] + 0.25) * a - 0.5 * L).reshape(-1, 3)
        r = r + rng.uniform(-0.02, 0.02, size=r.shape)
    else:
        # n is not 4 k^3: the first n sites of a simple cubic lattice
        L = (n / w["rho"]) ** (1 / 3)
        m = int(np.ceil(n ** (1 / 3) - 1e-9))
        g = (np.arange(m) + 0.5) * (L / m) - 0.5 * L
        r = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)[:n]
        r = r + rng.uniform(-0.02, 0.02, size=r.shape)
    v = rng.normal(0, np.sqrt(w["T"]), size=(n, 3))
    v -= v.mean(axis=0)
    v *= np.sqrt(3 * (n - 1) * w["T"] / np.sum(v * v))
    species = np.zeros(n, dtype=np.uint32)
    if w["nspecies"] == 2:
        species[rng.permutation(n)[: n // 5]] = 1
    return r, v, species, L


def make_engine(w, L, seed=7, precision="dsfloat", cell_occupancy=None):
    import halmd_gb300 as hg
    eng = hg.Engine(precision)
    extra = {}
    if w.get("occupancy"):
        extra["neighbour_occupancy"] = w["occupancy"]
    if cell_occupancy:
        extra["cell_occupancy"] = cell_occupancy
    if w["nspecies"] == 2:
        d = hg.system_desc(w["n"], L, epsilon=KA["eps"], sigma=KA["sigma"], r_cut=w.get("rc", 2.5),
                           truncation=w["trunc"], smoothing=0.005, skin=w["skin"], timestep=w["dt"],
                           integrator="andersen" if w["rate"] > 0 else "verlet", temperature=w["T"],
                           collision_rate=w["rate"], seed=seed, **extra)
    else:
        d = hg.system_desc(w["n"], L, r_cut=w.get("rc", 2.5), truncation=w["trunc"], skin=w["skin"],
                           timestep=w["dt"], integrator="andersen" if w["rate"] > 0 else "verlet",
                           temperature=w["T"], collision_rate=w["rate"], seed=seed, **extra)
    eng.add_system(d)
    eng.commit()
    return eng


def equilibrated_state(w, r, v, species, L, seed=7):
    """The reference benchmarks start from configurations equilibrated at T
    (examples/benchmarks/*/generate_configuration.lua): the synthetic start
    (relaxed by steepest descent for KA) advanced with Andersen collisions."""
    e = w["equilibrate"]
    weq = dict(w, rate=e["rate"], dt=e["dt"])
    eng = make_engine(weq, L, seed=seed)
    eng.set("species", species)
    eng.set("position", r)
    if w["nspecies"] == 2:
        eng.minimize(RELAX_STEPS, RELAX_STEP_SIZE, RELAX_MAX_MOVE)
    eng.set("velocity", v)
    eng.step(e["steps"])
    r, v = eng.get("position"), eng.get("velocity")
    eng.close()
    return r, v


class ClockSampler:
    """SM clocks and throttle reasons sampled during the timed region.

    Reads NVML through ctypes every 5 ms in a thread (the timed regions of
    the small workloads last well under a second); falls back to
    `nvidia-smi -lms 50` where NVML cannot be loaded.  Only reads settings.
    """

    # nvmlClocksEventReasons bits
    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x40: "sw_thermal_slowdown", 0x80: "hw_thermal_slowdown"}
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        import threading
        self.rows = []          # (sm_mhz, reason bits)
        self.max_mhz = None
        self.p = None
        self.thread = None
        self.stop_flag = threading.Event()
        vis = os.environ.get("CUDA_VISIBLE_DEVICES", "")
        index = int(vis.split(",")[device]) if vis and vis.split(",")[device].strip().isdigit() else device
        if self._nvml_start(index):
            first = threading.Event()
            self.thread = threading.Thread(target=self._poll, args=(first,), daemon=True)
            self.thread.start()
            first.wait(2.0)
            return
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(index), "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "50"],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.p.stdout.readline()   # started: the first sample precedes the timed region
        except OSError:
            self.p = None

    def _nvml_start(self, index):
        import ctypes
        try:
            lib = ctypes.CDLL("libnvidia-ml.so.1")
            if lib.nvmlInit_v2() != 0:
                return False
            h = ctypes.c_void_p()
            if lib.nvmlDeviceGetHandleByIndex_v2(ctypes.c_uint(index), ctypes.byref(h)) != 0:
                return False
            mx = ctypes.c_uint()
            if lib.nvmlDeviceGetMaxClockInfo(h, ctypes.c_int(1), ctypes.byref(mx)) != 0:   # NVML_CLOCK_SM
                return False
            self.max_mhz = float(mx.value)
            self.reasons_fn = getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
                lib.nvmlDeviceGetCurrentClocksThrottleReasons
            self.lib, self.h = lib, h
            return True
        except (OSError, AttributeError):
            return False

    def _poll(self, first):
        import ctypes
        mhz, bits = ctypes.c_uint(), ctypes.c_ulonglong()
        while True:
            if self.lib.nvmlDeviceGetClockInfo(self.h, ctypes.c_int(1), ctypes.byref(mhz)) == 0 and \
                    self.reasons_fn(self.h, ctypes.byref(bits)) == 0:
                self.rows.append((float(mhz.value), int(bits.value)))
            first.set()
            if self.stop_flag.wait(0.005):
                return

    def stop(self):
        if self.thread is not None:
            self.stop_flag.set()
            self.thread.join()
            self.lib.nvmlShutdown()
            if not self.rows:
                return None
            reasons = sorted({name for _, b in self.rows for bit, name in self.REASONS.items() if b & bit})
            return {"sm_mhz": float(np.median([r[0] for r in self.rows])), "sm_max_mhz": self.max_mhz,
                    "samples": len(self.rows), "reasons": reasons, "source": "nvml, 5 ms"}
        if self.p is None:
            return None
        self.p.terminate()
        try:
            out, _ = self.p.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
            out, _ = self.p.communicate()
        rows = [[x.strip() for x in line.split(",")] for line in out.strip().splitlines() if line.strip()]
        rows = [r for r in rows if len(r) == 7]
        if not rows:
            return None
        sm = [float(r[0]) for r in rows if r[0].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for k, name in enumerate(names):
                if r[3 + k].lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": float(rows[0][1]),
                "samples": len(rows), "reasons": sorted(reasons), "source": "nvidia-smi, 50 ms"}


def dram_traffic(workload):
    """DRAM bytes per force launch from the committed ncu capture of this workload, or None."""
    path = os.path.join(REPO, "profiles", "dram_traffic.json")
    try:
        with open(path) as fh:
            rec = json.load(fh).get(workload)
    except (OSError, ValueError):
        return None, None
    if not rec:
        return None, None
    return float(rec["dram_bytes_per_launch"]), rec["from"]


def peaks():
    try:
        with open(MEASURED) as fh:
            p = json.load(fh)
        return float(p["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def cpu_baseline(w, r, v, species, L, budget_s=15.0):
    """FP64 single-thread host backend restatement on a bounded sample."""
    import oracle
    if w["nspecies"] == 2:
        pot = oracle.Potential(KA["eps"], KA["sigma"], w.get("rc", 2.5), w["trunc"], h=0.005)
    else:
        pot = oracle.Potential(1.0, 1.0, w.get("rc", 2.5), w["trunc"])
    n = w["n"]
    mass = np.ones(n)
    t0 = time.perf_counter()
    oracle.md_run(r, v, species, mass, [L] * 3, pot, w["skin"], w["dt"], 2, temperature=w["T"],
                  coll_rate=w["rate"], seed=1)
    t_probe = time.perf_counter() - t0
    steps = int(max(2, min(2000, (budget_s / max(t_probe, 1e-3)) * 2)))
    t0 = time.perf_counter()
    oracle.md_run(r, v, species, mass, [L] * 3, pot, w["skin"], w["dt"], steps, temperature=w["T"],
                  coll_rate=w["rate"], seed=1)
    dt = time.perf_counter() - t0
    return {"value": n * steps / dt, "unit": "particle-steps/s", "cores": 1, "kind": "port",
            "sample": "%s, %d MD steps from the synthetic start (list builds included), FP64, 1 thread" %
                      (w["name"], steps)}


def force_accuracy(eng, w):
    """Force error of the engine's current state against the FP64 oracle, on
    the CPU beside the baseline: max_i |F_i - F64_i| / max(|F64_i|, F_rms),
    with F64 at the double-single state (hi + lo words) and, for comparison,
    at the float hi words alone (what a kernel reading the hi words computes)."""
    import oracle
    n = w["n"]
    pot = _ref_potential(w)
    eng.force(aux=True)
    f = eng.get("force")
    Lf = np.array(eng.info().box_f32, dtype=np.float32)
    pos4 = eng.get_raw("position_hi")[eng.get("reverse_id")]
    species = eng.get("species")
    out = {}
    for key, r in (("vs_fp64_of_dsfloat_state", eng.get("position")),
                   ("vs_fp64_at_float_hi_words", pos4[:, :3].astype(np.float64))):
        ref = oracle.forces(r, species, Lf.astype(np.float64), pot, pos4=pos4, Lf=Lf, aux=False)["force"]
        norm = np.linalg.norm(ref, axis=1)
        e = np.linalg.norm(f - ref, axis=1) / np.maximum(norm, np.sqrt(np.mean(norm ** 2)))
        out[key] = {"max": float(e.max()), "median": float(np.median(e))}
    out["metric"] = "max_i |F_i - F64_i| / max(|F64_i|, F_rms), n = %d" % n
    return out


def _ref_potential(w):
    import oracle
    if w["nspecies"] == 2:
        return oracle.Potential(KA["eps"], KA["sigma"], w.get("rc", 2.5), w["trunc"], h=0.005)
    return oracle.Potential(1.0, 1.0, w.get("rc", 2.5), w["trunc"])


def ref_steps_per_sample(args, w):
    """MD steps of the reference arm per bench step: those of the GPU arm
    (--md-steps) up to 1e7 particle-steps per bench step (about 7 s of one
    core), fewer for larger systems."""
    return max(1, min(int(args.md_steps), int(1e7 // w["n"])))


def _ref_worker(wname, k, warmup, steps, per, relax, barrier, queue):
    """One replica of the reference arm (a spawned process): its own seeded
    copy of the workload, FP64 host-backend restatement, one thread."""
    import oracle
    w = workload(wname)
    r, v, species, L = initial_state(w, seed=2024 + k)
    pot = _ref_potential(w)
    mass = np.ones(w["n"])
    if w["nspecies"] == 2 and relax:
        r, _, _ = oracle.minimize(r, species, [L] * 3, pot, w["skin"], relax, RELAX_STEP_SIZE, RELAX_MAX_MOVE)
    for _ in range(warmup):
        oracle.md_run(r, v, species, mass, [L] * 3, pot, w["skin"], w["dt"], 1, temperature=w["T"],
                      coll_rate=w["rate"], seed=1)
    barrier.wait()
    t0 = time.perf_counter()
    for j in range(steps):
        oracle.md_run(r, v, species, mass, [L] * 3, pot, w["skin"], w["dt"], per, temperature=w["T"],
                      coll_rate=w["rate"], seed=1 + j)
    queue.put(time.perf_counter() - t0)


def run_reference(args, w):
    """The reference arm: the reference's host backend (its FP64 restatement,
    single-threaded as the reference is) as one independent replica per
    host core, started together; value = all replicas' particle-steps over
    the slowest replica's time."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    cores = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)
    per = ref_steps_per_sample(args, w)
    # the random KA start relaxed by FP64 steepest descent, as long as the
    # GPU arm relaxes its own (each replica in parallel: ~0.14 s a step at 64k)
    relax = RELAX_STEPS if w["nspecies"] == 2 else 0
    barrier = ctx.Barrier(cores)
    queue = ctx.Queue()
    procs = [ctx.Process(target=_ref_worker, args=(args.workload, k, args.warmup, args.steps, per, relax, barrier, queue))
             for k in range(cores)]
    for p in procs:
        p.start()
    times = [queue.get() for _ in procs]
    for p in procs:
        p.join()
    dt = max(times)
    n = w["n"]
    value = cores * n * per * args.steps / dt
    sample = ("%s: %d independent replicas (one per host core), each %d x %d MD steps, FP64 host-backend "
              "restatement, one thread per replica (the reference host backend is single-threaded)%s"
              % (w["name"], cores, args.steps, per, ", starts relaxed by %d descent steps" % relax if relax else ""))
    line = {"metric": "particle-steps/s", "value": value, "unit": "particle-steps/s", "impl": "reference",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * dt / (per * args.steps), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": dict(workload_config(w, per), parallelism="replicas: one per host core (%d)" % cores),
            "cpu_baseline": {"value": value, "unit": "particle-steps/s", "cores": cores, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def workload_config(w, md_steps):
    """The workload part of a line's config, the same for both arms."""
    return {"workload": w["name"], "n": w["n"], "density": w["rho"], "temperature": w["T"], "dt": w["dt"],
            "md_steps_per_bench_step": md_steps, "truncation": w["trunc"], "skin": w["skin"],
            "r_cut": w.get("rc", 2.5)}


def ensemble_specs(count=256, seed=256):
    """Replicas of the batched-ensemble workload: N log-uniform in [500, 32000],
    density uniform in [0.7, 1.2], T uniform in [0.5, 2.0], LJ or KA by a coin
    flip (KA: 80:20, smooth_r4, Andersen at T; LJ: shifted cut-off, NVE)."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        n = int(np.floor(np.exp(rng.uniform(np.log(500), np.log(32000)))))
        rho = float(rng.uniform(0.7, 1.2))
        T = float(rng.uniform(0.5, 2.0))
        ka = bool(rng.integers(0, 2))
        L = (n / rho) ** (1 / 3)
        m = int(np.ceil(n ** (1 / 3)))
        g = (np.arange(m) + 0.5) * (L / m) - 0.5 * L
        sites = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
        r = sites[rng.permutation(len(sites))[:n]] + rng.uniform(-0.02, 0.02, size=(n, 3))
        v = rng.normal(0, np.sqrt(T), size=(n, 3))
        v -= v.mean(axis=0)
        sp = np.zeros(n, dtype=np.uint32)
        if ka:
            sp[rng.permutation(n)[: n // 5]] = 1
            d = dict(epsilon=KA["eps"], sigma=KA["sigma"], r_cut=2.5, truncation="smooth_r4", smoothing=0.005,
                     skin=0.3, timestep=0.002, integrator="andersen", temperature=T, collision_rate=1.0,
                     seed=1000 + k)
        else:
            d = dict(r_cut=2.5, truncation="shifted", skin=0.3, timestep=0.002)
        out.append(dict(n=n, L=L, r=r, v=v, sp=sp, desc=d))
    return out


def run_ensemble(args, emit=True):
    """ENS-256: all replicas in one engine (one launch per phase, graph-captured
    step chunks) against looping the one-system path over the same replicas.
    Returns the line (rank 0), printed unless emit is false."""
    import torch
    import halmd_gb300 as hg
    from halmd_gb300.shard import combine, partition, rank_env
    from halmd_gb300.tune import autotune_force_lanes, autotune_list_build
    rank, world, local = rank_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    specs = ensemble_specs()
    count = len(specs)
    # replicas only: each rank takes a share of the replicas (bin-packed by size)
    specs = [specs[k] for k in partition([s["n"] for s in specs], world)[rank]]
    ntot = sum(s["n"] for s in specs)
    M = args.md_steps

    def load(eng, k, s):
        eng.set("species", s["sp"], k)
        eng.set("position", s["r"], k)
        eng.set("velocity", s["v"], k)

    batch = hg.Engine("dsfloat")
    for s in specs:
        batch.add_system(hg.system_desc(s["n"], s["L"], **s["desc"]))
    batch.commit()
    if args.neighbour_scan:
        batch.set_option("neighbour_scan", args.neighbour_scan)
    for k, s in enumerate(specs):
        load(batch, k, s)
    batch.step(M)
    list_ms = {}
    if not args.neighbour_scan:
        _, list_ms = autotune_list_build(batch, use_cache=False)
    lanes, lane_ms = autotune_force_lanes(batch, use_cache=False)
    if args.phases:
        # module-path breakdown of the batched step (one launch per phase for all replicas)
        chains0 = batch.get_option("rebuild_chains")
        batch.profile(True)
        for _ in range(args.phases):
            batch.integrate()
            batch.force()
            batch.finalize()
        out = {"workload": "ENS-256", "particles": ntot, "md_steps": args.phases, "force_lanes": lanes,
               "list_block": batch.get_option("list_block"),
               "rebuild_chains": batch.get_option("rebuild_chains") - chains0}
        for ph in ("integrate", "rebuild", "force", "finalize"):
            ms, cnt = batch.profile_get(ph)
            out[ph + "_ms_per_call"] = ms / max(cnt, 1)
            out[ph + "_ms_per_step"] = ms / max(args.phases, 1)
        print(json.dumps(out))
        batch.close()
        return
    for _ in range(args.warmup):
        batch.step(M)
    stream = torch.cuda.ExternalStream(batch.stream)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    chains0, kernels0 = batch.get_option("rebuild_chains"), batch.get_option("step_kernels")
    clocks = ClockSampler(0)
    total_ms = 0.0
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        batch.step(M)
        e1.record(stream)
        e1.synchronize()
        total_ms += e0.elapsed_time(e1)
    clk = clocks.stop()
    chains = batch.get_option("rebuild_chains") - chains0
    inf = batch.info(0)
    work_all, ms_all = combine(ntot * M * args.steps, total_ms, device="cuda")
    batched = work_all / (ms_all * 1e-3)
    ntot_all = combine(ntot, 0.0, device="cuda")[0]
    # step-graph kernels, plus the rebuild chain in every step where any replica rebuilt
    launches = (batch.get_option("step_kernels") - kernels0) + chains * inf.rebuild_kernels
    scan_used = batch.get_option("neighbour_scan")
    batch.close()

    # the plain path: one engine per replica, stepped one after another (the
    # same list-build scan as the batch)
    engines = []
    for s in specs:
        e = hg.Engine("dsfloat")
        e.add_system(hg.system_desc(s["n"], s["L"], **s["desc"]))
        e.commit()
        e.set_option("neighbour_scan", scan_used)
        load(e, 0, s)
        e.step(M)
        engines.append(e)
    for e in engines:
        e.step(M)
    torch.cuda.synchronize()
    loop_steps = max(1, args.steps // 2)
    t0 = time.perf_counter()
    for _ in range(loop_steps):
        for e in engines:
            e.step(M)
    torch.cuda.synchronize()
    loop_s = time.perf_counter() - t0
    lwork, lms = combine(ntot * M * loop_steps, 1e3 * loop_s, device="cuda")
    looped = lwork / (lms * 1e-3)
    for e in engines:
        e.close()
    if world > 1:
        dist.destroy_process_group()
    if rank != 0:
        return
    line = {"metric": "particle-steps/s", "value": batched, "unit": "particle-steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_all / (M * args.steps),
            "higher_is_better": True, "scaling": "strong" if world > 1 else "weak", "vs_baseline": None,
            "dtype": "f32 (dsfloat state)", "data": "synthetic",
            "config": {"workload": "ENS-256", "replicas": count, "particles": int(ntot_all),
                       "parallelism": "replicas bin-packed over %d GPUs" % world if world > 1 else "single",
                       "md_steps_per_bench_step": M, "force_lanes": lanes,
                       "autotune_force_ms": {str(k): v for k, v in lane_ms.items()},
                       "neighbour_scan": scan_used, "autotune_list_ms": list_ms,
                       "l2": "flushed (256 MB write) between timed bench steps"},
            "looped_plain_path": {"value": looped, "unit": "particle-steps/s",
                                  "note": "256 engines of one replica each, hmd_step(%d) in turn" % M},
            "batch_speedup": batched / looped, "gpu_launches": launches, "clocks": clk}
    if emit:
        print(json.dumps(line))
    return line


def serve_jobs(count, steps_scale, rate=50.0, seed=2000):
    """Served-workload stream: Poisson arrivals at `rate` per second, N
    log-uniform in [1e3, 2e5], density uniform in [0.8, 1.2], T uniform in
    [0.5, 1.5], steps log-uniform in [1e3, 1e5] times `steps_scale`, LJ or KA by
    a coin flip; all drawn from `seed`."""
    from halmd_gb300.serve import Job
    rng = np.random.default_rng(seed)
    t = 0.0
    jobs = []
    for k in range(count):
        t += rng.exponential(1.0 / rate)
        n = int(np.floor(np.exp(rng.uniform(np.log(1e3), np.log(2e5)))))
        rho = float(rng.uniform(0.8, 1.2))
        T = float(rng.uniform(0.5, 1.5))
        steps = max(1, int(np.exp(rng.uniform(np.log(1e3), np.log(1e5))) * steps_scale))
        ka = bool(rng.integers(0, 2))
        L = (n / rho) ** (1 / 3)
        m = int(np.ceil(n ** (1 / 3)))
        g = (np.arange(m) + 0.5) * (L / m) - 0.5 * L
        sites = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
        r = sites[rng.permutation(len(sites))[:n]] + rng.uniform(-0.02, 0.02, size=(n, 3))
        v = rng.normal(0, np.sqrt(T), size=(n, 3))
        v -= v.mean(axis=0)
        sp = np.zeros(n, dtype=np.uint32)
        if ka:
            sp[rng.permutation(n)[: n // 5]] = 1
            d = dict(epsilon=KA["eps"], sigma=KA["sigma"], r_cut=2.5, truncation="smooth_r4", smoothing=0.005,
                     skin=0.3, timestep=0.002, integrator="andersen", temperature=T, collision_rate=1.0,
                     seed=5000 + k)
        else:
            d = dict(r_cut=2.5, truncation="shifted", skin=0.3, timestep=0.002)
        jobs.append(Job(k, n, L, d, r, v, sp, steps, arrival=t))
    return jobs


def run_serve(args, emit=True):
    """SERVE: continuous batching under an 80% HBM budget against a FIFO run
    of the one-system path, same job stream."""
    import torch
    from halmd_gb300.serve import Server, run_fifo
    from halmd_gb300.shard import combine, partition, rank_env
    rank, world, local = rank_env()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    def my_jobs():
        # replicas only: each rank serves a share of the stream (bin-packed by work)
        all_jobs = serve_jobs(args.serve_jobs, args.serve_steps_scale)
        return [all_jobs[k] for k in partition([j.work for j in all_jobs], world)[rank]]

    def gather_latency(js):
        lat = [j.completed - j.arrival for j in js]
        if dist is None:
            return lat
        out = [None] * world
        dist.all_gather_object(out, lat)
        return [x for part in out for x in part]

    def pct(lat):
        a = np.array(lat)
        return {"p50": float(np.percentile(a, 50)), "p99": float(np.percentile(a, 99)), "mean": float(a.mean())}

    jobs = my_jobs()
    work = sum(j.work for j in jobs)
    srv = Server(budget_fraction=0.8, max_slots=args.serve_max_slots, max_jobs=1024, neighbour_capacity=288,
                 chunk=args.md_steps)
    clocks = ClockSampler(0)
    limit = args.serve_time_limit or None
    st = srv.run(jobs, realtime=True, time_limit=limit)
    clk = clocks.stop()
    done_jobs = [j for j in jobs if j.completed is not None]
    lat = pct(gather_latency(done_jobs)) if done_jobs else {"p50": None, "p99": None, "mean": None}
    budget = srv.budget
    srv.close()
    work, makespan = combine(st["work"], st["makespan"], device="cuda")
    chunks = int(combine(st["chunks"], 0.0, device="cuda")[0])
    fifo_jobs = my_jobs()
    fst = run_fifo(fifo_jobs, time_limit=limit)
    fdone = [j for j in fifo_jobs if j.completed is not None]
    flat = pct(gather_latency(fdone)) if fdone else {"p50": None, "p99": None, "mean": None}
    fwork, fmakespan = combine(fst["work"], fst["makespan"], device="cuda")
    njobs = int(combine(len(jobs), 0.0, device="cuda")[0])
    if dist is not None:
        dist.destroy_process_group()
    if rank != 0:
        return
    completed, fcompleted = st["completed"], fst["completed"]
    st = {"makespan": makespan, "chunks": chunks}
    fst = {"makespan": fmakespan}
    line = {"metric": "particle-steps/s", "value": work / st["makespan"], "unit": "particle-steps/s", "n_gpus": world,
            "steps": st["chunks"], "warmup": 0, "ms_per_step": 1e3 * st["makespan"] / max(st["chunks"], 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32 (dsfloat state)",
            "data": "synthetic",
            "config": {"workload": "SERVE", "jobs": njobs, "arrival_rate_per_s": 50,
                       "parallelism": "jobs bin-packed over %d GPUs" % world if world > 1 else "single",
                       "steps_scale": args.serve_steps_scale, "particle_steps": work, "chunk_md_steps": args.md_steps,
                       "hbm_budget": budget, "time_limit_s": limit},
            "latency_s": {"p50": lat["p50"], "p99": lat["p99"], "mean": lat["mean"],
                          "over": "jobs completed%s" % (" within the time limit" if limit else "")},
            "completed_jobs": completed if world == 1 else None,
            "makespan_s": st["makespan"],
            "fifo_plain_path": {"value": fwork / fst["makespan"], "unit": "particle-steps/s",
                                "latency_s": flat, "makespan_s": fst["makespan"],
                                "completed_jobs": fcompleted if world == 1 else None,
                                "particle_steps": fwork},
            "throughput_ratio_vs_fifo": (work / st["makespan"]) / (fwork / fst["makespan"]), "clocks": clk}
    if emit:
        print(json.dumps(line))
    return line


def run_phases(args, w):
    """Per-phase breakdown of the MD step through the module-level calls."""
    r, v, species, L = initial_state(w)
    eng = make_engine(w, L, cell_occupancy=args.cell_occupancy or None)
    if args.force_lanes:
        eng.set_option("force_lanes", args.force_lanes)
        eng.set_option("list_block", args.list_block)
    if args.neighbour_scan:
        eng.set_option("neighbour_scan", args.neighbour_scan)
    eng.set("species", species)
    eng.set("position", r)
    if w["nspecies"] == 2:
        eng.minimize(RELAX_STEPS, RELAX_STEP_SIZE, RELAX_MAX_MOVE)
    eng.set("velocity", v)
    eng.step(50)
    for _ in range(5):
        eng.integrate(); eng.force(); eng.finalize()
    inf0 = eng.info()
    eng.profile(True)
    for _ in range(args.phases):
        eng.integrate()
        eng.force()
        eng.finalize()
    inf1 = eng.info()
    out = {"workload": w["name"], "n": w["n"], "md_steps": args.phases,
           "rebuilds": int(inf1.rebuilds - inf0.rebuilds), "force_lanes": eng.get_option("force_lanes"),
           "list_block": eng.get_option("list_block"), "neighbour_scan": eng.get_option("neighbour_scan"),
           "cell_occupancy": args.cell_occupancy or 0.5}
    for ph in ("integrate", "rebuild", "force", "finalize"):
        ms, cnt = eng.profile_get(ph)
        out[ph + "_ms_per_call"] = ms / max(cnt, 1)
        out[ph + "_ms_per_step"] = ms / max(args.phases, 1)
    print(json.dumps(out))
    eng.close()


def run_variants(args, w):
    """The precision variants of one workload from the same start: float
    positions, dsfloat positions (the default engine) and the FP64 variant
    (HMD_PRECISION_DOUBLE), each run for --variants MD steps of NVE.  Per
    variant: the energy drift |E(t) - E(0)| / |E(0)| fitted per 1e5 steps,
    its difference from the FP64 run's, and the force error of the start
    state against FP64 forces of the same state (the FP64 engine with the
    float cut-off test, so the pair sets agree)."""
    import halmd_gb300 as hg
    import torch
    steps, every = int(args.variants), max(1, int(args.variants) // 100)
    r, v, species, L = initial_state(w)
    wv = dict(w, rate=0.0)                      # NVE: drift is a property of the integrator and arithmetic
    # the common start: the synthetic state (KA: relaxed) after 200 steps of
    # the dsfloat engine, so that forces are those of a fluid, not a lattice
    eng = make_engine(wv, L)
    eng.set("species", species)
    eng.set("position", r)
    if w["nspecies"] == 2:
        eng.minimize(RELAX_STEPS, RELAX_STEP_SIZE, RELAX_MAX_MOVE)
    eng.set("velocity", v)
    eng.step(200)
    r, v = eng.get("position"), eng.get("velocity")
    eng.close()

    def engine(precision, float_cutoff=False):
        eng = make_engine(wv, L, precision=precision)
        if float_cutoff:
            eng.set_option("float_cutoff", 1)
        eng.set("species", species)
        eng.set("position", r)
        eng.set("velocity", v)
        return eng

    out = {}
    ref64 = engine("double", float_cutoff=True)
    for precision in ("float", "dsfloat", "double"):
        eng = engine(precision)
        eng.force(aux=True)
        f = eng.get("force")
        ref64.set("position", eng.get("position"))
        ref64.force()
        f64 = ref64.get("force")
        norm = np.linalg.norm(f64, axis=1)
        err = np.linalg.norm(f - f64, axis=1) / np.maximum(norm, np.sqrt(np.mean(norm ** 2)))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        t, e = [], []
        for k in range(steps // every + 1):
            if k:
                eng.step(every - 1)
            eng.step(1, aux_last=True)
            th = eng.thermo()
            t.append(k * every)
            e.append(0.5 * th["mv2"] + th["epot"])
        wall = time.perf_counter() - t0
        t, e = np.array(t, dtype=float), np.array(e)
        (slope, _), cov = np.polyfit(t, e, 1, cov=True)
        out[precision] = {"drift_per_1e5_steps": float(slope * 1e5 / abs(e[0])),
                          "drift_stderr": float(np.sqrt(cov[0, 0]) * 1e5 / abs(e[0])),
                          "max_abs_dE_over_E0": float(np.max(np.abs(e - e[0])) / abs(e[0])),
                          "force_err_vs_fp64": {"max": float(err.max()), "median": float(np.median(err))},
                          "ms_per_step": 1e3 * wall / steps}
        eng.close()
    ref64.close()
    for precision in ("float", "dsfloat"):
        out[precision]["drift_minus_fp64"] = out[precision]["drift_per_1e5_steps"] - out["double"]["drift_per_1e5_steps"]
    print(json.dumps({"workload": w["name"], "n": w["n"], "md_steps": steps, "sample_every": every,
                      "ensemble": "NVE from the same start", "variants": out}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300")
    ap.add_argument("--workload", default="ka64k",
                    help="ka64k, lj1m, lj4k, ens256, serve; ref-lj64k, ref-ka256k: the reference's own benchmarks")
    ap.add_argument("--md-steps", type=int, default=100, help="MD steps per bench step")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-lj1m", action="store_true", help="default workload: skip the LJ-1M sub-record")
    ap.add_argument("--no-batched", action="store_true",
                    help="default workload: skip the ENS-256 and SERVE sub-records")
    ap.add_argument("--sub-serve-time-limit", type=float, default=30.0,
                    help="default workload: seconds of the SERVE sub-record's stream prefix (each of the served "
                         "and FIFO runs)")
    ap.add_argument("--variants", type=int, default=0,
                    help="run the float, dsfloat and FP64 variants of the workload for N MD steps from the same "
                         "start and print their energy drift and force error, then exit")
    ap.add_argument("--phases", type=int, default=0,
                    help="run N MD steps through the module calls (integrate / force / finalize, one launch "
                         "each, no graph) with the per-phase CUDA-event timers, print the breakdown and exit; "
                         "this is the run profilers can attribute kernel by kernel")
    ap.add_argument("--force-lanes", type=int, default=0,
                    help="threads per particle in the force kernel (0: autotune in the bench, engine default "
                         "in --phases)")
    ap.add_argument("--list-block", type=int, default=0, help="list block width (0 auto, 4, 8) with --force-lanes")
    ap.add_argument("--fuse-steps", type=int, default=1, help="1: fused finalize + integrate in chunks")
    ap.add_argument("--cell-occupancy", type=float, default=0.0,
                    help="binning cell occupancy (the reference's parameter; 0: autotuned in the bench among "
                         "0.5, 1, 1.5 and 2, 0.5 elsewhere)")
    ap.add_argument("--neighbour-scan", type=int, default=0,
                    help="list build: 1 per lane, 2 shared per warp; 0: autotuned in the bench, the engine's "
                         "choice by system size in --phases")
    ap.add_argument("--serve-jobs", type=int, default=200)
    ap.add_argument("--serve-steps-scale", type=float, default=0.1)
    ap.add_argument("--serve-max-slots", type=int, default=1 << 24)
    ap.add_argument("--serve-time-limit", type=float, default=0.0,
                    help="SERVE: stop both runs after this many seconds (a prefix of the stream; 0: run to the end)")
    args = ap.parse_args()
    if args.workload == "serve":
        if args.impl == "reference":
            raise SystemExit("the served workload has no reference arm")
        return run_serve(args)
    if args.workload == "ens256":
        if args.impl == "reference":
            raise SystemExit("the ensemble workload has no reference arm")
        return run_ensemble(args)
    w = workload(args.workload)
    if args.phases:
        return run_phases(args, w)
    if args.variants:
        return run_variants(args, w)

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return run_reference(args, w)

    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    line = measure(args, w, world, rank, local, dist, args.steps, args.warmup, not args.no_cpu_baseline)
    if world == 1 and args.workload == "ka64k" and not args.no_lj1m:
        # the metric's second configuration: LJ-1M, fewer bench steps (each is
        # 100 MD steps of a million particles)
        sub = measure(args, workload("lj1m"), world, rank, local, dist, min(args.steps, 10), 3,
                      not args.no_cpu_baseline)
        line["lj1m"] = {k: sub[k] for k in ("value", "unit", "ms_per_step", "steps", "warmup", "config", "e2e",
                                            "gpu_launches", "roofline", "clocks", "cpu_baseline", "accuracy", "run")
                        if k in sub}
    if world == 1 and args.workload == "ka64k" and not args.no_batched:
        # the batched and served forms of the metric, short: ENS-256 with 3
        # bench steps, and SERVE's 2000-job stream over a time-bounded prefix
        import copy
        a = copy.copy(args)
        a.steps, a.warmup, a.phases, a.neighbour_scan = 3, 3, 0, 0
        try:
            ens = run_ensemble(a, emit=False)
            line["ens256"] = {k: ens[k] for k in ("value", "unit", "ms_per_step", "steps", "config",
                                                  "looped_plain_path", "batch_speedup", "gpu_launches", "clocks")}
        except Exception as ex:   # a failed sub-record must not take the headline with it
            line["ens256"] = {"error": "%s: %s" % (type(ex).__name__, str(ex)[:200])}
        a = copy.copy(args)
        a.serve_jobs, a.serve_steps_scale, a.serve_time_limit = 2000, 1.0, args.sub_serve_time_limit
        try:
            srv = run_serve(a, emit=False)
            line["serve"] = {k: srv[k] for k in ("value", "unit", "config", "latency_s", "completed_jobs",
                                                 "makespan_s", "fifo_plain_path", "throughput_ratio_vs_fifo",
                                                 "clocks")}
        except Exception as ex:
            line["serve"] = {"error": "%s: %s" % (type(ex).__name__, str(ex)[:200])}
    if rank == 0:
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


def measure(args, w, world, rank, local, dist, steps, warmup, with_cpu):
    """The GPU arm on one workload: K timed bench steps after W warm-up
    steps; returns the JSON line (rank 0 holds the max over ranks)."""
    import torch
    r, v, species, L = initial_state(w, seed=2024 + rank)
    if w.get("equilibrate"):
        r, v = equilibrated_state(w, r, v, species, L, seed=7 + rank)
    eng = make_engine(w, L, seed=7 + rank, cell_occupancy=args.cell_occupancy or None)
    eng.set_option("fuse_steps", args.fuse_steps)
    if args.neighbour_scan:
        eng.set_option("neighbour_scan", args.neighbour_scan)
    n = w["n"]
    eng.set("species", species)
    eng.set("position", r)
    if w["nspecies"] == 2 and not w.get("equilibrate"):
        eng.minimize(RELAX_STEPS, RELAX_STEP_SIZE, RELAX_MAX_MOVE)
        r = eng.get("position")
    eng.set("velocity", v)
    eng.step(max(1, args.md_steps))   # equilibrate lists / first rebuilds
    from halmd_gb300.tune import autotune_cell_occupancy, autotune_force_lanes, autotune_list_build
    cell_occ, cell_ms = args.cell_occupancy or 0.5, {}
    if not args.cell_occupancy:
        # binning cell size: engines of each candidate cell occupancy on this state
        r_now, v_now = eng.get("position"), eng.get("velocity")

        def build(occ):
            e = make_engine(w, L, seed=7 + rank, cell_occupancy=occ)
            if args.neighbour_scan:
                e.set_option("neighbour_scan", args.neighbour_scan)
            e.set("species", species)
            e.set("position", r_now)
            e.set("velocity", v_now)
            return e

        cell_occ, cell_ms = autotune_cell_occupancy(build)
        if cell_occ != 0.5:
            eng.close()
            eng = build(cell_occ)
            eng.set_option("fuse_steps", args.fuse_steps)
            eng.step(max(1, args.md_steps))
    list_ms = {}
    if not args.neighbour_scan:
        _, list_ms = autotune_list_build(eng, use_cache=False)
    if args.force_lanes:
        eng.set_option("force_lanes", args.force_lanes)
        eng.set_option("list_block", args.list_block)
        lanes, lane_ms = args.force_lanes, {}
    else:
        lanes, lane_ms = autotune_force_lanes(eng, use_cache=False)
    stream = torch.cuda.ExternalStream(eng.stream)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()

    M = args.md_steps
    for _ in range(warmup):
        eng.step(M)
    inf0 = eng.info()
    k0, c0 = eng.get_option("step_kernels"), eng.get_option("rebuild_chains")
    barrier()
    clocks = ClockSampler(local)
    total_ms = 0.0
    for _ in range(steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        eng.step(M)
        e1.record(stream)
        e1.synchronize()
        total_ms += e0.elapsed_time(e1)
    barrier()
    clk = clocks.stop()
    inf1 = eng.info()
    t = torch.tensor([total_ms], dtype=torch.float64, device="cuda")
    if dist is not None:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    total_ms = float(t.item())
    md_steps = M * steps
    value = world * n * md_steps / (total_ms * 1e-3)
    rebuilds = int(inf1.rebuilds - inf0.rebuilds)
    launches = (eng.get_option("step_kernels") - k0) + (eng.get_option("rebuild_chains") - c0) * inf1.rebuild_kernels

    # e2e: the public API with host buffers; H2D of the phase space, M steps, D2H of it
    e2e_ms = 0.0
    h2d = d2h = 0
    # the phase space lives in page-locked host memory (torch pin_memory),
    # which hmd_set / hmd_get copy with one DMA each
    pos = torch.empty((n, 3), dtype=torch.float64, pin_memory=True).numpy()
    vel = torch.empty((n, 3), dtype=torch.float64, pin_memory=True).numpy()
    eng.get("position", out=pos)
    eng.get("velocity", out=vel)
    for _ in range(max(1, steps // 2)):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        eng.set("position", pos)
        eng.set("velocity", vel)
        eng.step(M)
        eng.get("position", out=pos)
        eng.get("velocity", out=vel)
        e2e_ms += 1e3 * (time.perf_counter() - t0)
    e2e_steps = M * max(1, steps // 2)
    # bytes the API moves per bench step: set(position) and set(velocity) copy 3 n doubles each up,
    # get(position) and get(velocity) 3 n doubles each down (converted on the device); the rebuild request
    # after set(position) reads and writes the per-system state table
    h2d = 2 * 24 * n + 48 * len(eng.systems)
    d2h = 2 * 24 * n + 48 * len(eng.systems)
    e2e_value = world * n * e2e_steps / (e2e_ms * 1e-3)

    # dominant kernel: the pair force, timed alone with events on the engine stream
    eng.profile(True)
    for _ in range(20):
        eng.force()
    f_ms, f_cnt = eng.profile_get("force")
    eng.profile(False)
    counts, _ = eng.neighbour_lists()
    K_l = float(counts.mean())
    bytes_per_launch = n * (16 + 4 * K_l + 16)
    achieved = bytes_per_launch / (f_ms / f_cnt * 1e-3) / 1e9
    peak, peak_kind = peaks()
    traffic_bytes, traffic_from = dram_traffic(w["name"])

    cpu = acc = None
    if rank == 0 and world == 1 and with_cpu:
        cpu = cpu_baseline(w, r, v, species, L)
        acc = force_accuracy(eng, w)

    line = {"metric": "particle-steps/s", "value": value, "unit": "particle-steps/s", "n_gpus": world,
            "steps": steps, "warmup": warmup, "ms_per_step": total_ms / md_steps,
            "higher_is_better": True, "scaling": "weak",
            "vs_baseline": value / w["published"] if w.get("published") and world == 1 else None,
            "dtype": "f32 (dsfloat state)",
            "data": "synthetic",
            "config": dict(workload_config(w, M), l2="flushed (256 MB write) between timed bench steps",
                           parallelism="replicas" if world > 1 else "single"),
            "run": {"precision": "dsfloat", "rebuilds_in_timed_region": rebuilds,
                    "force_lanes": lanes, "list_block": eng.get_option("list_block"),
                    "autotune_force_ms": {str(k): v for k, v in lane_ms.items()},
                    "neighbour_scan": eng.get_option("neighbour_scan"),
                    "autotune_list_ms": list_ms,
                    "cell_occupancy": cell_occ, "autotune_cell_ms": cell_ms},
            "e2e": {"value": e2e_value, "unit": "particle-steps/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h,
                    "note": "per bench step: hmd_set(position, velocity) + hmd_step(%d) + "
                            "hmd_get(position, velocity), host arrays page-locked" % M},
            "gpu_launches": launches,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic_bytes, "traffic_unit": "bytes per launch",
                         "traffic_from": traffic_from, "kernel": "k_force",
                         "peak_source": peak_kind,
                         "bytes_per_launch": bytes_per_launch, "mean_list_length": K_l,
                         "force_ms": f_ms / f_cnt},
            "clocks": clk}
    if cpu is not None:
        line["cpu_baseline"] = cpu
    if acc is not None:
        line["accuracy"] = acc
    eng.close()
    return line


if __name__ == "__main__":
    main()
