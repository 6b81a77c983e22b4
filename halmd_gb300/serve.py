"""Continuous-batching job server: many independent MD jobs on one GPU.

Jobs (an LJ or Kob-Andersen system with its initial phase space and a step
count) are admitted into one engine with reserved capacity as soon as slots,
cells and table entries are free, advance together in captured graph chunks
(one launch per phase for all jobs), and leave when their step count is
reached; their phase space stays resident in HBM meanwhile.  Each job's
result does not depend on which other jobs shared the GPU: kernels are
deterministic per system, random streams are keyed by (job seed, particle
tag, job step), and a job that finishes in the middle of a chunk is frozen
on the device until the chunk ends.

No counterpart exists in the reference (one simulation per process); the
server is built on the engine's C ABI (hmd_engine_reserve / add_system /
remove_system / step / progress).
"""
import collections
import time

import numpy as np

from ._lib import Engine, HmdError, system_desc

HMD_ERR_NOMEM = -4


class Job:
    """One simulation request."""

    def __init__(self, jid, n, box, desc, position, velocity, species, steps, arrival=0.0):
        self.jid = jid
        self.n = int(n)
        self.box = box
        self.desc = dict(desc)
        self.position = np.asarray(position, dtype=np.float64)
        self.velocity = np.asarray(velocity, dtype=np.float64)
        self.species = np.asarray(species, dtype=np.uint32)
        self.steps = int(steps)
        self.arrival = float(arrival)
        self.admitted = None
        self.completed = None
        self.result = None          # dict(position, velocity, thermo) at completion

    @property
    def work(self):
        return self.n * self.steps

    def system_desc(self):
        return system_desc(self.n, self.box, **self.desc)


def device_memory_bytes():
    try:
        import torch
        return int(torch.cuda.mem_get_info()[1])
    except Exception:
        return 0


class Server:
    """Admit, advance and retire jobs in one engine with reserved capacity.

    budget_fraction: share of the GPU's memory the engine may reserve;
    max_slots caps the reservation (the engine's launch grids span it);
    engine_factory(precision) makes the engine (the C-ABI Engine)."""

    def __init__(self, budget_fraction=0.8, max_slots=1 << 24, max_jobs=1024, neighbour_capacity=288,
                 precision="dsfloat", chunk=100, force_lanes=None, total_bytes=None, engine_factory=Engine):
        total = total_bytes if total_bytes is not None else device_memory_bytes()
        # device bytes per slot: phase space (+ copies), list slots and snapshots
        per_slot = 360 + 4 * neighbour_capacity
        budget_slots = int(budget_fraction * total // per_slot) if total else max_slots
        slots = max(2048, min(max_slots, budget_slots))
        self.engine = engine_factory(precision)
        self.engine.reserve(slots, max_jobs, neighbour_capacity)
        if force_lanes:
            self.engine.set_option("force_lanes", force_lanes)
        self.engine.commit()
        self.chunk = int(chunk)
        self.table = max_jobs
        self.running = {}
        self.queue = collections.deque()
        self.done = []
        self.budget = dict(total_bytes=total, fraction=budget_fraction, slots=slots, per_slot=per_slot)

    def close(self):
        self.engine.close()

    def submit(self, job):
        self.queue.append(job)

    def _admit(self, now):
        admitted = 0
        while self.queue:
            job = self.queue[0]
            try:
                k = self.engine.add(job.system_desc())
            except HmdError as e:
                if e.code == HMD_ERR_NOMEM:
                    break          # wait for capacity to free up
                raise
            self.engine.set("species", job.species, k)
            self.engine.set("position", job.position, k)
            self.engine.set("velocity", job.velocity, k)
            self.engine.set_steps_left(job.steps, k)
            job.admitted = now
            self.running[k] = job
            self.queue.popleft()
            admitted += 1
        return admitted

    def _collect(self, now):
        if not self.running:
            return 0
        step, left = self.engine.progress(self.table)
        finished = [k for k in self.running if left[k] == 0]
        for k in finished:
            job = self.running.pop(k)
            job.result = dict(position=self.engine.get("position", k), velocity=self.engine.get("velocity", k),
                              image=self.engine.get("image", k), step=int(step[k]))
            job.completed = now
            self.engine.remove(k)
            self.done.append(job)
        return len(finished)

    def run(self, jobs, clock=time.perf_counter, realtime=True, time_limit=None):
        """Serve `jobs` (arrival times in seconds from the start).  With
        realtime=False arrivals are released as soon as the previous ones are
        admitted (throughput mode).  With a time_limit the run stops after
        the chunk that crosses it; `work` counts the particle-steps done by
        then (finished jobs and the steps of the running ones)."""
        pending = collections.deque(sorted(jobs, key=lambda j: j.arrival))
        t0 = clock()
        chunks = 0
        while pending or self.queue or self.running:
            now = clock() - t0
            if time_limit is not None and now >= time_limit:
                break
            while pending and (pending[0].arrival <= now or not realtime):
                self.submit(pending.popleft())
            self._admit(now)
            if self.running:
                self.engine.step(self.chunk)
                chunks += 1
                self._collect(clock() - t0)
            elif pending:
                time.sleep(max(0.0, min(0.01, pending[0].arrival - (clock() - t0))))
            elif self.queue:
                raise RuntimeError("job %d does not fit the reserved capacity" % self.queue[0].jid)
        makespan = clock() - t0
        work = sum(j.work for j in self.done)
        if self.running:
            step, _ = self.engine.progress(self.table)
            work += sum(job.n * int(step[k]) for k, job in self.running.items())
        return dict(makespan=makespan, chunks=chunks, work=work, completed=len(self.done))


def latency_stats(jobs):
    lat = np.array([j.completed - j.arrival for j in jobs])
    return dict(p50=float(np.percentile(lat, 50)), p99=float(np.percentile(lat, 99)), mean=float(lat.mean()))


def run_fifo(jobs, precision="dsfloat", clock=time.perf_counter, force_lanes=None, time_limit=None, chunk=1000):
    """The plain path: one engine per job, jobs one after another in arrival
    order (a job starts at max(arrival, previous completion)).  With a
    time_limit a job runs in chunks of `chunk` steps and the run stops after
    the chunk that crosses the limit; `work` counts the particle-steps done."""
    t0 = clock()
    work, completed = 0, 0
    for job in sorted(jobs, key=lambda j: j.arrival):
        now = clock() - t0
        if time_limit is not None and now >= time_limit:
            break
        if job.arrival > now:
            time.sleep(job.arrival - now)
        job.admitted = clock() - t0
        eng = Engine(precision)
        eng.add_system(job.system_desc())
        if force_lanes:
            eng.set_option("force_lanes", force_lanes)
        eng.commit()
        eng.set("species", job.species)
        eng.set("position", job.position)
        eng.set("velocity", job.velocity)
        if time_limit is None:
            eng.step(job.steps)
            done = job.steps
        else:
            done = 0
            while done < job.steps and clock() - t0 < time_limit:
                k = min(chunk, job.steps - done)
                eng.step(k)
                eng.info()                       # the chunk has run
                done += k
        work += job.n * done
        if done == job.steps:
            job.result = dict(position=eng.get("position"), velocity=eng.get("velocity"), image=eng.get("image"),
                              step=int(eng.info().step))
            job.completed = clock() - t0
            completed += 1
        eng.close()
    return dict(makespan=clock() - t0, work=work, completed=completed)
