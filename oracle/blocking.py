"""Blocking scheme and correlation restated in plain Python (test infrastructure).

Follows observables/dynamics/blocking_scheme.cpp:35-200 (levels, sampling
condition, process / skip / finalise) and observables/dynamics/correlation.hpp:208-224
(first entry of a full block against every entry).  The correlation
function is a callback fn(sample_a, sample_b) -> list of (count, mean, M2)
per shell; results accumulate with the pairwise merge of
numeric/accumulator.hpp:96-108.
"""
import math


def merge(acc, n2, m2, v2):
    n, m, v = acc
    if n2 > 0:
        c = n + n2
        v = v + v2 + (m - m2) ** 2 * n * n2 / c
        m = (n * m + n2 * m2) / c
        n = c
    return [n, m, v]


class BlockingScheme:
    def __init__(self, timestep, max_lag_time, resolution, block_size, shift, separation, origin_step=0):
        if block_size < 2 or shift == 0 or shift >= block_size or resolution <= 0:
            raise ValueError("bad blocking parameters")
        self.dt = timestep
        self.block_size = block_size
        self.separation = separation
        max_interval = int(round(max_lag_time / timestep))
        s = int(round(resolution / timestep))
        self.interval = []
        while s <= max_interval:
            self.interval.append(s)
            if shift > 1 and s * shift <= max_interval:
                self.interval.append(s * shift)
            s *= block_size
        if not self.interval:
            raise ValueError("Sampling interval of dynamic correlations is too large.")
        self.origin = [origin_step] * len(self.interval)
        self.blocks = [[] for _ in self.interval]
        self.fns = []
        self.results = []

    def add(self, fn, nshell=1):
        self.fns.append(fn)
        self.results.append([[[[0.0, 0.0, 0.0] for _ in range(nshell)] for _ in range(self.block_size)]
                             for _ in self.interval])
        return len(self.fns) - 1

    def time(self):
        return [[iv * j * self.dt for j in range(self.block_size)] for iv in self.interval]

    def sample(self, step, acquire):
        cache = {}
        for i, iv in enumerate(self.interval):
            if step >= self.origin[i] and (step - self.origin[i]) % iv == 0:
                if step not in cache:
                    cache[step] = acquire()
                self.blocks[i].append(cache[step])
                if len(self.blocks[i]) == self.block_size:
                    self.process(i)

    def finalise(self):
        for i in range(len(self.interval)):
            while self.blocks[i]:
                self.process(i)

    def process(self, level):
        blk = self.blocks[level]
        for k, fn in enumerate(self.fns):
            for j, b in enumerate(blk):
                for sh, (n2, m2, v2) in enumerate(fn(blk[0], b)):
                    acc = self.results[k][level][j][sh]
                    self.results[k][level][j][sh] = merge(acc, n2, m2, v2)
        iv = self.interval[level]
        skip = max((self.separation + iv - 1) // iv, 1)
        self.origin[level] += skip * iv
        del blk[:skip]

    def mean_error_count(self, k):
        out = []
        for lvl in self.results[k]:
            row = []
            for lag in lvl:
                cell = []
                for n, m, v in lag:
                    err = math.sqrt((v / n) / (n - 1)) if n > 1 else 0.0
                    cell.append((m, err, n))
                row.append(cell)
            out.append(row)
        return out
