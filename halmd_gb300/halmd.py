"""Module-style front end with the names, keyword arguments and defaults of the
reference's Lua API for the MD step, over the engine's C ABI.

    from halmd_gb300 import halmd
    box = halmd.mdsim.box(length=[L, L, L])
    particle = halmd.mdsim.particle(dimension=3, particles=n, species=2)
    particle.data["species"] = species
    particle.data["position"] = r
    potential = halmd.mdsim.potentials.pair.lennard_jones(
        epsilon=[[1, 1.5], [1.5, 0.5]], sigma=[[1, 0.8], [0.8, 0.88]]).truncate("smooth_r4", cutoff=2.5, h=0.005)
    force = halmd.mdsim.forces.pair(box=box, particle=particle, potential=potential, neighbour={"skin": 0.3})
    integrator = halmd.mdsim.integrators.verlet_nvt_andersen(
        box=box, particle=particle, timestep=0.002, temperature=0.7, rate=1)
    thermo = halmd.observables.thermodynamics(box=box, group=particle)
    halmd.observables.sampler.run(1000)
    print(thermo.potential_energy(), thermo.temperature())

Lua tables become Python keywords, or a dict with the same keys.  A
positional first entry, as in `truncate({"smooth_r4", cutoff = 2.5, h = 0.005})`,
becomes the first positional argument.  The modules mirror:

    lua/halmd/mdsim/box.lua.in                 box{length | edges}
    lua/halmd/mdsim/particle.lua.in:63-68      particle{dimension, particles, species=1, precision, label="all"}
    lua/halmd/mdsim/potentials/pair/lennard_jones.lua.in:56-60
                                               lennard_jones{epsilon=1, sigma=1, species}
    .../adapters/truncate.lua.in:287-305       :truncate{kind="shifted", cutoff, h}
    lua/halmd/mdsim/neighbour.lua.in:88-102    neighbour{skin=0.5, occupancy, disable_sorting}
    lua/halmd/mdsim/forces/pair.lua.in:36-40   forces.pair{box, particle, potential, neighbour}
    lua/halmd/mdsim/integrators/verlet.lua.in:57-59, verlet_nvt_andersen.lua.in:52-56
    lua/halmd/observables/thermodynamics.lua.in:60-130 (formulas)
    lua/halmd/observables/sampler.lua.in        sampler.run(steps), sampler.on_sample(fn, every)
    lua/halmd/observables/dynamics/*.lua.in     blocking_scheme, mean_square_displacement,
                                               mean_quartic_displacement, velocity_autocorrelation,
                                               intermediate_scattering_function

All modules of one script share one engine, committed when the simulation
first needs the device (the first `sampler.run` or read of device data).
Several `particle` instances become independent systems of that engine and
advance together.  Instances coupled by pair forces, as
`forces.pair{particle = {p1, p2}, ...}` wires them (pair_trunc.hpp:60-61,
154-162; test/integration/modularity/two_particles.lua), become one system
whose particles are the instances' in order: every ordered pair of the
coupled instances needs its force, all with one potential, box, neighbour
configuration and integrator, which is the same physics as one instance of
several species.  `reset()` starts a new script.
"""
import numpy as np

from ._lib import Dynamics, Engine, system_desc


def _args(args, kw):
    out = dict(args or {})
    out.update(kw)
    return out


class _Script:
    """The modules of one script and the engine they share."""

    def __init__(self):
        self.particles = []
        self.forces = []             # (p1, p2): forces on p1 from p2
        self.engine = None
        self.observers = []          # (every, fn) called after steps that are multiples of every
        self.blocking = []
        self.step = 0

    def committed(self):
        return self.engine is not None

    def commit(self):
        if self.engine is not None:
            return self.engine
        if not self.particles:
            raise RuntimeError("no particle instance")
        precisions = {p.precision for p in self.particles}
        if len(precisions) != 1:
            raise ValueError("all particle instances of a script share one precision")
        groups = self.groups()
        eng = Engine("dsfloat" if precisions.pop() == "double-single" else "float")
        for g in groups:
            index = eng.add_system(g[0]._desc(sum(p.nparticle for p in g)))
            offset = 0
            for p in g:
                p._index, p._offset, p._group = index, offset, g
                offset += p.nparticle
        eng.commit()
        for g in groups:
            for name in ("species", "mass", "position", "image", "velocity"):
                if all(name not in p._pending for p in g):
                    continue
                if len(g) == 1:
                    eng.set(name, g[0]._pending[name], g[0]._index)
                    continue
                if name == "position" and not all(name in p._pending for p in g):
                    raise ValueError("positions of only some of the coupled particle instances are set")
                parts = [p._pending[name] if name in p._pending else _default(name, p.nparticle) for p in g]
                eng.set(name, np.concatenate([np.asarray(x) for x in parts]), g[0]._index)
            for p in g:
                p._pending.clear()
                for call in p._setup:
                    call(eng, p._index)
                p._setup.clear()
        self.engine = eng
        for b in self.blocking:
            b._attach()
        return eng


    def groups(self):
        """The particle instances as engine systems: instances coupled by pair
        forces form one group (checked to be one system of several species)."""
        parent = {id(p): p for p in self.particles}

        def root(p):
            while parent[id(p)] is not p:
                p = parent[id(p)]
            return p

        for a, b in self.forces:
            ra, rb = root(a), root(b)
            if ra is not rb:
                parent[id(rb)] = ra
        groups, seen = [], {}
        for p in self.particles:
            r = root(p)
            if id(r) not in seen:
                seen[id(r)] = []
                groups.append(seen[id(r)])
            seen[id(r)].append(p)
        wired = {(id(a), id(b)) for a, b in self.forces}
        for g in groups:
            if len(g) == 1:
                continue
            missing = [(a.label, b.label) for a in g for b in g if (id(a), id(b)) not in wired]
            if missing:
                raise ValueError("coupled particle instances need a pair force for every ordered pair; missing %s"
                                 % missing)
            first = g[0]
            for p in g[1:]:
                for what in ("_box", "_potential", "_integrator"):
                    if getattr(p, what) is None or getattr(first, what) is None:
                        raise RuntimeError("particle '%s' needs a box, a pair force and an integrator" % p.label)
                if p._potential is not first._potential and _potential_key(p._potential) != _potential_key(
                        first._potential):
                    raise ValueError("coupled particle instances must share one potential")
                if list(p._box.length) != list(first._box.length):
                    raise ValueError("coupled particle instances must share one box")
                if (p._neighbour or {}) != (first._neighbour or {}):
                    raise ValueError("coupled particle instances must share one neighbour configuration")
                if _integrator_key(p._integrator) != _integrator_key(first._integrator):
                    raise ValueError("coupled particle instances must use the same integrator")
                if p.nspecies != first.nspecies:
                    raise ValueError("coupled particle instances must declare the same number of species")
                if p._setup:
                    raise ValueError("set-up modules (lattice, boltzmann) act on whole systems: set the "
                                     "positions and velocities of coupled particle instances directly")
            if first._setup:
                raise ValueError("set-up modules (lattice, boltzmann) act on whole systems: set the "
                                 "positions and velocities of coupled particle instances directly")
        return groups


def _default(name, n):
    if name == "species":
        return np.zeros(n, dtype=np.uint32)
    if name == "mass":
        return np.ones(n)
    return np.zeros((n, 3))


def _potential_key(pot):
    return (pot.potential, np.asarray(pot.epsilon).tolist(), np.asarray(pot.sigma).tolist(), pot.kind, pot.cutoff,
            pot.h, sorted(pot.params.items()))


def _integrator_key(integ):
    return tuple(sorted((k, v) for k, v in vars(integ).items() if k != "particle"))


_script = _Script()


def reset():
    """Forget every module; the next ones form a new script (a new engine)."""
    global _script
    if _script.engine is not None:
        for b in _script.blocking:
            b._close()
        _script.engine.close()
    _script = _Script()


class _Namespace:
    def __init__(self, **kw):
        self.__dict__.update(kw)


# ---- mdsim ------------------------------------------------------------------

class box:
    """halmd.mdsim.box{length = {Lx, Ly, Lz}} (or diagonal `edges`)."""

    def __init__(self, args=None, **kw):
        a = _args(args, kw)
        if "length" in a:
            self.length = [float(x) for x in a["length"]]
        elif "edges" in a:
            e = np.asarray(a["edges"], dtype=float)
            if np.count_nonzero(e - np.diag(np.diagonal(e))):
                raise ValueError("only cuboid boxes are supported")
            self.length = list(np.diagonal(e))
        else:
            raise ValueError("box: missing argument 'length' or 'edges'")
        if len(self.length) != 3:
            raise ValueError("box: 3 edge lengths expected")

    @property
    def volume(self):
        return float(np.prod(self.length))


class _Data:
    def __init__(self, particle):
        self._p = particle

    def __getitem__(self, name):
        return self._p.get(name)

    def __setitem__(self, name, value):
        self._p.set(name, value)

    def __getattr__(self, name):
        return self._p.get(name)


class particle:
    """halmd.mdsim.particle{dimension, particles, species = 1, precision, label = "all"}."""

    def __init__(self, args=None, **kw):
        a = _args(args, kw)
        if int(a.get("dimension", 3)) != 3:
            raise ValueError("unsupported space dimension: '%d'" % int(a["dimension"]))
        self.nparticle = int(a["particles"])
        self.nspecies = int(a.get("species", 1))
        self.precision = a.get("precision", "double-single")
        if self.precision not in ("double-single", "single"):
            raise ValueError("unsupported floating-point precision: '%s'" % self.precision)
        self.label = a.get("label", "all")
        self.memory = "gpu"
        self.data = _Data(self)
        self._pending = {}
        self._setup = []       # set-up calls (lattice, Boltzmann) waiting for the engine
        self._index = None
        self._offset = 0       # first particle of this instance in its engine system
        self._group = [self]   # the instances that share the system (coupled by pair forces)
        self._box = self._potential = self._neighbour = self._integrator = None
        _script.particles.append(self)

    def set(self, name, value):
        value = np.asarray(value)
        if not _script.committed():
            self._pending[name] = value
        elif len(self._group) == 1:
            _script.engine.set(name, value, self._index)
        else:
            full = np.array(_script.engine.get(name, self._index), copy=True)
            full[self._offset:self._offset + self.nparticle] = value
            _script.engine.set(name, full, self._index)

    def get(self, name):
        if not _script.committed() and name in self._pending:
            return self._pending[name]
        full = _script.commit().get(name, self._index)
        if len(self._group) == 1:
            return full
        return full[self._offset:self._offset + self.nparticle]

    def _desc(self, nparticle=None):
        if self._box is None or self._potential is None or self._integrator is None:
            raise RuntimeError("particle '%s' needs a box, a pair force and an integrator" % self.label)
        pot, nb, integ = self._potential, self._neighbour or {}, self._integrator
        # an untruncated potential: the pair_full force (forces/pair.lua.in:78-83)
        kw = dict(epsilon=pot.epsilon, sigma=pot.sigma, r_cut=0.0 if pot.kind is None else pot.cutoff,
                  truncation=pot.kind or "none",
                  skin=nb.get("skin", 0.5), timestep=integ.timestep, integrator=integ.kind,
                  sort=not nb.get("disable_sorting", False), potential=pot.potential, **pot.params)
        if pot.kind == "smooth_r4":
            kw["smoothing"] = pot.h
        if nb.get("occupancy") is not None:
            kw["neighbour_occupancy"] = nb["occupancy"]
        if integ.kind in ("andersen", "boltzmann"):
            kw.update(temperature=integ.temperature, collision_rate=integ.rate, seed=integ.seed)
        if integ.kind == "hoover":
            kw.update(temperature=integ.temperature, resonance_frequency=integ.resonance_frequency)
        return system_desc(nparticle or self.nparticle, self._box.length, nspecies=self.nspecies, **kw)


class _Potential:
    def __init__(self, epsilon, sigma, species, potential="lennard_jones", params=None):
        self.epsilon, self.sigma, self.species = epsilon, sigma, species
        self.potential, self.params = potential, dict(params or {})
        self.kind, self.cutoff, self.h = None, None, None

    def truncate(self, args=None, **kw):
        """:truncate{kind = "shifted", cutoff, h} (truncate.lua.in:287-305)."""
        if isinstance(args, str):
            args = {1: args}
        a = _args(args, kw)
        if "cutoff" not in a:
            raise ValueError("missing keyword argument 'cutoff'")
        kind = a.get(1, a.get("kind", "shifted"))
        if kind not in ("sharp", "shifted", "smooth_r4", "force_shifted"):
            raise ValueError("invalid truncation type '%s'" % kind)
        out = _Potential(self.epsilon, self.sigma, self.species, self.potential, self.params)
        out.kind, out.cutoff = kind, a["cutoff"]
        if kind == "smooth_r4":
            if "h" not in a:
                raise ValueError("missing keyword argument 'h'")
            out.h = float(a["h"])
        return out

    @property
    def r_cut(self):
        return self.cutoff


def lennard_jones(args=None, **kw):
    """halmd.mdsim.potentials.pair.lennard_jones{epsilon = 1, sigma = 1, species}."""
    a = _args(args, kw)
    eps = np.atleast_2d(np.asarray(a.get("epsilon", 1.0), dtype=float))
    sig = np.atleast_2d(np.asarray(a.get("sigma", 1.0), dtype=float))
    species = int(a.get("species", max(eps.shape[0], sig.shape[0])))
    return _Potential(eps, sig, species)


def _species(a, *mats):
    return int(a.get("species", max(np.atleast_2d(np.asarray(m)).shape[0] for m in mats)))


def mie(args=None, **kw):
    """halmd.mdsim.potentials.pair.mie{epsilon = 1, sigma = 1, index_repulsion, index_attraction, species}
    (mie.lua.in:66-72; both indices even, repulsion > attraction)."""
    a = _args(args, kw)
    for k in ("index_repulsion", "index_attraction"):
        if k not in a:
            raise ValueError("missing keyword argument '%s'" % k)
    eps = np.atleast_2d(np.asarray(a.get("epsilon", 1.0), dtype=float))
    sig = np.atleast_2d(np.asarray(a.get("sigma", 1.0), dtype=float))
    params = dict(index_repulsion=a["index_repulsion"], index_attraction=a["index_attraction"])
    return _Potential(eps, sig, _species(a, eps, sig), "mie", params)


def morse(args=None, **kw):
    """halmd.mdsim.potentials.pair.morse{epsilon = 1, sigma = 1, r_min (or minimum), distortion = 1, species}
    (morse.lua.in:75-81, 168-185)."""
    a = _args(args, kw)
    r_min = a.get("r_min", a.get("minimum"))
    if r_min is None:
        raise ValueError("missing keyword argument 'r_min'")
    eps = np.atleast_2d(np.asarray(a.get("epsilon", 1.0), dtype=float))
    sig = np.atleast_2d(np.asarray(a.get("sigma", 1.0), dtype=float))
    params = dict(r_min=r_min, distortion=a.get("distortion", 1.0))
    return _Potential(eps, sig, _species(a, eps, sig), "morse", params)


def power_law(args=None, **kw):
    """halmd.mdsim.potentials.pair.power_law{epsilon = 1, sigma = 1, index = 12, species} (power_law.lua.in:56-61)."""
    a = _args(args, kw)
    eps = np.atleast_2d(np.asarray(a.get("epsilon", 1.0), dtype=float))
    sig = np.atleast_2d(np.asarray(a.get("sigma", 1.0), dtype=float))
    return _Potential(eps, sig, _species(a, eps, sig), "power_law", dict(index=a.get("index", 12)))


def neighbour(args=None, **kw):
    """halmd.mdsim.neighbour{skin = 0.5, occupancy, disable_sorting = false} (as keyword table)."""
    return _args(args, kw)


def pair(args=None, **kw):
    """halmd.mdsim.forces.pair{box, particle, potential, neighbour}: the truncated
    force (pair_trunc) for a potential with a cutoff, else the untruncated
    force over all pairs (pair_full; forces/pair.lua.in:78-83)."""
    a = _args(args, kw)
    pot = a["potential"]
    parts = list(a["particle"]) if isinstance(a["particle"], (list, tuple)) else [a["particle"]]
    if len(parts) == 1:
        parts = parts * 2
    if len(parts) != 2:
        raise ValueError("forces.pair: one particle instance or a pair {p1, p2} expected")
    p1, p2 = parts
    for p in (p1, p2):
        if p._potential is None:
            p._box, p._potential, p._neighbour = a["box"], pot, dict(a.get("neighbour") or {})
    _script.forces.append((p1, p2))
    return _Namespace(particle=p1 if p1 is p2 else (p1, p2), potential=pot)


class _Integrator:
    def __init__(self, kind, a):
        if "timestep" not in a:
            raise ValueError("missing keyword argument 'timestep'")
        self.kind = kind
        self.timestep = float(a["timestep"])
        self.particle = a["particle"]
        a["particle"]._box = a.get("box", a["particle"]._box)
        a["particle"]._integrator = self
        if kind in ("andersen", "boltzmann"):
            self.temperature = float(a["temperature"])
            self.rate = float(a["rate"])
            self.seed = int(a.get("seed", 0))
        if kind == "hoover":
            self.temperature = float(a["temperature"])
            self.resonance_frequency = float(a["resonance_frequency"])


def verlet(args=None, **kw):
    """halmd.mdsim.integrators.verlet{box, particle, timestep}."""
    return _Integrator("verlet", _args(args, kw))


def verlet_nvt_andersen(args=None, **kw):
    """halmd.mdsim.integrators.verlet_nvt_andersen{box, particle, timestep, temperature, rate}."""
    return _Integrator("andersen", _args(args, kw))


def verlet_nvt_hoover(args=None, **kw):
    """halmd.mdsim.integrators.verlet_nvt_hoover{box, particle, timestep, temperature, resonance_frequency}
    (verlet_nvt_hoover.lua.in:170-180; both thermostat arguments are required)."""
    a = _args(args, kw)
    for k in ("temperature", "resonance_frequency"):
        if k not in a:
            raise ValueError("missing keyword argument '%s'" % k)
    return _Integrator("hoover", a)


def verlet_nvt_boltzmann(args=None, **kw):
    """halmd.mdsim.integrators.verlet_nvt_boltzmann{box, particle, timestep, temperature, rate}:
    velocity Verlet with Maxwell-Boltzmann velocities every max(1, round(1 / (rate timestep))) steps."""
    a = _args(args, kw)
    for k in ("temperature", "rate"):
        if k not in a:
            raise ValueError("missing keyword argument '%s'" % k)
    return _Integrator("boltzmann", a)


def euler(args=None, **kw):
    """halmd.mdsim.integrators.euler{box, particle, timestep}: r += v dt."""
    return _Integrator("euler", _args(args, kw))


class _SetUp:
    def __init__(self, particle, call):
        self.particle, self._call = particle, call

    def set(self):
        """Run on the device now, or when the engine is built."""
        if _script.committed():
            self._call(_script.engine, self.particle._index)
        else:
            self.particle._setup.append(self._call)


def lattice(args=None, **kw):
    """halmd.mdsim.positions.lattice{box, particle, slab = {1, 1, 1}}:set(): fcc sites filling the slab
    (mdsim/host/positions/lattice.cpp; positions/lattice.lua.in)."""
    a = _args(args, kw)
    slab = a.get("slab")
    p = a["particle"]
    if "box" in a:
        p._box = a["box"]
    return _SetUp(p, lambda eng, s: eng.lattice(slab, s))


def boltzmann(args=None, **kw):
    """halmd.mdsim.velocities.boltzmann{particle, temperature}:set(): Maxwell-Boltzmann velocities
    with zero total momentum (velocities/boltzmann.lua.in)."""
    a = _args(args, kw)
    if "temperature" not in a:
        raise ValueError("missing keyword argument 'temperature'")
    T, seed = float(a["temperature"]), int(a.get("seed", 0))
    return _SetUp(a["particle"], lambda eng, s: eng.boltzmann(T, seed, s))


mdsim = _Namespace(
    box=box, particle=particle, neighbour=neighbour,
    positions=_Namespace(lattice=lattice), velocities=_Namespace(boltzmann=boltzmann),
    potentials=_Namespace(pair=_Namespace(lennard_jones=lennard_jones, mie=mie, morse=morse, power_law=power_law)),
    forces=_Namespace(pair=pair),
    integrators=_Namespace(verlet=verlet, verlet_nvt_andersen=verlet_nvt_andersen,
                           verlet_nvt_hoover=verlet_nvt_hoover, verlet_nvt_boltzmann=verlet_nvt_boltzmann,
                           euler=euler),
)


# ---- observables -------------------------------------------------------------

class thermodynamics:
    """halmd.observables.thermodynamics{box, group}: per-particle means from the
    FP64 device reductions (observables/thermodynamics.lua.in:60-130)."""

    def __init__(self, args=None, **kw):
        a = _args(args, kw)
        self.box = a["box"]
        self.group = a["group"]

    def _sums(self):
        eng = _script.commit()
        g = self.group
        if len(g._group) == 1:
            return eng.thermo(g._index)
        # one of several coupled instances: FP64 sums of its particles on the
        # host, from the per-particle arrays of the last sampled step
        v, m = g.get("velocity"), np.asarray(g.get("mass"), dtype=np.float64)
        stress = g.get("stress_pot")
        mv = m[:, None] * v
        return {"mv2": float(np.sum(mv * v)), "momentum": mv.sum(axis=0), "mass": float(m.sum()),
                "epot": float(np.sum(g.get("potential_energy"))),
                "virial": float(np.sum(stress[:, 0] + stress[:, 1] + stress[:, 2]))}

    def particle_number(self):
        return self.group.nparticle

    def volume(self):
        return self.box.volume

    def density(self):
        return self.group.nparticle / self.box.volume

    def kinetic_energy(self):
        return 0.5 * self._sums()["mv2"] / self.group.nparticle

    def potential_energy(self):
        return self._sums()["epot"] / self.group.nparticle

    def internal_energy(self):
        t = self._sums()
        return (0.5 * t["mv2"] + t["epot"]) / self.group.nparticle

    def temperature(self):
        return 2.0 * self.kinetic_energy() / 3.0

    def virial(self):
        return self._sums()["virial"] / self.group.nparticle

    def pressure(self):
        t = self._sums()
        n = self.group.nparticle
        return n / self.box.volume * ((t["mv2"] / n) / 3.0 + (t["virial"] / n) / 3.0)

    def center_of_mass_velocity(self):
        t = self._sums()
        return t["momentum"] / t["mass"]

    def mean_mass(self):
        return self._sums()["mass"] / self.group.nparticle


class _Sampler:
    """halmd.observables.sampler: run(steps) and on_sample(fn, every, start)."""

    def on_sample(self, fn, every=1, start=0):
        _script.observers.append((int(every), int(start), fn))

    def run(self, steps):
        eng = _script.commit()
        steps = int(steps)
        if _script.step == 0 and not getattr(_script, "started", False):
            # the initial state is a sample too (sampler.lua.in: setup, then sample)
            _script.started = True
            eng.force(aux=True)
            for every, start, fn in _script.observers:
                if every and start == 0:
                    fn()
        stops = {steps}
        for every, start, _ in _script.observers:
            k = _script.step + ((start - _script.step) % every if every else 0)
            while k <= _script.step + steps and every:
                if k > _script.step:
                    stops.add(k - _script.step)
                k += every
        for b in _script.blocking:
            stops.update(b._stops(_script.step, steps))
        done = 0
        for stop in sorted(stops):
            if stop > done:
                eng.step(stop - done, aux_last=True)
                done = stop
            now = _script.step + done
            for every, start, fn in _script.observers:
                if every and now >= start and (now - start) % every == 0:
                    fn()
            for b in _script.blocking:
                b._sample(now)
        _script.step += steps


sampler = _Sampler()


class mean_square_displacement:
    """halmd.observables.dynamics.mean_square_displacement{particle (group)}."""

    def __init__(self, args=None, **kw):
        a = _args(args, kw)
        self.group = a.get("group", a.get("particle"))
        self.first, self.last = int(a.get("first", 0)), int(a.get("last", self.group.nparticle))


class mean_quartic_displacement(mean_square_displacement):
    """halmd.observables.dynamics.mean_quartic_displacement{particle (group)}."""


class velocity_autocorrelation(mean_square_displacement):
    """halmd.observables.dynamics.velocity_autocorrelation{particle (group)}."""


class intermediate_scattering_function:
    """halmd.observables.dynamics.intermediate_scattering_function{particle, wavenumber,
    tolerance, max_count, norm}: shells of reciprocal-lattice vectors (wavevector.cpp:40-160)."""

    def __init__(self, args=None, **kw):
        a = _args(args, kw)
        self.group = a.get("group", a.get("particle"))
        self.wavenumber = [float(k) for k in np.atleast_1d(a["wavenumber"])]
        self.tolerance = float(a.get("tolerance", 0.01))
        self.max_count = int(a.get("max_count", 7))
        self.norm = float(a.get("norm", self.group.nparticle))
        self.first, self.last = int(a.get("first", 0)), int(a.get("last", self.group.nparticle))


class blocking_scheme:
    """halmd.observables.dynamics.blocking_scheme{max_lag, every, size = 10, shift, separation,
    correlations} (blocking_scheme.lua.in:83-93 defaults: shift = floor(sqrt(size)),
    separation = size); `every` is the sampling interval in steps."""

    def __init__(self, args=None, **kw):
        a = _args(args, kw)
        self.max_lag = float(a["max_lag"])
        self.every = int(a.get("every", 1))
        self.size = int(a.get("size", 10))
        self.shift = int(a.get("shift", int(np.floor(np.sqrt(self.size)))))
        self.separation = int(a.get("separation", self.size))
        self.correlations = list(a.get("correlations", []))
        groups = {id(c.group) for c in self.correlations}
        if len(groups) != 1:
            raise ValueError("blocking_scheme: correlations of one particle instance expected")
        self.group = self.correlations[0].group
        self._dyn = None
        self._tcf = []
        _script.blocking.append(self)
        if _script.committed():
            self._attach()

    def _attach(self):
        eng = _script.engine
        dt = self.group._integrator.timestep
        self._dyn = Dynamics(eng, self.max_lag, self.every * dt, block_size=self.size, shift=self.shift,
                             separation=self.separation, s=self.group._index)
        for c in self.correlations:
            # tags of the instance within its engine system (coupled instances share one)
            first, last = c.first + c.group._offset, c.last + c.group._offset
            if isinstance(c, mean_quartic_displacement):
                self._tcf.append(self._dyn.add_mqd(first, last))
            elif isinstance(c, velocity_autocorrelation):
                self._tcf.append(self._dyn.add_vacf(first, last))
            elif isinstance(c, mean_square_displacement):
                self._tcf.append(self._dyn.add_msd(first, last))
            else:
                self._tcf.append(self._dyn.add_isf(c.wavenumber, tolerance=c.tolerance, max_count=c.max_count,
                                                   first=first, last=last, norm=c.norm))
        self._dyn.sample()

    def _stops(self, step0, steps):
        k = ((step0 // self.every) + 1) * self.every
        return {s - step0 for s in range(k, step0 + steps + 1, self.every)}

    def _sample(self, now):
        if self._dyn is not None and now % self.every == 0:
            self._dyn.sample()

    def finalise(self):
        self._dyn.finalise()

    def time(self):
        return self._dyn.time()

    def result(self, k):
        """(mean, error, count) arrays [levels, size, shells] of correlation k."""
        return self._dyn.result(self._tcf[k])

    def _close(self):
        if self._dyn is not None:
            self._dyn.close()


class phase_space:
    """halmd.observables.phase_space{box, group}: acquire() a tag-ordered sample of the
    group's particles (observables/phase_space.lua.in, gpu/phase_space.cpp), set(sample)."""

    FIELDS = ("position", "velocity", "image", "species", "mass")

    def __init__(self, args=None, **kw):
        a = _args(args, kw)
        self.box = a["box"]
        self.group = a.get("group", a.get("particle"))

    def acquire(self):
        return {name: self.group.get(name) for name in self.FIELDS}

    def set(self, sample):
        for name in ("species", "mass", "position", "image", "velocity"):
            if name in sample:
                self.group.set(name, sample[name])


observables = _Namespace(
    thermodynamics=thermodynamics, sampler=sampler, phase_space=phase_space,
    dynamics=_Namespace(blocking_scheme=blocking_scheme, mean_square_displacement=mean_square_displacement,
                        mean_quartic_displacement=mean_quartic_displacement,
                        velocity_autocorrelation=velocity_autocorrelation,
                        intermediate_scattering_function=intermediate_scattering_function),
)
