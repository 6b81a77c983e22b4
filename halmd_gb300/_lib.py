"""ctypes binding of libhalmd_gb300.so (the C ABI in include/halmd_gb300.h).

The shared library is built in-tree by halmd_gb300.build; there is no fallback:
loading fails loudly if it is missing or cannot be opened.
"""
import ctypes
import os
import re

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
LIB_PATH = os.path.join(PKG, "libhalmd_gb300.so")
HEADER = os.path.join(REPO, "include", "halmd_gb300.h")

HMD_OK = 0
PRECISION = {"float": 0, "single": 0, "dsfloat": 1, "double-single": 1, "double": 2, "fp64": 2}
TRUNCATION = {"sharp": 0, "shifted": 1, "smooth_r4": 2, "force_shifted": 3, "none": 4}
INTEGRATOR = {"verlet": 0, "verlet_nvt_andersen": 1, "andersen": 1, "verlet_nvt_hoover": 2, "hoover": 2,
              "verlet_nvt_boltzmann": 3, "boltzmann": 3, "euler": 4}
POTENTIAL = {"lennard_jones": 0, "mie": 1, "morse": 2, "power_law": 3}
MAX_SPECIES = 4
NTHERMO = 14
PLACEHOLDER = 0xFFFFFFFF


class HmdError(RuntimeError):
    """Error returned by the C ABI (negative status code)."""

    def __init__(self, code, msg):
        super().__init__("%s (status %d)" % (msg, code))
        self.code = code


class SystemDesc(ctypes.Structure):
    _fields_ = [
        ("nparticle", ctypes.c_uint32),
        ("nspecies", ctypes.c_uint32),
        ("box", ctypes.c_double * 3),
        ("epsilon", ctypes.c_double * 16),
        ("sigma", ctypes.c_double * 16),
        ("r_cut", ctypes.c_double * 16),
        ("truncation", ctypes.c_int32),
        ("smoothing", ctypes.c_double),
        ("skin", ctypes.c_double),
        ("cell_occupancy", ctypes.c_double),
        ("neighbour_occupancy", ctypes.c_double),
        ("timestep", ctypes.c_double),
        ("integrator", ctypes.c_int32),
        ("temperature", ctypes.c_double),
        ("collision_rate", ctypes.c_double),
        ("seed", ctypes.c_uint64),
        ("sort", ctypes.c_int32),
        ("potential", ctypes.c_int32),
        ("index_repulsion", ctypes.c_uint32 * 16),
        ("index_attraction", ctypes.c_uint32 * 16),
        ("index", ctypes.c_uint32 * 16),
        ("r_min", ctypes.c_double * 16),
        ("distortion", ctypes.c_double * 16),
        ("resonance_frequency", ctypes.c_double),
    ]


class SystemInfo(ctypes.Structure):
    _fields_ = [
        ("nparticle", ctypes.c_uint32),
        ("nspecies", ctypes.c_uint32),
        ("slot_offset", ctypes.c_uint32),
        ("slots", ctypes.c_uint32),
        ("ncell", ctypes.c_int32 * 3),
        ("cell_size", ctypes.c_uint32),
        ("neighbour_capacity", ctypes.c_uint32),
        ("hilbert_depth", ctypes.c_uint32),
        ("max_neighbours", ctypes.c_uint32),
        ("max_cell_occupancy", ctypes.c_uint32),
        ("step", ctypes.c_uint64),
        ("rebuilds", ctypes.c_uint64),
        ("sort_key_bits", ctypes.c_uint32),
        ("rebuild_kernels", ctypes.c_uint32),
        ("box_f32", ctypes.c_float * 3),
        ("rr_cut_skin", ctypes.c_float * 16),
        ("rr_cut", ctypes.c_float * 16),
    ]


def header_symbols():
    """Names of all entry points declared in include/halmd_gb300.h."""
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^HMD_API\s+\w+\s+(hmd_\w+)\s*\(", text, flags=re.M)))


_lib = None


def load():
    """Open the library (no compute is launched)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError("libhalmd_gb300.so is not built (run `python -c \"import __graft_entry__ as g; g.build()\"`)")
    L = ctypes.CDLL(LIB_PATH)
    P = ctypes.c_void_p
    U = ctypes.c_uint32
    I = ctypes.c_int
    S = ctypes.c_size_t
    D = ctypes.c_double
    sig = {
        "hmd_system_desc_init": (None, [P]),
        "hmd_last_error": (I, [P, P, S]),
        "hmd_engine_create": (I, [I, I, P]),
        "hmd_engine_destroy": (I, [P]),
        "hmd_engine_add_system": (I, [P, P, P]),
        "hmd_engine_commit": (I, [P]),
        "hmd_engine_stream": (I, [P, P]),
        "hmd_engine_reserve": (I, [P, U, U, U]),
        "hmd_engine_remove_system": (I, [P, U]),
        "hmd_engine_capacity": (I, [P, P]),
        "hmd_engine_progress": (I, [P, P, P, U]),
        "hmd_engine_set_option": (I, [P, ctypes.c_char_p, ctypes.c_int64]),
        "hmd_engine_get_option": (I, [P, ctypes.c_char_p, P]),
        "hmd_info": (I, [P, U, P]),
        "hmd_set": (I, [P, U, ctypes.c_char_p, P, S]),
        "hmd_get": (I, [P, U, ctypes.c_char_p, P, S]),
        "hmd_get_raw": (I, [P, U, ctypes.c_char_p, P, S]),
        "hmd_step": (I, [P, ctypes.c_uint64, I]),
        "hmd_integrate": (I, [P]),
        "hmd_force": (I, [P, I]),
        "hmd_finalize": (I, [P]),
        "hmd_request_rebuild": (I, [P, U]),
        "hmd_set_steps_left": (I, [P, U, U]),
        "hmd_minimize": (I, [P, U, U, D, D]),
        "hmd_max_displacement": (I, [P, U, P]),
        "hmd_thermo": (I, [P, U, P]),
        "hmd_integrator_state": (I, [P, U, P]),
        "hmd_positions_lattice": (I, [P, U, P]),
        "hmd_velocities_boltzmann": (I, [P, U, D, ctypes.c_uint64]),
        "hmd_neighbour_lists": (I, [P, U, P, P, U]),
        "hmd_hilbert_keys": (I, [P, U, P]),
        "hmd_profile_enable": (I, [P, I]),
        "hmd_profile_get": (I, [P, ctypes.c_char_p, P, P]),
        "hmd_dynamics_create": (I, [P, U, D, D, U, U, U, P]),
        "hmd_dynamics_destroy": (I, [P]),
        "hmd_dynamics_levels": (I, [P, P, P]),
        "hmd_dynamics_time": (I, [P, P]),
        "hmd_dynamics_add_msd": (I, [P, U, U, P]),
        "hmd_dynamics_add_mqd": (I, [P, U, U, P]),
        "hmd_dynamics_add_vacf": (I, [P, U, U, P]),
        "hmd_dynamics_add_isf": (I, [P, P, U, D, U, U, U, D, P]),
        "hmd_dynamics_sample": (I, [P]),
        "hmd_dynamics_finalise": (I, [P]),
        "hmd_dynamics_result": (I, [P, ctypes.c_int32, P, P, P]),
        "hmd_dynamics_shells": (I, [P, ctypes.c_int32, P, P]),
        "hmd_msd_pair_noalloc": (I, [P, P, U, P, P]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def last_error(handle=None):
    buf = ctypes.create_string_buffer(1024)
    load().hmd_last_error(handle, buf, 1024)
    return buf.value.decode()


def check(rc, handle=None):
    if rc != HMD_OK:
        raise HmdError(rc, last_error(handle))
    return rc


def system_desc(nparticle, box, epsilon=1.0, sigma=1.0, r_cut=2.5, truncation="shifted", smoothing=0.005,
                skin=0.5, cell_occupancy=0.5, neighbour_occupancy=0.4, timestep=0.001, integrator="verlet",
                temperature=1.0, collision_rate=0.0, seed=0, sort=True, nspecies=None, potential="lennard_jones",
                index_repulsion=12, index_attraction=6, index=12, r_min=None, distortion=1.0,
                resonance_frequency=0.0):
    """Build an hmd_system_desc from keyword arguments (Lua module names).

    potential: lennard_jones (epsilon, sigma), mie (index_repulsion m,
    index_attraction n: even, m > n), morse (r_min, required; distortion B),
    power_law (index n); every truncation applies to each.  truncation "none"
    is the untruncated potential over all pairs (pair_full): r_cut and skin
    are then ignored.
    """
    L = load()
    d = SystemDesc()
    L.hmd_system_desc_init(ctypes.byref(d))
    eps = np.atleast_2d(np.asarray(epsilon, dtype=np.float64))
    ns = nspecies or eps.shape[0]
    def mat(x):
        m = np.asarray(x, dtype=np.float64)
        if m.size == 1:
            m = np.full((ns, ns), float(m.reshape(-1)[0]))
        return m.reshape(ns, ns)
    eps, sig, rc = mat(epsilon), mat(sigma), mat(r_cut)
    d.nparticle = int(nparticle)
    d.nspecies = ns
    b = np.broadcast_to(np.asarray(box, dtype=np.float64), (3,))
    for q in range(3):
        d.box[q] = float(b[q])
    for a in range(ns):
        for c in range(ns):
            d.epsilon[a * ns + c] = eps[a, c]
            d.sigma[a * ns + c] = sig[a, c]
            d.r_cut[a * ns + c] = rc[a, c]
    d.truncation = TRUNCATION[truncation]
    d.smoothing = smoothing
    d.skin = skin
    d.cell_occupancy = cell_occupancy
    d.neighbour_occupancy = neighbour_occupancy
    d.timestep = timestep
    d.integrator = INTEGRATOR[integrator]
    d.temperature = temperature
    d.collision_rate = collision_rate
    d.seed = int(seed)
    d.sort = 1 if sort else 0
    d.resonance_frequency = float(resonance_frequency)
    d.potential = POTENTIAL[potential]
    if potential == "morse" and r_min is None:
        raise ValueError("morse needs r_min")
    m_rep, m_att, m_idx = mat(index_repulsion), mat(index_attraction), mat(index)
    m_rmin, m_dist = mat(0.0 if r_min is None else r_min), mat(distortion)
    for a in range(ns):
        for c in range(ns):
            k = a * ns + c
            d.index_repulsion[k] = int(m_rep[a, c])
            d.index_attraction[k] = int(m_att[a, c])
            d.index[k] = int(m_idx[a, c])
            d.r_min[k] = m_rmin[a, c]
            d.distortion[k] = m_dist[a, c]
    return d


class Engine:
    """One engine handle: systems that advance together on one GPU."""

    def __init__(self, precision="dsfloat", device=0):
        self._L = load()
        self._h = ctypes.c_void_p()
        check(self._L.hmd_engine_create(PRECISION[precision], int(device), ctypes.byref(self._h)))
        self.precision = precision
        self.systems = []
        self.committed = False

    def close(self):
        if self._h:
            self._L.hmd_engine_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        return check(rc, self._h)

    def add_system(self, desc):
        idx = ctypes.c_uint32()
        self._check(self._L.hmd_engine_add_system(self._h, ctypes.byref(desc), ctypes.byref(idx)))
        self.systems.append(desc)
        return idx.value

    def commit(self):
        self._check(self._L.hmd_engine_commit(self._h))
        self.committed = True

    def reserve(self, slots, systems, neighbour_capacity=0):
        self._check(self._L.hmd_engine_reserve(self._h, int(slots), int(systems), int(neighbour_capacity)))
        self.capacity_mode = True

    def add(self, desc):
        """Add a system; on a committed engine with reserved capacity it joins
        between steps and keeps its index until removed."""
        idx = ctypes.c_uint32()
        self._check(self._L.hmd_engine_add_system(self._h, ctypes.byref(desc), ctypes.byref(idx)))
        k = idx.value
        while len(self.systems) <= k:
            self.systems.append(None)
        self.systems[k] = desc
        return k

    def remove(self, s):
        self._check(self._L.hmd_engine_remove_system(self._h, int(s)))
        self.systems[s] = None

    def progress(self, n):
        step = np.zeros(n, dtype=np.uint64)
        left = np.zeros(n, dtype=np.uint32)
        self._check(self._L.hmd_engine_progress(self._h, _ptr(step), _ptr(left), int(n)))
        return step, left

    def capacity(self):
        out = np.zeros(8, dtype=np.uint64)
        self._check(self._L.hmd_engine_capacity(self._h, _ptr(out)))
        keys = ("slots", "slots_used", "cells", "cells_used", "neighbour_capacity", "systems", "system_table",
                "bytes_per_slot")
        return {k: int(v) for k, v in zip(keys, out)}

    def set_option(self, name, value):
        self._check(self._L.hmd_engine_set_option(self._h, name.encode(), int(value)))

    def get_option(self, name):
        v = ctypes.c_int64()
        self._check(self._L.hmd_engine_get_option(self._h, name.encode(), ctypes.byref(v)))
        return v.value

    @property
    def stream(self):
        s = ctypes.c_void_p()
        self._check(self._L.hmd_engine_stream(self._h, ctypes.byref(s)))
        return s.value or 0

    def info(self, s=0):
        i = SystemInfo()
        self._check(self._L.hmd_info(self._h, s, ctypes.byref(i)))
        return i

    def n(self, s=0):
        return self.systems[s].nparticle

    def set(self, name, array, s=0):
        dtype = np.uint32 if name == "species" else np.float64
        a = np.ascontiguousarray(array, dtype=dtype)
        self._check(self._L.hmd_set(self._h, s, name.encode(), _ptr(a), a.size))

    def get(self, name, s=0, out=None):
        """Tag-ordered array `name` of system s; into `out` (C-contiguous, right shape and
        dtype, e.g. page-locked host memory) when given."""
        n = self.n(s)
        shapes = {"position": (n, 3), "unwrapped_position": (n, 3), "velocity": (n, 3), "image": (n, 3),
                  "force": (n, 3), "mass": (n,), "species": (n,), "potential_energy": (n,),
                  "stress_pot": (n, 6), "reverse_id": (n,), "id": (self.info(s).slots,) if out is None else out.shape}
        dtype = np.uint32 if name in ("species", "reverse_id", "id") else np.float64
        if out is not None:
            if out.shape != shapes[name] or out.dtype != dtype or not out.flags.c_contiguous:
                raise ValueError("out must be a C-contiguous %s array of shape %s" % (np.dtype(dtype), shapes[name]))
            a = out
        else:
            a = np.zeros(shapes[name], dtype=dtype)
        self._check(self._L.hmd_get(self._h, s, name.encode(), _ptr(a), a.size))
        return a

    def get_raw(self, name, s=0):
        inf = self.info(s)
        if name == "cells":
            a = np.zeros(inf.ncell[0] * inf.ncell[1] * inf.ncell[2] * inf.cell_size, dtype=np.uint32)
        else:
            a = np.zeros((inf.slots, 4), dtype=np.float32)
        self._check(self._L.hmd_get_raw(self._h, s, name.encode(), _ptr(a), a.nbytes))
        return a

    def step(self, nsteps, aux_last=False):
        self._check(self._L.hmd_step(self._h, int(nsteps), 1 if aux_last else 0))

    def integrate(self):
        self._check(self._L.hmd_integrate(self._h))

    def force(self, aux=False):
        self._check(self._L.hmd_force(self._h, 1 if aux else 0))

    def finalize(self):
        self._check(self._L.hmd_finalize(self._h))

    def request_rebuild(self, s=0):
        self._check(self._L.hmd_request_rebuild(self._h, s))

    def set_steps_left(self, steps, s=0):
        self._check(self._L.hmd_set_steps_left(self._h, s, int(steps) & 0xFFFFFFFF))

    def minimize(self, steps=1000, step_size=1e-3, max_move=0.05, s=0):
        """Steepest-descent relaxation of system s (positions only)."""
        self._check(self._L.hmd_minimize(self._h, s, int(steps), float(step_size), float(max_move)))

    def max_displacement(self, s=0):
        d = ctypes.c_double()
        self._check(self._L.hmd_max_displacement(self._h, s, ctypes.byref(d)))
        return d.value

    def thermo(self, s=0):
        out = np.zeros(NTHERMO)
        self._check(self._L.hmd_thermo(self._h, s, _ptr(out)))
        return dict(mv2=out[0], momentum=out[1:4].copy(), mass=out[4], epot=out[5], virial=out[6],
                    stress=out[7:13].copy(), count=out[13])

    def lattice(self, slab=None, s=0):
        """positions.lattice: fcc sites filling the slab (fractions of the box edges) at the box centre."""
        sl = None if slab is None else np.ascontiguousarray(np.broadcast_to(np.asarray(slab, dtype=np.float64), (3,)))
        self._check(self._L.hmd_positions_lattice(self._h, s, _ptr(sl) if sl is not None else None))

    def boltzmann(self, temperature, seed=0, s=0):
        """velocities.boltzmann set(): Maxwell-Boltzmann velocities at temperature, zero momentum."""
        self._check(self._L.hmd_velocities_boltzmann(self._h, s, float(temperature), int(seed)))

    def integrator_state(self, s=0):
        """Chain positions xi, velocities v_xi and energy per particle (Nose-Hoover);
        the centre-of-mass velocity of the last draw (Maxwell-Boltzmann)."""
        out = np.zeros(8)
        self._check(self._L.hmd_integrator_state(self._h, s, _ptr(out)))
        return dict(xi=out[0:2].copy(), v_xi=out[2:4].copy(), internal_energy=out[4], vcm=out[5:8].copy())

    def neighbour_lists(self, maxn=None, s=0):
        n = self.n(s)
        maxn = maxn or self.info(s).neighbour_capacity
        counts = np.zeros(n, dtype=np.uint32)
        lists = np.zeros((n, maxn), dtype=np.uint32)
        self._check(self._L.hmd_neighbour_lists(self._h, s, _ptr(counts), _ptr(lists), maxn))
        return counts, lists

    def profile(self, enable=True):
        self._check(self._L.hmd_profile_enable(self._h, 1 if enable else 0))

    def profile_get(self, phase):
        ms = ctypes.c_double()
        cnt = ctypes.c_uint64()
        self._check(self._L.hmd_profile_get(self._h, phase.encode(), ctypes.byref(ms), ctypes.byref(cnt)))
        return ms.value, cnt.value

    def hilbert_keys(self, s=0):
        k = np.zeros(self.n(s), dtype=np.uint32)
        self._check(self._L.hmd_hilbert_keys(self._h, s, _ptr(k)))
        return k


class Dynamics:
    """Blocking scheme with MSD / ISF correlations over one system."""

    def __init__(self, engine, max_lag_time, resolution, block_size=10, shift=None, separation=None, s=0):
        self.engine = engine
        self._L = load()
        shift = int(np.floor(np.sqrt(block_size))) if shift is None else shift
        separation = block_size if separation is None else separation
        self._h = ctypes.c_void_p()
        check(self._L.hmd_dynamics_create(engine._h, s, float(max_lag_time), float(resolution), int(block_size),
                                          int(shift), int(separation), ctypes.byref(self._h)), engine._h)
        lv = ctypes.c_uint32()
        bs = ctypes.c_uint32()
        self._L.hmd_dynamics_levels(self._h, ctypes.byref(lv), ctypes.byref(bs))
        self.levels, self.block_size = lv.value, bs.value
        self.shells = {}

    def close(self):
        if self._h:
            self._L.hmd_dynamics_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        return check(rc, self.engine._h)

    def time(self):
        t = np.zeros((self.levels, self.block_size))
        self._check(self._L.hmd_dynamics_time(self._h, _ptr(t)))
        return t

    def add_msd(self, first, last):
        return self._add_particle_tcf(self._L.hmd_dynamics_add_msd, first, last)

    def add_mqd(self, first, last):
        return self._add_particle_tcf(self._L.hmd_dynamics_add_mqd, first, last)

    def add_vacf(self, first, last):
        return self._add_particle_tcf(self._L.hmd_dynamics_add_vacf, first, last)

    def _add_particle_tcf(self, fn, first, last):
        k = ctypes.c_int32()
        self._check(fn(self._h, int(first), int(last), ctypes.byref(k)))
        self.shells[k.value] = 1
        return k.value

    def add_isf(self, wavenumber, tolerance, max_count, first, last, norm):
        w = np.ascontiguousarray(np.atleast_1d(wavenumber), dtype=np.float64)
        k = ctypes.c_int32()
        self._check(self._L.hmd_dynamics_add_isf(self._h, _ptr(w), w.size, float(tolerance), int(max_count),
                                                 int(first), int(last), float(norm), ctypes.byref(k)))
        ns = ctypes.c_uint32()
        self._L.hmd_dynamics_shells(self._h, k.value, ctypes.byref(ns), None)
        self.shells[k.value] = ns.value
        return k.value

    def wavenumbers(self, tcf):
        out = np.zeros(self.shells[tcf])
        self._check(self._L.hmd_dynamics_shells(self._h, tcf, None, _ptr(out)))
        return out

    def sample(self):
        self._check(self._L.hmd_dynamics_sample(self._h))

    def finalise(self):
        self._check(self._L.hmd_dynamics_finalise(self._h))

    def result(self, tcf):
        shape = (self.levels, self.block_size, self.shells[tcf])
        mean = np.zeros(shape)
        err = np.zeros(shape)
        cnt = np.zeros(shape, dtype=np.uint64)
        self._check(self._L.hmd_dynamics_result(self._h, tcf, _ptr(mean), _ptr(err), _ptr(cnt)))
        return mean, err, cnt
