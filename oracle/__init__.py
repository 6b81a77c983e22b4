"""ctypes view of the CPU oracle (oracle/oracle.cpp).

TEST INFRASTRUCTURE ONLY: the checker for the CUDA product.  Only tests/,
``__graft_entry__.smoke()`` and the CPU legs of ``bench.py`` import this
package; the product (``halmd_gb300``) never does.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "liboracle.so")

TRUNC = {"sharp": 0, "shifted": 1, "smooth_r4": 2, "force_shifted": 3, "none": 4}
PLACEHOLDER = 0xFFFFFFFF


def build(force=False):
    """Compile liboracle.so with the committed Makefile (gcc only)."""
    src = os.path.join(_HERE, "oracle.cpp")
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
        subprocess.check_call(["make", "-s", "-C", _HERE, "all"])
    return _LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        P = ctypes.c_void_p
        I = ctypes.c_int
        D = ctypes.c_double
        L.orc_pot_sizeof.restype = ctypes.c_size_t
        L.orc_pot_init.argtypes = [P, I, P, P, P, I, D]
        L.orc_pot_init_any.argtypes = [P, I, I, P, P, P, I, D, P, P, P, P]
        L.orc_pot_eval.argtypes = [P, D, I, I, P, P]
        L.orc_accumulate.argtypes = [I, P, P]
        L.orc_binning_sizing.argtypes = [I, P, D, D, D, P]
        L.orc_binning_f32.argtypes = [I, P, P, P, I, P, P]
        L.orc_neighbour_full_f32.argtypes = [I, P, P, I, P, I, P, P]
        L.orc_forces.argtypes = [I, P, P, P, P, I, P, P, P, P, P, P]
        L.orc_forces.restype = ctypes.c_long
        L.orc_dsfun.argtypes = [I, I, P, P, P]
        L.orc_integrate_f32.argtypes = [I, I, P, P, P, P, ctypes.c_float, ctypes.c_float, P]
        L.orc_finalize_f32.argtypes = [I, I, P, P, P, ctypes.c_float]
        L.orc_max_displacement2_f32.argtypes = [I, P, P, P]
        L.orc_max_displacement2_f32.restype = ctypes.c_float
        L.orc_philox4x32_10.argtypes = [P, P, P]
        L.orc_andersen_finalize_f32.argtypes = [I, I, P, P, P, P, ctypes.c_float, ctypes.c_float,
                                                ctypes.c_uint32, ctypes.c_uint64, ctypes.c_uint64, P]
        L.orc_hilbert_depth.argtypes = [D]
        L.orc_hilbert_depth.restype = ctypes.c_uint
        L.orc_hilbert_map_unit.argtypes = [I, P, ctypes.c_uint, P]
        L.orc_hilbert_keys_f32.argtypes = [I, P, P, ctypes.c_uint, P]
        L.orc_stable_argsort_u32.argtypes = [I, P, P]
        L.orc_kinetic.argtypes = [I, P, P, P]
        L.orc_msd.argtypes = [I, I, P, P, P]
        L.orc_density_modes.argtypes = [I, I, P, I, P, P]
        L.orc_isf.argtypes = [I, P, P, P, D, P]
        L.orc_wavevectors.argtypes = [I, P, P, D, I, P, I, P, P]
        L.orc_fcc_lattice.argtypes = [I, D, P]
        L.orc_md_run.argtypes = [I, P, P, P, P, P, P, P, D, D, I, D, D, ctypes.c_uint64, P]
        L.orc_lattice.argtypes = [I, P, P, P]
        L.orc_lattice.restype = ctypes.c_long
        L.orc_boltzmann.argtypes = [I, P, D, ctypes.c_uint64, P]
        L.orc_md_run_any.argtypes = [I, P, P, P, P, P, P, P, D, D, I, I, D, D, D, ctypes.c_uint64, P, P]
        L.orc_minimize.argtypes = [I, P, P, P, P, P, D, I, D, D, P]
        L.orc_tcf.argtypes = [I, I, I, P, P, P]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


POTENTIAL = {"lennard_jones": 0, "mie": 1, "morse": 2, "power_law": 3}


class Potential:
    """A pair potential with a truncation, FP64 (host potential restatement).

    potential: lennard_jones (epsilon, sigma), mie (+ index_repulsion,
    index_attraction), morse (+ r_min, distortion), power_law (+ index).
    """

    def __init__(self, epsilon, sigma, r_cut, truncation="shifted", h=0.005, potential="lennard_jones",
                 index_repulsion=None, index_attraction=None, index=None, r_min=None, distortion=None):
        self.eps = np.ascontiguousarray(epsilon, dtype=np.float64)
        self.ns = int(round(np.sqrt(self.eps.size)))
        self.sigma = np.ascontiguousarray(sigma, dtype=np.float64).reshape(self.ns, self.ns)
        rc = np.asarray(r_cut, dtype=np.float64)
        if rc.size == 1:
            rc = np.full((self.ns, self.ns), float(rc))
        self.r_cut_sigma = np.ascontiguousarray(rc.reshape(self.ns, self.ns))
        self.truncation = truncation
        self.potential = potential
        self.h = h

        def mat(v, dtype, default):
            a = np.asarray(default if v is None else v, dtype=dtype)
            if a.size == 1:
                a = np.full((self.ns, self.ns), a.reshape(()))
            return np.ascontiguousarray(a.reshape(self.ns, self.ns), dtype=dtype)

        idx_m = mat(index if potential == "power_law" else index_repulsion, np.uint32, 12)
        idx_n = mat(index_attraction, np.uint32, 6)
        self.r_min = mat(r_min, np.float64, 1.0)
        self.distortion = mat(distortion, np.float64, 1.0)
        self._buf = np.zeros(lib().orc_pot_sizeof(), dtype=np.uint8)
        rc_ = lib().orc_pot_init_any(_p(self._buf), POTENTIAL[potential], self.ns, _p(self.eps), _p(self.sigma),
                                     _p(self.r_cut_sigma), TRUNC[truncation], float(h), _p(idx_m), _p(idx_n),
                                     _p(self.r_min), _p(self.distortion))
        if rc_ != 0:
            raise ValueError("bad potential parameters")

    @property
    def ptr(self):
        return _p(self._buf)

    @property
    def r_cut(self):
        return self.sigma * self.r_cut_sigma

    def __call__(self, rr, a, b):
        f = ctypes.c_double()
        e = ctypes.c_double()
        lib().orc_pot_eval(self.ptr, float(rr), int(a), int(b), ctypes.byref(f), ctypes.byref(e))
        return f.value, e.value


def accumulate(values):
    x = np.ascontiguousarray(values, dtype=np.float64)
    out = np.zeros(6)
    lib().orc_accumulate(x.size, _p(x), _p(out))
    return dict(count=out[0], mean=out[1], variance=out[2], sigma=out[3], error_of_mean=out[4], sum=out[5])


def binning_sizing(n, L, r_cut_max, skin, occupancy):
    L = np.ascontiguousarray(L, dtype=np.float64)
    ncell = np.zeros(3, dtype=np.int32)
    cs = lib().orc_binning_sizing(int(n), _p(L), float(r_cut_max), float(skin), float(occupancy), _p(ncell))
    return ncell, cs


def binning_f32(pos4, ncell, cell_len, cell_size):
    pos4 = np.ascontiguousarray(pos4, dtype=np.float32)
    n = pos4.shape[0]
    ncell = np.ascontiguousarray(ncell, dtype=np.int32)
    cell_len = np.ascontiguousarray(cell_len, dtype=np.float32)
    cells = np.zeros(int(np.prod(ncell)) * cell_size, dtype=np.uint32)
    cell_of = np.zeros(n, dtype=np.uint32)
    maxocc = lib().orc_binning_f32(n, _p(pos4), _p(ncell), _p(cell_len), int(cell_size), _p(cells), _p(cell_of))
    return cells, cell_of, maxocc


def neighbour_full_f32(pos4, Lf, rr_cut_skin, maxn):
    pos4 = np.ascontiguousarray(pos4, dtype=np.float32)
    n = pos4.shape[0]
    Lf = np.ascontiguousarray(Lf, dtype=np.float32)
    rrcs = np.ascontiguousarray(rr_cut_skin, dtype=np.float32)
    ns = int(round(np.sqrt(rrcs.size)))
    counts = np.zeros(n, dtype=np.uint32)
    lists = np.zeros((n, maxn), dtype=np.uint32)
    mx = lib().orc_neighbour_full_f32(n, _p(pos4), _p(Lf), ns, _p(rrcs), int(maxn), _p(counts), _p(lists))
    return counts, lists, mx


def forces(r, species, L, pot, pos4=None, Lf=None, aux=True):
    """FP64 forces; with pos4/Lf the cutoff decision follows the float GPU rule."""
    r = np.ascontiguousarray(r, dtype=np.float64)
    n = r.shape[0]
    sp = np.ascontiguousarray(species, dtype=np.uint32)
    L = np.ascontiguousarray(L, dtype=np.float64)
    f = np.zeros((n, 3))
    en = np.zeros(n) if aux else None
    st = np.zeros((n, 6)) if aux else None
    tot = np.zeros(2)
    decide = 1 if pos4 is not None else 0
    if decide:
        pos4 = np.ascontiguousarray(pos4, dtype=np.float32)
        Lf = np.ascontiguousarray(Lf, dtype=np.float32)
    npairs = lib().orc_forces(n, _p(r), _p(sp), _p(L), pot.ptr, decide, _p(pos4), _p(Lf),
                              _p(f), _p(en), _p(st), _p(tot))
    return dict(force=f, en_pot=en, stress=st, epot=tot[0], virial=tot[1], npairs=npairs)


def dsfun(op, a, b):
    a = np.ascontiguousarray(a, dtype=np.float32)
    b = np.ascontiguousarray(b, dtype=np.float32)
    c = np.zeros_like(a)
    lib().orc_dsfun({"add": 0, "sub": 1, "mul": 2}[op], a.shape[0], _p(a), _p(b), _p(c))
    return c


def integrate_f32(r4, v4, img4, f4, dt, Lf, ds=True):
    """r4/v4: (2n,4) float32 [hi rows | lo rows]; modified copies returned."""
    r4 = np.array(r4, dtype=np.float32, copy=True)
    v4 = np.array(v4, dtype=np.float32, copy=True)
    img4 = np.array(img4, dtype=np.float32, copy=True)
    f4 = np.ascontiguousarray(f4, dtype=np.float32)
    n = img4.shape[0]
    Lf = np.ascontiguousarray(Lf, dtype=np.float32)
    lib().orc_integrate_f32(n, int(ds), _p(r4), _p(v4), _p(img4), _p(f4), np.float32(dt),
                            np.float32(np.float64(dt) / 2), _p(Lf))
    return r4, v4, img4


def finalize_f32(r4, v4, f4, dt, ds=True):
    v4 = np.array(v4, dtype=np.float32, copy=True)
    r4 = np.ascontiguousarray(r4, dtype=np.float32)
    f4 = np.ascontiguousarray(f4, dtype=np.float32)
    n = f4.shape[0]
    lib().orc_finalize_f32(n, int(ds), _p(r4), _p(v4), _p(f4), np.float32(np.float64(dt) / 2))
    return v4


def max_displacement2_f32(r4, r04, Lf):
    r4 = np.ascontiguousarray(r4, dtype=np.float32)
    r04 = np.ascontiguousarray(r04, dtype=np.float32)
    Lf = np.ascontiguousarray(Lf, dtype=np.float32)
    return lib().orc_max_displacement2_f32(r04.shape[0], _p(r4), _p(r04), _p(Lf))


def philox4x32_10(ctr, key):
    c = np.ascontiguousarray(ctr, dtype=np.uint32)
    k = np.ascontiguousarray(key, dtype=np.uint32)
    out = np.zeros(4, dtype=np.uint32)
    lib().orc_philox4x32_10(_p(c), _p(k), _p(out))
    return out


def andersen_threshold(coll_prob):
    return int(min(4294967295.0, np.floor(coll_prob * 4294967296.0)))


def andersen_finalize_f32(r4, v4, f4, ids, dt, temperature, coll_prob, seed, step, ds=True):
    v4 = np.array(v4, dtype=np.float32, copy=True)
    r4 = np.ascontiguousarray(r4, dtype=np.float32)
    f4 = np.ascontiguousarray(f4, dtype=np.float32)
    ids = np.ascontiguousarray(ids, dtype=np.uint32)
    n = f4.shape[0]
    coll = np.zeros(n, dtype=np.uint8)
    lib().orc_andersen_finalize_f32(n, int(ds), _p(r4), _p(v4), _p(f4), _p(ids), np.float32(np.float64(dt) / 2),
                                    np.float32(np.sqrt(temperature)), andersen_threshold(coll_prob),
                                    int(seed), int(step), _p(coll))
    return v4, coll.astype(bool)


def hilbert_depth(max_length):
    return lib().orc_hilbert_depth(float(max_length))


def hilbert_map_unit(s3, depth):
    s3 = np.ascontiguousarray(s3, dtype=np.float32)
    keys = np.zeros(s3.shape[0], dtype=np.uint32)
    lib().orc_hilbert_map_unit(s3.shape[0], _p(s3), int(depth), _p(keys))
    return keys


def hilbert_keys_f32(pos4, Lf, depth):
    pos4 = np.ascontiguousarray(pos4, dtype=np.float32)
    Lf = np.ascontiguousarray(Lf, dtype=np.float32)
    keys = np.zeros(pos4.shape[0], dtype=np.uint32)
    lib().orc_hilbert_keys_f32(pos4.shape[0], _p(pos4), _p(Lf), int(depth), _p(keys))
    return keys


def stable_argsort_u32(keys):
    keys = np.ascontiguousarray(keys, dtype=np.uint32)
    perm = np.zeros(keys.size, dtype=np.uint32)
    lib().orc_stable_argsort_u32(keys.size, _p(keys), _p(perm))
    return perm


def msd(r1, r2, first=0, last=None):
    r1 = np.ascontiguousarray(r1, dtype=np.float64)
    r2 = np.ascontiguousarray(r2, dtype=np.float64)
    last = r1.shape[0] if last is None else last
    out = np.zeros(3)
    lib().orc_msd(int(first), int(last), _p(r1), _p(r2), _p(out))
    return dict(count=out[0], mean=out[1], variance=out[2])


def tcf(kind, a, b, first=0, last=None):
    """kind "msd", "mqd" (|b - a|^4) or "vacf" (a . b) over particles [first, last)."""
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    last = a.shape[0] if last is None else last
    out = np.zeros(3)
    lib().orc_tcf({"msd": 0, "mqd": 2, "vacf": 3}[kind], int(first), int(last), _p(a), _p(b), _p(out))
    return dict(count=out[0], mean=out[1], variance=out[2])


def density_modes(pos4, q3, first=0, last=None):
    pos4 = np.ascontiguousarray(pos4, dtype=np.float32)
    q3 = np.ascontiguousarray(q3, dtype=np.float32)
    last = pos4.shape[0] if last is None else last
    out = np.zeros((q3.shape[0], 2))
    lib().orc_density_modes(int(first), int(last), _p(pos4), q3.shape[0], _p(q3), _p(out))
    return out


def isf(shells, rho1, rho2, norm):
    sh = np.ascontiguousarray(shells, dtype=np.int32)
    rho1 = np.ascontiguousarray(rho1, dtype=np.float64)
    rho2 = np.ascontiguousarray(rho2, dtype=np.float64)
    out = np.zeros((sh.shape[0], 3))
    lib().orc_isf(sh.shape[0], _p(sh), _p(rho1), _p(rho2), float(norm), _p(out))
    return out


def wavevectors(radii, box_length, tolerance, max_count, filt=(1, 1, 1), max_out=100000):
    radii = np.ascontiguousarray(radii, dtype=np.float64)
    unit = np.ascontiguousarray(2 * np.pi / np.asarray(box_length, dtype=np.float64))
    filt = np.ascontiguousarray(filt, dtype=np.int32)
    q = np.zeros((max_out, 3))
    shell = np.zeros((radii.size, 2), dtype=np.int32)
    total = lib().orc_wavevectors(radii.size, _p(radii), _p(unit), float(tolerance), int(max_count), _p(filt),
                                  max_out, _p(q), _p(shell))
    return q[:total], shell


def lattice(n, box, slab=(1.0, 1.0, 1.0)):
    """positions.lattice: (positions [n, 3], number of sites)."""
    out = np.zeros((n, 3))
    box = np.ascontiguousarray(np.broadcast_to(np.asarray(box, dtype=np.float64), (3,)))
    slab = np.ascontiguousarray(np.broadcast_to(np.asarray(slab, dtype=np.float64), (3,)))
    sites = lib().orc_lattice(int(n), _p(box), _p(slab), _p(out))
    return out, int(sites)


def boltzmann(mass, temperature, seed):
    mass = np.ascontiguousarray(mass, dtype=np.float64)
    out = np.zeros((mass.size, 3))
    lib().orc_boltzmann(int(mass.size), _p(mass), float(temperature), int(seed), _p(out))
    return out


def fcc_lattice(ncell, L):
    r = np.zeros((4 * ncell ** 3, 3))
    lib().orc_fcc_lattice(int(ncell), float(L), _p(r))
    return r


def minimize(r, species, L, pot, skin, nsteps, step=1e-3, max_move=0.05, image=None):
    """FP64 steepest descent; returns (r, image, dict(epot, fmax))."""
    r = np.array(r, dtype=np.float64, copy=True)
    n = r.shape[0]
    image = np.zeros((n, 3)) if image is None else np.array(image, dtype=np.float64, copy=True)
    sp = np.ascontiguousarray(species, dtype=np.uint32)
    L = np.ascontiguousarray(L, dtype=np.float64)
    stats = np.zeros(2)
    lib().orc_minimize(n, _p(r), _p(image), _p(sp), _p(L), pot.ptr, float(skin), int(nsteps), float(step),
                       float(max_move), _p(stats))
    return r, image, dict(epot=stats[0], fmax=stats[1])


INTEGRATOR = {"verlet": 0, "andersen": 1, "hoover": 2, "boltzmann": 3, "euler": 4}


def md_run(r, v, species, mass, L, pot, skin, dt, nsteps, temperature=0.0, coll_rate=0.0, seed=0, image=None,
           integrator=None, resonance_frequency=0.0):
    """FP64 host-backend MD run; integrator verlet (default), andersen (when
    coll_rate > 0 and no integrator is named), hoover, boltzmann or euler."""
    r = np.array(r, dtype=np.float64, copy=True)
    v = np.array(v, dtype=np.float64, copy=True)
    n = r.shape[0]
    image = np.zeros((n, 3)) if image is None else np.array(image, dtype=np.float64, copy=True)
    sp = np.ascontiguousarray(species, dtype=np.uint32)
    m = np.ascontiguousarray(mass, dtype=np.float64)
    L = np.ascontiguousarray(L, dtype=np.float64)
    if integrator is None:
        integrator = "andersen" if coll_rate > 0 else "verlet"
    stats = np.zeros(3)
    chain = np.zeros(5)
    lib().orc_md_run_any(n, _p(r), _p(v), _p(image), _p(sp), _p(m), _p(L), pot.ptr, float(skin), float(dt),
                         int(nsteps), INTEGRATOR[integrator], float(temperature), float(coll_rate),
                         float(resonance_frequency), int(seed), _p(stats), _p(chain))
    return r, v, image, dict(rebuilds=stats[0], epot=stats[1], ekin=stats[2], xi=chain[0:2], v_xi=chain[2:4],
                             en_nhc=chain[4])
