"""The module-style front end maps the Lua API's names and defaults onto the
system description (no GPU: only the library's descriptor initialiser runs)."""
import numpy as np
import pytest

from halmd_gb300 import _lib


@pytest.fixture
def halmd():
    import os
    if not os.path.exists(_lib.LIB_PATH):
        from halmd_gb300 import build
        build.build()
    from halmd_gb300 import halmd as h
    h.reset()
    yield h
    h.reset()


def ka_script(halmd, n=1000, L=9.4):
    box = halmd.mdsim.box(length=[L, L, L])
    particle = halmd.mdsim.particle(dimension=3, particles=n, species=2)
    pot = halmd.mdsim.potentials.pair.lennard_jones(epsilon=[[1, 1.5], [1.5, 0.5]], sigma=[[1, 0.8], [0.8, 0.88]])
    pot = pot.truncate({1: "smooth_r4", "cutoff": 2.5, "h": 0.005})
    halmd.mdsim.forces.pair(box=box, particle=particle, potential=pot, neighbour={"skin": 0.3})
    halmd.mdsim.integrators.verlet_nvt_andersen(box=box, particle=particle, timestep=0.002, temperature=0.7, rate=1.0)
    return particle


def test_description_follows_the_modules(halmd):
    d = ka_script(halmd)._desc()
    assert d.nparticle == 1000 and d.nspecies == 2
    assert list(d.box) == [9.4, 9.4, 9.4]
    assert d.truncation == _lib.TRUNCATION["smooth_r4"] and d.smoothing == 0.005
    assert [d.epsilon[k] for k in range(4)] == [1, 1.5, 1.5, 0.5]
    assert [d.sigma[k] for k in range(4)] == [1, 0.8, 0.8, 0.88]
    assert [d.r_cut[k] for k in range(4)] == [2.5] * 4        # in units of sigma_ab, as the Lua cutoff
    assert d.skin == 0.3 and d.timestep == 0.002
    assert d.integrator == _lib.INTEGRATOR["andersen"] and d.temperature == 0.7 and d.collision_rate == 1.0
    assert d.sort == 1


def test_lua_defaults(halmd):
    box = halmd.mdsim.box({"length": [10, 10, 10]})
    p = halmd.mdsim.particle({"particles": 100})
    assert p.nspecies == 1 and p.precision == "double-single" and p.label == "all"
    pot = halmd.mdsim.potentials.pair.lennard_jones().truncate(cutoff=2.5)
    assert pot.kind == "shifted"                                  # truncate.lua.in:289
    assert np.all(pot.epsilon == 1) and np.all(pot.sigma == 1)
    halmd.mdsim.forces.pair(box=box, particle=p, potential=pot)
    halmd.mdsim.integrators.verlet(box=box, particle=p, timestep=0.001)
    d = p._desc()
    assert d.skin == 0.5                                          # neighbour.lua.in:162
    assert d.neighbour_occupancy == 0.4 and d.cell_occupancy == 0.5
    assert d.integrator == _lib.INTEGRATOR["verlet"]


def test_argument_errors(halmd):
    with pytest.raises(ValueError):
        halmd.mdsim.particle(dimension=2, particles=10)
    with pytest.raises(ValueError):
        halmd.mdsim.potentials.pair.lennard_jones().truncate("shifted")        # no cutoff
    with pytest.raises(ValueError):
        halmd.mdsim.potentials.pair.lennard_jones().truncate("cubic", cutoff=2.5)
    with pytest.raises(ValueError):
        halmd.mdsim.potentials.pair.lennard_jones().truncate("smooth_r4", cutoff=2.5)  # no h
    box = halmd.mdsim.box(length=[5, 5, 5])
    p = halmd.mdsim.particle(particles=10)
    with pytest.raises(RuntimeError):
        p._desc()                                                  # no force / integrator yet


def test_untruncated_potential_maps_onto_pair_full(halmd):
    # forces/pair.lua.in:78-83: a potential without r_cut takes the pair_full force
    box = halmd.mdsim.box(length=[5, 5, 5])
    p = halmd.mdsim.particle(particles=10)
    halmd.mdsim.forces.pair(box=box, particle=p, potential=halmd.mdsim.potentials.pair.lennard_jones())
    halmd.mdsim.integrators.verlet(box=box, particle=p, timestep=0.001)
    d = p._desc()
    assert d.truncation == 4


@pytest.mark.parametrize("name,kw,check", [
    ("mie", dict(index_repulsion=[[12, 10], [10, 14]], index_attraction=6),
     lambda d: [d.index_repulsion[k] for k in range(4)] == [12, 10, 10, 14] and d.index_attraction[3] == 6),
    ("morse", dict(r_min=1.1, distortion=[[1, 1.41], [1.41, 1.5]]),
     lambda d: d.r_min[0] == 1.1 and [d.distortion[k] for k in range(4)] == [1, 1.41, 1.41, 1.5]),
    ("power_law", dict(index=[[12, 9], [9, 6]]), lambda d: [d.index[k] for k in range(4)] == [12, 9, 9, 6]),
])
def test_other_potentials_map_onto_the_description(halmd, name, kw, check):
    box = halmd.mdsim.box(length=[10, 10, 10])
    p = halmd.mdsim.particle(particles=500, species=2)
    pot = getattr(halmd.mdsim.potentials.pair, name)(epsilon=[[1, 1.5], [1.5, 0.5]], **kw)
    pot = pot.truncate({1: "force_shifted", "cutoff": 2.5})
    halmd.mdsim.forces.pair(box=box, particle=p, potential=pot)
    halmd.mdsim.integrators.verlet(box=box, particle=p, timestep=0.001)
    d = p._desc()
    assert d.potential == _lib.POTENTIAL[name] and d.truncation == _lib.TRUNCATION["force_shifted"]
    assert check(d)


def test_other_potentials_defaults_and_errors(halmd):
    assert halmd.mdsim.potentials.pair.power_law().params["index"] == 12      # power_law.lua.in:140
    assert halmd.mdsim.potentials.pair.morse(minimum=1.2).params["distortion"] == 1.0   # morse.lua.in:178-185
    with pytest.raises(ValueError):
        halmd.mdsim.potentials.pair.morse()                                  # r_min has no default
    with pytest.raises(ValueError):
        halmd.mdsim.potentials.pair.mie(index_repulsion=12)                  # both indices are required


def two_instances(halmd, wire, na=800, nb=200, L=9.4):
    """The KA mixture as two particle instances A and B (test/integration/
    modularity/two_particles.lua): one box, one potential, forces for the
    ordered pairs in `wire`, a Verlet integrator each."""
    box = halmd.mdsim.box(length=[L, L, L])
    pa = halmd.mdsim.particle(particles=na, species=2, label="A")
    pb = halmd.mdsim.particle(particles=nb, species=2, label="B")
    pot = halmd.mdsim.potentials.pair.lennard_jones(epsilon=[[1, 1.5], [1.5, 0.5]], sigma=[[1, 0.8], [0.8, 0.88]])
    pot = pot.truncate("smooth_r4", cutoff=2.5, h=0.005)
    inst = {"A": pa, "B": pb}
    for l1, l2 in wire:
        halmd.mdsim.forces.pair(box=box, particle=[inst[l1], inst[l2]], potential=pot, neighbour={"skin": 0.3})
    for p in (pa, pb):
        halmd.mdsim.integrators.verlet(box=box, particle=p, timestep=0.002)
    return pa, pb


def test_coupled_instances_form_one_system(halmd):
    pa, pb = two_instances(halmd, [("A", "A"), ("A", "B"), ("B", "A"), ("B", "B")])
    groups = halmd._script.groups()
    assert len(groups) == 1 and groups[0] == [pa, pb]
    d = pa._desc(sum(p.nparticle for p in groups[0]))
    assert d.nparticle == 1000 and d.nspecies == 2 and d.truncation == _lib.TRUNCATION["smooth_r4"]


def test_coupled_instances_need_every_ordered_pair(halmd):
    two_instances(halmd, [("A", "A"), ("A", "B"), ("B", "B")])
    with pytest.raises(ValueError, match="every ordered pair"):
        halmd._script.groups()


def test_coupled_instances_share_the_integrator(halmd):
    pa, pb = two_instances(halmd, [("A", "A"), ("A", "B"), ("B", "A"), ("B", "B")])
    halmd.mdsim.integrators.verlet(particle=pb, timestep=0.001)
    with pytest.raises(ValueError, match="same integrator"):
        halmd._script.groups()


def test_uncoupled_instances_stay_separate_systems(halmd):
    pa, pb = two_instances(halmd, [("A", "A"), ("B", "B")])
    assert halmd._script.groups() == [[pa], [pb]]
