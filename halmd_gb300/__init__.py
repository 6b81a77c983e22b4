"""halmd_gb300 — GB300-native molecular-dynamics step with HALMD's module API.

The compute path is the CUDA library libhalmd_gb300.so (C ABI in
include/halmd_gb300.h), built in-tree for sm_103a; ``halmd_gb300.mdsim`` and
``halmd_gb300.observables`` mirror the reference's Lua modules
(halmd.mdsim.particle, potentials.pair.lennard_jones, neighbour,
integrators.*, observables.dynamics.*) on top of it.
"""
from ._lib import Dynamics, Engine, HmdError, load, system_desc  # noqa: F401

__all__ = ["Engine", "Dynamics", "HmdError", "load", "system_desc"]
