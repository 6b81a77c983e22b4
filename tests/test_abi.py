"""The C-ABI library loads and exports every entry point of include/halmd_gb300.h (no GPU needed)."""
import ctypes
import os
import subprocess

import pytest

from halmd_gb300 import _lib


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(_lib.LIB_PATH):
        from halmd_gb300 import build
        build.build()
    return _lib.load()


def test_header_declares_entry_points():
    names = _lib.header_symbols()
    assert "hmd_engine_create" in names and "hmd_step" in names
    assert len(names) >= 30


def test_library_exports_every_declared_symbol(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True, text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    missing = [s for s in _lib.header_symbols() if s not in exported]
    assert not missing, missing
    for s in _lib.header_symbols():
        assert hasattr(lib, s)


def test_desc_defaults_match_reference(lib):
    d = _lib.SystemDesc()
    lib.hmd_system_desc_init(ctypes.byref(d))
    assert d.skin == 0.5            # neighbour.lua.in: skin default 0.5
    assert d.neighbour_occupancy == 0.4   # from_binning.cpp:285-287
    assert d.cell_occupancy == 0.5  # binning.lua.in:83
    assert d.truncation == _lib.TRUNCATION["shifted"]   # truncate.lua.in:289
    assert d.sort == 1


def test_null_handles_are_rejected(lib):
    assert lib.hmd_step(None, 1, 0) == -1
    assert lib.hmd_engine_create(0, 0, None) == -1
    assert "null" in _lib.last_error()


def test_struct_layout_matches_header(lib):
    # the ctypes mirrors must have the C sizes and field offsets (catches drift
    # between header and binding)
    exe = os.path.join(_lib.REPO, "_build", "layout_check")
    os.makedirs(os.path.dirname(exe), exist_ok=True)
    lines = ['#include "halmd_gb300.h"', "#include <stdio.h>", "#include <stddef.h>", "int main(void){"]
    for cname, cls in (("hmd_system_desc", _lib.SystemDesc), ("hmd_system_info", _lib.SystemInfo)):
        lines.append('printf("%%zu\\n", sizeof(%s));' % cname)
        for field, _ in cls._fields_:
            lines.append('printf("%%zu\\n", offsetof(%s, %s));' % (cname, field))
    lines.append("return 0;}")
    c_path = exe + ".c"
    with open(c_path, "w") as fh:
        fh.write("\n".join(lines) + "\n")
    subprocess.run(["gcc", "-I", os.path.join(_lib.REPO, "include"), "-o", exe, c_path], check=True)
    got = [int(x) for x in subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()]
    want = []
    for cls in (_lib.SystemDesc, _lib.SystemInfo):
        want.append(ctypes.sizeof(cls))
        want.extend(getattr(cls, f).offset for f, _ in cls._fields_)
    assert got == want


def test_enum_constants_agree_with_the_header():
    # the binding's and the oracle's name -> value maps against the header's
    # #defines (the oracle's own integrator enum is internal and not checked)
    import re
    import oracle
    text = open(os.path.join(os.path.dirname(_lib.LIB_PATH), "..", "include", "halmd_gb300.h")).read()

    def defines(prefix):
        return {m.group(1).lower(): int(m.group(2))
                for m in re.finditer(r"#define HMD_%s_(\w+)\s+(\d+)" % prefix, text)}

    trunc, pot, integ = defines("TRUNC"), defines("POTENTIAL"), defines("INTEGRATOR")
    assert trunc == _lib.TRUNCATION == oracle.TRUNC
    assert pot == _lib.POTENTIAL == oracle.POTENTIAL
    short = {k: v for k, v in _lib.INTEGRATOR.items() if not k.startswith("verlet_")}
    assert integ == short


def test_c_harness_calls_every_entry_point_and_links(lib):
    """The C harness (tests/c_abi/harness.c) names every declared entry point
    and compiles and links against the header and the library with a C
    compiler; it runs on a GPU in test_gpu_c_abi.py."""
    import _c_harness
    missing = sorted(set(_lib.header_symbols()) - _c_harness.called_symbols())
    assert not missing, missing
    assert os.path.exists(_c_harness.build())
