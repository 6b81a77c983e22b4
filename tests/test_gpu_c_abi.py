"""Every entry point of include/halmd_gb300.h called from C on a GPU: the
harness tests/c_abi/harness.c, built with the system C compiler against the
header and the library (no Python binding in between)."""
import subprocess

import pytest

import _c_harness

pytestmark = pytest.mark.gpu


def test_c_harness_runs():
    exe = _c_harness.build()
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "harness ok" in r.stdout
