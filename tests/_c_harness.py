"""Build the C harness (tests/c_abi/harness.c) with the system C compiler
against include/halmd_gb300.h and the in-tree library."""
import os
import re
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
SRC = os.path.join(HERE, "c_abi", "harness.c")
OUT = os.path.join(REPO, "_build", "c_abi_harness")


def cuda_home():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def build():
    from halmd_gb300 import _lib
    if not os.path.exists(_lib.LIB_PATH):
        from halmd_gb300 import build as b
        b.build()
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    cuda = cuda_home()
    lib_dir = os.path.dirname(_lib.LIB_PATH)
    cmd = [os.environ.get("CC", "cc"), "-std=c99", "-O1", "-Wall", "-Werror", "-I" + os.path.join(REPO, "include"),
           "-I" + os.path.join(cuda, "include"), SRC, "-o", OUT, "-L" + lib_dir, "-lhalmd_gb300",
           "-L" + os.path.join(cuda, "lib64"), "-lcudart", "-lm", "-Wl,-rpath," + lib_dir]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return OUT


def called_symbols():
    """hmd_* names the harness calls."""
    with open(SRC) as fh:
        return set(re.findall(r"\b(hmd_[a-z_0-9]+)\s*\(", fh.read()))
