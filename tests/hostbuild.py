"""Host (g++) builds of device headers for the CPU tests: tests/host_*.cpp
include a header of prism3d_gb300/csrc with the CUDA qualifiers mapped to
host forms and export plain C functions."""
import ctypes
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def cuda_include():
    for d in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if d and os.path.exists(os.path.join(d, "include", "cuda_runtime.h")):
            return os.path.join(d, "include")
    return None


def build(source, out_dir):
    """Compile tests/<source> into out_dir and load it (skips the test when
    g++ or the CUDA headers are missing)."""
    cxx = shutil.which("g++")
    inc = cuda_include()
    if not cxx or not inc:
        pytest.skip("needs g++ and the CUDA headers")
    out = os.path.join(str(out_dir), os.path.splitext(source)[0] + ".so")
    src = os.path.join(ROOT, "tests", source)
    subprocess.run([cxx, "-O2", "-std=c++17", "-shared", "-fPIC", "-I", inc, src, "-o", out],
                   check=True, capture_output=True)
    return ctypes.CDLL(out)


def ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def root_lib(out_dir):
    """tests/host_root.cpp, initialised with the line parameters and the CO
    ladder."""
    import numpy as np
    from prism3d_gb300 import tables
    L = build("host_root.cpp", out_dir)
    lp = [np.ascontiguousarray(a, dtype=np.float64) for a in tables.line_params()]
    co = np.ascontiguousarray(tables.co_ladder(), dtype=np.float64)
    L.hr_init(*[ptr(a) for a in lp], ptr(co))
    return L
