"""The split-statistics and distance passes divide through div_rcp
(Markstein's correctly rounded division from a reciprocal) and
div_faithful_fix (a faithful quotient from the approximate reciprocal, then
the nearer of it and its neighbour by exact remainders).  This checks both
bit for bit against CUDA's correctly rounded division on 2^28 operand pairs
each."""

import ctypes
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("mode", [0, 1], ids=["markstein", "faithful_fix"])
def test_division_matches_correctly_rounded_division(tmp_path, mode):
    src = os.path.join(ROOT, "tests", "cuda", "div_check.cu")
    lib = str(tmp_path / "libdivcheck.so")
    nvcc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    subprocess.run([nvcc, "-std=c++17", "-gencode=arch=compute_103a,code=sm_103a", "-O3", "--fmad=false",
                    "-Xcompiler", "-fPIC", "-shared", "-I" + os.path.join(ROOT, "openpgl_gb300", "csrc"), src, "-o", lib],
                   check=True)
    dll = ctypes.CDLL(lib)
    dll.div_check.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    mism = np.zeros(1, np.uint64)
    bad = np.zeros(24, np.float32)
    assert dll.div_check(1 << 28, 12345 + mode, mode, mism.ctypes.data, bad.ctypes.data) == 0
    assert int(mism[0]) == 0, bad.reshape(8, 3)
