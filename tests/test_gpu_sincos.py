"""The guided queries' sampled directions take sin and cos of the azimuth
from lib_sincosf: on the device the float evaluation sincos_df where Ziv's
rounding test decides, else the double-precision functions rounded once.
This checks, bit for bit, that the result equals the double path on every
float of [0, 8) (the azimuths are in [0, 2 pi]) and on samples of the other
inputs (at least 8, negative, huge, infinite and NaN), which take the double
path directly."""

import ctypes
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
EIGHT = int(np.float32(8.0).view(np.uint32))


@pytest.fixture(scope="module")
def dll(tmp_path_factory):
    src = os.path.join(ROOT, "tests", "cuda", "sincos_check.cu")
    lib = str(tmp_path_factory.mktemp("sincos") / "libsincoscheck.so")
    nvcc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    subprocess.run([nvcc, "-std=c++17", "-gencode=arch=compute_103a,code=sm_103a", "-O3", "--fmad=false",
                    "-Xcompiler", "-fPIC", "-shared", "-I" + os.path.join(ROOT, "openpgl_gb300", "csrc"), src, "-o",
                    lib], check=True)
    d = ctypes.CDLL(lib)
    d.sincos_check.argtypes = [ctypes.c_uint32, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p]
    return d


def check(dll, begin, count):
    counts = np.zeros(2, np.uint64)
    bad = np.zeros(8, np.float32)
    assert dll.sincos_check(begin, count, counts.ctypes.data, bad.ctypes.data) == 0
    assert int(counts[0]) == 0, bad[: min(8, int(counts[0]))]
    return int(counts[1])


def test_every_float_below_eight_matches_the_double_path(dll):
    decided = check(dll, 0, EIGHT)
    assert decided >= EIGHT - EIGHT // 10000, decided  # the float evaluation answers nearly all


@pytest.mark.parametrize("begin", [EIGHT, 0x4E000000, 0x7F000000, 0x80000000, 0xBF000000, 0xFF000000],
                         ids=["8_up", "huge", "to_inf_nan", "neg_zero_tiny", "neg_half", "neg_inf_nan"])
def test_other_inputs_take_the_double_path(dll, begin):
    count = min(1 << 24, (1 << 32) - begin)
    assert check(dll, begin, count) == 0
