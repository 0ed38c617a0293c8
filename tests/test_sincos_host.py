"""The float sine and cosine of the guided queries' sampled directions
(sincos_df in pgl_math.cuh: Cody-Waite reduction, Taylor series in
double-float arithmetic, Ziv's rounding test) built for the host with the
library's flags: its double-float values against long double on a grid of
the floats in [0, 8) and against mpmath around the multiples of pi/2, and
every result the rounding test decides equal to the exact value rounded to
nearest.  The GPU test checks the device build on every float of [0, 8)
against the double path.  Host code only: runs without a GPU."""

import ctypes
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUDA_INCLUDE = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
EIGHT = int(np.float32(8.0).view(np.uint32))


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("sincos") / "libsincoshost.so")
    subprocess.run(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math", "-pthread",
                    "-I" + os.path.join(ROOT, "openpgl_gb300", "csrc"), "-I" + CUDA_INCLUDE,
                    os.path.join(ROOT, "tests", "cuda", "sincos_host_check.cpp"), "-o", out], check=True)
    dll = ctypes.CDLL(out)
    dll.sincos_host_check.argtypes = [ctypes.c_uint32] * 3 + [ctypes.c_int] + [ctypes.c_void_p] * 3
    dll.sincos_host_values.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    return dll


def test_grid_of_floats_below_eight(lib):
    out = np.zeros(3, np.uint64)
    err = np.zeros(2)
    first = np.zeros(1, np.float32)
    assert lib.sincos_host_check(0, EIGHT, 101, os.cpu_count() or 1, out.ctypes.data, err.ctypes.data,
                                 first.ctypes.data) == 0
    n, undecided, wrong = (int(v) for v in out)
    assert n == (EIGHT + 100) // 101
    assert wrong == 0, f"first decided result that is not correctly rounded: x = {first[0]!r}"
    # the rounding test widens by 2^-38: the error must stay well inside it
    assert err[0] < 2.0 ** -40 and err[1] < 2.0 ** -40, err
    assert undecided < 1e-4 * n, undecided


def test_around_multiples_of_half_pi_against_mpmath(lib):
    mpmath = pytest.importorskip("mpmath")
    mpmath.mp.prec = 160
    xs = []
    for k in range(1, 6):
        u = int(np.float32(k * np.pi / 2).view(np.uint32))
        xs += list(range(u - 300, u + 301))
    xs += [0, 1, 2, 0x00800000, 0x39800000, 0x39000000, 0x3F000000, EIGHT - 1]  # 0, denormals, 2^-12, 2^-13, 0.5
    x = np.array(xs, np.uint32).view(np.float32)
    parts = np.zeros((len(x), 4), np.float32)
    res = np.zeros((len(x), 3), np.float32)
    lib.sincos_host_values(x.ctypes.data, len(x), parts.ctypes.data, res.ctypes.data)
    # outside +0 <= x < 8 (-0 included: its sine keeps the sign on the double path) nothing is decided
    outside = np.array([0x80000000, 0x80000001, 0xBF800000, EIGHT, 0x7F800000, 0x7FC00000], np.uint32).view(np.float32)
    ores = np.zeros((len(outside), 3), np.float32)
    lib.sincos_host_values(outside.ctypes.data, len(outside), np.zeros((len(outside), 4), np.float32).ctypes.data,
                           ores.ctypes.data)
    assert not ores[:, 2].any()

    def nearest_float(v):
        f = np.float32(float(v))
        cands = [f, np.nextafter(f, np.float32(np.inf)), np.nextafter(f, np.float32(-np.inf))]
        return min(cands, key=lambda c: abs(mpmath.mpf(float(c)) - v))

    worst = 0.0
    for i, xv in enumerate(x):
        m = mpmath.mpf(float(xv))
        exact = (mpmath.sin(m), mpmath.cos(m))
        for j, e in enumerate(exact):
            got = mpmath.mpf(float(parts[i, 2 * j])) + mpmath.mpf(float(parts[i, 2 * j + 1]))
            if e != 0:
                worst = max(worst, float(abs((got - e) / e)))
            elif got != 0:
                worst = 1.0
            if res[i, 2] == 1:
                r = np.float32(res[i, j])
                assert r.view(np.uint32) == nearest_float(e).view(np.uint32), (float(xv), j)
    assert worst < 2.0 ** -44, worst
