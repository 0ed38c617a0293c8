"""Builds libopenpgl_gb300.so in-tree (openpgl_gb300/_build/) for sm_103a.

CUDA translation units are compiled with nvcc (--fmad=false: no contraction of
a*b+c, explicit FMAs only; IEEE division and square root), the host units
with g++ -ffp-contract=off, all in parallel, then linked with nvcc.
"""

from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libopenpgl_gb300.so")
LIBM_TABLE = os.path.join(OUT, "libm_exceptions.bin")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

CUDA_SOURCES = ["em_kernel.cu", "spatial_kernels.cu", "query_kernels.cu", "noalloc.cu", "path_kernels.cu", "dqt_kernels.cu"]
HOST_SOURCES = ["field.cpp", "api.cpp", "serve.cpp", "pathsegments.cpp"]
GENCODE = "-gencode=arch=compute_103a,code=sm_103a"


def _cuda_home():
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found")


def _run(cmd):
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("command failed: " + " ".join(cmd) + "\n" + p.stdout + p.stderr)
    return p.stdout + p.stderr


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, ptxas_info=False):
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(OUT, exist_ok=True)
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh"))]
    headers += [os.path.join(INCLUDE, "openpgl_gb300.h")]
    jobs = []
    objs = []
    for src in CUDA_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src + ".o")
        objs.append(o)
        if _stale(o, [s] + headers):
            cmd = [nvcc, "-std=c++17", GENCODE, "-O3", "-lineinfo", "--fmad=false", "-Xcompiler", "-fPIC",
                   "-Xcompiler", "-ffp-contract=off", "-c", s, "-o", o]
            if ptxas_info:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)
    for src in HOST_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src + ".o")
        objs.append(o)
        if _stale(o, [s] + headers):
            jobs.append(["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-Wall",
                         "-I" + os.path.join(cuda, "include"), "-c", s, "-o", o])
    if jobs:
        with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            for out in ex.map(_run, jobs):
                if verbose and out.strip():
                    print(out)
    if _stale(LIB, objs):
        _run([nvcc, GENCODE, "-shared", "-Xlinker", "--no-undefined", "-o", LIB] + objs + ["-lcudart", "-ldl"])
    # the plain per-object query driver the benchmark times (links the library)
    drv_src = os.path.join(CSRC, "plain_query_driver.cpp")
    drv = os.path.join(OUT, "plain_query_driver")
    if _stale(drv, [drv_src, LIB]):
        _run(["g++", "-std=c++17", "-O2", "-Wall", "-I" + INCLUDE, "-I" + os.path.join(cuda, "include"), drv_src, "-o",
              drv, "-L" + OUT, "-lopenpgl_gb300", "-Wl,-rpath,$ORIGIN", "-lpthread"])
    # the host C library's expf/cosf exceptions (read by the library at CUDA set-up)
    gen_src = os.path.join(CSRC, "gen_libm_exceptions.cpp")
    gen = os.path.join(OUT, "gen_libm_exceptions")
    if _stale(gen, [gen_src]):
        _run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-Wall", gen_src, "-o", gen, "-lpthread"])
    if _stale(LIBM_TABLE, [gen]):
        _run([gen, LIBM_TABLE, str(os.cpu_count() or 1)])
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, ptxas_info="--ptxas" in sys.argv))
