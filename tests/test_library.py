"""The C-ABI library builds, loads without a GPU and exports every entry
point the public headers declare (no compute calls)."""

import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = [os.path.join(ROOT, "include", "openpgl", f) for f in sorted(os.listdir(os.path.join(ROOT, "include", "openpgl")))]
HEADERS.append(os.path.join(ROOT, "include", "openpgl_gb300.h"))


def declared_symbols():
    names = set()
    for h in HEADERS:
        text = open(h).read()
        # a declaration spans from the export macro to the opening parenthesis
        for m in re.finditer(r"OPENPGL_CORE_INTERFACE[^;(]*?\b(pgl[A-Za-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    from openpgl_gb300 import build

    path = build.build()
    return ctypes.CDLL(path)


def test_headers_declare_api():
    syms = declared_symbols()
    assert len(syms) > 80
    for must in ("pglFieldUpdate", "pglDeviceNewField", "pglFieldInitSurfaceSamplingDistribution",
                 "pglVolumeSamplingDistributionSamplePDF", "pglFieldCompare", "pglSampleStorageAddSamples",
                 "pglFieldSampleSurfaceBatch", "pglFieldSampleBatchDevice"):
        assert must in syms


def test_library_exports_every_declared_symbol(lib):
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_library_has_no_undefined_own_symbols(lib):
    from openpgl_gb300 import build

    out = subprocess.run(["nm", "-D", "--undefined-only", build.LIB], capture_output=True, text=True).stdout
    own = [l for l in out.splitlines() if "pgl" in l]
    assert not own, own


def test_headers_compile_as_cpp():
    src = "#include <openpgl/openpgl.h>\n#include <openpgl_gb300.h>\nint main(){PGLFieldArguments a; pglFieldArgumentsSetDefaults(a, PGL_SPATIAL_STRUCTURE_KDTREE, PGL_DIRECTIONAL_DISTRIBUTION_PARALLAX_AWARE_VMM, true, 32000); return 0;}\n"
    p = subprocess.run(["g++", "-std=c++11", "-fsyntax-only", "-I" + os.path.join(ROOT, "include"), "-x", "c++", "-"],
                       input=src, capture_output=True, text=True)
    assert p.returncode == 0, p.stderr


def test_front_end_binds_all_symbols():
    import openpgl_gb300 as pgl

    lib = pgl.load()
    for name in pgl.C_API:
        assert hasattr(lib, name)
