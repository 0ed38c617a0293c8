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


def test_reference_cpp_wrapper_builds_and_links(lib, tmp_path):
    """The reference's own C++ wrapper (include/openpgl/cpp/*.h, unchanged),
    on top of this repository's C headers, compiles and links against the
    library: a renderer's code that uses openpgl::cpp builds as it is.  Runs
    where the reference sources are; the program is linked, not run (no GPU
    here).  The wrapper's Region::GetValid / GetDistribution and the C
    functions behind them are inside comment blocks in the reference itself
    (cpp/Region.h:64-80, include/openpgl/region.h:24-26, api/api.cpp:277-294),
    so nothing declares or calls them."""
    import shutil
    import sys

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle

    ref = pyoracle.reference_sources()
    if not ref:
        pytest.skip("reference sources not present")
    from openpgl_gb300 import build

    inc = tmp_path / "include"
    shutil.copytree(os.path.join(ROOT, "include"), inc)
    shutil.copytree(os.path.join(ref, "openpgl", "include", "openpgl", "cpp"), inc / "openpgl" / "cpp")
    src = tmp_path / "renderer.cpp"
    src.write_text(r'''
#include <openpgl/cpp/OpenPGL.h>
#include <vector>
int main() {
  openpgl::cpp::Device device(PGL_DEVICE_TYPE_CPU_8);
  openpgl::cpp::FieldConfig cfg;
  cfg.Init(PGL_SPATIAL_STRUCTURE_KDTREE, PGL_DIRECTIONAL_DISTRIBUTION_PARALLAX_AWARE_VMM, true, 32000);
  openpgl::cpp::Field field(&device, cfg);
  openpgl::cpp::SampleStorage storage;
  std::vector<PGLSampleData> samples(1000);
  storage.AddSamples(samples.data(), samples.size());
  field.Update(storage);
  storage.Clear();
  openpgl::cpp::SurfaceSamplingDistribution ssd(&field);
  float s1d = 0.5f;
  pgl_point3f p = {0.5f, 0.5f, 0.5f};
  pgl_vec3f n = {0.f, 0.f, 1.f}, d;
  pgl_point2f u = {0.3f, 0.7f};
  if (ssd.Init(&field, p, s1d)) {
    ssd.ApplyCosineProduct(n);
    float pdf = ssd.SamplePDF(u, d);
    pdf += ssd.PDF(d) + ssd.IncomingRadiancePDF(d);
    (void)ssd.GetId();
    (void)pdf;
  }
  openpgl::cpp::VolumeSamplingDistribution vsd(&field);
  if (vsd.Init(&field, p, s1d)) {
    vsd.ApplySingleLobeHenyeyGreensteinProduct(n, 0.5f);
    (void)vsd.SamplePDF(u, d);
  }
  openpgl::cpp::Field copy(&device, "field.bin");
  bool same = field == copy;
  openpgl::cpp::PathSegmentStorage paths;
  paths.Reserve(16);
  openpgl::cpp::PathSegment *seg = paths.NextSegment();
  (void)seg;
  return same ? 0 : 1;
}
''')
    exe = tmp_path / "renderer"
    p = subprocess.run(["g++", "-std=c++11", "-I" + str(inc), str(src), "-o", str(exe), "-L" + os.path.dirname(build.LIB),
                        "-lopenpgl_gb300", "-Wl,--no-undefined"], capture_output=True, text=True)
    assert p.returncode == 0, p.stderr[-3000:]
