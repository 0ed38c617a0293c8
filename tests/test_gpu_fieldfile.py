"""Field files on the device: pglDeviceNewFieldFromFile reads the reference's
layout (VecSize 8 lanes), so a field written by the reference library itself
answers guided queries as the reference does, and a GPU field survives a
store/load round trip unchanged and keeps training identically."""

import gzip
import json
import os
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
MANIFEST = json.load(open(os.path.join(GOLDEN, "manifest.json")))
# every field type of the goldens: parallax-aware VMM, plain VMM, directional quadtree
CASES = sorted(MANIFEST["cases"])


@pytest.fixture(scope="module")
def pgl():
    import openpgl_gb300

    openpgl_gb300.load()
    return openpgl_gb300


@pytest.mark.parametrize("name", CASES)
def test_reference_field_file_answers_like_the_reference(pgl, name, tmp_path):
    sys.path.insert(0, GOLDEN)
    import make_golden

    path = tmp_path / "ref.field"
    ref_bytes = gzip.open(os.path.join(GOLDEN, f"{name}.field.gz")).read()
    path.write_bytes(ref_bytes)
    dev = pgl.Device()
    field = pgl.Field.from_file(dev, str(path))
    _, queries = make_golden.build_inputs(MANIFEST["cases"][name])
    g = np.load(os.path.join(GOLDEN, f"{name}.queries.npz"))
    for volume, key in ((False, "surface"), (True, "volume")):
        out = field.sample_batch(queries, volume=volume, cosine=not volume)
        ref = g[key]
        assert np.array_equal(out["ok"], ref["ok"]), key
        ok = ref["ok"] == 1
        assert np.array_equal(out["id"][ok], ref["id"][ok]), key
        assert np.array_equal(out["sample1d"][ok].view(np.uint32), ref["sample1d"][ok].view(np.uint32)), key
        if ok.any():
            rel = np.abs(out["pdf"][ok] - ref["pdf"][ok]) / ref["pdf"][ok]
            assert rel.max() <= 1e-3, key
    # what was read is written back byte for byte
    assert field.field_bytes() == ref_bytes


def test_store_load_round_trip_and_continued_training(pgl, tmp_path):
    from openpgl_gb300 import synthetic as syn

    dev = pgl.Device()
    a = pgl.Field(dev, pgl.FieldConfig(True, 4000))
    st = pgl.SampleStorage()
    st.add_samples(syn.cube_face_samples(80000, 900, volume_fraction=0.25))
    a.update(st)
    path = str(tmp_path / "a.field")
    a.store(path)
    b = pgl.Field.from_file(dev, path)
    assert a.compare(b)
    assert a.field_bytes() == b.field_bytes()
    assert b.iteration == a.iteration
    q = syn.queries(2048, 901)
    assert a.sample_batch(q).tobytes() == b.sample_batch(q).tobytes()
    # both continue with the same frame and stay equal
    st.clear()
    st.add_samples(syn.cube_face_samples(80000, 902, volume_fraction=0.25))
    a.update(st)
    b.update(st)
    assert a.compare(b)
    assert a.field_bytes() == b.field_bytes()


def test_bad_files_are_rejected(pgl, tmp_path):
    dev = pgl.Device()
    p = tmp_path / "bad.field"
    p.write_bytes(b"not a field")
    with pytest.raises(RuntimeError):
        pgl.Field.from_file(dev, str(p))
    ref = gzip.open(os.path.join(GOLDEN, "cube_single.field.gz")).read()
    p.write_bytes(ref[: len(ref) // 2])
    with pytest.raises(RuntimeError):
        pgl.Field.from_file(dev, str(p))
    # a node count far beyond what the file holds is refused before anything
    # is allocated for it (no attempt at a 2^29-node tree)
    import struct

    import fieldfile

    surf = fieldfile.read_field_file(ref)["surface"]
    n = len(surf["nodes"])
    first = struct.pack("<fI", float(surf["nodes"]["split"][0]), int(surf["nodes"]["bits"][0]))
    at = ref.index(struct.pack("<Q", n) + first)
    p.write_bytes(ref[:at] + struct.pack("<Q", 1 << 29) + ref[at + 8:])
    with pytest.raises(RuntimeError, match="truncated"):
        pgl.Field.from_file(dev, str(p))
