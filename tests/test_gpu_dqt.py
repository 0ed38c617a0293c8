"""The directional quadtree field type on the GPU (PGL_DIRECTIONAL_DISTRIBUTION_QUADTREE,
Device.h:185-210; directional/dqt/): against the reference's own field files
and queries (tests/golden cube_dqt at the factory's defaults, cube_dqt_per_leaf
at non-default arguments) and against the oracle on fresh seeds.

Bar: the kd-tree and the leaf sample statistics bit-exact; per region the
quadtree's structure (child layout) equal, node weights and training
statistics within 1e-3 relative (in practice bit-exact: the sample's point on
the square is the only quantity computed with another implementation of a C
library function, atan2f, restated from its published algorithm); guided
queries pick the same region with the same sample1D, pdf and direction within
1e-3."""

import gzip
import json
import os
import sys

import numpy as np
import pytest

from helpers import compare_dqt_fields, compare_queries

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
MANIFEST = json.load(open(os.path.join(GOLDEN, "manifest.json")))
DQT_CASES = sorted(n for n, c in MANIFEST["cases"].items() if c.get("dqt", False))
TOL = 1e-3


@pytest.fixture(scope="module")
def pgl():
    import openpgl_gb300

    openpgl_gb300.load()
    return openpgl_gb300


def _check(a_bytes, b_bytes):
    for side in ("surface", "volume"):
        r = compare_dqt_fields(a_bytes, b_bytes, side)
        assert r["tree_equal"] and r["numbering_equal"], (side, r)
        if r["regions"] == 0:
            continue
        assert r["structure_equal"] and r["stats_equal"] and r["valid_equal"], (side, r)
        assert r["worst_rel"] <= TOL, (side, r)
        print(side, r)


def _train(pgl, frames, leaf, dqt_args=None):
    dev = pgl.Device()
    field = pgl.Field(dev, pgl.FieldConfig(True, leaf, dqt=True, dqt_args=dqt_args))
    st = pgl.SampleStorage()
    for f in frames:
        st.add_samples(f)
        field.update(st)
        st.clear()
    return dev, field


@pytest.mark.parametrize("name", DQT_CASES)
def test_quadtree_field_and_queries_match_reference(pgl, name):
    sys.path.insert(0, GOLDEN)
    import make_golden

    case = MANIFEST["cases"][name]
    frames, queries = make_golden.build_inputs(case)
    dev, field = _train(pgl, frames, case["leaf"], case.get("dqt_args"))
    ref = gzip.open(os.path.join(GOLDEN, f"{name}.field.gz")).read()
    _check(field.field_bytes(), ref)
    g = np.load(os.path.join(GOLDEN, f"{name}.queries.npz"))
    for volume, key in ((False, "surface"), (True, "volume")):
        out = field.sample_batch(queries, volume=volume, cosine=not volume)
        r = compare_queries(out, g[key])
        assert r["ok_equal"] and r["id_equal"] and r["sample1d_equal"], (key, r)
        assert r["worst_pdf_rel"] <= TOL and r["worst_dir"] <= 1e-3, (key, r)
        print(key, r)


@pytest.mark.parametrize("dqt_args", [None, (0, 0, 0.01, 0.0, 12), (1, 1, 0.02, 0.5, 8)])
def test_quadtree_matches_oracle_on_fresh_seeds(pgl, dqt_args):
    import pyoracle
    from openpgl_gb300 import synthetic as syn

    frames = [syn.cube_face_samples(100000, 700 + i, volume_fraction=0.25) for i in range(3)]
    dev, field = _train(pgl, frames, 5000, dqt_args)
    orc = pyoracle.OracleField(5000, deterministic=True, threads=os.cpu_count() or 4, dqt=True, dqt_args=dqt_args)
    for f in frames:
        orc.update(f)
    _check(field.field_bytes(), orc.field_bytes())
    q = syn.queries(32768, 703)
    for volume in (False, True):
        r = compare_queries(field.sample_batch(q, volume=volume, cosine=not volume), orc.query(q, volume=volume,
                                                                                           cosine=not volume))
        assert r["ok_equal"] and r["id_equal"] and r["sample1d_equal"], (volume, r)
        assert r["worst_pdf_rel"] <= TOL and r["worst_dir"] <= 1e-3, (volume, r)


def test_quadtree_file_round_trip_and_per_object_api(pgl, tmp_path):
    """A quadtree field stored and read back (pglFieldStoreToFile /
    pglDeviceNewFieldFromFile) compares equal, answers the same queries and
    keeps training to the same field; per-object calls (Init, SamplePDF, PDF,
    IncomingRadiancePDF, no cosine product) give the batch's bits."""
    from openpgl_gb300 import synthetic as syn

    frames = [syn.cube_face_samples(60000, 720 + i, volume_fraction=0.25) for i in range(3)]
    dev, field = _train(pgl, frames[:2], 4000)
    path = tmp_path / "q.field"
    assert field.store(str(path))
    loaded = pgl.Field.from_file(dev, str(path))
    assert field.compare(loaded) and loaded.compare(field)
    assert loaded.field_bytes() == field.field_bytes()
    q = syn.queries(4096, 721)
    assert loaded.sample_batch(q).tobytes() == field.sample_batch(q).tobytes()
    for f in (field, loaded):
        st = pgl.SampleStorage()
        st.add_samples(frames[2])
        f.update(st)
    assert field.field_bytes() == loaded.field_bytes()
    out = field.sample_batch(q)
    ssd = pgl.SurfaceSamplingDistribution(field)
    n = 0
    for i in range(0, len(q), 64):
        ok, s1d = ssd.init(tuple(q["position"][i]), float(q["sample1d"][i]))
        assert ok == bool(out["ok"][i])
        if not ok:
            continue
        ssd.apply_cosine_product(tuple(q["normal"][i]))  # not supported: no effect
        d, pdf = ssd.sample_pdf(tuple(q["u"][i]))
        assert np.float32(pdf) == out["pdf"][i]
        assert np.array_equal(np.array(d, np.float32), out["dir"][i])
        assert np.float32(ssd.pdf(d)) == out["pdfLi"][i]
        assert np.float32(ssd.incoming_radiance_pdf(d)) == out["pdfLi"][i]
        n += 1
    assert n > 10
    ssd.release()


def test_quadtree_vertices_match_single_queries_and_oracle(pgl):
    """Path vertices on a quadtree field (four SamplePDF calls per Init): call
    k equals the oracle's single guided query with the k-th 2D random number
    and the GPU's own single-sample batch bit for bit."""
    import pyoracle
    from openpgl_gb300 import synthetic as syn

    frames = [syn.cluster_samples(1 << 18, 730 + i) for i in range(2)]
    dev, field = _train(pgl, frames, 8000)
    orc = pyoracle.OracleField(8000, deterministic=True, threads=os.cpu_count() or 4, dqt=True)
    for f in frames:
        orc.update(f)
    v = syn.vertices(1 << 15, 731)
    out = field.sample_vertices(v)
    assert out["ok"].sum() > len(v) // 2
    for k in range(4):
        q = syn.vertex_queries(v, k)
        got = np.zeros(len(v), dtype=pgl.QUERY_RESULT_DTYPE)
        got["ok"], got["id"], got["sample1d"] = out["ok"], out["id"], out["sample1d"]
        got["dir"], got["pdf"] = out["sample"][:, k, :3], out["sample"][:, k, 3]
        r = compare_queries(got, orc.query(q))
        assert r["ok_equal"] and r["id_equal"] and r["sample1d_equal"], (k, r)
        assert r["worst_pdf_rel"] <= TOL and r["worst_dir"] <= 1e-3, (k, r)
        one = field.sample_batch(q)
        ok = one["ok"] == 1
        assert np.array_equal(one["pdf"][ok].view(np.uint32), got["pdf"][ok].view(np.uint32)), k
        assert np.array_equal(one["dir"][ok].view(np.uint32), got["dir"][ok].view(np.uint32)), k
