"""The oracle (CPU restatement of the reference's field path, oracle/) against
golden outputs of the reference library itself (tests/golden, made by
tests/golden/make_golden.py from the compiled reference sources).  Bit-exact:
the same field file (tree, regions, mixtures, statistics) and the same guided
query results.  CPU only."""

import gzip
import hashlib
import json
import os

import numpy as np
import pytest

import fieldfile
import pyoracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
MANIFEST = json.load(open(os.path.join(GOLDEN, "manifest.json")))
CASES = sorted(MANIFEST["cases"])


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def inputs(name):
    import make_golden

    case = MANIFEST["cases"][name]
    return make_golden.build_inputs(case), case


@pytest.fixture(scope="module", autouse=True)
def _golden_path():
    import sys

    sys.path.insert(0, GOLDEN)
    yield


def oracle_for(case):
    return pyoracle.OracleField(case["leaf"], deterministic=True, threads=4, parallax=case.get("parallax", True),
                                dqt=case.get("dqt", False), dqt_args=case.get("dqt_args"))


def golden(name):
    field = gzip.open(os.path.join(GOLDEN, f"{name}.field.gz")).read()
    q = np.load(os.path.join(GOLDEN, f"{name}.queries.npz"))
    return field, q["surface"], q["volume"]


@pytest.mark.parametrize("name", CASES)
def test_generators_reproduce_golden_inputs(name):
    (frames, queries), case = inputs(name)
    assert [sha(f) for f in frames] == case["frame_sha256"]
    assert sha(queries) == case["queries_sha256"]


@pytest.mark.parametrize("name", CASES)
def test_oracle_field_is_the_reference_field(name):
    (frames, queries), case = inputs(name)
    orc = oracle_for(case)
    for f in frames:
        orc.update(f)
    mine = fieldfile.strip_timings(orc.field_bytes())
    ref, _, _ = golden(name)
    assert hashlib.sha256(ref).hexdigest() == case["field_sha256"]
    assert mine == ref


@pytest.mark.parametrize("name", CASES)
def test_oracle_queries_are_the_reference_queries(name):
    (frames, queries), case = inputs(name)
    orc = oracle_for(case)
    for f in frames:
        orc.update(f)
    _, rs, rv = golden(name)
    s = orc.query(queries, volume=False, cosine=True)
    v = orc.query(queries, volume=True, cosine=False)
    assert s.tobytes() == rs.tobytes()
    assert v.tobytes() == rv.tobytes()


@pytest.mark.parametrize("name", CASES)
def test_oracle_hg_queries_are_the_reference_queries(name):
    """Volume queries with the single-lobe Henyey-Greenstein product
    (VMMVolumeSamplingDistribution.h:54-80) over mean cosines -0.99 .. 0.99."""
    (frames, queries), case = inputs(name)
    orc = oracle_for(case)
    for f in frames:
        orc.update(f)
    rh = np.load(os.path.join(GOLDEN, f"{name}.queries.npz"))["volume_hg"]
    h = orc.query_hg(queries, pyoracle.hg_mean_cosines(len(queries)))
    assert h.tobytes() == rh.tobytes()


def test_golden_field_structure():
    """The parsed reference file is self-consistent: leaves index regions,
    every region's sample statistics count matches the leaf histogram of its
    frame, and the canonical tree has one leaf per region."""
    ref, _, _ = golden("cube_single")
    f = fieldfile.read_field_file(ref)["surface"]
    canon = fieldfile.canonical_tree(f)
    assert canon["leaf"].sum() == len(f["regions"])
    assert sorted(canon["region"].tolist()) == list(range(len(f["regions"])))
    (frames, _), _ = inputs("cube_single")
    pos = np.stack([frames[0]["position"][:, i] for i in range(3)], axis=1)
    leaf = fieldfile.leaf_of_positions(f, pos)
    hist = np.bincount(leaf, minlength=len(f["regions"]))
    n = np.array([r["stats"]["n"] for r in f["regions"]])
    assert np.array_equal(hist.astype(np.float32), n)


@pytest.mark.skipif(not pyoracle.reference_available(), reason="reference library not built here")
def test_oracle_matches_live_reference_on_fresh_seed():
    from openpgl_gb300 import synthetic as syn

    frames = [syn.cube_face_samples(20000, 777 + i, volume_fraction=0.3) for i in range(2)]
    q = syn.queries(1024, 779)
    field, _, rs, rv, rh = pyoracle.run_reference(frames, q, max_samples_per_leaf=3000)
    orc = pyoracle.OracleField(3000, deterministic=True, threads=2)
    for f in frames:
        orc.update(f)
    assert fieldfile.strip_timings(orc.field_bytes()) == fieldfile.strip_timings(field)
    assert orc.query(q).tobytes() == rs.tobytes()
    assert orc.query(q, volume=True, cosine=False).tobytes() == rv.tobytes()
    assert orc.query_hg(q, pyoracle.hg_mean_cosines(len(q))).tobytes() == rh.tobytes()


@pytest.mark.skipif(not pyoracle.reference_available(), reason="reference library not built here")
@pytest.mark.parametrize("dqt_args", [None, (0, 0, 0.01, 0.0, 12), (1, 0, 0.01, 1.0, 12), (0, 1, 0.01, 1.0, 12),
                                      (1, 1, 0.02, 0.5, 8), (0, 0, 0.003, 2.0, 6)])
def test_oracle_quadtree_matches_live_reference_on_fresh_seed(dqt_args):
    """The directional quadtree field type (DQTFactory.h, DQT.h) on a fresh
    seed, at the default factory arguments and each branch of the factory's
    dispatch (leaf estimator x split metric x zero / non-zero footprint,
    DQTFactory.h:168-185): the same field file and the same query results."""
    from openpgl_gb300 import synthetic as syn

    frames = [syn.cube_face_samples(16000, 881 + i, volume_fraction=0.3) for i in range(3)]
    q = syn.queries(1024, 884)
    field, _, rs, rv, rh = pyoracle.run_reference(frames, q, max_samples_per_leaf=2500, dqt=True, dqt_args=dqt_args)
    orc = pyoracle.OracleField(2500, deterministic=True, threads=2, dqt=True, dqt_args=dqt_args)
    for f in frames:
        orc.update(f)
    assert fieldfile.strip_timings(orc.field_bytes()) == fieldfile.strip_timings(field)
    assert orc.query(q).tobytes() == rs.tobytes()
    assert orc.query(q, volume=True, cosine=False).tobytes() == rv.tobytes()
    assert orc.query_hg(q, pyoracle.hg_mean_cosines(len(q))).tobytes() == rh.tobytes()


def region_flags(field_bytes, side):
    f = fieldfile.read_field_file(field_bytes)[side]
    return np.array([r["valid"] for r in f["regions"]]), fieldfile.canonical_tree(f)


@pytest.mark.skipif(not pyoracle.reference_available(), reason="reference library not built here")
@pytest.mark.parametrize("dqt", [False, True])
def test_oracle_poisoned_samples_like_reference(dqt):
    """Poisoned samples (NaN direction or weight, infinite distance, zero
    weight) invalidate the same regions in the oracle as in the reference, and
    guided queries give the same results.  For quadtrees the whole field file is
    identical.  For VMMs the invalidated regions' mixtures are not compared:
    the reference's 8-wide SIMD EM and the oracle's lane loop carry NaNs
    through different lanes, so those regions' bytes differ while the tree,
    the sample statistics, the validity flags and every query agree."""
    from openpgl_gb300 import synthetic as syn

    from helpers import poisoned_frames

    frames = poisoned_frames()
    q = syn.queries(2048, 993)
    field, _, rs, rv, _ = pyoracle.run_reference(frames, q, max_samples_per_leaf=3000, dqt=dqt)
    orc = pyoracle.OracleField(3000, deterministic=True, threads=2, dqt=dqt)
    for f in frames:
        orc.update(f)
    mine = fieldfile.strip_timings(orc.field_bytes())
    ref = fieldfile.strip_timings(field)
    if dqt:
        assert mine == ref
    invalid = 0
    for side in ("surface", "volume"):
        va, ca = region_flags(mine, side)
        vb, cb = region_flags(ref, side)
        assert np.array_equal(ca["dim"], cb["dim"]) and np.array_equal(ca["split"], cb["split"])
        assert np.array_equal(va, vb)
        invalid += int((~va).sum())
        A = fieldfile.read_field_file(mine)[side]["regions"]
        B = fieldfile.read_field_file(ref)[side]["regions"]
        for ra, rb in zip(A, B):
            for key in ("mean", "var", "bounds"):
                assert ra["stats"][key].tobytes() == rb["stats"][key].tobytes()
    assert invalid > 0 or dqt  # the poison reached at least one VMM region
    assert orc.query(q).tobytes() == rs.tobytes()
    assert orc.query(q, volume=True, cosine=False).tobytes() == rv.tobytes()
