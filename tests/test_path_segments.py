"""Path segment storage (the reference's per-path sample producer,
PathSegmentDataStorage.h:161-385) in the library's host API against the
reference's own outputs (tests/golden/paths.npz, made by make_golden.py from
the compiled reference): the same samples, bit for bit, for all eight flag
sets, and the same pixel estimates.  Host code only: runs without a GPU."""

import hashlib
import json
import os

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
MANIFEST = json.load(open(os.path.join(GOLDEN, "manifest.json")))


@pytest.fixture(scope="module")
def pgl():
    import openpgl_gb300

    openpgl_gb300.load()
    return openpgl_gb300


@pytest.fixture(scope="module")
def paths():
    import sys

    sys.path.insert(0, GOLDEN)
    import make_golden

    case = MANIFEST["paths"]
    segs, begin = make_golden.build_paths(case)
    sha = lambda a: hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()
    assert sha(segs) == case["segments_sha256"] and sha(begin) == case["begin_sha256"]
    g = np.load(os.path.join(GOLDEN, "paths.npz"))
    return segs, begin, case, g


def test_host_storage_matches_reference(pgl, paths):
    segs, begin, case, g = paths
    st = pgl.PathSegmentStorage(reserve=int(np.diff(begin).max()) + 1)
    st.set_max_distance(case["max_distance"])
    assert st.max_distance() == np.float32(case["max_distance"])
    got_counts = np.zeros_like(g["counts"])
    got = []
    for fl in range(8):
        for p in range(len(begin) - 1):
            st.clear()
            st.add_segments(segs[int(begin[p]):int(begin[p + 1])])
            assert st.num_segments() == int(begin[p + 1] - begin[p])
            n = st.prepare_samples(bool(fl & 1), bool(fl & 2), bool(fl & 4))
            s = st.samples()
            assert n == len(s) == st.num_samples()
            got_counts[fl, p] = n
            got.append(s)
            if fl < 2:
                est = np.array(st.pixel_estimate(fl == 1), dtype=np.float32)
                assert est.tobytes() == g["pixel"][fl, p].tobytes(), (fl, p)
    assert np.array_equal(got_counts, g["counts"])
    assert np.concatenate(got).tobytes() == g["samples"].tobytes()
    st.release()


def test_validation(pgl, paths):
    segs, begin, case, g = paths
    st = pgl.PathSegmentStorage(reserve=32)
    st.set_max_distance(case["max_distance"])
    st.add_segments(segs[int(begin[3]):int(begin[4])])
    assert st.validate_segments()
    st.prepare_samples()
    assert st.validate_samples()
    bad = segs[int(begin[3]):int(begin[4])].copy()
    bad["roughness"][0] = 2.0
    st.clear()
    st.add_segments(bad)
    assert not st.validate_segments()
    st.release()


def test_storage_bounds(pgl, paths):
    """Segments beyond the reserved size are not stored (NextSegment returns
    null); samples beyond it are dropped."""
    segs, begin, case, g = paths
    st = pgl.PathSegmentStorage(reserve=3)
    with pytest.raises(RuntimeError):
        st.add_segments(segs[:4])
    assert st.num_segments() == 3
    st.release()
