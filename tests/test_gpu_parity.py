"""GPU parity: the GB300 library against the oracle (a bit-exact CPU
restatement of the reference, pinned by tests/test_oracle_golden.py) on
seeded inputs.

Bar (per the field's specification): kd-tree split planes, leaf sample counts
and sample-to-leaf assignment bit-exact; per leaf, the relative PDF error on a
fixed 64x64 direction grid at most 1e-3; guided queries choose the same region
and return the same pdf within 1e-3 relative (directions within 1e-3)."""

import os

import numpy as np
import pytest

from helpers import compare_fields, compare_queries, summary

pytestmark = pytest.mark.gpu

PDF_TOL = 1e-3


@pytest.fixture(scope="module")
def pgl():
    import openpgl_gb300

    openpgl_gb300.load()
    return openpgl_gb300


def _train(pgl, frames, leaf, deterministic=True):
    import pyoracle

    dev = pgl.Device()
    field = pgl.Field(dev, pgl.FieldConfig(deterministic=deterministic, max_samples_per_leaf=leaf))
    storage = pgl.SampleStorage()
    orc = pyoracle.OracleField(leaf, deterministic=deterministic, threads=os.cpu_count() or 8)
    for f in frames:
        storage.add_samples(f)
        field.update(storage)
        storage.clear()
        orc.update(f)
    return dev, field, orc


def _check_field(field, orc, side="surface"):
    """The bar on every leaf: tree, numbering and sample statistics equal, no
    leaf above PDF_TOL (the message names the leaves and their lobe counts)."""
    r = compare_fields(field.field_bytes(), orc.field_bytes(), side, tol=PDF_TOL)
    s = summary(r)
    assert r["tree_equal"], (side, s)
    assert r["numbering_equal"], (side, s)
    if r["regions"]:
        assert r["stats_equal"], (side, s)
        assert not r["over_tol"] and r["worst_pdf_rel"] <= PDF_TOL, (side, s)
    print(side, "regions", r["regions"], "bit-exact", r.get("bit_exact_regions"), "K flips", r.get("k_flips"),
          "worst pdf rel %.2e" % r.get("worst_pdf_rel", 0.0))
    return r


def _check_queries(out, ref, what=""):
    r = compare_queries(out, ref)
    assert r["ok_equal"] and r["id_equal"] and r["sample1d_equal"], (what, r)
    assert r["worst_pdf_rel"] <= PDF_TOL and r["worst_dir"] <= 1e-3, (what, r)
    return r


@pytest.mark.parametrize("n,leaf", [(262144, 32000), (131072, 4000), (1048576, 16000)])
def test_first_build_matches_oracle(pgl, n, leaf):
    from openpgl_gb300 import synthetic as syn

    dev, field, orc = _train(pgl, [syn.cube_face_samples(n, 21)], leaf)
    _check_field(field, orc)


def test_single_update_configuration(pgl):
    """The single-Update configuration at its full size: 1,048,576 cube-face
    samples, maxSamplesPerLeaf 32000, one Update, then 1,048,576 guided queries
    (cosine product, one SamplePDF each)."""
    from openpgl_gb300 import synthetic as syn

    dev, field, orc = _train(pgl, [syn.cube_face_samples(1 << 20, 1001)], 32000)
    _check_field(field, orc)
    q = syn.queries(1 << 20, 1002)
    r = _check_queries(field.sample_batch(q), orc.query(q), "1M queries")
    print(r)


def test_leaf_log_likelihood_matches_oracle(pgl):
    """Per region, the weighted log-likelihood of its reprojected samples under
    the GPU's mixture against the same under the oracle's mixture (both
    evaluated in FP64): within 1e-4 relative."""
    from helpers import leaf_log_likelihoods
    from openpgl_gb300 import synthetic as syn

    frame = syn.cube_face_samples(262144, 23)
    dev, field, orc = _train(pgl, [frame], 8000)
    a = leaf_log_likelihoods(field.field_bytes(), frame)
    b = leaf_log_likelihoods(orc.field_bytes(), frame)
    assert a.keys() == b.keys() and len(a) > 10
    # relative to the LL's scale (sum of |w log pdf|; the LL itself can be near 0)
    rel = [abs(a[r][0] - b[r][0]) / max(b[r][1], 1e-30) for r in b]
    assert max(rel) <= 1e-4, sorted(rel)[-5:]


def test_multiframe_surface_and_volume(pgl):
    from openpgl_gb300 import synthetic as syn

    frames = [syn.cube_face_samples(131072, 30 + i, volume_fraction=0.25) for i in range(3)]
    dev, field, orc = _train(pgl, frames, 4000)
    for side in ("surface", "volume"):
        _check_field(field, orc, side)


def test_clustered_update(pgl):
    from openpgl_gb300 import synthetic as syn

    frames = [syn.cluster_samples(200000, 40 + i, num_clusters=256) for i in range(2)]
    dev, field, orc = _train(pgl, frames, 2000)
    _check_field(field, orc)


def test_clustered_many_leaves(pgl):
    """The clustered distribution at 4096 clusters (Zipf masses, 1-6 lobes,
    near-delta lobes), 2,097,152 samples in two frames at maxSamplesPerLeaf
    16000 (leaves from a few hundred to 16000 samples), then queries drawn
    from the clusters."""
    from openpgl_gb300 import synthetic as syn

    frames = [syn.cluster_samples(1 << 20, 140 + i, volume_fraction=0.25) for i in range(2)]
    dev, field, orc = _train(pgl, frames, 16000)
    for side in ("surface", "volume"):
        _check_field(field, orc, side)
    q = syn.queries(1 << 18, 142, model_seed=1234)
    for volume in (False, True):
        _check_queries(field.sample_batch(q, volume=volume, cosine=not volume),
                       orc.query(q, volume=volume, cosine=not volume), f"volume={volume}")


def test_guided_queries_match_oracle(pgl):
    from openpgl_gb300 import synthetic as syn

    dev, field, orc = _train(pgl, [syn.cube_face_samples(262144, 50)], 8000)
    q = syn.queries(8192, 51)
    _check_queries(field.sample_batch(q), orc.query(q))


def test_poisoned_samples_flag_the_oracles_regions(pgl):
    """Samples with NaN directions or weights, infinite distances and zero
    weights in the second frame: the Update completes, the tree and the sample
    statistics are the oracle's, the same regions are flagged invalid (the
    oracle flags the reference's, tests/test_oracle_golden.py), and guided
    queries agree."""
    import fieldfile
    from helpers import poisoned_frames
    from openpgl_gb300 import synthetic as syn

    dev, field, orc = _train(pgl, poisoned_frames(), 3000)
    a, b = field.field_bytes(), orc.field_bytes()
    invalid = 0
    for side in ("surface", "volume"):
        r = compare_fields(a, b, side)
        assert r["tree_equal"] and r["stats_equal"], (side, r)
        va = [x["valid"] for x in fieldfile.read_field_file(a)[side]["regions"]]
        vb = [x["valid"] for x in fieldfile.read_field_file(b)[side]["regions"]]
        assert va == vb, side
        invalid += vb.count(False)
    assert invalid > 0
    q = syn.queries(2048, 993)
    for volume in (False, True):
        _check_queries(field.sample_batch(q, volume=volume, cosine=not volume),
                       orc.query(q, volume=volume, cosine=not volume), f"volume={volume}")


def test_per_object_api_matches_batch(pgl):
    from openpgl_gb300 import synthetic as syn

    dev, field, orc = _train(pgl, [syn.cube_face_samples(65536, 60)], 8000)
    q = syn.queries(64, 61)
    out = field.sample_batch(q)
    ssd = pgl.SurfaceSamplingDistribution(field)
    for i in range(len(q)):
        ok, s1d = ssd.init(tuple(q["position"][i]), float(q["sample1d"][i]))
        assert ok == bool(out["ok"][i])
        if not ok:
            continue
        ssd.apply_cosine_product(tuple(q["normal"][i]))
        d, pdf = ssd.sample_pdf(tuple(q["u"][i]))
        assert np.float32(pdf) == out["pdf"][i]
        assert np.array_equal(np.array(d, np.float32), out["dir"][i])
        assert ssd.get_id() == out["id"][i]
        assert np.float32(ssd.incoming_radiance_pdf(d)) == out["pdfLi"][i]
    ssd.release()


def test_field_compare_and_determinism(pgl):
    from openpgl_gb300 import synthetic as syn

    s = syn.cube_face_samples(100000, 70)
    dev = pgl.Device()
    fields = []
    for _ in range(2):
        f = pgl.Field(dev, pgl.FieldConfig(True, 6000))
        st = pgl.SampleStorage()
        st.add_samples(s)
        f.update(st)
        fields.append(f)
    assert fields[0].compare(fields[1])
    assert fields[0].field_bytes() == fields[1].field_bytes()


def test_one_leaf_fields(pgl):
    """Fields whose root never splits (one surface and one volume region over
    several frames): the region's sample statistics, bounds included, and its
    mixture match the oracle bit for bit."""
    from openpgl_gb300 import synthetic as syn

    frames = [syn.cube_face_samples(50000, 90 + i, volume_fraction=0.25) for i in range(3)]
    dev, field, orc = _train(pgl, frames, 1000000)
    for side in ("surface", "volume"):
        r = compare_fields(field.field_bytes(), orc.field_bytes(), side)
        assert r["regions"] == 1, (side, r)
        assert r["tree_equal"] and r["stats_equal"], (side, r)
        assert r["bit_exact_regions"] == 1, (side, r)


def test_hg_product_matches_oracle_and_per_object(pgl, tmp_path):
    """Volume queries with the single-lobe Henyey-Greenstein product on the
    oracle's own field (loaded from its field file, so the regions are the
    same bits and only the query arithmetic is compared): the batch against
    the oracle (same region and sample1D, pdfs within 1e-3), and the
    per-object calls (Init, ApplySingleLobeHenyeyGreensteinProduct, SamplePDF,
    PDF, IncomingRadiancePDF) against the batch bit for bit.  The fields the
    GPU trains itself are checked with the product against the reference's
    golden outputs in test_gpu_golden.py."""
    import pyoracle
    from openpgl_gb300 import synthetic as syn

    orc = pyoracle.OracleField(4000, deterministic=True, threads=8)
    for i in range(2):
        orc.update(syn.cube_face_samples(131072, 70 + i, volume_fraction=0.5))
    path = tmp_path / "oracle.field"
    path.write_bytes(orc.field_bytes())
    dev = pgl.Device()
    field = pgl.Field.from_file(dev, str(path))
    q = syn.queries(8192, 71)
    g = pyoracle.hg_mean_cosines(len(q))
    out = field.sample_batch_hg(q, g)
    ref = orc.query_hg(q, g)
    assert np.array_equal(out["ok"], ref["ok"])
    ok = ref["ok"] == 1
    assert ok.sum() > 1000
    assert np.array_equal(out["id"][ok], ref["id"][ok])
    assert np.array_equal(out["sample1d"][ok].view(np.uint32), ref["sample1d"][ok].view(np.uint32))
    rel = np.abs(out["pdf"][ok] - ref["pdf"][ok]) / ref["pdf"][ok]
    assert rel.max() <= PDF_TOL, np.quantile(rel, [0.5, 0.99, 0.999, 1.0])
    relli = np.abs(out["pdfLi"][ok] - ref["pdfLi"][ok]) / ref["pdfLi"][ok]
    assert relli.max() <= PDF_TOL
    assert np.abs(out["dir"][ok] - ref["dir"][ok]).max() <= 1e-3
    vsd = pgl.VolumeSamplingDistribution(field)
    assert vsd.supports_hg_product()
    for i in range(0, len(q), 128):
        ok_i, s1d = vsd.init(tuple(q["position"][i]), float(q["sample1d"][i]))
        assert ok_i == bool(out["ok"][i])
        if not ok_i:
            continue
        vsd.apply_hg_product(tuple(q["normal"][i]), float(g[i]))
        d, pdf = vsd.sample_pdf(tuple(q["u"][i]))
        assert np.float32(pdf) == out["pdf"][i]
        assert np.array_equal(np.array(d, np.float32), out["dir"][i])
        assert np.float32(vsd.pdf(d)) == out["pdf"][i]
        assert np.float32(vsd.incoming_radiance_pdf(d)) == out["pdfLi"][i]
    vsd.release()


def test_multiframe_configuration(pgl):
    """The multi-frame configuration the bench times, at its full size: 8
    frames of 2,097,152 samples (25 % inside-volume), maxSamplesPerLeaf
    32000, the storage cleared after every Update; then 1,048,576 guided
    queries.  Every leaf of both sub-fields within the bar (in fact every
    mixture bit-exact) and every query within it."""
    from openpgl_gb300 import synthetic as syn

    frames = [syn.cube_face_samples(2097152, 9000 + f, volume_fraction=0.25) for f in range(8)]
    dev, field, orc = _train(pgl, frames, 32000)
    for side in ("surface", "volume"):
        r = _check_field(field, orc, side)
        assert r["bit_exact_regions"] == r["regions"], (side, summary(r))
    q = syn.queries(1 << 20, 4242)
    _check_queries(field.sample_batch(q), orc.query(q), "1M queries")


def test_path_vertex_queries(pgl):
    """Path-vertex queries (Init, cosine product, four SamplePDF calls on the
    clustered field, vertices from the clusters): SamplePDF call k equals the
    oracle's single guided query with the k-th 2D random number (sampling
    does not change the distribution), region and sample1D bit for bit,
    pdfs within the bar."""
    from openpgl_gb300 import synthetic as syn

    frames = [syn.cluster_samples(1 << 19, 160 + i) for i in range(2)]
    dev, field, orc = _train(pgl, frames, 8000)
    v = syn.vertices(1 << 16, 161)
    out = field.sample_vertices(v)
    assert out["ok"].sum() > len(v) // 2
    for k in range(4):
        q = syn.vertex_queries(v, k)
        ref = orc.query(q)
        got = np.zeros(len(v), dtype=pgl.QUERY_RESULT_DTYPE)
        got["ok"], got["id"], got["sample1d"] = out["ok"], out["id"], out["sample1d"]
        got["dir"], got["pdf"] = out["sample"][:, k, :3], out["sample"][:, k, 3]
        r = compare_queries(got, ref)
        assert r["ok_equal"] and r["id_equal"] and r["sample1d_equal"], (k, r)
        assert r["worst_pdf_rel"] <= PDF_TOL and r["worst_dir"] <= 1e-3, (k, r)
        # and the batch with one sample per query, on the GPU, bit for bit
        one = field.sample_batch(q)
        ok = one["ok"] == 1
        assert np.array_equal(one["pdf"][ok].view(np.uint32), got["pdf"][ok].view(np.uint32)), k
        assert np.array_equal(one["dir"][ok].view(np.uint32), got["dir"][ok].view(np.uint32)), k


@pytest.mark.parametrize("sizes", [(1, 2, 7, 100, 50000), (0, 40000, 0, 3, 40000)])
def test_tiny_and_empty_frames(pgl, sizes):
    """Frames of a handful of samples, and empty frames, between ordinary
    ones (the first Update may see a single sample: the scene bounds skip the
    last sample, so a one-sample first frame leaves them degenerate): tree,
    sample statistics, mixtures and queries as the oracle's after every
    frame."""
    from openpgl_gb300 import synthetic as syn

    frames = [syn.cube_face_samples(n, 400 + i, volume_fraction=0.3) if n else
              np.zeros(0, dtype=syn.cube_face_samples(1, 0).dtype) for i, n in enumerate(sizes)]
    import pyoracle

    dev = pgl.Device()
    field = pgl.Field(dev, pgl.FieldConfig(True, 4000))
    storage = pgl.SampleStorage()
    orc = pyoracle.OracleField(4000, deterministic=True, threads=os.cpu_count() or 8)
    q = syn.queries(4096, 499)
    for f in frames:
        if len(f):
            storage.add_samples(f)
        field.update(storage)
        storage.clear()
        orc.update(f)
        assert field.iteration == orc.iteration
        for side in ("surface", "volume"):
            _check_field(field, orc, side)
        for vol in (False, True):
            _check_queries(field.sample_batch(q, volume=vol, cosine=not vol), orc.query(q, volume=vol, cosine=not vol),
                           f"after {len(f)} samples")


def test_explicit_scene_bounds_and_outside_queries(pgl):
    """Scene bounds set before the first Update (pglFieldSetSceneBounds) give
    the oracle's tree and regions; queries outside the bounds fail their
    Init, and a negative sample1D takes the leaf's own region (no stochastic
    neighbour choice), as in the oracle."""
    import pyoracle
    from openpgl_gb300 import synthetic as syn

    lo, hi = (-0.5, -0.25, -1.0), (1.5, 1.25, 2.0)
    dev = pgl.Device()
    field = pgl.Field(dev, pgl.FieldConfig(True, 4000))
    field.set_scene_bounds(lo, hi)
    orc = pyoracle.OracleField(4000, deterministic=True, threads=os.cpu_count() or 8)
    orc.set_scene_bounds(lo, hi)
    storage = pgl.SampleStorage()
    for i in range(2):
        f = syn.cube_face_samples(60000, 410 + i, volume_fraction=0.25)
        storage.add_samples(f)
        field.update(storage)
        storage.clear()
        orc.update(f)
    for side in ("surface", "volume"):
        _check_field(field, orc, side)
    q = syn.queries(8192, 420)
    q["position"][:1024] += np.float32(5.0)  # outside the scene bounds
    q["sample1d"][1024:2048] = np.float32(-1.0)  # no neighbour choice
    for vol in (False, True):
        out = field.sample_batch(q, volume=vol, cosine=not vol)
        _check_queries(out, orc.query(q, volume=vol, cosine=not vol), f"volume={vol}")
        assert not out["ok"][:1024].any()
