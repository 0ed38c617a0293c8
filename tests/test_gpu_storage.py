"""Sample storage files and the compare entry points on the GPU library.

* pglNewSampleStorageFromFile reads the file the reference wrote
  (tests/golden/storage.samples.gz) and pglSampleStorageStoreToFile writes
  the same bytes back; a storage filled by pglSampleStorageAddSamples writes
  them too.
* pglSampleStorageCompare follows SampleDataStorage::operator==
  (SampleDataStorage.h:230-279): order-free (both sides sorted by
  SampleDataLess), member-wise float equality (+0 equals -0), and, as in the
  reference, only over the first storage's records (a storage equals one
  that holds more records after its own).
* pglFieldCompare (Field.h:552-601) is false for a field whose regions differ
  from another's in one region, true for a field and its copy read back from
  a file."""

import numpy as np
import pytest

from test_storage_file import expected_storage_bytes, golden_storage, storage_inputs

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pgl():
    import openpgl_gb300

    openpgl_gb300.load()
    return openpgl_gb300


def test_storage_file_round_trip(pgl, tmp_path):
    samples, meta = storage_inputs()
    golden = golden_storage()
    src = tmp_path / "ref.storage"
    src.write_bytes(golden)
    st = pgl.SampleStorage.from_file(str(src))
    assert (st.size_surface, st.size_volume) == (meta["surface"], meta["volume"])
    out = tmp_path / "gpu.storage"
    assert st.store(str(out))
    assert out.read_bytes() == golden
    mine = pgl.SampleStorage()
    mine.add_samples(samples)
    out2 = tmp_path / "gpu2.storage"
    assert mine.store(str(out2))
    assert out2.read_bytes() == golden == expected_storage_bytes(samples)
    assert st.compare(mine) and mine.compare(st)
    st.release()
    mine.release()


def test_storage_compare_semantics(pgl):
    samples, _ = storage_inputs()

    def storage(recs):
        s = pgl.SampleStorage()
        s.add_samples(np.ascontiguousarray(recs))
        return s

    a = storage(samples)
    shuffled = samples[np.random.default_rng(3).permutation(len(samples))]
    b = storage(shuffled)
    assert a.compare(b) and b.compare(a)
    changed = samples.copy()
    changed["weight"][17] = np.float32(changed["weight"][17]) * np.float32(1.5)
    c = storage(changed)
    assert not a.compare(c) and not c.compare(a)
    # +0 and -0 compare equal member by member
    z = samples.copy()
    z["direction"][5] = (0.0, 0.0, 1.0)
    zn = z.copy()
    zn["direction"][5] = (-0.0, 0.0, 1.0)
    assert storage(z).compare(storage(zn))
    # the reference compares over the first storage's records only: the
    # sorted prefix of a larger storage compares equal, the other way round too
    order = np.lexsort((samples["distance"], samples["pdf"], samples["weight"]))
    small = samples[order][: len(samples) // 2]
    d = storage(small)
    assert d.compare(a) and a.compare(d)
    for s in (a, b, c, d):
        s.release()


def _field(pgl, dev, samples, leaf=600):
    f = pgl.Field(dev, pgl.FieldConfig(True, leaf))
    st = pgl.SampleStorage()
    st.add_samples(samples)
    f.update(st)
    st.release()
    return f


def test_field_compare_detects_one_region(pgl, tmp_path):
    """Two fields trained on the same positions, one with the weight of one
    sample changed: same tree, one region's mixture differs, so the fields
    compare unequal; each compares equal to its copy from a field file."""
    from openpgl_gb300 import synthetic as syn

    import fieldfile

    s = syn.cube_face_samples(20000, 808)
    dev = pgl.Device()
    a = _field(pgl, dev, s)
    s2 = s.copy()
    s2["weight"][1234] = np.float32(s2["weight"][1234]) * np.float32(3.0)
    b = _field(pgl, dev, s2)
    fa = fieldfile.read_field_file(a.field_bytes())["surface"]
    fb = fieldfile.read_field_file(b.field_bytes())["surface"]
    ca, cb = fieldfile.canonical_tree(fa), fieldfile.canonical_tree(fb)
    assert np.array_equal(ca["dim"], cb["dim"]) and np.array_equal(ca["split"], cb["split"])
    differing = [i for i, (ra, rb) in enumerate(zip(fa["regions"], fb["regions"]))
                 if any(not np.array_equal(ra["vmm"][k], rb["vmm"][k]) for k in ("w", "kappa", "mx"))]
    assert len(differing) == 1, differing
    assert not a.compare(b) and not b.compare(a)
    path = tmp_path / "a.field"
    assert a.store(str(path))
    a2 = pgl.Field.from_file(dev, str(path))
    assert a.compare(a2) and a2.compare(a)
    for f in (a, b, a2):
        f.release()


def test_page_locked_records_are_read_in_place():
    """Records in page-locked host memory go to the device without a staging
    copy (the split kernels read them over the host link): the storage and
    the trained field equal those made from ordinary host memory."""
    import torch

    import openpgl_gb300 as pgl
    from openpgl_gb300 import synthetic as syn

    samples = syn.cube_face_samples(300000, 77, volume_fraction=0.3)
    pinned = torch.empty(samples.nbytes, dtype=torch.uint8, pin_memory=True)
    view = pinned.numpy().view(samples.dtype)
    view[:] = samples
    dev = pgl.Device()
    a, b = pgl.SampleStorage(), pgl.SampleStorage()
    a.add_samples(samples)
    b.add_samples(view)
    assert a.compare(b) and b.compare(a)
    assert a.size_surface == b.size_surface and a.size_volume == b.size_volume
    fa = pgl.Field(dev, pgl.FieldConfig(True, 8000))
    fb = pgl.Field(dev, pgl.FieldConfig(True, 8000))
    fa.update(a)
    fb.update(b)
    assert fa.field_bytes() == fb.field_bytes()


def test_page_locked_query_buffers_are_used_in_place():
    """Guided queries and path vertices whose buffers are page-locked host
    memory are read and written in place by the kernels: the same bytes as
    with ordinary host memory."""
    import torch

    import openpgl_gb300 as pgl
    from openpgl_gb300 import synthetic as syn

    dev = pgl.Device()
    field = pgl.Field(dev, pgl.FieldConfig(True, 8000))
    st = pgl.SampleStorage()
    st.add_samples(syn.cube_face_samples(200000, 81, volume_fraction=0.3))
    field.update(st)
    q = syn.queries(50000, 82)
    qp = torch.from_numpy(q.view(np.uint8)).pin_memory().numpy().view(q.dtype)
    rp = torch.empty(len(q) * 32, dtype=torch.uint8).pin_memory().numpy().view(pgl.QUERY_RESULT_DTYPE)
    for vol in (False, True):
        ref = field.sample_batch(q, volume=vol, cosine=not vol)
        field.sample_batch(qp, volume=vol, cosine=not vol, out=rp)
        assert rp.tobytes() == ref.tobytes()
    v = syn.vertices(30000, 83)
    vp = torch.from_numpy(v.view(np.uint8)).pin_memory().numpy().view(v.dtype)
    ref = field.sample_vertices(v)
    got = field.sample_vertices(vp)
    assert got.tobytes() == ref.tobytes()
