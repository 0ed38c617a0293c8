"""Path segments -> samples on the device (pglPathSegmentsPrepareSamplesDevice,
...PropagateSamplesDevice) against the reference's golden outputs, bit for
bit: the same samples in the same order (path by path, each path's in the
reference's order) for all eight flag sets; and propagation into a sample
storage that an Update then trains on."""

import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")


@pytest.fixture(scope="module")
def pgl():
    import openpgl_gb300

    openpgl_gb300.load()
    return openpgl_gb300


def _paths():
    import sys

    sys.path.insert(0, GOLDEN)
    import make_golden

    case = json.load(open(os.path.join(GOLDEN, "manifest.json")))["paths"]
    segs, begin = make_golden.build_paths(case)
    return segs, begin, case, np.load(os.path.join(GOLDEN, "paths.npz"))


def test_device_path_samples_match_reference(pgl):
    import torch

    segs, begin, case, g = _paths()
    num_paths = len(begin) - 1
    d_segs = torch.from_numpy(segs.view(np.uint8)).cuda()
    d_begin = torch.from_numpy(begin.astype(np.uint32).view(np.int32)).cuda()
    d_out = torch.zeros(len(segs) * 40, dtype=torch.uint8, device="cuda")
    d_off = torch.zeros(num_paths + 1, dtype=torch.int32, device="cuda")
    from openpgl_gb300.synthetic import PGL_SAMPLE_DTYPE

    got = []
    for fl in range(8):
        pgl.path_samples_device(d_segs.data_ptr(), d_begin.data_ptr(), num_paths, case["max_distance"],
                                d_out.data_ptr(), d_off.data_ptr(), bool(fl & 1), bool(fl & 2), bool(fl & 4))
        torch.cuda.synchronize()
        off = d_off.cpu().numpy().view(np.uint32)
        assert np.array_equal(np.diff(off), g["counts"][fl]), fl
        got.append(d_out.cpu().numpy()[:int(off[-1]) * 40].view(PGL_SAMPLE_DTYPE))
    assert np.concatenate(got).tobytes() == g["samples"].tobytes()


def test_host_and_device_propagation_train_the_same_field(pgl):
    """Per-path PropagateSamples (host) and the device batch fill two sample
    storages with the same samples; Updates on them give the same field."""
    import torch

    from openpgl_gb300 import synthetic as syn

    segs, begin = syn.path_segments(20000, 17)
    num_paths = len(begin) - 1
    dev = pgl.Device()
    host_storage, dev_storage = pgl.SampleStorage(), pgl.SampleStorage()
    st = pgl.PathSegmentStorage(reserve=16)
    st.set_max_distance(3.0)
    for p in range(num_paths):
        st.add_segments(segs[int(begin[p]):int(begin[p + 1])])
        st.propagate(host_storage)
    d_segs = torch.from_numpy(segs.view(np.uint8)).cuda()
    d_begin = torch.from_numpy(begin.astype(np.uint32).view(np.int32)).cuda()
    n = pgl.load().pglPathSegmentsPropagateSamplesDevice(d_segs.data_ptr(), d_begin.data_ptr(), num_paths, 3.0,
                                                         dev_storage.h, False, False, True)
    assert n > 10000
    fields = []
    for storage in (host_storage, dev_storage):
        f = pgl.Field(dev, pgl.FieldConfig(True, 2000))
        f.update(storage)
        fields.append(f.field_bytes())
    assert fields[0] == fields[1]
