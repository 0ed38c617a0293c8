"""Failure detection without a GPU fault: the EM kernel's bounded wait, on a
flag that nothing sets, gives up after its limit and records an error that
the host reads; the context stays usable for the next Update."""

import time

import pytest

pytestmark = pytest.mark.gpu


def test_bounded_wait_runs_out_and_context_survives():
    import openpgl_gb300 as pgl
    from openpgl_gb300 import synthetic as syn

    pgl.load()
    t0 = time.perf_counter()
    code = pgl.bounded_wait_runs_out(50_000_000)  # 50 ms
    dt = time.perf_counter() - t0
    assert code == 2  # the slot wait ran out
    assert 0.05 <= dt < 10.0
    dev = pgl.Device()
    field = pgl.Field(dev, pgl.FieldConfig(deterministic=True, max_samples_per_leaf=4000))
    storage = pgl.SampleStorage()
    storage.add_samples(syn.cube_face_samples(20000, 7))
    field.update(storage)
    assert field.validate()
