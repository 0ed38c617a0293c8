"""EM schedule parameters change the Update's speed, never its result: fields
trained with other schedules (helper blocks per region, chunk size, pipeline
stages, queue order by measured cost) and a field whose Update was
autotuned are byte-identical to the field trained with the defaults."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pgl():
    import openpgl_gb300

    openpgl_gb300.load()
    return openpgl_gb300


def _frames():
    from openpgl_gb300 import synthetic as syn

    return [syn.cube_face_samples(131072, 400 + i, volume_fraction=0.25) for i in range(3)]


def _train(pgl, frames, tuning=None, autotune_at=None):
    dev = pgl.Device()
    field = pgl.Field(dev, pgl.FieldConfig(True, 4000))
    if tuning:
        field.set_em_tuning(**tuning)
    st = pgl.SampleStorage()
    for k, f in enumerate(frames):
        if autotune_at == k:
            field.autotune_next_update()
        st.add_samples(f)
        field.update(st)
        st.clear()
    return dev, field


def test_schedules_give_the_same_field(pgl):
    frames = _frames()
    _, ref = _train(pgl, frames)
    ref_bytes = ref.field_bytes()
    for tuning in (dict(max_helpers=0), dict(max_helpers=2, chunk_div=2), dict(max_helpers=16, stage_cap=2),
                   dict(max_helpers=8, chunk_div=4, order_by_cost=1)):
        _, f = _train(pgl, frames, tuning)
        assert f.em_tuning() == dict(dict(max_helpers=4, chunk_div=1, stage_cap=8, order_by_cost=0), **tuning)
        assert f.field_bytes() == ref_bytes, tuning


def test_autotuned_update_gives_the_same_field(pgl):
    frames = _frames()
    _, ref = _train(pgl, frames)
    _, tuned = _train(pgl, frames, autotune_at=1)
    assert tuned.field_bytes() == ref.field_bytes()
    trials = tuned.tuning_trials()
    # 3 helper counts x 2 chunk sizes, twice (by count, by measured cost)
    assert len(trials) == 12
    best = min(trials, key=lambda t: t["ms"])
    chosen = tuned.em_tuning()
    assert {k: best[k] for k in chosen} == chosen
    assert all(t["ms"] > 0.0 for t in trials)


def test_out_of_range_tuning_is_rejected(pgl):
    dev = pgl.Device()
    field = pgl.Field(dev, pgl.FieldConfig(True, 4000))
    for bad in (dict(max_helpers=-1), dict(chunk_div=0), dict(chunk_div=5), dict(stage_cap=1), dict(order_by_cost=2)):
        with pytest.raises(ValueError):
            field.set_em_tuning(**bad)
    assert field.em_tuning() == dict(max_helpers=4, chunk_div=1, stage_cap=8, order_by_cost=0)


def test_plain_launches_give_the_same_field(pgl):
    """The plain form (per Update and sub-field one EM launch with one block
    per region, no work queue or helpers) trains the same field as the
    batched launch."""
    frames = _frames()[:2]
    _, ref = _train(pgl, frames)
    dev = pgl.Device()
    field = pgl.Field(dev, pgl.FieldConfig(True, 4000))
    field.set_plain_update(True)
    st = pgl.SampleStorage()
    for f in frames:
        st.add_samples(f)
        field.update(st)
        st.clear()
    assert field.field_bytes() == ref.field_bytes()
