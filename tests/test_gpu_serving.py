"""The guiding server (continuous batching over a double-buffered field): each
request's results equal the same queries answered alone, whatever else is in
flight; requests larger than one launch are split and reassembled; while an
Update runs in the background, every request is answered from one field state,
the one its reported version names."""

import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _trained(pgl, syn, seed, frames=1):
    dev = pgl.Device()
    f = pgl.Field(dev, pgl.FieldConfig(True, 4000))
    st = pgl.SampleStorage()
    for k in range(frames):
        st.add_samples(syn.cube_face_samples(60000, seed + k, volume_fraction=0.25))
        f.update(st)
        st.clear()
    return dev, f


def test_results_alone_equal_results_in_the_mix():
    import openpgl_gb300 as pgl
    from openpgl_gb300 import synthetic as syn

    dev, field = _trained(pgl, syn, 5000)
    rng = np.random.default_rng(7)
    sizes = np.exp(rng.uniform(np.log(50), np.log(40000), size=24)).astype(int)
    batches = [(syn.queries(int(n), 6000 + i), bool(i % 3 == 2)) for i, n in enumerate(sizes)]
    alone = [field.sample_batch(q, volume=vol, cosine=not vol) for q, vol in batches]

    server = pgl.GuidingServer(field, hbm_budget_bytes=1 << 20)  # ~15k queries per launch
    results = [None] * len(batches)

    def worker(idx):
        for i in idx:
            q, vol = batches[i]
            t, out = server.submit(q, volume=vol, cosine=not vol)
            lat, ver = server.wait(t)
            results[i] = (out, lat, ver)

    threads = [threading.Thread(target=worker, args=(list(range(k, len(batches), 4)),)) for k in range(4)]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    for i, (out, lat, ver) in enumerate(results):
        assert out.tobytes() == alone[i].tobytes(), i
        assert ver == field.iteration
        assert lat > 0.0
    s = server.stats()
    assert s["queries"] == sizes.sum() and s["requests"] == len(batches)
    assert s["launches"] < len(batches) + sizes.sum() // 15000 + 2
    server.release()


def test_queries_during_background_update_come_from_one_field_state():
    import openpgl_gb300 as pgl
    from openpgl_gb300 import synthetic as syn

    dev, field = _trained(pgl, syn, 5100)
    _, after = _trained(pgl, syn, 5100, frames=2)  # the same training plus the next frame
    q = syn.queries(20000, 5200)
    expect = {field.iteration: field.sample_batch(q), after.iteration: after.sample_batch(q)}
    assert field.iteration + 1 == after.iteration

    server = pgl.GuidingServer(field, hbm_budget_bytes=1 << 22)
    server.add_samples(syn.cube_face_samples(60000, 5101, volume_fraction=0.25))
    ticket = server.update()
    seen = set()
    for _ in range(12):
        t, out = server.submit(q)
        _, ver = server.wait(t)
        assert ver in expect
        assert out.tobytes() == expect[ver].tobytes()
        seen.add(ver)
    server.wait_update(ticket)
    t, out = server.submit(q)
    _, ver = server.wait(t)
    assert ver == after.iteration and out.tobytes() == expect[ver].tobytes()
    assert server.stats()["updates"] == 1
    server.release()
    assert field.compare(after)
