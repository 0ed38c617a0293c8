"""The guiding server (continuous batching over a double-buffered field): each
request's results equal the same queries answered alone, whatever else is in
flight; requests larger than one launch are split and reassembled; while an
Update runs in the background, every request is answered from one field state,
the one its reported version names."""

import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _trained(pgl, syn, seed, frames=1, dqt=False):
    dev = pgl.Device()
    f = pgl.Field(dev, pgl.FieldConfig(True, 4000, dqt=dqt))
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

    # a budget that leaves a few thousand queries per launch (the field's own
    # memory, its two snapshots and two launches' buffers all count)
    server = pgl.GuidingServer(field, hbm_budget_bytes=64 << 20)
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
    cap = int(s["launch_capacity"])
    assert cap >= 1024, cap
    assert s["launches"] < len(batches) + sizes.sum() // cap + 2
    assert s["device_bytes"] <= s["budget_bytes"]
    server.release()


@pytest.mark.parametrize("dqt", [False, True])
def test_queries_during_background_update_come_from_one_field_state(dqt):
    """Queries served while the field trains in the background come from one
    field state each (before or after the Update), for mixture fields and for
    directional quadtree fields."""
    import openpgl_gb300 as pgl
    from openpgl_gb300 import synthetic as syn

    dev, field = _trained(pgl, syn, 5100, dqt=dqt)
    _, after = _trained(pgl, syn, 5100, frames=2, dqt=dqt)  # the same training plus the next frame
    q = syn.queries(20000, 5200)
    expect = {field.iteration: field.sample_batch(q), after.iteration: after.sample_batch(q)}
    assert field.iteration + 1 == after.iteration

    server = pgl.GuidingServer(field, hbm_budget_bytes=256 << 20)
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


def test_vertices_in_the_mix_and_the_budget():
    """Path-vertex requests (four SamplePDF calls per vertex) served beside
    single-sample requests give the same bytes as the direct call; a training
    batch whose Update would not fit in the budget is refused, and the
    server's device memory stays within the budget."""
    import openpgl_gb300 as pgl
    from openpgl_gb300 import synthetic as syn

    dev, field = _trained(pgl, syn, 5300)
    verts = [syn.vertices(int(n), 5400 + i) for i, n in enumerate((3000, 70000, 20000))]
    qs = [syn.queries(int(n), 5500 + i) for i, n in enumerate((5000, 90000))]
    alone_v = [field.sample_vertices(v) for v in verts]
    alone_q = [field.sample_batch(q) for q in qs]
    server = pgl.GuidingServer(field, hbm_budget_bytes=96 << 20)
    tickets = []
    for i in range(3):
        tickets.append(("v", i) + server.submit_vertices(verts[i]))
        if i < 2:
            tickets.append(("q", i) + server.submit(qs[i]))
    for kind, i, t, out in tickets:
        server.wait(t)
        ref = alone_v[i] if kind == "v" else alone_q[i]
        assert out.tobytes() == ref.tobytes(), (kind, i)
    s = server.stats()
    assert s["device_bytes"] <= s["budget_bytes"]
    with pytest.raises(RuntimeError, match="budget"):
        server.add_samples(syn.cube_face_samples(1 << 20, 5600))
    server.add_samples(syn.cube_face_samples(20000, 5601, volume_fraction=0.25))
    server.wait_update(server.update())
    assert server.stats()["updates"] == 1
    server.release()


def test_quadtree_field_served_alone_equals_in_the_mix():
    """A directional quadtree field behind the server: query and path-vertex
    requests of mixed sizes from several threads give the direct calls'
    bytes."""
    import openpgl_gb300 as pgl
    from openpgl_gb300 import synthetic as syn

    dev, field = _trained(pgl, syn, 5300, frames=2, dqt=True)
    rng = np.random.default_rng(11)
    sizes = np.exp(rng.uniform(np.log(50), np.log(20000), size=12)).astype(int)
    batches = [syn.queries(int(n), 5400 + i) for i, n in enumerate(sizes)]
    verts = [syn.vertices(int(n), 5500 + i) for i, n in enumerate(sizes[:6])]
    alone_q = [field.sample_batch(q) for q in batches]
    alone_v = [field.sample_vertices(v) for v in verts]
    server = pgl.GuidingServer(field, hbm_budget_bytes=256 << 20)
    got_q, got_v = [None] * len(batches), [None] * len(verts)

    def worker(k):
        for i in range(k, len(batches), 3):
            t, out = server.submit(batches[i])
            server.wait(t)
            got_q[i] = out
        for i in range(k, len(verts), 3):
            t, out = server.submit_vertices(verts[i])
            server.wait(t)
            got_v[i] = out

    threads = [threading.Thread(target=worker, args=(k,)) for k in range(3)]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    for a, b in zip(alone_q, got_q):
        assert a.tobytes() == b.tobytes()
    for a, b in zip(alone_v, got_v):
        assert a.tobytes() == b.tobytes()
    server.release()


def test_page_locked_requests_are_served_in_place():
    """Requests whose buffers are page-locked host memory are read and
    written in place by the server's launches (no staging copies): the same
    bytes as the direct calls, mixed with requests in ordinary memory."""
    import torch

    import openpgl_gb300 as pgl
    from openpgl_gb300 import synthetic as syn

    def pinned(a):
        return torch.from_numpy(a.view(np.uint8)).pin_memory().numpy().view(a.dtype)

    dev, field = _trained(pgl, syn, 5600, frames=2)
    qs = [syn.queries(n, 5700 + i) for i, n in enumerate((2000, 30000, 500, 12000))]
    vs = [syn.vertices(n, 5800 + i) for i, n in enumerate((4000, 25000))]
    alone_q = [field.sample_batch(q) for q in qs]
    alone_v = [field.sample_vertices(v) for v in vs]
    server = pgl.GuidingServer(field, hbm_budget_bytes=256 << 20)
    tickets = []
    for i, q in enumerate(qs):
        src = pinned(q) if i % 2 == 0 else q
        out = pinned(np.zeros(len(q), dtype=pgl.QUERY_RESULT_DTYPE)) if i % 2 == 0 else None
        tickets.append(("q", i, server.submit(src, out=out) if out is not None else server.submit(src)))
    for i, v in enumerate(vs):
        out = pinned(np.zeros(len(v), dtype=pgl.VERTEX_RESULT_DTYPE))
        tickets.append(("v", i, server.submit_vertices(pinned(v), out=out)))
    for kind, i, (t, out) in tickets:
        server.wait(t)
        ref = alone_q[i] if kind == "q" else alone_v[i]
        assert out.tobytes() == ref.tobytes(), (kind, i)
    server.release()
