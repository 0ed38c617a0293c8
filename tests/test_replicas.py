"""The replica path of the benchmark (openpgl_gb300/replicas.py) with two
gloo ranks on the CPU: barrier, maximum of the ranks' timings, whole-job
arithmetic, and a rank that leaves before the timings are gathered (the
survivor gets an error from the collective instead of waiting for ever)."""

import os
import socket

import pytest
import torch.multiprocessing as mp

from openpgl_gb300 import replicas


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _env(rank, world, port):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))


def _max_rank(rank, world, port, out):
    _env(rank, world, port)
    replicas.init("gloo", timeout_s=30)
    replicas.barrier()
    # rank r reports step, e2e and query times that differ per rank
    got = replicas.max_over_ranks([10.0 + rank, 20.0 - rank, 5.0 * (rank + 1)])
    replicas.barrier()
    out.put((rank, got))
    replicas.shutdown()


def _leaving_rank(rank, world, port, out):
    _env(rank, world, port)
    replicas.init("gloo", timeout_s=5)
    replicas.barrier()
    if rank == 1:
        replicas.shutdown()
        return  # leaves between steps, with no collective in flight
    try:
        replicas.max_over_ranks([1.0])
        out.put((rank, "no error"))
    except Exception as e:  # noqa: BLE001 - any error from the collective is the signal
        out.put((rank, type(e).__name__))


def _run(fn, world=2, timeout=120):
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=fn, args=(r, world, port, out)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout)
    for p in procs:
        if p.is_alive():
            p.kill()
            pytest.fail("a rank did not finish")
    res = {}
    while not out.empty():
        r, v = out.get()
        res[r] = v
    return res, [p.exitcode for p in procs]


def test_max_over_ranks_two_gloo_ranks():
    res, codes = _run(_max_rank)
    assert codes == [0, 0]
    assert res[0] == res[1] == [11.0, 20.0, 10.0]


def test_rank_leaving_surfaces_as_an_error_on_the_other():
    res, codes = _run(_leaving_rank)
    assert codes == [0, 0]
    assert res[0] != "no error"


def test_whole_job_value_is_weak_scaling():
    # one replica: 16.8M samples per 100 ms = 100 ms per 16.8M
    unit = 16_777_216
    assert replicas.whole_job_ms_per_unit(100.0, unit, unit, 1) == 100.0
    # four replicas of the same work in the same time: the job processes 4x the samples
    assert replicas.whole_job_ms_per_unit(100.0, unit, unit, 4) == 25.0
    # the slowest replica sets the time
    assert replicas.whole_job_ms_per_unit(max(100.0, 120.0), unit // 2, unit, 2) == 120.0
    assert not replicas.active()
