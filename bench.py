#!/usr/bin/env python3
"""Benchmark of the field-training (Update) and guided-query path on one GB300.

Workload (multi-frame, plain drop-in): 8 frames x 2,097,152 PGLSampleData
records (16,777,216 samples per step) from the cube-face generator, 25 % of
them flagged inside-volume (interior positions, one lobe with kappa 20);
maxSamplesPerLeaf 32000, deterministic.  One step = a fresh field, then for
every frame: clear the storage, add that frame's samples, pglFieldUpdate.
The metric is milliseconds per 16M (2^24) samples, lower is better.  Beside it
the guided queries of the cube workload (1,048,576 queries: Init + cosine
product + Sample + PDF) on the trained field, as queries/s.

`value` is timed with CUDA events on the library's stream with the samples
already in device memory; `e2e` adds each frame's host-to-device copy from
pinned memory (pglSampleStorageAddSamples on host records) and the read-back
of the per-region update reports.  The inputs (16.8M x 40 B = 671 MB) are
larger than L2 (129 MB), so no flush is needed between steps.

Beside the headline, `clustered` times the clustered workload: one Update of
a fresh field on 16,777,216 surface samples around 4096 Gaussian clusters
(Zipf masses, 1-6 lobes each), maxSamplesPerLeaf 32000, with the default EM
schedule and with the schedule the EM autotuner picks on the Update before
(the fields are compared byte for byte).  `widened` times the rows built
beyond the core path: volume guided queries with the Henyey-Greenstein
product, training samples made from path segments on the device, the
multi-frame step with the plain VMM field type, and the multi-frame step in
the plain drop-in form (per Update and sub-field one EM launch with one block
per region, no work queue and no helper blocks) beside the batched one.

`--impl reference` times the CPU restatement of the reference algorithm (the
oracle, built with the reference's arithmetic) with all host threads on a
bounded sample of the same workload.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

FRAMES = 8
FRAME_SAMPLES = 2_097_152
SAMPLES_PER_STEP = FRAMES * FRAME_SAMPLES  # 16,777,216
UNIT_SAMPLES = 16_777_216
MAX_SAMPLES_PER_LEAF = 32000
QUERIES = 1_048_576
METRIC = "Update ms/16M samples; guided queries/s @p99; batched vs plain GPU vs host CPU"
UNIT = "ms/16M samples"
WORKLOAD = ("multi-frame: 8 frames x 2,097,152 samples (25% inside-volume, cube faces, 3-lobe vMF per octant), "
            "maxSamplesPerLeaf 32000, deterministic; plus 1,048,576 guided queries (cosine product, 1 SamplePDF)")
# algorithmic bytes of one EM launch: each sample's position+distance and
# direction+weight read once (2 x 16 B), each region's directional state
# (3008 B) read and written once
EM_BYTES_PER_SAMPLE = 32
REGION_STATE_BYTES = 3008
# DRAM bytes (read + write) per sample of an EM launch, measured by ncu
# (dram__bytes_read.sum + dram__bytes_write.sum) on the first Update's launch of
# this workload (`bench.py --em-capture`: 2,097,152 samples, 115.7 MB)
EM_TRAFFIC_PER_SAMPLE = 55.2


# the port against the compiled reference (CPU_8, AVX2) on x86, first frame
# of this workload, 8 threads: 2005 ms against 518 ms
PORT_NOTE = "oracle port; the compiled reference ran 3.3-3.9x faster than this port per frame on x86"


def log(msg):
    """Progress of the benchmark's legs (stderr; the JSON line goes to stdout)."""
    print(f"[bench {time.strftime('%H:%M:%S')}] {msg}", file=sys.stderr, flush=True)


def host_info():
    """Host cores and CPU model string (lscpu, else /proc/cpuinfo)."""
    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                model = line.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.SubprocessError):
        pass
    if model is None:
        try:
            for line in open("/proc/cpuinfo"):
                if line.lower().startswith(("model name", "cpu part")):
                    model = line.split(":", 1)[1].strip()
                    break
        except OSError:
            pass
    return {"nproc": os.cpu_count(), "cpu_model": model or "unknown", "machine": os.uname().machine}


def frame_seed(f):
    return 9000 + f


def make_frames():
    from openpgl_gb300 import synthetic as syn

    return [syn.cube_face_samples(FRAME_SAMPLES, frame_seed(f), volume_fraction=0.25) for f in range(FRAMES)]


def make_queries():
    from openpgl_gb300 import synthetic as syn

    return syn.queries(QUERIES, 4242)


# ----------------------------------------------------------------- clocks
class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons while running."""

    FIELDS = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.thread.join(timeout=5)
        sm, smax, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) != 6:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for name, v in zip(names, parts[2:]):
                if v.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ----------------------------------------------------------------- clustered workload
CLUSTER_SAMPLES = 16_777_216
CLUSTER_SEED = 77


def run_clustered(pgl, dev, stream, steps, warmup):
    """One Update of a fresh field per step on the clustered samples (already
    in device memory): default EM schedule, then the schedule the autotuner
    picks (its sweep runs inside one untimed Update)."""
    import torch

    from openpgl_gb300 import synthetic as syn

    samples = syn.cluster_samples(CLUSTER_SAMPLES, CLUSTER_SEED)
    d = torch.from_numpy(samples.view(np.uint8)).to("cuda")
    storage = pgl.SampleStorage()
    torch.cuda.synchronize()

    def update(tuning=None, autotune=False, plain=False):
        field = pgl.Field(dev, pgl.FieldConfig(deterministic=True, max_samples_per_leaf=MAX_SAMPLES_PER_LEAF))
        if tuning:
            field.set_em_tuning(**tuning)
        if plain:
            field.set_plain_update(True)
        if autotune:
            field.autotune_next_update()
        storage.clear()
        storage.add_samples_device(d.data_ptr(), CLUSTER_SAMPLES)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        field.update(storage)
        b.record(stream)
        torch.cuda.synchronize()
        return field, a.elapsed_time(b)

    def timed(tuning=None):
        for _ in range(warmup):
            update(tuning)
        first, times, ems = None, [], []
        for _ in range(steps):
            field, t = update(tuning)
            times.append(t)
            ems.append(field.phases(False)["em_kernel"])
            first = first or field
        return first, statistics.median(times), statistics.median(ems)

    ref, ms_default, em_default = timed()
    tuned_field, tune_ms = update(autotune=True)
    chosen = tuned_field.em_tuning()
    trials = tuned_field.tuning_trials()
    same = tuned_field.field_bytes() == ref.field_bytes()
    field, ms_tuned, em_tuned = timed(chosen)
    same = same and field.field_bytes() == ref.field_bytes()
    # the plain drop-in form on the same Update (per sub-field one EM launch,
    # one block per region)
    plain_times = []
    for _ in range(2):
        pf, t = update(plain=True)
        plain_times.append(t)
    plain_same = pf.field_bytes() == ref.field_bytes()
    out = {"workload": "clustered: 16,777,216 surface samples around 4096 Gaussian clusters (Zipf(1.1) masses, "
                       "1-6 vMF lobes each), maxSamplesPerLeaf 32000, deterministic; one Update of a fresh field",
           "regions": int(ref.phases(False)["regions"]),
           "update_ms": round(ms_default, 3), "em_kernel_ms": round(em_default, 3),
           "autotuned": {"update_ms": round(ms_tuned, 3), "em_kernel_ms": round(em_tuned, 3), "schedule": chosen,
                         "trials": len(trials), "tuning_update_ms": round(tune_ms, 1),
                         "best_trial_ms": round(min(t["ms"] for t in trials), 3) if trials else None},
           "same_field": bool(same),
           "plain_update": {"update_ms": round(min(plain_times), 3), "same_field": bool(plain_same),
                            "batched_speedup": round(min(plain_times) / ms_default, 2)}}
    return out, ref


# ----------------------------------------------------------------- widened rows
PATHS = 131_072


def run_widened(pgl, dev, stream, field, queries, frames, d_frames, steps, warmup):
    """The rows built beyond the core path, each timed on the device with CUDA
    events: volume guided queries with the Henyey-Greenstein product (mean
    cosines uniform in [-0.9, 0.9]), training samples made from 131,072
    synthetic paths, one multi-frame step with the plain VMM field type and
    one with the directional quadtree field type (plus its guided queries),
    and the plain drop-in form of the Update."""
    import torch

    from openpgl_gb300 import synthetic as syn

    out = {}
    # HG product queries on the trained field's volume sub-field
    n = len(queries)
    g = (np.random.Generator(np.random.PCG64(4343)).random(n) * 1.8 - 0.9).astype(np.float32)
    qd = torch.from_numpy(queries.view(np.uint8)).to("cuda")
    gd = torch.from_numpy(g).to("cuda")
    rd = torch.empty(n * 32, dtype=torch.uint8, device="cuda")
    for _ in range(max(warmup, 3)):
        field.sample_batch_hg_device(qd.data_ptr(), gd.data_ptr(), n, rd.data_ptr(), stream=dev.cuda_stream())
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = max(steps, 5)
    a.record(stream)
    for _ in range(reps):
        field.sample_batch_hg_device(qd.data_ptr(), gd.data_ptr(), n, rd.data_ptr(), stream=dev.cuda_stream())
    b.record(stream)
    torch.cuda.synchronize()
    ms = a.elapsed_time(b) / reps
    out["hg_queries"] = {"queries_per_s": round(n / (ms * 1e-3)), "batch": n, "ms_per_batch": round(ms, 3)}
    # samples from path segments
    segs, begin = syn.path_segments(PATHS, 6161)
    d_segs = torch.from_numpy(segs.view(np.uint8)).to("cuda")
    d_begin = torch.from_numpy(begin.astype(np.uint32).view(np.int32)).to("cuda")
    d_out = torch.empty(len(segs) * 40, dtype=torch.uint8, device="cuda")
    d_off = torch.empty(PATHS + 1, dtype=torch.int32, device="cuda")

    def prep():
        pgl.path_samples_device(d_segs.data_ptr(), d_begin.data_ptr(), PATHS, 3.0, d_out.data_ptr(), d_off.data_ptr(),
                                stream=dev.cuda_stream())

    for _ in range(max(warmup, 3)):
        prep()
    a.record(stream)
    for _ in range(reps):
        prep()
    b.record(stream)
    torch.cuda.synchronize()
    ms = a.elapsed_time(b) / reps
    made = int(d_off[-1].item())
    out["path_samples"] = {"paths": PATHS, "segments": len(segs), "samples": made, "ms": round(ms, 3),
                           "segments_per_s": round(len(segs) / (ms * 1e-3)),
                           "segment_bytes_gbs": round(len(segs) * 136 / (ms * 1e-3) / 1e9, 1)}
    # the plain VMM field type on the multi-frame workload (one step after one warm-up)
    plain = pgl.Field(dev, pgl.FieldConfig(deterministic=True, max_samples_per_leaf=MAX_SAMPLES_PER_LEAF,
                                           parallax=False))
    storage = pgl.SampleStorage()

    def step(fld):
        fld.reset()
        for f, d in zip(frames, d_frames):
            storage.clear()
            storage.add_samples_device(d.data_ptr(), len(f))
            fld.update(storage)

    step(plain)
    torch.cuda.synchronize()
    a.record(stream)
    step(plain)
    b.record(stream)
    torch.cuda.synchronize()
    out["plain_vmm_update"] = {"value": round(a.elapsed_time(b), 3), "unit": UNIT}
    # the directional quadtree field type on the multi-frame workload (one step
    # after one warm-up), and its guided queries on the trained field
    quad = pgl.Field(dev, pgl.FieldConfig(deterministic=True, max_samples_per_leaf=MAX_SAMPLES_PER_LEAF, dqt=True))
    step(quad)
    torch.cuda.synchronize()
    a.record(stream)
    step(quad)
    b.record(stream)
    torch.cuda.synchronize()
    dqt_ms = a.elapsed_time(b)
    rq = torch.empty(n * 32, dtype=torch.uint8, device="cuda")
    for _ in range(max(warmup, 3)):
        quad.sample_batch_device(qd.data_ptr(), n, rq.data_ptr(), stream=dev.cuda_stream())
    a.record(stream)
    for _ in range(reps):
        quad.sample_batch_device(qd.data_ptr(), n, rq.data_ptr(), stream=dev.cuda_stream())
    b.record(stream)
    torch.cuda.synchronize()
    qms = a.elapsed_time(b) / reps
    out["dqt_update"] = {"value": round(dqt_ms, 3), "unit": UNIT,
                         "queries_per_s": round(n / (qms * 1e-3)), "ms_per_query_batch": round(qms, 3),
                         "factory": "rejection-sampling estimator, mean split metric, threshold 0.01, "
                                    "footprint 1, 12 levels"}
    out["_dqt_field"] = quad.field_bytes()
    out["_dqt_queries"] = np.frombuffer(rq.cpu().numpy().tobytes(), dtype=pgl.QUERY_RESULT_DTYPE).copy()
    quad.release()
    # the plain drop-in form of the Update: per sub-field one EM launch with a
    # block per region (all SMs; no queue, no helper blocks, no shared passes)
    per_region = pgl.Field(dev, pgl.FieldConfig(deterministic=True, max_samples_per_leaf=MAX_SAMPLES_PER_LEAF))
    per_region.set_plain_update(True)
    step(per_region)
    torch.cuda.synchronize()
    times = []
    for _ in range(max(2, min(steps, 3))):
        a.record(stream)
        step(per_region)
        b.record(stream)
        torch.cuda.synchronize()
        times.append(a.elapsed_time(b))
    out["plain_update"] = {"value": round(statistics.median(times), 3), "unit": UNIT,
                           "form": "per Update and sub-field one EM launch with one block per region (all SMs, "
                                   "no work queue, no helper blocks)",
                           "same_field": per_region.field_bytes() == field_bytes_of(pgl, dev, frames, d_frames)}
    return out


def run_single_update(pgl, dev, stream, steps):
    """The single-Update configuration: 1,048,576 cube-face surface samples,
    maxSamplesPerLeaf 32000, one Update of a fresh field (batched form and the
    plain drop-in form, samples already in device memory), then 1,048,576
    guided queries (cosine product, one SamplePDF) on device buffers.  Returns
    the numbers, the frame and the batched form's field bytes (for the oracle
    comparison of the CPU leg)."""
    import torch

    from openpgl_gb300 import synthetic as syn

    frame = syn.cube_face_samples(1 << 20, 1001)
    d = torch.from_numpy(frame.view(np.uint8)).to("cuda")
    q = syn.queries(1 << 20, 1002)
    qd = torch.from_numpy(q.view(np.uint8)).to("cuda")
    rd = torch.empty(len(q) * 32, dtype=torch.uint8, device="cuda")
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    st = pgl.SampleStorage()
    out, fields = {}, {}
    for form in ("batched", "plain"):
        field = pgl.Field(dev, pgl.FieldConfig(deterministic=True, max_samples_per_leaf=32000))
        field.set_plain_update(form == "plain")
        times = []
        for i in range(max(3, min(steps, 5)) + 1):
            field.reset()
            st.clear()
            st.add_samples_device(d.data_ptr(), len(frame))
            torch.cuda.synchronize()
            a.record(stream)
            field.update(st)
            b.record(stream)
            torch.cuda.synchronize()
            if i:  # the first Update is a warm-up
                times.append(a.elapsed_time(b))
        out[f"{form}_update_ms"] = round(statistics.median(times), 3)
        fields[form] = field
    field = fields["batched"]
    for _ in range(3):
        field.sample_batch_device(qd.data_ptr(), len(q), rd.data_ptr(), stream=dev.cuda_stream())
    reps = 10
    a.record(stream)
    for _ in range(reps):
        field.sample_batch_device(qd.data_ptr(), len(q), rd.data_ptr(), stream=dev.cuda_stream())
    b.record(stream)
    torch.cuda.synchronize()
    qms = a.elapsed_time(b) / reps
    out.update(batched_speedup=round(out["plain_update_ms"] / out["batched_update_ms"], 2),
               same_field=fields["plain"].field_bytes() == field.field_bytes(),
               queries_per_s=round(len(q) / (qms * 1e-3)), ms_per_query_batch=round(qms, 3),
               workload="1,048,576 cube-face surface samples, maxSamplesPerLeaf 32000, one Update of a fresh "
                        "field; 1,048,576 guided queries (cosine product, one SamplePDF)")
    gq = np.frombuffer(rd.cpu().numpy().tobytes(), dtype=pgl.QUERY_RESULT_DTYPE).copy()
    fb = field.field_bytes()
    for f in fields.values():
        f.release()
    st.release()
    return out, (frame, q, fb, gq)


def single_update_cpu(frame, q, gpu_field_bytes, gpu_queries):
    """The oracle on the single-Update configuration (all host threads, one
    Update of a fresh field, timed) and the comparison of its field and
    queries with the GPU's."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import pyoracle
    from helpers import compare_fields, compare_queries

    threads = os.cpu_count()
    orc = pyoracle.OracleField(32000, deterministic=True, threads=threads)
    t0 = time.perf_counter()
    orc.update(frame)
    ms = (time.perf_counter() - t0) * 1e3
    t0 = time.perf_counter()
    ref = orc.query(q)
    qps = len(q) / (time.perf_counter() - t0)
    r = compare_fields(gpu_field_bytes, orc.field_bytes(), "surface")
    par = {k: r.get(k) for k in ("tree_equal", "numbering_equal", "stats_equal", "regions", "bit_exact_regions",
                                 "worst_pdf_rel")}
    par["queries"] = compare_queries(gpu_queries, ref)
    orc.close()
    return {"update_ms": round(ms, 1), "queries_per_s": round(qps), "cores": threads, "kind": "port"}, par


def field_bytes_of(pgl, dev, frames, d_frames):
    """The batched form's field after the multi-frame step (for comparisons)."""
    f = pgl.Field(dev, pgl.FieldConfig(deterministic=True, max_samples_per_leaf=MAX_SAMPLES_PER_LEAF))
    st = pgl.SampleStorage()
    for fr, d in zip(frames, d_frames):
        st.clear()
        st.add_samples_device(d.data_ptr(), len(fr))
        f.update(st)
    out = f.field_bytes()
    f.release()
    st.release()
    return out


# ----------------------------------------------------------------- CPU baseline
def cpu_baseline(frames, budget_s=20.0, threads=None):
    """Times the oracle (the CPU restatement of the reference's Update, with the
    reference's arithmetic) on the frames of the workload, as many as fit in
    about budget_s, and scales to ms per 16M samples.  Returns the baseline
    and the oracle field (trained on all frames when they fit)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle

    threads = threads or os.cpu_count()
    orc = pyoracle.OracleField(MAX_SAMPLES_PER_LEAF, deterministic=True, threads=threads)
    done, t_total = 0, 0.0
    for f in frames:
        t0 = time.perf_counter()
        orc.update(f)
        t_total += time.perf_counter() - t0
        done += 1
        if t_total >= budget_s:
            break
    samples = done * FRAME_SAMPLES
    value = t_total * 1e3 * UNIT_SAMPLES / samples
    return ({"value": value, "unit": UNIT, "cores": threads, "kind": "port",
             "sample": f"frames 1-{done} of 8 ({samples} samples, fresh field), oracle Update wall time scaled to "
                       f"16,777,216 samples",
             "note": PORT_NOTE, "host": host_info()}, orc if done == len(frames) else None)


def parity_block(orc, gpu_field_bytes, gpu_queries, queries):
    """The GPU's field after the timed step against the oracle's field trained
    on the same frames (surface and volume: tree, numbering and leaf sample
    statistics equal, regions with equal mixture bytes, worst per-leaf
    relative PDF error on the 64x64 grid, leaves above 1e-3 and lobe-count
    flips), and the GPU's guided-query batch against the oracle's on the same
    queries (ok flags, region ids and sample1D bits equal, worst pdf error).
    Also times the oracle's queries on 131,072 of them."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from helpers import compare_fields, compare_queries

    out = {}
    for side in ("surface", "volume"):
        r = compare_fields(gpu_field_bytes, orc.field_bytes(), side)
        out[side] = {k: r.get(k) for k in ("tree_equal", "numbering_equal", "stats_equal", "regions",
                                           "bit_exact_regions", "worst_pdf_rel")}
        out[side]["leaves_over_1e-3"] = r.get("over_tol", [])[:8]
        out[side]["k_flips"] = r.get("k_flips", [])[:8]
    n = 131072
    t0 = time.perf_counter()
    orc.query(queries[:n])
    qps = n / (time.perf_counter() - t0)
    ref = orc.query(queries)
    out["queries"] = compare_queries(gpu_queries, ref)
    out["queries"]["count"] = len(queries)
    return out, qps


def dqt_parity(frames, queries, gpu_field_bytes, gpu_queries):
    """The oracle's quadtree field on the same 8 frames (timed: the quadtree
    field type's CPU baseline, all host threads) against the GPU's
    (compare_dqt_fields per side), and the guided queries against the
    oracle's."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import pyoracle
    from helpers import compare_dqt_fields, compare_queries

    threads = os.cpu_count()
    orc = pyoracle.OracleField(MAX_SAMPLES_PER_LEAF, deterministic=True, threads=threads, dqt=True)
    t0 = time.perf_counter()
    for f in frames:
        orc.update(f)
    ms = (time.perf_counter() - t0) * 1e3 * UNIT_SAMPLES / (len(frames) * FRAME_SAMPLES)
    base = {"value": round(ms, 1), "unit": UNIT, "cores": threads, "kind": "port",
            "sample": "frames 1-8 of 8, fresh quadtree field"}
    par = {side: compare_dqt_fields(gpu_field_bytes, orc.field_bytes(), side) for side in ("surface", "volume")}
    par["queries"] = compare_queries(gpu_queries, orc.query(queries))
    orc.close()
    return base, par


# ----------------------------------------------------------------- serving
def run_serving(pgl, field, frames, queries, seconds=6.0, submitters=8, update_every=100):
    """Guided queries through the guiding server (continuous batching over a
    double-buffered field) from `submitters` threads, each sending batches of
    log-uniform size in [1024, 262144] back to back (closed loop: the load is
    the saturating one), while a 2M-sample Update runs in the background every
    `update_every` batches.  Beside it the plain drop-in: the per-object API
    (one Init + cosine product + SamplePDF launch chain per query)."""
    import threading

    rng = np.random.default_rng(99)
    sizes = np.exp(rng.uniform(np.log(1024), np.log(262144), size=4096)).astype(int)
    server = pgl.GuidingServer(field, hbm_budget_bytes=4 << 30)
    lock = threading.Lock()
    state = {"next": 0, "batches": 0, "stop": False, "tickets": []}
    t_end = time.perf_counter() + seconds

    def submitter():
        while time.perf_counter() < t_end:
            with lock:
                i = state["next"]
                state["next"] += 1
                state["batches"] += 1
                upd = state["batches"] % update_every == 0
            n = int(sizes[i % len(sizes)])
            off = (i * 7919) % (len(queries) - n)
            t, out = server.submit(queries[off:off + n])
            server.wait(t)
            if upd:
                server.add_samples(frames[i % len(frames)])
                state["tickets"].append(server.update())

    t0 = time.perf_counter()
    threads = [threading.Thread(target=submitter) for _ in range(submitters)]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    wall = time.perf_counter() - t0
    for t in state["tickets"]:
        server.wait_update(t)
    st = server.stats()
    server.release()

    # plain drop-in: per-object calls
    n_plain = 2000
    ssd = pgl.SurfaceSamplingDistribution(field)
    q = queries[:n_plain]
    t0 = time.perf_counter()
    for i in range(n_plain):
        ok, _ = ssd.init(tuple(q["position"][i]), float(q["sample1d"][i]))
        if ok:
            ssd.apply_cosine_product(tuple(q["normal"][i]))
            ssd.sample_pdf(tuple(q["u"][i]))
    plain_qps = n_plain / (time.perf_counter() - t0)
    ssd.release()
    return {"queries_per_s": round(st["queries"] / wall), "p50_ms": round(st["p50_ms"], 3),
            "p99_ms": round(st["p99_ms"], 3), "p999_ms": round(st["p999_ms"], 3), "requests": int(st["requests"]),
            "launches": int(st["launches"]), "background_updates": int(st["updates"]), "submitters": submitters,
            "batch_sizes": "log-uniform 1024-262144", "plain_per_object_queries_per_s": round(plain_qps),
            "served_vs_plain": round(st["queries"] / wall / plain_qps, 1)}


# ----------------------------------------------------------------- serving workload
SERVE_BUDGET = 40 << 30
SERVE_POOL = 1 << 20       # vertices the request stream draws its batches from
SERVE_MIN, SERVE_MAX = 1024, 1 << 20
UPDATE_EVERY = 500         # batches between interleaved Updates
UPDATE_SAMPLES = 2_097_152


def run_serving_c3(pgl, field, batches_per_rate=1000, loads=(0.25, 0.5, 0.75, 0.9, 1.0, 1.25), plain_seconds=3.0):
    """The serving workload on the clustered field: batches of path vertices
    (sizes log-uniform in 1,024-1,048,576; position from the clusters, normal,
    wo, roughness, sample1D, four 2D random numbers; per vertex Init + cosine
    product + 4 SamplePDF) arriving by Poisson at rates swept to saturation,
    a 2,097,152-sample Update interleaved every 500 batches, a 40 GB HBM
    budget.  Per rate: offered and achieved vertices/s and p50/p99/p99.9
    request latency (arrival to results in host memory).  Beside it the plain
    drop-in: the per-object C API driven from C++ threads (one vertex at a
    time, as a renderer's threads call the reference)."""
    import queue as queue_mod

    import torch

    from openpgl_gb300 import synthetic as syn

    pool = torch.from_numpy(syn.vertices(SERVE_POOL, 3303).view(np.uint8)).pin_memory()
    verts = pool.numpy().view(syn.PGL_VERTEX_DTYPE)
    out_pool = torch.empty(8 * SERVE_POOL * 76, dtype=torch.uint8).pin_memory()
    outs = out_pool.numpy().view(pgl.VERTEX_RESULT_DTYPE)
    rng = np.random.default_rng(3304)
    train = [syn.cluster_samples(UPDATE_SAMPLES, 3400 + k) for k in range(2)]
    server = pgl.GuidingServer(field, hbm_budget_bytes=SERVE_BUDGET)

    def run(rate, nb):
        """nb batches arriving at `rate` batches/s (None: all at once)."""
        sizes = np.exp(rng.uniform(np.log(SERVE_MIN), np.log(SERVE_MAX), size=nb)).astype(np.int64)
        gaps = rng.exponential(1.0 / rate, size=nb) if rate else np.zeros(nb)
        arrivals = np.cumsum(gaps)
        done_q = queue_mod.Queue()
        lat = np.zeros(nb)
        out_at = [0]
        updates = []

        def waiter():
            while True:
                item = done_q.get()
                if item is None:
                    return
                i, t, t_arr, t_sub = item
                ms, _ = server.wait(t)
                lat[i] = ms + (t_sub - t_arr) * 1e3

        th = threading.Thread(target=waiter)
        th.start()
        server.reset_stats()
        t0 = time.perf_counter()
        for i in range(nb):
            n = int(sizes[i])
            now = time.perf_counter() - t0
            if arrivals[i] > now:
                time.sleep(arrivals[i] - now)
            off = int(rng.integers(0, SERVE_POOL - n + 1))
            o = out_at[0] if out_at[0] + n <= len(outs) else 0
            out_at[0] = o + n
            t_sub = time.perf_counter() - t0
            t, _ = server.submit_vertices(verts[off:off + n], outs[o:o + n])
            done_q.put((i, t, t0 + arrivals[i] if rate else t0, t0 + t_sub))
            if (i + 1) % UPDATE_EVERY == 0:
                server.add_samples(train[(i // UPDATE_EVERY) % len(train)])
                updates.append(server.update())
        done_q.put(None)
        th.join()
        wall = time.perf_counter() - t0
        for u in updates:
            server.wait_update(u)
        st = server.stats()
        return sizes, lat, wall, st

    # service capacity: all batches of a closed burst
    sizes, lat, wall, st = run(None, max(100, batches_per_rate // 4))
    capacity = len(sizes) / wall
    log(f"serving capacity {capacity:.1f} batches/s ({float(sizes.sum()) / wall / 1e6:.1f} M vertices/s)")
    points = []
    for load in loads:
        rate = load * capacity
        sizes, lat, wall, st = run(rate, batches_per_rate)
        log(f"load {load}: {float(sizes.sum()) / wall / 1e6:.1f} M vertices/s, p99 {np.percentile(lat, 99):.2f} ms")
        points.append({"load": load, "offered_batches_per_s": round(rate, 1),
                       "offered_vertices_per_s": round(rate * float(sizes.mean())),
                       "vertices_per_s": round(float(sizes.sum()) / wall),
                       "p50_ms": round(float(np.percentile(lat, 50)), 3),
                       "p99_ms": round(float(np.percentile(lat, 99)), 3),
                       "p999_ms": round(float(np.percentile(lat, 99.9)), 3),
                       "batches": int(len(sizes)), "updates": int(st["updates"])})
    mem = server.stats()
    server.release()
    # the plain drop-in: per-object calls from C++ threads (the field through its file)
    plain = run_plain_driver(pgl, field, verts[:65536], seconds=plain_seconds)
    out = {"workload": "path vertices on the clustered field: batches log-uniform in 1,024-1,048,576 vertices, "
                       "Poisson arrivals swept to saturation, Init + cosine product + 4 SamplePDF per vertex, "
                       "a 2,097,152-sample Update every 500 batches, 40 GB HBM budget",
           "batches_per_rate": batches_per_rate, "saturation_batches_per_s": round(capacity, 1),
           "points": points, "device_bytes": int(mem["device_bytes"]), "budget_bytes": int(mem["budget_bytes"]),
           "plain": plain}
    if plain:
        # matched p99: the plain form serving the same request sizes one vertex
        # at a time takes n / (vertices/s) per request; the served form's best
        # throughput among the rates whose p99 is no worse than that
        plain_p99 = float(np.percentile(sizes, 99)) / plain["vertices_per_s"] * 1e3
        ok = [p for p in points if p["p99_ms"] <= plain_p99]
        best = max(ok, key=lambda p: p["vertices_per_s"]) if ok else None
        out["matched_p99"] = {"plain_p99_request_ms": round(plain_p99, 1),
                              "served_vertices_per_s": best["vertices_per_s"] if best else None,
                              "served_vs_plain": round(best["vertices_per_s"] / plain["vertices_per_s"], 1)
                              if best else None}
    return out


def run_plain_driver(pgl, field, verts, seconds=3.0, threads=None):
    """Runs the per-object query driver (C++ threads, one vertex at a time)
    on a copy of `field` read from its file."""
    import tempfile

    exe = os.path.join(ROOT, "openpgl_gb300", "_build", "plain_query_driver")
    if not os.path.exists(exe):
        return None
    threads = threads or min(16, os.cpu_count() or 1)
    with tempfile.TemporaryDirectory() as td:
        fpath, vpath = os.path.join(td, "f.field"), os.path.join(td, "v.bin")
        field.store(fpath)
        with open(vpath, "wb") as f:
            f.write(np.uint64(len(verts)).tobytes())
            f.write(np.ascontiguousarray(verts).tobytes())
        r = subprocess.run([exe, fpath, vpath, str(threads), str(seconds)], capture_output=True, text=True,
                           timeout=seconds + 120)
    if r.returncode != 0:
        return {"error": r.stderr[-300:]}
    done, wall, vps, p50, p99, p999 = (float(x) for x in r.stdout.split())
    return {"threads": threads, "vertices": int(done), "vertices_per_s": round(vps, 1),
            "p50_us": p50, "p99_us": p99, "p999_us": p999,
            "form": "per-object C API (Init, ApplyCosineProduct, 4 SamplePDF) from C++ threads, one vertex per "
                    "call chain"}


# ----------------------------------------------------------------- scale workload
SCALE_SAMPLES = 64 << 20
SCALE_FRAMES = 16
SCALE_LEAF = 16000


def cluster_frame_device(n, seed, model, volume_fraction=0.25):
    """A frame of the clustered distribution made on the device (torch's
    seeded generator): cluster by mass, Gaussian offset, a lobe of the
    cluster's mixture by weight, a vMF direction, lognormal(0,2) weight, pdf
    1/(4 pi), distance U[0.05, 2], 25 % flagged inside-volume.  Records of
    40 bytes (PGLSampleData).  Deterministic for a seed on a given device; it
    stands in for the host generator, which is too slow at 64M samples."""
    import torch

    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    dev = "cuda"
    cdf = torch.cumsum(model["mass"], 0)
    c = torch.clamp(torch.searchsorted(cdf, torch.rand(n, device=dev, generator=g) * cdf[-1]), max=len(cdf) - 1)
    pos = model["centers"][c] + model["sigma"][c, None] * torch.randn(n, 3, device=dev, generator=g)
    lw = model["lobe_w"][c]
    lcdf = torch.cumsum(lw, 1)
    u = torch.rand(n, 1, device=dev, generator=g) * lcdf[:, -1:]
    lobe = torch.clamp((lcdf < u).sum(1), max=5)
    mu = model["mu"][c, lobe]
    kappa = model["kappa"][c, lobe]
    ux = torch.rand(n, device=dev, generator=g)
    w = torch.clamp(1.0 + torch.log(ux + (1.0 - ux) * torch.exp(-2.0 * kappa)) / kappa, -1.0, 1.0)
    phi = 2.0 * np.pi * torch.rand(n, device=dev, generator=g)
    r = torch.sqrt(torch.clamp(1.0 - w * w, min=0.0))
    local = torch.stack([r * torch.cos(phi), r * torch.sin(phi), w], 1)
    # frame around mu
    a = torch.where(mu[:, 2:3].abs() < 0.999, torch.tensor([0.0, 0.0, 1.0], device=dev),
                    torch.tensor([1.0, 0.0, 0.0], device=dev))
    t1 = torch.nn.functional.normalize(torch.cross(a, mu, dim=1), dim=1)
    t2 = torch.cross(mu, t1, dim=1)
    d = local[:, :1] * t1 + local[:, 1:2] * t2 + local[:, 2:3] * mu
    rec = torch.empty(n, 10, dtype=torch.float32, device=dev)
    rec[:, 0:3] = pos
    rec[:, 3:6] = d
    rec[:, 6] = torch.exp(2.0 * torch.randn(n, device=dev, generator=g))
    rec[:, 7] = 0.07957747154594767
    rec[:, 8] = 0.05 + 1.95 * torch.rand(n, device=dev, generator=g)
    flags = (torch.rand(n, device=dev, generator=g) < volume_fraction).to(torch.int32) * 2
    rec[:, 9] = flags.view(torch.float32)
    return rec


def run_scale(pgl, dev, serve_rate=None, frames=SCALE_FRAMES, n=SCALE_SAMPLES):
    """The scale workload: 16 frames of 64M clustered samples (25 % volume),
    maxSamplesPerLeaf 16000, each frame's Update run by the guiding server
    (40 GB budget covering the double-buffered field, the sample storage and
    the query buffers) while path-vertex batches keep arriving at
    `serve_rate` batches/s (half of the serving workload's saturation)."""
    import torch

    from openpgl_gb300 import synthetic as syn

    m = syn.cluster_model(1234)
    model = {k: torch.from_numpy(np.asarray(v, dtype=np.float32)).cuda() for k, v in m.items()}
    field = pgl.Field(dev, pgl.FieldConfig(deterministic=True, max_samples_per_leaf=SCALE_LEAF))
    # the query load takes about half of the GPU: the EM leaves half the SMs to it
    server = pgl.GuidingServer(field, hbm_budget_bytes=SERVE_BUDGET, reserved_sms=76 if serve_rate else 0)
    pool = torch.from_numpy(syn.vertices(SERVE_POOL, 3313).view(np.uint8)).pin_memory()
    verts = pool.numpy().view(syn.PGL_VERTEX_DTYPE)
    outs = torch.empty(4 * SERVE_POOL * 76, dtype=torch.uint8).pin_memory().numpy().view(pgl.VERTEX_RESULT_DTYPE)
    stop = threading.Event()
    lat = []
    rng = np.random.default_rng(3314)

    def load():
        """Poisson batches of path vertices until stopped (from the second frame on)."""
        out_at = 0
        t_next = time.perf_counter()
        pendingq = []
        while not stop.is_set():
            t_next += rng.exponential(1.0 / serve_rate)
            now = time.perf_counter()
            if t_next > now:
                time.sleep(t_next - now)
            nv = int(np.exp(rng.uniform(np.log(SERVE_MIN), np.log(SERVE_MAX))))
            off = int(rng.integers(0, SERVE_POOL - nv + 1))
            o = out_at if out_at + nv <= len(outs) else 0
            out_at = o + nv
            t, _ = server.submit_vertices(verts[off:off + nv], outs[o:o + nv])
            pendingq.append(t)
            while len(pendingq) > 64:
                ms, _ = server.wait(pendingq.pop(0))
                lat.append(ms)
        for t in pendingq:
            ms, _ = server.wait(t)
            lat.append(ms)

    per_frame, em_ms, regions, peak = [], [], [], 0
    th = None
    try:
        for f in range(frames):
            rec = cluster_frame_device(n, 5000 + f, model)
            torch.cuda.synchronize()
            server.add_samples_device(rec.data_ptr(), n)
            del rec
            t0 = time.perf_counter()
            server.wait_update(server.update())
            per_frame.append((time.perf_counter() - t0) * 1e3)
            ph = [field.phases(False), field.phases(True)]
            em_ms.append(ph[0]["em_kernel"])
            regions.append(int(ph[0]["regions"] + ph[1]["regions"]))
            peak = max(peak, int(server.stats()["device_bytes"]))
            log(f"scale frame {f}: update {per_frame[-1]:.1f} ms, em {em_ms[-1]:.1f} ms, {regions[-1]} regions")
            if f == 0 and serve_rate:
                th = threading.Thread(target=load, daemon=True)
                th.start()
    finally:
        stop.set()
        if th:
            th.join()
    server.release()
    field.release()
    lat = np.array(lat) if lat else np.zeros(1)
    total = sum(per_frame)
    return {"workload": "16 frames x 67,108,864 clustered samples (25% inside-volume), maxSamplesPerLeaf 16000, "
                        "Updates through the guiding server (40 GB budget) with path-vertex batches arriving "
                        "at half the serving workload's saturation from the second frame on (EM launches "
                        "leave 76 of 152 SMs to the queries)",
            "frames": frames, "samples_per_frame": n, "update_ms_per_frame": [round(x, 1) for x in per_frame],
            "em_kernel_ms_per_frame": [round(x, 1) for x in em_ms], "regions_per_frame": regions,
            "ms_per_16M_samples": round(total * UNIT_SAMPLES / (frames * n), 3),
            "concurrent_queries": {"batches_per_s": round(serve_rate, 1) if serve_rate else None,
                                   "requests": int(len(lat)), "p50_ms": round(float(np.percentile(lat, 50)), 3),
                                   "p99_ms": round(float(np.percentile(lat, 99)), 3),
                                   "p999_ms": round(float(np.percentile(lat, 99.9)), 3)},
            "peak_device_bytes": peak, "budget_bytes": SERVE_BUDGET,
            "data": "generated on the device from the cluster model (torch seeded generator)"}


# ----------------------------------------------------------------- GPU arm
def run_gpu(args, rank, world, local_rank):
    import torch

    import openpgl_gb300 as pgl
    from openpgl_gb300 import replicas

    torch.cuda.set_device(local_rank)
    frames = make_frames()
    queries = make_queries()
    dev = pgl.Device()
    stream = torch.cuda.ExternalStream(dev.cuda_stream())
    field = pgl.Field(dev, pgl.FieldConfig(deterministic=True, max_samples_per_leaf=MAX_SAMPLES_PER_LEAF))
    storage = pgl.SampleStorage()
    d_frames = [torch.from_numpy(f.view(np.uint8)).to("cuda") for f in frames]
    torch.cuda.synchronize()

    def step():
        field.reset()
        for f, d in zip(frames, d_frames):
            storage.clear()
            storage.add_samples_device(d.data_ptr(), len(f))
            field.update(storage)

    def barrier():
        replicas.barrier("cuda")

    log("warm-up steps")
    for _ in range(args.warmup):
        step()
    log("timed steps")
    clocks = ClockSampler(local_rank)
    clocks.start()
    barrier()
    launches0 = pgl.kernel_launch_count()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        step()
    ev1.record(stream)
    barrier()
    launches = pgl.kernel_launch_count() - launches0
    ms = ev0.elapsed_time(ev1) / args.steps
    clk = clocks.stop()
    gpu_field_bytes = field.field_bytes()
    # one more (untimed) step for the EM launch's counters: its CUDA-event time
    # per Update and the work its passes did (the step is deterministic, so the
    # timed steps did the same work)
    em_work = em_counters(field, storage, frames, d_frames)

    log(f"step {ms:.2f} ms; counter step and queries")
    # ---- guided queries on the trained field (device buffers)
    qdev = torch.from_numpy(queries.view(np.uint8)).to("cuda")
    rdev = torch.empty(QUERIES * 32, dtype=torch.uint8, device="cuda")
    for _ in range(max(args.warmup, 3)):
        field.sample_batch_device(qdev.data_ptr(), QUERIES, rdev.data_ptr(), stream=dev.cuda_stream())
    torch.cuda.synchronize()
    lat = []
    q0, q1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = max(args.steps, 5)
    for _ in range(reps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        field.sample_batch_device(qdev.data_ptr(), QUERIES, rdev.data_ptr(), stream=dev.cuda_stream())
        b.record(stream)
        lat.append((a, b))
    torch.cuda.synchronize()
    lat_ms = sorted(a.elapsed_time(b) for a, b in lat)
    q_ms = statistics.median(lat_ms)
    gpu_queries = np.frombuffer(rdev.cpu().numpy().tobytes(), dtype=pgl.QUERY_RESULT_DTYPE).copy()
    query_work = query_counters(field, gpu_queries)
    # host-buffer queries (page-locked host memory, read and written over the host link)
    q_pinned = torch.from_numpy(queries.view(np.uint8)).pin_memory().numpy().view(queries.dtype)
    r_pinned = torch.empty(len(queries) * 32, dtype=torch.uint8).pin_memory().numpy().view(pgl.QUERY_RESULT_DTYPE)
    field.sample_batch(q_pinned, out=r_pinned)
    t0 = time.perf_counter()
    for _ in range(reps):
        field.sample_batch(q_pinned, out=r_pinned)
    q_e2e_ms = (time.perf_counter() - t0) * 1e3 / reps
    e2e_same = r_pinned.tobytes() == gpu_queries.tobytes()

    # ---- rows beyond the core path: HG queries, path-segment samples, plain VMM,
    # and the plain drop-in form of the Update beside the batched one
    log("widened rows")
    widened = None
    if args.widened:
        widened = run_widened(pgl, dev, stream, field, queries, frames, d_frames, args.steps, args.warmup)
        widened["plain_update"]["batched_speedup"] = round(widened["plain_update"]["value"] / ms, 2)

    # ---- the single-Update configuration (1M samples, one Update, 1M queries)
    log("single-Update configuration")
    single, single_data = run_single_update(pgl, dev, stream, args.steps) if args.widened else (None, None)

    # ---- clustered workload, default and autotuned EM schedule
    log("clustered workload")
    clustered, clustered_field = run_clustered(pgl, dev, stream, args.steps, 1) if args.clustered else (None, None)

    # ---- served guided queries (continuous batching, background updates)
    log("serving (closed loop)")
    serving = run_serving(pgl, field, frames[:2], queries, seconds=args.serve_seconds) if args.serve_seconds > 0 else None
    serving_c3 = None
    if clustered_field is not None and args.serve_batches > 0:
        log("serving workload on the clustered field")
        serving_c3 = run_serving_c3(pgl, clustered_field, batches_per_rate=args.serve_batches)
    scale = None
    if args.scale_frames > 0:
        rate = 0.5 * serving_c3["saturation_batches_per_s"] if serving_c3 else None
        log("scale workload")
        scale = run_scale(pgl, dev, serve_rate=rate, frames=args.scale_frames)

    log("end to end")
    # ---- end to end: host (pinned) sample records through the C API
    pinned = [torch.from_numpy(f.view(np.uint8)).pin_memory() for f in frames]
    host_views = [p.numpy().view(frames[0].dtype) for p in pinned]
    d2h = [0]

    def e2e_step():
        field.reset()
        for f in host_views:
            storage.clear()
            storage.add_samples(f)
            field.update(storage)
            for vol in (False, True):
                rep = field.reports(vol)
                d2h[0] += rep.nbytes if hasattr(rep, "nbytes") else 0

    e2e_step()
    barrier()
    d2h[0] = 0
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0 = time.perf_counter()
    e0.record(stream)
    for _ in range(args.steps):
        e2e_step()
    e1.record(stream)
    barrier()
    e2e_ms = e0.elapsed_time(e1) / args.steps
    e2e_wall = (time.perf_counter() - t0) * 1e3 / args.steps

    ms, e2e_ms, q_ms = replicas.max_over_ranks([ms, e2e_ms, q_ms], "cuda")
    if rank != 0:
        return None

    sm_mhz = clk.get("sm_mhz") or measured_peak("sm_max_mhz", 2070.0)[0]
    roofline = em_roofline(em_work, sm_mhz, ms)
    query_roof = kernel_roofline(query_work["flop"], query_work["sfu"], query_work["bytes"], q_ms, sm_mhz)
    query_roof.update(kernel="query_g_kernel", mean_lobes=query_work["mean_lobes"],
                      work="per query with K lobes and one SamplePDF: 62K + (50 + 12K) + 64 flop, "
                           "7K + (6 + K) SFU, 36 B in + 32 B out")
    out = {
        "metric": METRIC,
        "value": round(replicas.whole_job_ms_per_unit(ms, SAMPLES_PER_STEP, UNIT_SAMPLES, world), 3),
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(ms, 3),
        "higher_is_better": False,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded generators of the configured shapes)",
        "config": {"workload": WORKLOAD, "samples_per_step": SAMPLES_PER_STEP, "frames": FRAMES,
                   "max_samples_per_leaf": MAX_SAMPLES_PER_LEAF, "l2": "inputs (671 MB) larger than L2",
                   "parallelism": f"replicas x{world}"},
        "roofline": roofline,
        "e2e": {"value": round(replicas.whole_job_ms_per_unit(e2e_ms, SAMPLES_PER_STEP, UNIT_SAMPLES, world), 3),
                "unit": UNIT,
                "h2d_bytes_per_step": SAMPLES_PER_STEP * 40, "d2h_bytes_per_step": d2h[0] // max(args.steps, 1),
                "wall_ms_per_step": round(e2e_wall, 3)},
        "queries": {"queries_per_s": round(QUERIES / (q_ms * 1e-3)), "batch": QUERIES,
                    "p50_ms": round(statistics.median(lat_ms), 3),
                    "p99_ms": round(lat_ms[min(len(lat_ms) - 1, int(0.99 * len(lat_ms)))], 3),
                    "e2e_queries_per_s": round(QUERIES / (q_e2e_ms * 1e-3)), "e2e_same_results": e2e_same,
                    "roofline": query_roof},
        "serving": serving,
        "serving_clustered": serving_c3,
        "scale": scale,
        "single_update": single,
        "clustered": clustered,
        "widened": widened,
        "gpu_launches": int(launches),
        "clocks": clk,
    }
    if not args.no_cpu_baseline:
        log("CPU baseline and parity")
        out["cpu_baseline"], orc = cpu_baseline(frames, budget_s=args.cpu_budget)
        if orc is not None:
            out["parity"], qps = parity_block(orc, gpu_field_bytes, gpu_queries, queries)
            out["cpu_baseline"]["queries_per_s"] = round(qps)
            orc.close()
        if single is not None:
            log("single-Update oracle and parity")
            single["cpu_baseline"], single["parity"] = single_update_cpu(*single_data)
        if widened is not None and "_dqt_field" in widened:
            log("quadtree oracle and parity")
            widened["dqt_update"]["cpu_baseline"], widened["dqt_update"]["parity"] = dqt_parity(
                frames, queries, widened["_dqt_field"], widened["_dqt_queries"])
    if widened is not None:
        widened.pop("_dqt_field", None)
        widened.pop("_dqt_queries", None)
    return out


# ----------------------------------------------------------------- roofline
# Counting convention of the path's measurement: an exp, log, sqrt, rsqrt, rcp
# or sincos is one SFU op, a division one rcp plus one FMA, an FMA two flop.
ESTEP_FLOP_LOBE, ESTEP_SFU_LOBE = 21, 1      # per (sample, lobe, E-step pass)
ESTEP_FLOP_SAMPLE, ESTEP_SFU_SAMPLE = 4, 2   # per (sample, E-step pass)
DIST_FLOP_LOBE, DIST_SFU_LOBE = 30, 1        # per (sample, lobe) of a distance pass
SPLIT_FLOP_LOBE, SPLIT_SFU_LOBE = 70, 3      # per (sample, lobe) of a split-statistics pass
SMS, FP32_LANES_PER_SM, SFU_PER_SM = 152, 128, 16


def derived_peaks(sm_mhz):
    """FP32 and SFU peaks derived from the SM count, the lanes per SM (128
    FP32, 16 SFU per clock) and the SM clock measured during the run (FMA = 2
    flop); HBM from the measured copy bandwidth."""
    hz = sm_mhz * 1e6
    hbm, src = measured_peak("hbm_gbs", 6800.0)
    return {"fp32_tflops": SMS * FP32_LANES_PER_SM * 2 * hz / 1e12, "sfu_tops": SMS * SFU_PER_SM * hz / 1e12,
            "hbm_gbs": hbm, "hbm_source": src, "sm_mhz": sm_mhz}


def kernel_roofline(flop, sfu, nbytes, ms, sm_mhz):
    """t_roof = max(F / F_peak, SFU / SFU_peak, B / B_peak) for one launch of
    `ms` milliseconds; the binding resource names the bound, `achieved` is that
    resource's rate and `frac` = t_roof / t_measured."""
    p = derived_peaks(sm_mhz)
    t = {"fp32": flop / (p["fp32_tflops"] * 1e12), "sfu": sfu / (p["sfu_tops"] * 1e12),
         "hbm": nbytes / (p["hbm_gbs"] * 1e9)}
    bound = max(t, key=t.get)
    sec = ms * 1e-3
    rate = {"fp32": (flop / sec / 1e12, p["fp32_tflops"], "TFLOP/s", "derived"),
            "sfu": (sfu / sec / 1e12, p["sfu_tops"], "Tops/s", "derived"),
            "hbm": (nbytes / sec / 1e9, p["hbm_gbs"], "GB/s", p["hbm_source"])}
    a, peak, unit, src = rate[bound]
    return {"bound": bound, "achieved": round(a, 4), "peak": round(peak, 2), "unit": unit, "peak_source": src,
            "frac": round(t[bound] / sec, 5), "t_roof_ms": round(t[bound] * 1e3, 5), "avg_launch_ms": round(ms, 4),
            "per_resource_frac": {k: round(v / sec, 5) for k, v in t.items()},
            "algorithmic": {"flop": int(flop), "sfu": int(sfu), "bytes": int(nbytes)}}


def em_counters(field, storage, frames, d_frames):
    """One step, keeping per Update the EM launch's CUDA-event time and the
    algorithmic work of its passes (per-region pass and lobe counters of the
    launch's profile)."""
    import torch

    out = []
    field.reset()
    for f, d in zip(frames, d_frames):
        storage.clear()
        storage.add_samples_device(d.data_ptr(), len(f))
        field.update(storage)
        torch.cuda.synchronize()
        live = [(v, field.phases(v)) for v in (False, True)]
        live = [(v, ph) for v, ph in live if ph["samples"] > 0]
        if not live:
            continue
        flop = sfu = nbytes = samples = 0
        for v, ph in live:
            prof = field.profile(v).astype(np.float64)
            cnt, ep, el, dl, sl = prof[:, 1], prof[:, 2], prof[:, 18], prof[:, 19], prof[:, 20]
            flop += float((cnt * (ESTEP_FLOP_LOBE * el + ESTEP_FLOP_SAMPLE * ep + DIST_FLOP_LOBE * dl
                                  + SPLIT_FLOP_LOBE * sl)).sum())
            sfu += float((cnt * (ESTEP_SFU_LOBE * el + ESTEP_SFU_SAMPLE * ep + DIST_SFU_LOBE * dl
                                 + SPLIT_SFU_LOBE * sl)).sum())
            nbytes += int(ph["samples"]) * EM_BYTES_PER_SAMPLE + int(ph["regions"]) * 2 * REGION_STATE_BYTES
            samples += int(ph["samples"])
        # one EM launch serves both sub-fields of an Update (both report its time)
        out.append({"ms": live[0][1]["em_kernel"], "update_ms": max(ph["total"] for _, ph in live),
                    "flop": flop, "sfu": sfu, "bytes": nbytes, "samples": samples})
    return out


def em_roofline(work, sm_mhz, step_ms):
    """Roofline of the average EM launch of a step (the dominant kernel)."""
    n = max(len(work), 1)
    avg = {k: sum(w[k] for w in work) / n for k in ("ms", "flop", "sfu", "bytes", "samples")}
    r = kernel_roofline(avg["flop"], avg["sfu"], avg["bytes"], avg["ms"], sm_mhz)
    r["kernel"] = "em_leaf_kernel"
    r["launches_per_step"] = len(work)
    r["em_share_of_step"] = round(sum(w["ms"] for w in work) / step_ms, 3)
    r["per_launch_ms"] = [round(w["ms"], 3) for w in work]
    r["traffic"] = round(EM_TRAFFIC_PER_SAMPLE * avg["samples"])
    r["traffic_source"] = ("ncu DRAM bytes per sample of the first Update's EM launch (2,097,152 samples), "
                           "times the samples of the average launch")
    r["work"] = ("per (sample, lobe, E-step pass) 21 flop + 1 SFU; per (sample, E-step pass) 4 flop + 2 SFU; "
                 "per (sample, lobe) of a distance pass 30 flop + 1 SFU, of a split-statistics pass 70 flop + "
                 "3 SFU; 32 B per sample and 2 x 3008 B per region of HBM; pass and lobe counts from the "
                 "launch's own per-region counters")
    return r


def query_counters(field, out):
    """Algorithmic work of the guided-query batch from the lobe count of each
    query's region (the last Update's per-region reports)."""
    rep = field.reports(False)
    k_of = {int(r[0]): int(r[4]) for r in rep}
    ok = out["ok"] == 1
    ks = np.array([k_of.get(int(i), 0) for i in out["id"][ok]], dtype=np.float64)
    flop = float((62 * ks + 50 + 12 * ks + 64).sum())
    sfu = float((7 * ks + 6 + ks).sum())
    return {"flop": flop, "sfu": sfu, "bytes": len(out) * (36 + 32), "mean_lobes": round(float(ks.mean()), 2)
            if len(ks) else 0.0}


def em_capture():
    """One Update of a fresh field on the first frame of the workload (2,097,152
    samples), for a profiler to capture that Update's EM launch."""
    import torch

    import openpgl_gb300 as pgl
    from openpgl_gb300 import synthetic as syn

    frame = syn.cube_face_samples(FRAME_SAMPLES, frame_seed(0), volume_fraction=0.25)
    d = torch.from_numpy(frame.view(np.uint8)).to("cuda")
    dev = pgl.Device()
    field = pgl.Field(dev, pgl.FieldConfig(deterministic=True, max_samples_per_leaf=MAX_SAMPLES_PER_LEAF))
    storage = pgl.SampleStorage()
    storage.add_samples_device(d.data_ptr(), len(frame))
    field.update(storage)
    torch.cuda.synchronize()
    field.release()


def measured_peak(key, fallback):
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            v = json.load(f).get(key)
        if v:
            return float(v), "measured"
    except (OSError, ValueError):
        pass
    return fallback, "fallback"


def run_reference(args, rank, world):
    if rank != 0:
        return None
    frames = make_frames()
    threads = os.cpu_count()
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle

    # each step is the GPU arm's step: a fresh field, then for every frame of
    # the workload an Update on that frame's samples
    def step():
        orc = pyoracle.OracleField(MAX_SAMPLES_PER_LEAF, deterministic=True, threads=threads)
        t0 = time.perf_counter()
        for f in frames:
            orc.update(f)
        dt = time.perf_counter() - t0
        return orc, dt

    for _ in range(args.warmup):
        step()[0].close()
    times = []
    orc = None
    for _ in range(args.steps):
        if orc is not None:
            orc.close()
        orc, dt = step()
        times.append(dt)
    ms = sum(times) * 1e3 / len(times)
    value = ms * UNIT_SAMPLES / SAMPLES_PER_STEP
    queries = make_queries()
    n = 131072
    t0 = time.perf_counter()
    orc.query(queries[:n])
    qps = n / (time.perf_counter() - t0)
    orc.close()
    return {
        "impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 3), "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded generators of the "
                                                                        "configured shapes)",
        "config": {"workload": WORKLOAD, "samples_per_step": SAMPLES_PER_STEP, "frames": FRAMES,
                   "max_samples_per_leaf": MAX_SAMPLES_PER_LEAF, "parallelism": "host threads"},
        "cpu_baseline": {"value": round(value, 3), "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": "the whole step per step: a fresh field, then Updates on frames 1-8 "
                                   "(16,777,216 samples)",
                         "note": PORT_NOTE, "host": host_info()},
        "queries": {"queries_per_s": round(qps), "sample": f"{n} guided queries on the trained field"},
        "e2e": {"value": round(value, 3), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-budget", type=float, default=20.0)
    ap.add_argument("--serve-seconds", type=float, default=6.0)
    ap.add_argument("--no-clustered", dest="clustered", action="store_false",
                    help="skip the clustered workload (default and autotuned EM schedule)")
    ap.add_argument("--serve-batches", type=int, default=1000,
                    help="batches per arrival rate of the serving workload on the clustered field (0: skip)")
    ap.add_argument("--scale-frames", type=int, default=SCALE_FRAMES,
                    help="frames of the 64M-sample scale workload (0: skip)")
    ap.add_argument("--no-widened", dest="widened", action="store_false",
                    help="skip the rows beyond the core path (HG queries, path samples, plain VMM, plain form)")
    ap.add_argument("--em-capture", action="store_true",
                    help="profiling case: one Update of a fresh field on the workload's first frame (one EM "
                         "launch), nothing timed or printed")
    args = ap.parse_args()
    if args.em_capture:
        em_capture()
        return
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        out = run_reference(args, rank, world)
    else:
        from openpgl_gb300 import replicas

        if world > 1:
            import torch

            torch.cuda.set_device(local_rank)
            replicas.init("nccl")
        out = run_gpu(args, rank, world, local_rank)
        replicas.shutdown()
    if out is not None:
        print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
