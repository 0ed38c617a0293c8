"""ctypes front end of the oracle library (oracle/_build/liboracle_pgl.so) and of
the reference harness (oracle/_ref/ref_harness, x86 hosts with the reference
tree only).  Test infrastructure: used by tests/, __graft_entry__.smoke() and
bench.py's CPU baseline, never by the product.
"""

from __future__ import annotations

import ctypes
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle_pgl.so")
REF_PATHS = os.path.join(HERE, "_ref", "ref_paths")
REF_HARNESS = os.path.join(HERE, "_ref", "ref_harness")

QUERY_OUT_DTYPE = np.dtype(
    [("ok", "<u4"), ("id", "<u4"), ("sample1d", "<f4"), ("dir", "<f4", (3,)), ("pdf", "<f4"), ("pdfLi", "<f4")]
)

_lib = None


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        lib = ctypes.CDLL(LIB_PATH)
        vp, u64 = ctypes.c_void_p, ctypes.c_uint64
        lib.orc_field_new.restype = vp
        lib.orc_field_new.argtypes = [ctypes.c_int, u64, ctypes.c_int]
        lib.orc_field_free.argtypes = [vp]
        lib.orc_field_update.argtypes = [vp, vp, u64]
        lib.orc_field_iteration.restype = u64
        lib.orc_field_iteration.argtypes = [vp]
        lib.orc_field_store.restype = u64
        lib.orc_field_store.argtypes = [vp, ctypes.c_char_p, u64]
        lib.orc_field_query.argtypes = [vp, ctypes.c_int, ctypes.c_int, vp, vp, u64]
        lib.orc_field_query_hg.argtypes = [vp, vp, vp, vp, u64]
        lib.orc_field_set_parallax.argtypes = [vp, ctypes.c_int]
        lib.orc_field_set_dqt.argtypes = [vp]
        lib.orc_field_set_dqt_args.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_float, ctypes.c_float,
                                               ctypes.c_uint32]
        lib.orc_field_leaf_of.argtypes = [vp, ctypes.c_int, vp, vp, u64]
        lib.orc_field_set_scene_bounds.argtypes = [vp, vp]
        for n in ("orc_fexp", "orc_flog", "orc_rcp", "orc_rsqrt"):
            getattr(lib, n).restype = ctypes.c_float
            getattr(lib, n).argtypes = [ctypes.c_float]
        _lib = lib
    return _lib


class OracleField:
    """Oracle restatement of a kd-tree field (deterministic CPU_8) with
    parallax-aware VMMs, plain VMMs (parallax=False) or directional quadtrees
    (dqt=True; dqt_args as for run_reference)."""

    def __init__(self, max_samples_per_leaf=32000, deterministic=True, threads=1, parallax=True, dqt=False,
                 dqt_args=None):
        self.lib = load()
        self.h = self.lib.orc_field_new(int(deterministic), int(max_samples_per_leaf), int(threads))
        if not parallax:
            self.lib.orc_field_set_parallax(self.h, 0)
        if dqt:
            self.lib.orc_field_set_dqt(self.h)
            if dqt_args:
                self.lib.orc_field_set_dqt_args(self.h, *dqt_args)

    def close(self):
        if self.h:
            self.lib.orc_field_free(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def set_scene_bounds(self, lower, upper):
        b = np.ascontiguousarray(np.concatenate([lower, upper]).astype(np.float32))
        self.lib.orc_field_set_scene_bounds(self.h, b.ctypes.data)

    def update(self, samples):
        s = np.ascontiguousarray(samples)
        self.lib.orc_field_update(self.h, s.ctypes.data, len(s))

    @property
    def iteration(self):
        return int(self.lib.orc_field_iteration(self.h))

    def field_bytes(self):
        n = self.lib.orc_field_store(self.h, None, 0)
        buf = ctypes.create_string_buffer(int(n))
        self.lib.orc_field_store(self.h, buf, n)
        return buf.raw

    def query(self, queries, volume=False, cosine=True):
        q = np.ascontiguousarray(queries)
        out = np.zeros(len(q), dtype=QUERY_OUT_DTYPE)
        self.lib.orc_field_query(self.h, int(volume), int(cosine), q.ctypes.data, out.ctypes.data, len(q))
        return out

    def query_hg(self, queries, mean_cosines):
        """Volume queries with the Henyey-Greenstein product (direction = the
        query's normal)."""
        q = np.ascontiguousarray(queries)
        g = np.ascontiguousarray(mean_cosines, dtype=np.float32)
        out = np.zeros(len(q), dtype=QUERY_OUT_DTYPE)
        self.lib.orc_field_query_hg(self.h, q.ctypes.data, g.ctypes.data, out.ctypes.data, len(q))
        return out

    def leaf_of(self, positions, volume=False):
        p = np.ascontiguousarray(np.asarray(positions, np.float32).reshape(-1, 3))
        out = np.zeros(len(p), dtype=np.int32)
        self.lib.orc_field_leaf_of(self.h, int(volume), p.ctypes.data, out.ctypes.data, len(p))
        return out


def hg_mean_cosines(n):
    """Mean cosine of the phase function for query i (the reference harness
    uses the same float arithmetic): -0.99 .. 0.99 in steps of 0.01."""
    i = np.arange(n, dtype=np.int64) % 199
    return i.astype(np.float32) * np.float32(0.01) - np.float32(0.99)


def run_reference_paths(segments, begin, max_distance):
    """Runs the reference's path segment storage (oracle/_ref/ref_paths) path
    by path for the eight flag sets (bit 0 useNEEMiWeights, bit 1
    guideDirectLight, bit 2 rrAffectsDirectContribution); returns (counts
    [8, numPaths], samples concatenated flag set by flag set and path by path,
    pixel estimates [2, numPaths, 3] for rrAffectsDirectContribution false and
    true)."""
    import sys

    sys.path.insert(0, os.path.dirname(HERE))
    from openpgl_gb300 import synthetic

    num_paths = len(begin) - 1
    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, "paths.bin")
        with open(path, "wb") as f:
            f.write(synthetic.paths_blob(segments, begin))
        subprocess.run([REF_PATHS, path, os.path.join(td, "ref"), repr(float(max_distance))], check=True)
        counts = np.fromfile(os.path.join(td, "ref.counts.bin"), dtype=np.uint32).reshape(8, num_paths)
        samples = np.fromfile(os.path.join(td, "ref.samples.bin"), dtype=synthetic.PGL_SAMPLE_DTYPE)
        pixel = np.fromfile(os.path.join(td, "ref.pixel.bin"), dtype=np.float32).reshape(2, num_paths, 3)
    return counts, samples, pixel


def run_reference_storage(samples):
    """The reference's SampleStorage holding ``samples`` (AddSamples), stored by
    SampleStorage::Store; returns (file bytes, (equal, surface size, volume
    size) of the storage read back from the file and compared with the
    original by operator==)."""
    import sys

    sys.path.insert(0, os.path.dirname(HERE))
    from openpgl_gb300 import synthetic

    with tempfile.TemporaryDirectory() as td:
        fpath = os.path.join(td, "frames.bin")
        with open(fpath, "wb") as f:
            f.write(synthetic.frames_blob([samples]))
        env = dict(os.environ, PGL_REF_STORE_SAMPLES="1", PGL_ORACLE_THREADS="1")
        subprocess.run([REF_HARNESS, fpath, os.path.join(td, "ref"), "8", "1", "32000", "1"], check=True, env=env)
        data = open(os.path.join(td, "ref.storage"), "rb").read()
        eq, ns, nv = (int(x) for x in open(os.path.join(td, "ref.storage_cmp")).read().split())
    return data, (eq, ns, nv)


def reference_sources():
    """The reference source tree as oracle/Makefile.ref finds it (its REF), or
    None when the sources are absent (as on the GPU hosts)."""
    try:
        out = subprocess.run(["make", "-s", "-C", HERE, "-f", "Makefile.ref", "print-ref"], capture_output=True,
                             text=True, timeout=60).stdout.strip()
    except (OSError, subprocess.SubprocessError):
        return None
    return out or None


def reference_available():
    return os.path.exists(REF_HARNESS)


def run_reference(frames, queries=None, max_samples_per_leaf=32000, deterministic=True, threads=1, device=8,
                  parallax=True, dqt=False, dqt_args=None):
    """Runs the reference library on ``frames`` (list of sample arrays) and
    returns (field file bytes, per-frame update ms, surface query out, volume
    query out, volume query out with the Henyey-Greenstein product of mean
    cosine hg_mean_cosines(n)).  ``dqt_args`` = (leafEstimator, splitMetric,
    splitThreshold, footprintFactor, maxLevels) overrides the quadtree
    factory's defaults."""
    import sys

    sys.path.insert(0, os.path.dirname(HERE))
    from openpgl_gb300 import synthetic

    with tempfile.TemporaryDirectory() as td:
        fpath = os.path.join(td, "frames.bin")
        with open(fpath, "wb") as f:
            f.write(synthetic.frames_blob(frames))
        args = [REF_HARNESS, fpath, os.path.join(td, "ref"), str(device), str(threads),
                str(max_samples_per_leaf), str(int(deterministic))]
        if queries is not None:
            qpath = os.path.join(td, "q.bin")
            with open(qpath, "wb") as f:
                f.write(synthetic.queries_blob(queries))
            args.append(qpath)
        env = dict(os.environ)
        env["PGL_ORACLE_THREADS"] = str(threads)
        env["PGL_REF_PLAIN_VMM"] = "0" if parallax else "1"
        env["PGL_REF_DQT"] = "1" if dqt else "0"
        env["PGL_REF_DQT_ARGS"] = ",".join(repr(v) for v in dqt_args) if dqt_args else ""
        subprocess.run(args, check=True, env=env)
        field = open(os.path.join(td, "ref.field"), "rb").read()
        times = [float(x) for x in open(os.path.join(td, "ref.times")).read().split()]
        sq = vq = hq = None
        if queries is not None:
            sq = np.fromfile(os.path.join(td, "ref.surfq.bin"), dtype=QUERY_OUT_DTYPE)
            vq = np.fromfile(os.path.join(td, "ref.volq.bin"), dtype=QUERY_OUT_DTYPE)
            hq = np.fromfile(os.path.join(td, "ref.volhgq.bin"), dtype=QUERY_OUT_DTYPE)
        return field, times, sq, vq, hq
