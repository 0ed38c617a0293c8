#!/usr/bin/env python3
"""Generates the golden fixtures of this directory by running the reference
Open PGL library itself (compiled from the reference sources by
oracle/Makefile.ref into oracle/_ref/, CPU_8 device, deterministic field,
serial scheduling) on seeded synthetic inputs.

Each case stores:
  <case>.field.gz   the reference's field file after the last frame
                    (pglFieldStoreToFile layout, update timings zeroed)
  <case>.queries.npz  "surface": guided surface queries (Init + cosine
                    product + SamplePDF + IncomingRadiancePDF per query),
                    "volume": guided volume queries (Init + SamplePDF +
                    IncomingRadiancePDF), "volume_hg": the same with the
                    single-lobe Henyey-Greenstein product first (direction =
                    the query's normal, mean cosine pyoracle.hg_mean_cosines)
and paths.npz the samples and pixel estimates of the reference's path
segment storage on synthetic paths (counts per flag set and path, samples,
pixel estimates), and storage.samples.gz a sample storage file written by the
reference's SampleStorage::Store (STORAGE below); manifest.json records the generator calls and the SHA-256
of every generated input, so a test can check that the generators still produce the
same inputs before it compares outputs.

Run from the repository root on a machine that has the reference sources:
    make -C oracle -f Makefile.ref REF=/path/to/openpgl
    python tests/golden/make_golden.py
"""

from __future__ import annotations

import gzip
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "oracle")]

# case name -> (generator, per-frame arguments, queries, maxSamplesPerLeaf)
CASES = {
    "cube_single": dict(gen="cube_face_samples", frames=[dict(n=65536, seed=101)],
                        queries=dict(n=4096, seed=102), leaf=8000),
    "cube_multiframe_volume": dict(gen="cube_face_samples",
                                   frames=[dict(n=32768, seed=110 + i, volume_fraction=0.25) for i in range(3)],
                                   queries=dict(n=4096, seed=113), leaf=4000),
    "clusters": dict(gen="cluster_samples", frames=[dict(n=60000, seed=120 + i, num_clusters=64) for i in range(2)],
                     queries=dict(n=4096, seed=122, model_seed=1234), leaf=2000),
    # the plain VMM field type (no parallax compensation)
    "cube_plain_vmm": dict(gen="cube_face_samples",
                           frames=[dict(n=32768, seed=130 + i, volume_fraction=0.25) for i in range(3)],
                           queries=dict(n=4096, seed=133), leaf=4000, parallax=False),
    # the directional quadtree field type (reference defaults of PGLDQTFactoryArguments)
    "cube_dqt": dict(gen="cube_face_samples", frames=[dict(n=32768, seed=140 + i, volume_fraction=0.25) for i in range(2)],
                     queries=dict(n=4096, seed=142), leaf=4000, dqt=True),
    # its other branches: PER_LEAF estimator, SECOND_MOMENT metric, threshold 0.02,
    # footprint 0.5, 8 levels
    "cube_dqt_per_leaf": dict(gen="cube_face_samples",
                              frames=[dict(n=32768, seed=150 + i, volume_fraction=0.25) for i in range(2)],
                              queries=dict(n=4096, seed=152), leaf=4000, dqt=True, dqt_args=[1, 1, 0.02, 0.5, 8]),
}


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def build_inputs(case):
    from openpgl_gb300 import synthetic as syn

    gen = getattr(syn, case["gen"])
    frames = [gen(**kw) for kw in case["frames"]]
    queries = syn.queries(**case["queries"])
    return frames, queries


# path segment case: generator arguments and the storage's max distance
PATHS = dict(num_paths=1024, seed=5, max_len=12, max_distance=3.0)


def build_paths(case):
    from openpgl_gb300 import synthetic as syn

    return syn.path_segments(case["num_paths"], case["seed"], case["max_len"])


# sample storage file case: generator arguments (2,000 records, 30 % inside-volume)
STORAGE = dict(n=2000, seed=7, volume_fraction=0.3)


def build_storage(case):
    from openpgl_gb300 import synthetic as syn

    return syn.cube_face_samples(**case)


def write_storage(pyoracle, manifest):
    """A sample storage file (SampleDataStorage.h:176-216) written by the
    reference's SampleStorage::Store, and what the reference reads back."""
    samples = build_storage(STORAGE)
    data, (eq, ns, nv) = pyoracle.run_reference_storage(samples)
    with gzip.GzipFile(os.path.join(HERE, "storage.samples.gz"), "wb", compresslevel=9, mtime=0) as f:
        f.write(data)
    manifest["storage"] = dict(STORAGE, samples_sha256=sha(samples), file_sha256=hashlib.sha256(data).hexdigest(),
                               reference_reads_back_equal=bool(eq), surface=ns, volume=nv)
    print("storage", len(data), "bytes,", ns, "surface,", nv, "volume, read back equal:", bool(eq))


def main():
    import argparse

    import fieldfile
    import pyoracle

    ap = argparse.ArgumentParser()
    ap.add_argument("--only", choices=["storage"], help="regenerate one fixture, keep the others and the manifest")
    args = ap.parse_args()
    if not pyoracle.reference_available():
        sys.exit("oracle/_ref/ref_harness is missing: build it with oracle/Makefile.ref first")
    if args.only == "storage":
        with open(os.path.join(HERE, "manifest.json")) as f:
            manifest = json.load(f)
        write_storage(pyoracle, manifest)
        with open(os.path.join(HERE, "manifest.json"), "w") as f:
            json.dump(manifest, f, indent=1)
        return
    manifest = {"generator": "openpgl_gb300.synthetic", "reference": "Open PGL 0.6.0, CPU_8, deterministic, serial",
                "cases": {}}
    for name, case in CASES.items():
        frames, queries = build_inputs(case)
        field, _, sq, vq, hq = pyoracle.run_reference(frames, queries, max_samples_per_leaf=case["leaf"],
                                                      parallax=case.get("parallax", True), dqt=case.get("dqt", False),
                                                      dqt_args=case.get("dqt_args"),
                                                  deterministic=True, threads=1, device=8)
        field = fieldfile.strip_timings(field)
        with gzip.open(os.path.join(HERE, f"{name}.field.gz"), "wb", compresslevel=9) as f:
            f.write(field)
        np.savez_compressed(os.path.join(HERE, f"{name}.queries.npz"), surface=sq, volume=vq, volume_hg=hq)
        manifest["cases"][name] = dict(case, frame_sha256=[sha(f) for f in frames], queries_sha256=sha(queries),
                                       field_sha256=hashlib.sha256(field).hexdigest())
        print(name, len(field), "bytes,", len(fieldfile.read_field_file(field)["surface"]["regions"]), "surface regions")
    # path segments -> samples (PathSegmentDataStorage), all eight flag sets
    segs, begin = build_paths(PATHS)
    counts, samples, pixel = pyoracle.run_reference_paths(segs, begin, PATHS["max_distance"])
    np.savez_compressed(os.path.join(HERE, "paths.npz"), counts=counts, samples=samples, pixel=pixel)
    manifest["paths"] = dict(PATHS, segments_sha256=sha(segs), begin_sha256=sha(begin))
    print("paths", len(begin) - 1, "paths,", len(segs), "segments,", len(samples), "samples")
    write_storage(pyoracle, manifest)
    with open(os.path.join(HERE, "manifest.json"), "w") as f:
        json.dump(manifest, f, indent=1)


if __name__ == "__main__":
    main()
