"""The sample storage file written by the reference (tests/golden/
storage.samples.gz, SampleStorage::Store on seeded records): its layout as
SampleDataStorage.h:176-216 and storeSampleDataStorageToFile (:57-70) write
it.  A header string with its terminating zero, then the surface records and
the volume records, each as a u64 count followed by 40-byte PGLSampleData
records, in the order they were added (records flagged inside-volume, flag
bit 1, go to the volume side)."""

import gzip
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
HEADER = b"OPENPGL_0.6.0_SAMPLE_STORAGE\0"


def golden_storage():
    return gzip.open(os.path.join(GOLDEN, "storage.samples.gz")).read()


def expected_storage_bytes(samples):
    """The file the reference writes for a storage holding `samples`."""
    vol = (samples["flags"] & 2) != 0
    out = [HEADER]
    for side in (samples[~vol], samples[vol]):
        out.append(np.uint64(len(side)).tobytes())
        out.append(np.ascontiguousarray(side).tobytes())
    return b"".join(out)


def storage_inputs():
    sys.path.insert(0, GOLDEN)
    import make_golden

    manifest = json.load(open(os.path.join(GOLDEN, "manifest.json")))
    samples = make_golden.build_storage(make_golden.STORAGE)
    return samples, manifest["storage"]


def test_reference_storage_file_layout():
    samples, meta = storage_inputs()
    assert make_golden_sha(samples) == meta["samples_sha256"]
    data = golden_storage()
    assert data == expected_storage_bytes(samples)
    assert meta["reference_reads_back_equal"]
    vol = (samples["flags"] & 2) != 0
    assert (meta["surface"], meta["volume"]) == (int((~vol).sum()), int(vol.sum()))


def make_golden_sha(a):
    import hashlib

    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()
