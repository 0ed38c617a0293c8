"""pglSplitSamplesDeviceNoAlloc (allocates nothing) against the existing
entry point pglSampleStorageAddSamplesDevice over two calls: the same surface
and volume records in the same order, and the same counts."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _records(storage, tmp_path):
    """Both sides of a storage, read back through its file (the reference's
    layout: a header string, then per side a u64 count and the records)."""
    path = tmp_path / "split.storage"
    assert storage.store(str(path))
    data = path.read_bytes()
    off = data.index(b"\0") + 1
    sides = []
    for _ in range(2):
        n = int(np.frombuffer(data, np.uint64, 1, off)[0])
        off += 8
        sides.append(np.frombuffer(data, storage_dtype(), n, off))
        off += n * 40
    return sides


def storage_dtype():
    from openpgl_gb300 import synthetic as syn

    return syn.PGL_SAMPLE_DTYPE


# two calls in a row each: ragged sizes (part of a tile), sizes whose scan
# gives some scan threads several tiles (more than 1024 tiles of 1024
# records), an exact multiple of the tile, and empty batches
@pytest.mark.parametrize("sizes", [(30000, 70001), (1024 * 1500 + 17, 65536), (0, 1024), (4096, 0)])
def test_no_alloc_split_matches_storage_ingest(sizes, tmp_path):
    import torch

    import openpgl_gb300 as pgl
    from openpgl_gb300 import synthetic as syn

    pgl.load()
    for call, n in enumerate(sizes):
        s = syn.cube_face_samples(max(n, 1), 3100 + call, volume_fraction=0.3)[:n]
        d_in = torch.from_numpy(s.view(np.uint8)).cuda()
        d_surf = torch.empty(max(n, 1) * 40, dtype=torch.uint8, device="cuda")
        d_vol = torch.empty(max(n, 1) * 40, dtype=torch.uint8, device="cuda")
        # counts start as garbage: the call must write both
        d_counts = torch.full((2,), -1, dtype=torch.int32, device="cuda")
        pgl.split_samples_device_noalloc(d_in.data_ptr(), n, d_surf.data_ptr(), d_vol.data_ptr(), d_counts.data_ptr())
        torch.cuda.synchronize()
        ns, nv = (int(x) for x in d_counts.cpu().numpy())
        surf = d_surf.cpu().numpy().view(storage_dtype())[:ns]
        vol = d_vol.cpu().numpy().view(storage_dtype())[:nv]

        storage = pgl.SampleStorage()
        if n:
            storage.add_samples_device(d_in.data_ptr(), n)
        assert (ns, nv) == (storage.size_surface, storage.size_volume)
        ref_surf, ref_vol = _records(storage, tmp_path)
        assert surf.tobytes() == ref_surf.tobytes()
        assert vol.tobytes() == ref_vol.tobytes()
        storage.release()


def test_no_alloc_split_rejects_oversized_batches():
    import openpgl_gb300 as pgl

    pgl.load()
    with pytest.raises(RuntimeError, match="67108864"):
        pgl.split_samples_device_noalloc(0, 67108864 + 1, 0, 0, 0)
