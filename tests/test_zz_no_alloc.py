"""pglSplitSamplesDeviceNoAlloc (allocates nothing) against the existing
entry point pglSampleStorageAddSamplesDevice over two calls: the same surface
and volume records in the same order, and the same counts."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _records(storage, volume, n):
    out = np.zeros(n, dtype=storage_dtype())
    for i in range(n):
        out[i] = storage.sample(i, volume=volume)
    return out


def storage_dtype():
    from openpgl_gb300 import synthetic as syn

    return syn.PGL_SAMPLE_DTYPE


@pytest.mark.parametrize("sizes", [(30000, 70001)])
def test_no_alloc_split_matches_storage_ingest(sizes):
    import torch

    import openpgl_gb300 as pgl
    from openpgl_gb300 import synthetic as syn

    pgl.load()
    for call, n in enumerate(sizes):
        s = syn.cube_face_samples(n, 3100 + call, volume_fraction=0.3)
        d_in = torch.from_numpy(s.view(np.uint8)).cuda()
        d_surf = torch.empty(n * 40, dtype=torch.uint8, device="cuda")
        d_vol = torch.empty(n * 40, dtype=torch.uint8, device="cuda")
        d_counts = torch.zeros(2, dtype=torch.int32, device="cuda")
        pgl.split_samples_device_noalloc(d_in.data_ptr(), n, d_surf.data_ptr(), d_vol.data_ptr(), d_counts.data_ptr())
        torch.cuda.synchronize()
        ns, nv = (int(x) for x in d_counts.cpu().numpy())
        surf = d_surf.cpu().numpy().view(storage_dtype())[:ns]
        vol = d_vol.cpu().numpy().view(storage_dtype())[:nv]

        storage = pgl.SampleStorage()
        storage.add_samples_device(d_in.data_ptr(), n)
        assert (ns, nv) == (storage.size_surface, storage.size_volume)
        assert surf.tobytes() == _records(storage, False, ns).tobytes()
        assert vol.tobytes() == _records(storage, True, nv).tobytes()
        storage.release()


def test_no_alloc_split_rejects_oversized_batches():
    import openpgl_gb300 as pgl

    pgl.load()
    with pytest.raises(RuntimeError, match="67108864"):
        pgl.split_samples_device_noalloc(0, 67108864 + 1, 0, 0, 0)
