"""ar_render_noalloc, the allocation-free render entry point (for callers that
must not call cudaMalloc / cudaFree, e.g. a frame loop that cannot afford the
device-wide synchronisation of cudaFree, or an application whose memory pool
owns all device memory).  Checked through the C ABI against ar_render on the
same scene, twice in a row (the shared scratch array keeps the previous call's
contents, so the second call proves it re-initialises what it must).
Collected last on purpose: if it fails, every other test has already run."""
import ctypes as C

import numpy as np
import pytest

from aperturerendererv3_gb300 import SceneRenderer, _lib, configs

pytestmark = pytest.mark.gpu


def test_noalloc_matches_ar_render_twice(cuda_device):
    import torch
    objs, cam = configs.cornell_triangles(), configs.CORNELL_CAMERA
    r = SceneRenderer(objs)
    lib = _lib.load()
    for size, spp in (((96, 64), 8), ((160, 120), 4)):  # one wave, then several waves
        ref = r.Render(size, cam["origin"], cam["direction"], spp, fov=cam["fov"], max_depth=8)
        p = r.params(size, cam["origin"], cam["direction"], spp, fov=cam["fov"], max_depth=8)
        for _ in range(2):
            out = torch.full((size[1], size[0], 3), float("nan"), dtype=torch.float64, device="cuda")
            code = lib.ar_render_noalloc(r._ctx, C.byref(p), out.data_ptr(), None)
            assert code == _lib.AR_OK, lib.ar_last_error(r._ctx)
            torch.cuda.synchronize()
            got = out.cpu().numpy()
            np.testing.assert_allclose(got, ref, rtol=1e-5, atol=1e-6)
            assert np.array_equal(got, ref)
    assert r.error_word() == 0


def test_noalloc_rejects_waves_beyond_the_scratch_limit(cuda_device):
    import torch
    objs, cam = configs.cornell_triangles(), configs.CORNELL_CAMERA
    r = SceneRenderer(objs)
    r.build()
    lib = _lib.load()
    p = r.params((32, 32), cam["origin"], cam["direction"], 1, fov=cam["fov"], max_depth=4,
                 wave_paths=43264 + 1)
    out = torch.zeros((32, 32, 3), dtype=torch.float64, device="cuda")
    assert lib.ar_render_noalloc(r._ctx, C.byref(p), out.data_ptr(), None) == _lib.AR_ERR_INVALID
    assert b"exceeds the scratch limit" in lib.ar_last_error(r._ctx)
