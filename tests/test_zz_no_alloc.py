"""ar_render_noalloc, the allocation-free render entry point (for callers that
must not call cudaMalloc / cudaFree, e.g. a frame loop that cannot afford the
device-wide synchronisation of cudaFree, or an application whose memory pool
owns all device memory).  Checked through the C ABI against ar_render on the
same scene, twice in a row (the shared scratch array keeps the previous call's
contents, so the second call proves it re-initialises what it must), and
checked to leave the device's free memory unchanged.
Collected last on purpose: if it fails, every other test has already run."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from aperturerendererv3_gb300 import SceneRenderer, _lib, configs
from aperturerendererv3_gb300.scene import Material, SceneObject, sdf

pytestmark = pytest.mark.gpu


def _noalloc(lib, r, p, size):
    import torch
    out = torch.full((size[1], size[0], 3), float("nan"), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    code = lib.ar_render_noalloc(r._ctx, C.byref(p), out.data_ptr(), None)
    assert code == _lib.AR_OK, lib.ar_last_error(r._ctx)
    torch.cuda.synchronize()
    free1 = torch.cuda.mem_get_info()[0]
    return out.cpu().numpy(), free0, free1


def test_noalloc_matches_ar_render_twice(cuda_device):
    objs, cam = configs.cornell_triangles(), configs.CORNELL_CAMERA
    r = SceneRenderer(objs)
    lib = _lib.load()
    for size, spp in (((96, 64), 8), ((160, 120), 4)):  # one wave, then several waves
        ref = r.Render(size, cam["origin"], cam["direction"], spp, fov=cam["fov"], max_depth=8)
        p = r.params(size, cam["origin"], cam["direction"], spp, fov=cam["fov"], max_depth=8)
        for call in range(2):
            got, free0, free1 = _noalloc(lib, r, p, size)
            np.testing.assert_allclose(got, ref, rtol=1e-5, atol=1e-6)
            assert np.array_equal(got, ref)
            if call == 1:  # after the first call has looked the scratch array up
                assert free1 == free0, f"device free memory changed by {free0 - free1} bytes"
    assert r.error_word() == 0


def test_noalloc_camera_inside_an_sdf_object(cuda_device):
    """The camera sits inside an SDF volume object (a sphere field): both entry
    points must start the paths inside it, so the images are identical."""
    cam = configs.CORNELL_CAMERA
    objs = configs.cornell_triangles()
    objs.append(SceneObject(tuple(cam["origin"]), (0.2, 0.2, 0.2),
                            Material.CreateGlassPureColor((0.9, 0.95, 1.0), 1.5, 0.5, 40.0), (0.0, 0.0, 0.0),
                            _lib.OBJECT_SDF, sdf.CreateSDFVolume(0)))
    r2 = SceneRenderer(objs)
    assert r2.AddVolumeToCacheManager((24, 24, 24), sdfFunctor=lambda u: np.linalg.norm(u, axis=1) - 0.4) == 0
    lib = _lib.load()
    size, spp = (48, 40), 4
    ref = r2.Render(size, cam["origin"], cam["direction"], spp, fov=cam["fov"], max_depth=8)
    p = r2.params(size, cam["origin"], cam["direction"], spp, fov=cam["fov"], max_depth=8)
    got, _, _ = _noalloc(lib, r2, p, size)
    assert np.array_equal(got, ref)
    assert r2.error_word() == 0


def _max_paths():
    hdr = (Path(__file__).resolve().parents[1] / "include" / "aperture" / "ar.h").read_text()
    return int(re.search(r"#define AR_NOALLOC_MAX_PATHS (\d+)", hdr).group(1))


def test_noalloc_rejects_waves_beyond_the_scratch_limit(cuda_device):
    import torch
    objs, cam = configs.cornell_triangles(), configs.CORNELL_CAMERA
    r = SceneRenderer(objs)
    r.build()
    lib = _lib.load()
    p = r.params((32, 32), cam["origin"], cam["direction"], 1, fov=cam["fov"], max_depth=4,
                 wave_paths=_max_paths() + 1)
    out = torch.zeros((32, 32, 3), dtype=torch.float64, device="cuda")
    assert lib.ar_render_noalloc(r._ctx, C.byref(p), out.data_ptr(), None) == _lib.AR_ERR_INVALID
    assert b"exceeds the scratch limit" in lib.ar_last_error(r._ctx)
