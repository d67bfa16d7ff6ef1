"""The denoiser on the GPU against the reference's own denoiser code (oracle/_ref).

* Records: the per-pixel G-buffer means and sample moments recorded during a
  GPU render equal the reference's records of the same render (first-hit ids
  are bit-exact, so albedo / metallic / roughness / shading-model halves and
  the sample counts are equal everywhere; normals, distances and moments follow
  the per-sample radiance, equal to a few float ulps).
* Records are independent of how samples split into waves and calls: one call
  of 8 samples equals two calls of 4 (first_frame 0 then 4) and a run with
  small waves, bit for bit.
* Filter: on the same image and records, the GPU filter equals the reference's
  filter loop bit for bit, on the records the GPU made, on the records the
  reference made, and at image sizes that cut the 32 x 8 tiles.
* The filtered image of a noisy render is smoother than the raw one.
"""
import numpy as np
import pytest

from aperturerendererv3_gb300 import SceneRenderer, configs
from oracle import ref_runner as rr

pytestmark = pytest.mark.gpu

CAM = configs.CORNELL_CAMERA


@pytest.fixture(scope="module")
def ref_available():
    if not rr.available():
        pytest.skip("reference oracle not built in this checkout")


def halves(g, lo, hi):
    return g["h"][..., lo:hi]


def test_records_match_the_reference(cuda_device, ref_available):
    objs = configs.cornell_triangles()
    size, spp = (40, 30), 8
    r = SceneRenderer(objs)
    img = r.Render(size, CAM["origin"], CAM["direction"], spp, fov=CAM["fov"], max_depth=8, denoise=True)
    g, m = r.denoise_records()
    _, _, st = rr.render(objs, size, CAM["origin"], CAM["direction"], spp, fov=CAM["fov"], max_depth=8, denoise=True)
    rg, rm = st["gbuffer"], st["moments"]
    assert np.array_equal(g["valid"], rg["valid"]) and np.array_equal(g["frames"], rg["frames"])
    assert np.array_equal(m["num"], rm["num"])
    # albedo, metallic, roughness, shading-model histogram: exact
    for lo, hi in ((0, 3), (6, 8), (8, 13)):
        assert np.array_equal(halves(g, lo, hi), halves(rg, lo, hi)), (lo, hi)
    # normals: the same half, or one half ulp apart
    diff = np.abs(halves(g, 3, 6).astype(np.int32) - halves(rg, 3, 6).astype(np.int32))
    assert (diff <= 1).all() and (diff == 0).mean() > 0.99
    assert np.allclose(g["depth"], rg["depth"], rtol=1e-5, atol=0)
    # moments follow the per-sample radiance (equal to a few ulps; a path may part ways)
    for f in ("mean", "m2n", "m3n"):
        close = np.isclose(m[f], rm[f], rtol=1e-3, atol=1e-5).all(-1)
        assert close.mean() > 0.97, (f, close.mean())
    assert np.isfinite(img).all()


def test_records_do_not_depend_on_waves_or_calls(cuda_device):
    objs = configs.cornell_triangles()
    size = (24, 16)
    a = SceneRenderer(objs)
    a.Render(size, CAM["origin"], CAM["direction"], 8, fov=CAM["fov"], max_depth=8, denoise=True)
    g1, m1 = a.denoise_records()
    b = SceneRenderer(objs)
    b.Render(size, CAM["origin"], CAM["direction"], 4, fov=CAM["fov"], max_depth=8, denoise=True)
    b.Render(size, CAM["origin"], CAM["direction"], 4, fov=CAM["fov"], max_depth=8, denoise=True, first_frame=4)
    g2, m2 = b.denoise_records()
    c = SceneRenderer(objs)
    c.Render(size, CAM["origin"], CAM["direction"], 8, fov=CAM["fov"], max_depth=8, denoise=True, wave_paths=1000)
    g3, m3 = c.denoise_records()
    for g, m in ((g2, m2), (g3, m3)):
        assert g.tobytes() == g1.tobytes()
        assert m.tobytes() == m1.tobytes()


@pytest.mark.parametrize("size", [(40, 30), (37, 13), (1, 1), (5, 41), (70, 9)])
def test_filter_equals_the_reference_filter(cuda_device, ref_available, size):
    objs = configs.cornell_triangles()
    r = SceneRenderer(objs)
    img = r.Render(size, CAM["origin"], CAM["direction"], 8, fov=CAM["fov"], max_depth=8, denoise=False)
    r.Render(size, CAM["origin"], CAM["direction"], 8, fov=CAM["fov"], max_depth=8, denoise=True)
    g, m = r.denoise_records()
    gpu = r.denoise(img)
    ref = rr.denoise(img, g, m)
    assert np.array_equal(gpu.astype(np.float32), ref)
    assert np.array_equal(gpu, gpu.astype(np.float32).astype(np.float64))


def test_filter_on_the_references_records(cuda_device, ref_available):
    objs = configs.reference_cornell()
    cam = configs.REFERENCE_CORNELL_CAMERA
    size = (48, 36)
    mean, _, st = rr.render(objs, size, cam["origin"], cam["direction"], 8, fov=cam["fov"], max_depth=16,
                            denoise=True)
    r = SceneRenderer(objs)
    r.set_denoise_records(st["gbuffer"], st["moments"])
    gpu = r.denoise(mean)
    ref = rr.denoise(mean, st["gbuffer"], st["moments"])
    assert np.array_equal(gpu.astype(np.float32), ref)


def test_filtered_image_is_smoother(cuda_device):
    objs = configs.cornell_triangles()
    r = SceneRenderer(objs)
    size = (64, 64)
    raw = r.Render(size, CAM["origin"], CAM["direction"], 4, fov=CAM["fov"], max_depth=8)
    den = r.Render(size, CAM["origin"], CAM["direction"], 4, fov=CAM["fov"], max_depth=8, denoise=True)

    def tv(x):
        y = x[..., 1]
        return np.abs(np.diff(y, axis=0)).mean() + np.abs(np.diff(y, axis=1)).mean()

    assert tv(den) < 0.7 * tv(raw)
    assert np.isfinite(den).all() and (den >= 0).all()


def test_device_tensors_and_errors(cuda_device):
    import torch
    objs = configs.cornell_triangles()
    r = SceneRenderer(objs)
    with pytest.raises(Exception):
        r.denoise(np.zeros((4, 4, 3)))          # nothing recorded yet
    img = r.Render((16, 8), CAM["origin"], CAM["direction"], 2, fov=CAM["fov"], max_depth=4, denoise=True)
    raw = r.Render((16, 8), CAM["origin"], CAM["direction"], 2, fov=CAM["fov"], max_depth=4)
    t = torch.as_tensor(raw, device="cuda")
    out = r.denoise(t)
    assert out.is_cuda and np.array_equal(out.cpu().numpy(), img)
    with pytest.raises(ValueError):
        r.denoise(np.zeros((8, 17, 3)))
