"""Progressive one-frame-per-call rendering (ar_render_frame, the reference's
SceneRenderer::Render(hdr, ldr, size, origin, dir, frameIndex, toneType, odd,
even, ...), core/scene.hpp:109-114, core/scene.cu:135-366) through the C ABI:

* N calls with frames 0..N-1 trace the same paths as one N-sample ar_render:
  the HDR buffer equals the reference's float32 running mean
  (lerp(hdr, sample, 1 / (1 + frame)), core/scene.cu:178-180) replayed over
  ar_render's per-sample output bit for bit, and the odd / even buffers
  likewise (core/scene.cu:181-191); the mean agrees with the FP64 mean to
  float rounding;
* the display image equals the reference's own display kernel
  (core/scene.cu:22-131, compiled into the oracle) for each tone type and
  after SetExposure;
* guided and denoised frames run and learn / record as the reference's
  settings make them."""
import numpy as np
import pytest

from aperturerendererv3_gb300 import SceneRenderer, configs
from oracle import ref_runner as rr

pytestmark = pytest.mark.gpu


def _lerp(a, b, v):
    a, b, v = np.float32(a), np.float32(b), np.float32(v)
    return (a * (np.float32(1.0) - v) + b * v).astype(np.float32)


def _replay(per):
    """The reference's float32 running means over per-sample XYZ (frames, H, W, 3)."""
    hdr = np.zeros(per.shape[1:], np.float32)
    odd = np.zeros_like(hdr)
    even = np.zeros_like(hdr)
    for f, s in enumerate(per.astype(np.float32)):
        s = np.maximum(s, np.float32(0.0))
        hdr = _lerp(hdr, s, np.float32(1.0) / np.float32(1 + f))
        half = np.float32(1.0) / np.float32(1 + (f >> 1))
        if f % 2 == 1:
            odd = _lerp(odd, s, half)
        else:
            even = _lerp(even, s, half)
    return hdr, odd, even


def test_frames_equal_one_render_and_the_reference_display(cuda_device):
    import torch
    objs, cam = configs.reference_cornell(), configs.REFERENCE_CORNELL_CAMERA
    size, n = (48, 40), 6
    r = SceneRenderer(objs)
    mean, per = r.Render(size, cam["origin"], cam["direction"], n, fov=cam["fov"], max_depth=16, per_sample=True)
    # frame 0 blends at rate 1: any finite previous contents are replaced
    hdr = torch.full((size[1], size[0], 3), 7.0, dtype=torch.float32, device="cuda")
    odd = torch.zeros_like(hdr)
    even = torch.zeros_like(hdr)
    ldr = torch.zeros((size[1], size[0]), dtype=torch.int32, device="cuda")
    for f in range(n):
        r.RenderFrame(hdr, ldr, size, cam["origin"], cam["direction"], f, 2, odd, even, fov=cam["fov"], max_depth=16)
    want_hdr, want_odd, want_even = _replay(per)
    got = hdr.cpu().numpy()
    assert np.array_equal(got, want_hdr)
    assert np.array_equal(odd.cpu().numpy(), want_odd) and np.array_equal(even.cpu().numpy(), want_even)
    np.testing.assert_allclose(got, mean, rtol=1e-5, atol=1e-6)
    if rr.available():
        assert np.array_equal(ldr.cpu().numpy().view(np.uint32), rr.frame_tonemap(got, 1.0, 2))
        for tone, exp in ((0, 1.0), (1, 1.7), (2, 0.4)):
            r.SetExposure(exp)
            r.RenderFrame(hdr, ldr, size, cam["origin"], cam["direction"], n, tone, fov=cam["fov"], max_depth=16)
            assert np.array_equal(ldr.cpu().numpy().view(np.uint32), rr.frame_tonemap(hdr.cpu().numpy(), exp, tone))
    assert r.error_word() == 0


def test_guided_and_denoised_frames(cuda_device):
    import torch
    objs, cam = configs.reference_cornell(), configs.REFERENCE_CORNELL_CAMERA
    size = (40, 32)
    r = SceneRenderer(objs)
    hdr = torch.zeros((size[1], size[0], 3), dtype=torch.float32, device="cuda")
    ldr = torch.zeros((size[1], size[0]), dtype=torch.int32, device="cuda")
    for f in range(4):
        r.RenderFrame(hdr, ldr, size, cam["origin"], cam["direction"], f, 2, fov=cam["fov"], max_depth=16, guide=1)
    assert r.guide_stats()[0] > 0  # the probes learn after every frame
    plain = torch.zeros_like(ldr)
    den = torch.zeros_like(ldr)
    hdr2 = hdr.clone()
    r.RenderFrame(hdr, plain, size, cam["origin"], cam["direction"], 4, 2, fov=cam["fov"], max_depth=16, guide=1)
    r.RenderFrame(hdr2, den, size, cam["origin"], cam["direction"], 4, 2, fov=cam["fov"], max_depth=16, guide=1,
                  denoise=True)
    assert torch.isfinite(hdr).all() and not torch.equal(plain, den)
    with pytest.raises(Exception):
        r.RenderFrame(hdr, ldr, size, cam["origin"], cam["direction"], -1, 2)
