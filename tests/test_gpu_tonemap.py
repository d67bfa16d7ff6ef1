"""The GPU display transform (ar_tonemap) against the reference's own pixel loop
of Camera::RenderToFile with core/tonemap.cuh's curves, compiled into the
reference oracle (oracle/_ref): every byte equal.  The FP64 restatement
(oracle/tonemap64.py) stays as a second, independent check (one 8-bit level)."""
import numpy as np
import pytest

from aperturerendererv3_gb300 import SceneRenderer, configs
from aperturerendererv3_gb300.scene import Camera
from oracle import ref_runner as rr
from oracle import tonemap64

pytestmark = pytest.mark.gpu


def _image():
    rng = np.random.default_rng(1)
    xyz = rng.gamma(0.7, 0.6, (48, 64, 3)).astype(np.float32).astype(np.float64)
    xyz[:4] = 0.0
    xyz[4:8] *= 50.0  # highlights through the shoulder of the curve
    xyz[8, :8] = [[1e-8, 0, 0], [0, 1e-8, 0], [70000.0, 70000.0, 70000.0], [0.3, 0.3, 0.3],
                  [1.0, 1.0, 1.0], [0.0, 0.5, 2.0], [5.0, 0.0, 0.0], [0.95047, 1.0, 1.08883]]
    return xyz


@pytest.mark.parametrize("tone", ["aces", "gamma", "linear"])
def test_tonemap_matches_reference(cuda_device, tone):
    xyz = _image()
    r = SceneRenderer(configs.cornell_triangles())
    gpu = r.tonemap(xyz, 1.3, tone)
    if rr.available():
        ref = rr.tonemap(xyz.astype(np.float32), 1.3, tone)
        assert np.array_equal(gpu, ref), int((gpu != ref).sum())
    assert np.abs(gpu.astype(int) - tonemap64.tonemap(xyz, 1.3, tone).astype(int)).max() <= 1


def test_camera_writes_bmp_and_pfm(cuda_device, tmp_path):
    cam_cfg = configs.CORNELL_CAMERA
    r = SceneRenderer(configs.cornell_triangles())
    cam = Camera(r, "main", 32, 24, cam_cfg["origin"], cam_cfg["direction"], fov=cam_cfg["fov"])
    img = cam.RenderToFile(str(tmp_path / "shot"), 4, max_depth=8)
    raw = (tmp_path / "shot.bmp").read_bytes()
    px = np.frombuffer(raw[54:], np.uint8).reshape(24, 32, 4)[..., [2, 1, 0, 3]]
    if rr.available():
        assert np.array_equal(px, rr.tonemap(img.astype(np.float32), 1.0, "aces"))
    assert np.abs(px.astype(int) - tonemap64.tonemap(img, 1.0, "aces").astype(int)).max() <= 1
    cam.RenderToFile(str(tmp_path / "shot.pfm"), 4, max_depth=8)
    assert (tmp_path / "shot.pfm").stat().st_size == len(b"PF\n32 24\n-1.0\n") + 32 * 24 * 12
