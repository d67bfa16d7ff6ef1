"""The GPU display transform against the FP64 restatement of the reference's
tonemaps (oracle/tonemap64.py): every channel within one 8-bit level."""
import numpy as np
import pytest

from aperturerendererv3_gb300 import SceneRenderer, configs
from aperturerendererv3_gb300.scene import Camera
from oracle import tonemap64

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("tone", ["aces", "gamma", "linear"])
def test_tonemap_matches_fp64(cuda_device, tone):
    rng = np.random.default_rng(1)
    xyz = rng.gamma(0.7, 0.6, (48, 64, 3))
    xyz[:4] = 0.0
    xyz[4:8] *= 50.0  # highlights through the shoulder of the curve
    r = SceneRenderer(configs.cornell_triangles())
    gpu = r.tonemap(xyz, 1.3, tone)
    ref = tonemap64.tonemap(xyz, 1.3, tone)
    assert np.abs(gpu.astype(int) - ref.astype(int)).max() <= 1


def test_camera_writes_bmp_and_pfm(cuda_device, tmp_path):
    cam_cfg = configs.CORNELL_CAMERA
    r = SceneRenderer(configs.cornell_triangles())
    cam = Camera(r, "main", 32, 24, cam_cfg["origin"], cam_cfg["direction"], fov=cam_cfg["fov"])
    img = cam.RenderToFile(str(tmp_path / "shot"), 4, max_depth=8)
    raw = (tmp_path / "shot.bmp").read_bytes()
    px = np.frombuffer(raw[54:], np.uint8).reshape(24, 32, 4)[..., [2, 1, 0, 3]]
    assert np.abs(px.astype(int) - tonemap64.tonemap(img, 1.0, "aces").astype(int)).max() <= 1
    cam.RenderToFile(str(tmp_path / "shot.pfm"), 4, max_depth=8)
    assert (tmp_path / "shot.pfm").stat().st_size == len(b"PF\n32 24\n-1.0\n") + 32 * 24 * 12
