"""Headless image output (host, no GPU): the BMP writer lays out the
reference's 32-bit top-down BGRA file (core/camera.cu:10-62) and the PFM writer
a little-endian bottom-up float map."""
import numpy as np

from aperturerendererv3_gb300.scene import write_bmp, write_pfm


def test_bmp_layout(tmp_path):
    rng = np.random.default_rng(0)
    rgba = rng.integers(0, 256, (5, 7, 4), dtype=np.uint8)
    p = tmp_path / "img.bmp"
    write_bmp(str(p), rgba)
    raw = p.read_bytes()
    assert raw[:2] == b"BM"
    assert int.from_bytes(raw[2:6], "little") == 54 + 5 * 7 * 4 == len(raw)
    assert int.from_bytes(raw[18:22], "little", signed=True) == 7
    assert int.from_bytes(raw[22:26], "little", signed=True) == -5  # top-down
    assert int.from_bytes(raw[28:30], "little") == 32
    px = np.frombuffer(raw[54:], np.uint8).reshape(5, 7, 4)
    assert np.array_equal(px[..., [2, 1, 0, 3]], rgba)


def test_pfm_layout(tmp_path):
    img = np.arange(4 * 3 * 3, dtype=np.float64).reshape(4, 3, 3)
    p = tmp_path / "img.pfm"
    write_pfm(str(p), img)
    raw = p.read_bytes()
    head = b"PF\n3 4\n-1.0\n"
    assert raw.startswith(head)
    data = np.frombuffer(raw[len(head):], "<f4").reshape(4, 3, 3)
    assert np.array_equal(data[::-1], img.astype(np.float32))
