"""Denoiser pieces that need no GPU.

* The t-quantile table the kernel uses (csrc/ar_t_quantile.h, written by
  csrc/gen_t_quantile.py) equals the reference's own table
  (core/denoise/t_quantile.cu) and Student's t quantiles at 1 - 0.0025.
* The reference's filter (oracle/_ref, denoise command) leaves an image whose
  pixels all carry identical records unchanged, and its records of a small
  render count every sample.
* The C ABI checks its arguments without a device.
"""
import re

import numpy as np
import pytest

from conftest import ROOT
from aperturerendererv3_gb300 import _lib
from oracle import ref_runner as rr

HEADER = ROOT / "aperturerendererv3_gb300" / "csrc" / "ar_t_quantile.h"
REF_TABLE = ROOT / "oracle" / "_ref" / "src" / "core" / "denoise" / "t_quantile.cu"


def header_table() -> np.ndarray:
    body = HEADER.read_text().split("{", 1)[1].split("}", 1)[0]
    vals = [float.fromhex(v.strip().rstrip("f")) for v in body.split(",") if v.strip()]
    return np.array(vals, np.float32)


def test_t_quantile_table_matches_student_t():
    stats = pytest.importorskip("scipy.stats")
    t = header_table()
    assert t.shape == (1024,)
    want = stats.t.ppf(1.0 - 0.0025, np.arange(1, 1025)).astype(np.float32)
    assert np.array_equal(t, want)


def test_t_quantile_table_matches_the_reference_table():
    if not REF_TABLE.exists():
        pytest.skip("reference sources not in this checkout")
    text = REF_TABLE.read_text()
    body = re.search(r"#define T005_LUT_INIT \{([^}]*)\}", text).group(1)
    ref = np.array([float(v.strip().rstrip("f")) for v in body.split(",") if v.strip()], np.float64).astype(np.float32)
    assert np.array_equal(header_table(), ref)


@pytest.fixture(scope="module")
def ref_available():
    if not rr.available():
        pytest.skip("reference oracle not built in this checkout")


def test_reference_filter_keeps_a_uniform_image(ref_available):
    h, w = 9, 13
    g = np.zeros((h, w), rr.GBUF_DTYPE)
    g["h"][..., :3] = np.float16(0.5).view(np.uint16)
    g["h"][..., 5] = np.float16(1.0).view(np.uint16)
    g["h"][..., 8] = np.float16(1.0).view(np.uint16)
    g["depth"] = 2.0
    g["valid"] = g["frames"] = 16
    m = np.zeros((h, w), rr.STAT_DTYPE)
    m["num"] = 16
    m["mean"] = -1.0
    m["m2n"] = 0.2
    m["m3n"] = 0.01
    img = np.full((h, w, 3), 0.37, np.float32)
    out = rr.denoise(img, g, m)
    assert np.allclose(out, img, rtol=1e-5, atol=0)


def test_reference_records_count_every_sample(ref_available):
    from aperturerendererv3_gb300 import configs
    cam = configs.CORNELL_CAMERA
    _, _, st = rr.render(configs.cornell_triangles(), (12, 8), cam["origin"], cam["direction"], 5, fov=cam["fov"],
                         max_depth=4, denoise=True)
    g, m = st["gbuffer"], st["moments"]
    assert (g["frames"] == 5).all() and (m["num"] == 5).all()
    hist = g["h"][..., 8:13].view(np.float16).astype(np.float32).sum(-1)
    assert np.allclose(hist, 1.0, atol=4e-3)


def test_denoise_abi_rejects_bad_arguments():
    lib = _lib.load()
    assert lib.ar_denoise(None, None, 0, None, 0, None) == _lib.AR_ERR_INVALID
    assert lib.ar_denoise_read(None, None, None, None, None) == _lib.AR_ERR_INVALID
    assert lib.ar_denoise_write(None, 1, 1, None, None) == _lib.AR_ERR_INVALID
    assert _lib.DENOISE_GBUF_DTYPE.itemsize == 40 and _lib.DENOISE_STAT_DTYPE.itemsize == 40
    assert _lib.DENOISE_GBUF_DTYPE == rr.GBUF_DTYPE and _lib.DENOISE_STAT_DTYPE == rr.STAT_DTYPE
