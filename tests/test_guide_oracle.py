"""The reference oracle's guided mode on the CPU (the checker the GPU guide
parity tests use): with no probes the reference's guided integrator draws
exactly what the unguided one draws (SCENE_PROBES_COUNTS = 0 skips every
probe query, core/render/render.cuh:553-562), it still collects radiance
records, one probe update turns those records into probes whose counts add up
to the records, and a frame over those probes samples differently."""
import numpy as np
import pytest

from aperturerendererv3_gb300 import configs
from oracle import ref_runner as rr


@pytest.fixture(scope="module")
def ref_available():
    if not rr.available():
        pytest.skip("reference oracle not built in this checkout")


def test_oracle_guided_loop(ref_available):
    objs, cam = configs.reference_cornell(), configs.REFERENCE_CORNELL_CAMERA
    size = (24, 24)
    empty = {"keys": np.zeros((0, 4), np.int32), "texels": np.zeros((0, 86, 4), np.float32),
             "counts": np.zeros(0, np.uint64)}
    kw = dict(fov=cam["fov"], max_depth=16, per_sample_frames=1)
    _, g0, st = rr.render(objs, size, cam["origin"], cam["direction"], 1, guide_probes=empty, **kw)
    _, p0, _ = rr.render(objs, size, cam["origin"], cam["direction"], 1, **kw)
    assert np.array_equal(g0, p0)
    rec = st["records"].reshape(-1)
    v = rec[rec["valid"] == 1]
    assert len(v) > 100
    assert np.all(v["radiance"] >= 0) and np.all(np.isfinite(v["radiance"]))
    probes = rr.guide_update(empty, v["key"], v["dir"], v["radiance"])
    assert int(probes["counts"].sum()) == len(v)
    assert len(np.unique(v["key"], axis=0)) == len(probes["keys"])
    t = probes["texels"]
    assert np.all(t[:, :85, :] >= 1e-5)  # GenerateMipmaps floors the leaf at PATH_GUIDING_PROBE_MIN_BRIGHTNESS
    np.testing.assert_allclose(t[:, 84, :3], t[:, :64, :3].mean(axis=1), rtol=1e-5)  # 1x1 mip = leaf mean
    _, g40, _ = rr.render(objs, size, cam["origin"], cam["direction"], 1, first_frame=40, guide_probes=probes, **kw)
    _, p40, _ = rr.render(objs, size, cam["origin"], cam["direction"], 1, first_frame=40, **kw)
    assert np.isfinite(g40).all() and not np.array_equal(g40, p40)
