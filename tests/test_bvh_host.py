"""The wide-BVH builder and the kernels' traversal code, run on the host:
closest-hit ids and t bit-exact against the reference BVH traversal (golden
fixture and, where the oracle is built, a live random case)."""
import ctypes as C

import numpy as np
import pytest

from conftest import GOLDEN
from aperturerendererv3_gb300 import _lib, configs


def host_trace(tris, rays):
    lib = _lib.load()
    tris = np.ascontiguousarray(tris, np.float32).reshape(-1, 9)
    rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
    ids = np.zeros(len(rays), np.int32)
    t = np.zeros(len(rays), np.float32)
    nv = C.c_int64()
    rc = lib.ar_host_trace_closest(tris.ctypes.data, len(tris), rays.ctypes.data, len(rays), ids.ctypes.data,
                                   t.ctypes.data, C.byref(nv))
    assert rc == 0
    return ids, t, nv.value


def test_golden_trace_bit_exact():
    g = np.load(GOLDEN / "trace_small.npz")
    ids, t, visits = host_trace(g["tris"], g["rays"])
    assert (g["ids"] >= 0).sum() > 100
    assert np.array_equal(ids, g["ids"])
    assert np.array_equal(t.view(np.uint32), g["t"].view(np.uint32))
    assert visits > 0


def test_dense_random_case_vs_live_oracle():
    from oracle import ref_runner as rr
    if not rr.available():
        pytest.skip("reference oracle not built in this checkout")
    tris = configs.random_triangles(50_000, seed=9)
    cam = configs.BVH_STRESS_CAMERA
    rays = configs.pinhole_rays(96, 64, cam["origin"], cam["direction"], cam["fov"])
    rays[::7, 3] = 1.2   # some rays with tmin inside the cloud
    rays[::5, 7] = 1.6   # and some with a tmax inside it
    ids, t, _ = host_trace(tris, rays)
    rids, rt, _ = rr.trace(tris, rays)
    assert (rids >= 0).mean() > 0.3
    assert np.array_equal(ids, rids)
    assert np.array_equal(t.view(np.uint32), rt.view(np.uint32))


def test_degenerate_inputs():
    # identical triangles (all centroids equal) and a zero-area triangle
    tri = np.array([0, 0, 0, 1, 0, 0, 0, 1, 0], np.float32)
    tris = np.tile(tri, (40, 1))
    tris[5] = [0.2, 0.2, 0, 0.2, 0.2, 0, 0.2, 0.2, 0]
    rays = np.array([[0.25, 0.25, 1.0, 0.0, 0.0, 0.0, -1.0, np.inf]], np.float32)
    ids, t, _ = host_trace(tris, rays)
    assert ids[0] == 0  # ties at equal t resolve to the smallest id
    assert abs(t[0] - 1.0) < 1e-6
