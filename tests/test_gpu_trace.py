"""Closest-hit / any-hit parity of the sm_103a wide-BVH traversal with the
reference BVH (core/render/intersection.cuh:148-310) and with brute force:
primitive ids bit-exact, t bit-exact (same watertight test on both sides)."""
import numpy as np
import pytest

from conftest import GOLDEN
from aperturerendererv3_gb300 import Material, SceneObject, SceneRenderer, TriangleMesh, configs

pytestmark = pytest.mark.gpu


def mesh_renderer(tris: np.ndarray) -> SceneRenderer:
    tris = np.ascontiguousarray(tris, np.float32).reshape(-1, 9)
    n = len(tris)
    mesh = TriangleMesh(tris.reshape(-1, 3), np.arange(3 * n, dtype=np.uint32).reshape(-1, 3),
                        np.zeros(n, np.int32), [Material.CreateDiffusePureColor((0.5, 0.5, 0.5))])
    return SceneRenderer([], mesh=mesh)


def gpu_trace(r: SceneRenderer, rays: np.ndarray):
    import torch
    d = torch.from_numpy(np.ascontiguousarray(rays, np.float32)).cuda()
    ids, t = r.trace_closest(d)
    hit = r.trace_any(d)
    torch.cuda.synchronize()
    return ids.cpu().numpy(), t.cpu().numpy(), hit.cpu().numpy()


def test_golden_closest_hit_bit_exact(cuda_device):
    g = np.load(GOLDEN / "trace_small.npz")
    r = mesh_renderer(g["tris"])
    ids, t, hit = gpu_trace(r, g["rays"])
    assert np.array_equal(ids, g["ids"])
    assert np.array_equal(t.view(np.uint32), g["t"].view(np.uint32))
    assert np.array_equal(hit.astype(bool), g["ids"] >= 0)
    assert r.error_word() == 0


def bounce_rays(tris, rays, ids, t, seed=5):
    """One cosine-hemisphere bounce ray per hit, from the hit point."""
    rng = np.random.default_rng(seed)
    hit = ids >= 0
    o = rays[hit, 0:3] + rays[hit, 4:7] * t[hit, None]
    v = tris[ids[hit]].reshape(-1, 3, 3).astype(np.float64)
    n = np.cross(v[:, 1] - v[:, 0], v[:, 2] - v[:, 0])
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    flip = np.einsum("ij,ij->i", n, rays[hit, 4:7]) > 0
    n[flip] *= -1
    u1, u2 = rng.random(len(n)), rng.random(len(n))
    r_, phi = np.sqrt(u1), 2 * np.pi * u2
    a = np.where(np.abs(n[:, 0:1]) > 0.9, [[0.0, 1.0, 0.0]], [[1.0, 0.0, 0.0]])
    tt = np.cross(n, a)
    tt /= np.linalg.norm(tt, axis=1, keepdims=True)
    bb = np.cross(n, tt)
    d = tt * (r_ * np.cos(phi))[:, None] + bb * (r_ * np.sin(phi))[:, None] + n * np.sqrt(1 - u1)[:, None]
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    out = np.zeros((len(d), 8), np.float32)
    out[:, 0:3] = o
    out[:, 3] = 1e-4
    out[:, 4:7] = d
    out[:, 7] = np.inf
    return out


def test_random_triangles_primary_and_bounce_vs_oracle(cuda_device):
    from oracle import ref_runner as rr
    tris = configs.random_triangles(200_000, seed=1)
    cam = configs.BVH_STRESS_CAMERA
    rays = configs.pinhole_rays(320, 180, cam["origin"], cam["direction"], cam["fov"])
    r = mesh_renderer(tris)
    ids, t, hit = gpu_trace(r, rays)
    assert np.array_equal(hit.astype(bool), ids >= 0)
    b = bounce_rays(tris, rays, ids, t)
    bids, bt, bhit = gpu_trace(r, b)
    assert (ids >= 0).mean() > 0.5
    if not rr.available():
        pytest.skip("reference oracle unavailable on this machine; golden test covers parity")
    rids, rt, _ = rr.trace(tris, rays)
    assert np.array_equal(ids, rids)
    assert np.array_equal(t.view(np.uint32), rt.view(np.uint32))
    rbids, rbt, _ = rr.trace(tris, b)
    assert np.array_equal(bids, rbids)
    assert np.array_equal(bt.view(np.uint32), rbt.view(np.uint32))
    assert r.error_word() == 0


def test_edge_cases_empty_ray_batch_and_miss_everything(cuda_device):
    import torch
    tris = configs.random_triangles(1000, seed=2)
    r = mesh_renderer(tris)
    ids, t = r.trace_closest(torch.zeros((0, 8), dtype=torch.float32, device="cuda"))
    assert ids.numel() == 0
    rays = np.zeros((64, 8), np.float32)
    rays[:, 0:3] = (5.0, 5.0, 5.0)
    rays[:, 4:7] = (0.0, 0.0, 1.0)  # pointing away from the unit cube
    rays[:, 7] = np.inf
    ids, t, hit = gpu_trace(r, rays)
    assert np.all(ids == -1) and np.all(hit == 0) and np.all(t == -1)
    # tmax shorter than any hit: no hit
    rays = configs.pinhole_rays(8, 8, (0.5, 0.5, 2.0), (0, 0, -1), 20.0)
    rays[:, 7] = 0.5
    ids, _, hit = gpu_trace(r, rays)
    assert np.all(ids == -1) and np.all(hit == 0)


def test_single_triangle_and_analytic_objects(cuda_device):
    import torch
    objs = [SceneObject.Triangle((0, 0, 0), (1, 0, 0), (0, 1, 0), Material()),
            SceneObject((3.0, 0.0, 0.0), (0.5, 0.5, 0.5), Material(), (0.0, 30.0, 0.0), 0),
            SceneObject((-3.0, 0.0, 0.0), (0.5, 0.5, 0.5), Material(), (0.0, 0.0, 0.0), 1)]
    r = SceneRenderer(objs)
    rays = np.array([[0.2, 0.2, 5.0, 0.0, 0.0, 0.0, -1.0, np.inf],
                     [3.0, 0.0, 5.0, 0.0, 0.0, 0.0, -1.0, np.inf],
                     [-3.0, 0.0, 5.0, 0.0, 0.0, 0.0, -1.0, np.inf],
                     [9.0, 9.0, 5.0, 0.0, 0.0, 0.0, -1.0, np.inf]], np.float32)
    ids, t, hit = gpu_trace(r, rays)
    assert list(ids) == [0, 1, 2, -1]
    assert abs(t[0] - 5.0) < 1e-6
    assert abs(t[2] - 4.5) < 1e-6
    assert list(hit) == [1, 1, 1, 0]
