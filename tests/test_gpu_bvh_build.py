"""The GPU BVH build (AR_BUILD_GPU: Morton codes, radix sort, Karras radix
tree, collapse to the 8-wide format) against the host binned-SAH build.

Closest hits do not depend on the tree, so the GPU-built BVH must return the
same primitive ids and distances for the same rays, and renders through it
must equal renders through the host-built BVH bit for bit; every primitive
appears in exactly one leaf slot.  Sizes from 1 primitive to the 8.4M-triangle
terrain; duplicate centroids (all Morton codes equal) included.
"""
import numpy as np
import pytest

from aperturerendererv3_gb300 import SceneRenderer, configs
from aperturerendererv3_gb300.scene import Material, TriangleMesh

pytestmark = pytest.mark.gpu


def mesh_of(tris):
    v = tris.reshape(-1, 3).astype(np.float32)
    return TriangleMesh(v, np.arange(len(v), dtype=np.uint32).reshape(-1, 3), np.zeros(len(tris), np.int32),
                        [Material.CreateDiffusePureColor((0.5, 0.5, 0.5))])


def both(objs, mesh):
    a = SceneRenderer(objs, mesh=mesh)
    a.build()
    b = SceneRenderer(objs, mesh=mesh)
    b.set_build_mode("gpu")
    b.build()
    return a, b


def random_rays(n, seed, lo=-0.2, hi=1.2):
    rng = np.random.default_rng(seed)
    o = rng.uniform(lo, hi, (n, 3))
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return np.concatenate([o, np.full((n, 1), 1e-4), d, np.full((n, 1), np.inf)], 1).astype(np.float32)


@pytest.mark.parametrize("n", [1, 2, 3, 4, 9, 100, 5000, 200_000])
def test_gpu_build_answers_like_the_host_build(cuda_device, n):
    import torch
    tris = configs.random_triangles(n, seed=n)
    a, b = both([], mesh_of(tris))
    sa, sb = a.stats(), b.stats()
    assert sb["slots"] == n and sa["slots"] == n
    rays = torch.as_tensor(random_rays(20_000, seed=1), device="cuda")
    ia, ta = a.trace_closest(rays)
    ib, tb = b.trace_closest(rays)
    assert torch.equal(ia, ib)
    assert torch.equal(ta, tb)
    assert torch.equal(a.trace_any(rays), b.trace_any(rays))
    assert b.error_word() == 0


def test_duplicate_centroids(cuda_device):
    import torch
    base = configs.random_triangles(1, seed=3)
    tris = np.repeat(base, 64, axis=0)  # 64 identical triangles: one Morton code
    a, b = both([], mesh_of(tris))
    rays = torch.as_tensor(random_rays(5000, seed=2), device="cuda")
    ia, ta = a.trace_closest(rays)
    ib, tb = b.trace_closest(rays)
    assert torch.equal(ia, ib) and torch.equal(ta, tb)


def test_renders_through_either_bvh_are_identical(cuda_device):
    objs, mesh = configs.terrain_scene(res=256, n_spheres=16, seed=5)
    a, b = both(objs, mesh)
    cam = configs.TERRAIN_CAMERA
    kw = dict(fov=cam["fov"], max_depth=8)
    ia = a.Render((64, 36), cam["origin"], cam["direction"], 4, **kw)
    ib = b.Render((64, 36), cam["origin"], cam["direction"], 4, **kw)
    assert np.array_equal(ia, ib)


def test_full_terrain_build(cuda_device):
    import torch
    objs, mesh = configs.terrain_scene()
    a, b = both(objs, mesh)
    assert b.stats()["slots"] == a.stats()["slots"]
    assert b.build_time_ms() < a.build_time_ms()
    cam = configs.TERRAIN_CAMERA
    rays = torch.as_tensor(configs.pinhole_rays(480, 270, cam["origin"], cam["direction"], cam["fov"]), device="cuda")
    ia, ta = a.trace_closest(rays)
    ib, tb = b.trace_closest(rays)
    assert torch.equal(ia, ib) and torch.equal(ta, tb)


@pytest.mark.parametrize("mode", ["host", "gpu"])
def test_refit_answers_like_a_rebuild(cuda_device, mode):
    """Move the terrain's vertices, refit, and compare with a fresh build of the
    moved mesh: same hits, same render."""
    import torch
    from aperturerendererv3_gb300.scene import TriangleMesh
    objs, mesh = configs.terrain_scene(res=256, n_spheres=16, seed=5)
    r = SceneRenderer(objs, mesh=mesh)
    r.set_build_mode(mode)
    r.build()
    rng = np.random.default_rng(3)
    v = np.asarray(mesh.vertices, np.float32).copy()
    v[:, 1] = v[:, 1] * 1.4 + rng.normal(0.0, 0.003, len(v)).astype(np.float32)
    r.refit_mesh(v)
    moved = TriangleMesh(v, mesh.indices, mesh.material_ids, mesh.materials, mesh.uv)
    fresh = SceneRenderer(objs, mesh=moved)
    fresh.build()
    cam = configs.TERRAIN_CAMERA
    rays = torch.as_tensor(configs.pinhole_rays(320, 180, cam["origin"], cam["direction"], cam["fov"]), device="cuda")
    ia, ta = r.trace_closest(rays)
    ib, tb = fresh.trace_closest(rays)
    assert torch.equal(ia, ib) and torch.equal(ta, tb)
    kw = dict(fov=cam["fov"], max_depth=6)
    assert np.array_equal(r.Render((48, 27), cam["origin"], cam["direction"], 2, **kw),
                          fresh.Render((48, 27), cam["origin"], cam["direction"], 2, **kw))
    with pytest.raises(Exception):
        r.refit_mesh(v[:-1])


@pytest.mark.parametrize("mode", ["host", "gpu"])
def test_rebuild_after_device_refit_uses_moved_vertices(cuda_device, mode):
    """A refit from device memory, then a rebuild through the C ABI alone (no
    new mesh upload): the context's host copy of the mesh follows the refit."""
    import ctypes as C
    import torch
    from aperturerendererv3_gb300 import _lib
    from aperturerendererv3_gb300.scene import TriangleMesh
    objs, mesh = configs.terrain_scene(res=128, n_spheres=8, seed=9)
    r = SceneRenderer(objs, mesh=mesh)
    r.build()
    v = np.asarray(mesh.vertices, np.float32).copy()
    v[:, 1] = v[:, 1] * 0.6 + 0.05
    r.refit_mesh(torch.as_tensor(v, device="cuda"))
    code = {"host": _lib.BUILD_HOST, "gpu": _lib.BUILD_GPU}[mode]
    assert r._lib.ar_scene_set_build_mode(r._ctx, code) == _lib.AR_OK
    assert r._lib.ar_scene_build(r._ctx) == _lib.AR_OK
    fresh = SceneRenderer(objs, mesh=TriangleMesh(v, mesh.indices, mesh.material_ids, mesh.materials, mesh.uv))
    fresh.build()
    cam = configs.TERRAIN_CAMERA
    rays = torch.as_tensor(configs.pinhole_rays(160, 90, cam["origin"], cam["direction"], cam["fov"]), device="cuda")
    ia, ta = r.trace_closest(rays)
    ib, tb = fresh.trace_closest(rays)
    assert torch.equal(ia, ib) and torch.equal(ta, tb)
    # the Python mesh follows too
    assert np.array_equal(np.asarray(r.mesh.vertices), v)
