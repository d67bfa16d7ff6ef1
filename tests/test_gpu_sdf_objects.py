"""SDF scene objects (OBJ_SDF: torus, cached volumes) on the GPU against the
reference's own IntersectSDFObject and volume cache run on the host (oracle/_ref).

* Volumes filled on the GPU from the reference's functors equal the host fill
  bit for bit; caller data round-trips.
* Per-sample radiance of a Cornell box holding a rotated torus, a diamond
  volume (the reference's example, 64^3) and a caller-data sphere volume
  matches the reference integrator.
* A volume added after the scene is built is picked up without a rebuild.
* Rays through many overlapping SDF objects resolve to the closest one.
"""
import numpy as np
import pytest

from aperturerendererv3_gb300 import SceneRenderer, configs
from aperturerendererv3_gb300 import _lib
from aperturerendererv3_gb300.scene import Material, SceneObject, sdf
from oracle import ref_runner as rr

pytestmark = pytest.mark.gpu

CAM = configs.CORNELL_CAMERA


@pytest.fixture(scope="module")
def ref_available():
    if not rr.available():
        pytest.skip("reference oracle not built in this checkout")


def sphere_field(u):
    return np.linalg.norm(u, axis=1) - 0.4


def sdf_scene(r):
    diamond = r.AddVolumeToCacheManager((64, 64, 64), sdfFunctor="diamond", sdfInfo=sdf.CreateDiamond())
    ball = r.AddVolumeToCacheManager((24, 20, 28), sdfFunctor=sphere_field)
    objs = configs.cornell_triangles()
    gold = Material.CreateGGXPureColor((0.9, 0.7, 0.3), 0.2, 1.0, 0.5)
    glassy = Material.CreateDiffusePureColor((0.3, 0.8, 0.6))
    objs.append(SceneObject((0.15, -0.3, 0.05), (0.2, 0.2, 0.2), gold, (70.0, 20.0, 0.0), _lib.OBJECT_SDF,
                            sdf.CreateTorus()))
    objs.append(SceneObject((-0.2, -0.25, -0.1), (0.16, 0.16, 0.16), glassy, (-90.0, 0.0, 15.0), _lib.OBJECT_SDF,
                            sdf.CreateSDFVolume(diamond)))
    objs.append(SceneObject((0.0, 0.15, -0.2), (0.12, 0.1, 0.14), Material.CreateDiffusePureColor((0.8, 0.8, 0.8)),
                            (0.0, 30.0, 0.0), _lib.OBJECT_SDF, sdf.CreateSDFVolume(ball)))
    vols = [(_lib.SDF_FN_DIAMOND, sdf.CreateDiamond(), (64, 64, 64)), (None, r.sdf_volume(ball), None)]
    return objs, vols


def test_gpu_volume_fill_equals_the_reference_fill(cuda_device, ref_available):
    r = SceneRenderer(configs.cornell_triangles())
    i = r.AddVolumeToCacheManager((64, 64, 64), sdfFunctor="diamond", sdfInfo=sdf.CreateDiamond())
    j = r.AddVolumeToCacheManager((32, 24, 16), sdfFunctor="torus", sdfInfo=(0.3, 0.1, 0.0, 0.0))
    k = r.AddVolumeToCacheManager((5, 6, 7), sdfFunctor=sphere_field)
    assert np.array_equal(r.sdf_volume(i), rr.sdf_volume(_lib.SDF_FN_DIAMOND, sdf.CreateDiamond(), (64, 64, 64)))
    assert np.array_equal(r.sdf_volume(j), rr.sdf_volume(_lib.SDF_FN_TORUS, (0.3, 0.1, 0.0, 0.0), (32, 24, 16)))
    assert r.sdf_volume(k).shape == (7, 6, 5)
    r.ClearVolumes()
    with pytest.raises(Exception):
        r.sdf_volume(0)


def test_per_sample_radiance_matches_the_reference(cuda_device, ref_available):
    r = SceneRenderer([])
    objs, vols = sdf_scene(r)
    r2 = SceneRenderer(objs)
    for fn, prm, dims in vols:
        if fn is None:
            r2.AddVolumeToCacheManager((prm.shape[2], prm.shape[1], prm.shape[0]), sdfFunctor=lambda u, v=prm: v)
        else:
            r2.AddVolumeToCacheManager(dims, sdfFunctor="diamond", sdfInfo=prm)
    size, spp = (40, 40), 4
    mean, ps = r2.Render(size, CAM["origin"], CAM["direction"], spp, fov=CAM["fov"], max_depth=8, per_sample=True)
    rmean, rps, _ = rr.render(objs, size, CAM["origin"], CAM["direction"], spp, fov=CAM["fov"], max_depth=8,
                              per_sample_frames=spp, volumes=vols)
    rel = (np.abs(ps.astype(np.float64) - rps) / np.maximum(np.abs(rps), 1e-6)).max(-1)
    assert (rel < 1e-4).mean() > 0.99, (rel < 1e-4).mean()
    assert abs(mean.mean() - rmean.mean()) < 1e-3 * rmean.mean()
    assert r2.error_word() == 0


def test_volume_added_after_the_build(cuda_device):
    objs = configs.cornell_triangles()
    objs.append(SceneObject((0.0, -0.25, 0.0), (0.2, 0.2, 0.2), Material.CreateDiffusePureColor((0.9, 0.2, 0.2)),
                            (0.0, 0.0, 0.0), _lib.OBJECT_SDF, sdf.CreateSDFVolume(0)))
    r = SceneRenderer(objs)
    before = r.Render((24, 24), CAM["origin"], CAM["direction"], 2, fov=CAM["fov"], max_depth=4)
    r.AddVolumeToCacheManager((32, 32, 32), sdfFunctor=sphere_field)
    after = r.Render((24, 24), CAM["origin"], CAM["direction"], 2, fov=CAM["fov"], max_depth=4)
    assert not np.array_equal(before, after)


def test_rays_through_many_overlapping_sdf_objects(cuda_device, ref_available):
    """Seven overlapping tori along the view axis: rays cross several SDF objects'
    bounds in the SDF objects' own BVH, and the closest march wins."""
    objs = configs.cornell_triangles()
    mat = Material.CreateDiffusePureColor((0.7, 0.5, 0.9))
    for k in range(7):
        objs.append(SceneObject((0.02 * k, -0.2 + 0.01 * k, 0.3 - 0.09 * k), (0.15, 0.15, 0.15), mat,
                                (90.0, 10.0 * k, 0.0), _lib.OBJECT_SDF, sdf.CreateTorus(1.0, 0.3, 0.06)))
    r = SceneRenderer(objs)
    size, spp = (32, 32), 2
    mean, ps = r.Render(size, CAM["origin"], CAM["direction"], spp, fov=CAM["fov"], max_depth=4, per_sample=True)
    rmean, rps, _ = rr.render(objs, size, CAM["origin"], CAM["direction"], spp, fov=CAM["fov"], max_depth=4,
                              per_sample_frames=spp)
    rel = (np.abs(ps.astype(np.float64) - rps) / np.maximum(np.abs(rps), 1e-6)).max(-1)
    assert (rel < 1e-4).mean() > 0.99, (rel < 1e-4).mean()
