"""Voxel path guiding on the GPU (core/guiding/*, core/render/render.cuh:553-638,
core/scene.cu:409-570): the first frame draws nothing extra (no probes yet), the
probes fill in after each frame, and guided images converge to the same mean as
unguided ones."""
import numpy as np
import pytest

from aperturerendererv3_gb300 import SceneRenderer, configs

pytestmark = pytest.mark.gpu


def scenes():
    return [("reference_cornell", configs.reference_cornell(), None, configs.REFERENCE_CORNELL_CAMERA),
            ("cornell_triangles", configs.cornell_triangles(), None, configs.CORNELL_CAMERA)]


@pytest.mark.parametrize("name,objs,mesh,cam", scenes())
def test_first_guided_frame_equals_unguided(cuda_device, name, objs, mesh, cam):
    r = SceneRenderer(objs, mesh=mesh)
    a = r.Render((48, 40), cam["origin"], cam["direction"], 1, fov=cam["fov"], max_depth=16)
    b = r.Render((48, 40), cam["origin"], cam["direction"], 1, fov=cam["fov"], max_depth=16, guide=1)
    assert np.array_equal(a, b)
    n, cap = r.guide_stats()
    assert 0 < n <= cap


@pytest.mark.parametrize("name,objs,mesh,cam", scenes())
def test_guided_render_learns_and_stays_unbiased(cuda_device, name, objs, mesh, cam):
    size, spp = (64, 64), 256
    r = SceneRenderer(objs, mesh=mesh)
    plain = r.Render(size, cam["origin"], cam["direction"], spp, fov=cam["fov"], max_depth=16)
    guided = r.Render(size, cam["origin"], cam["direction"], spp, fov=cam["fov"], max_depth=16, guide=1,
                      first_frame=0)
    n, _ = r.guide_stats()
    assert n > 50
    assert r.error_word() == 0
    assert np.all(np.isfinite(guided))
    m_plain, m_guided = plain[..., 1].mean(), guided[..., 1].mean()
    assert abs(m_guided - m_plain) < 0.03 * m_plain, (m_plain, m_guided)
    # probes persist across calls until reset
    assert r.MarkNeedResetGuiding() == n
    assert r.guide_stats()[0] == 0


def test_guide_on_terrain_mesh(cuda_device):
    objs, mesh = configs.terrain_scene(res=96, n_spheres=8, seed=7)
    cam = configs.TERRAIN_CAMERA
    r = SceneRenderer(objs, mesh=mesh)
    img = r.Render((96, 54), cam["origin"], cam["direction"], 8, fov=cam["fov"], max_depth=16, guide=1)
    assert np.all(np.isfinite(img)) and img.mean() > 0
    assert r.guide_stats()[0] > 0
    assert r.error_word() == 0


@pytest.mark.parametrize("name,objs,mesh,cam", scenes())
def test_mlp_guide_trains_and_stays_unbiased(cuda_device, name, objs, mesh, cam):
    """guide=2: the network trains after every frame (eight Adam steps), takes over
    from the voxel probes after its warm-up, and the image converges to the
    same mean as unguided rendering."""
    size, spp = (64, 64), 256
    r = SceneRenderer(objs, mesh=mesh)
    plain = r.Render(size, cam["origin"], cam["direction"], spp, fov=cam["fov"], max_depth=16)
    guided = r.Render(size, cam["origin"], cam["direction"], spp, fov=cam["fov"], max_depth=16, guide=2)
    steps, loss = r.mlp_stats()
    assert steps == 8 * spp  # eight Adam steps per frame
    assert np.isfinite(loss)  # Poisson log-likelihood: may be negative
    assert r.error_word() == 0
    assert np.all(np.isfinite(guided))
    m_plain, m_guided = plain[..., 1].mean(), guided[..., 1].mean()
    assert abs(m_guided - m_plain) < 0.03 * m_plain, (m_plain, m_guided)
    r.MarkNeedResetGuiding()
    assert r.mlp_stats()[0] == 0


def test_mlp_guide_on_terrain(cuda_device):
    objs, mesh = configs.terrain_scene(res=96, n_spheres=8, seed=7)
    cam = configs.TERRAIN_CAMERA
    r = SceneRenderer(objs, mesh=mesh)
    img = r.Render((96, 54), cam["origin"], cam["direction"], 16, fov=cam["fov"], max_depth=16, guide=2)
    assert np.all(np.isfinite(img)) and img.mean() > 0
    assert r.mlp_stats()[0] == 8 * 16
    assert r.error_word() == 0


@pytest.mark.parametrize("name,objs,mesh,cam", scenes()[:1])
def test_guide_update_windows(cuda_device, name, objs, mesh, cam):
    """guide_frames = k: the guide updates after every k frames and the k frames
    share waves.  k = 1 is the per-frame update; the first window of k frames has
    no probes yet and draws exactly what the unguided render draws; the windowed
    render learns and stays unbiased."""
    size = (48, 40)
    kw = dict(fov=cam["fov"], max_depth=16)
    r = SceneRenderer(objs, mesh=mesh)
    a = r.Render(size, cam["origin"], cam["direction"], 6, guide=1, **kw)
    r.MarkNeedResetGuiding()
    b = r.Render(size, cam["origin"], cam["direction"], 6, guide=1, guide_frames=1, **kw)
    assert np.array_equal(a, b)
    r.MarkNeedResetGuiding()
    plain = r.Render(size, cam["origin"], cam["direction"], 4, **kw)
    w4 = r.Render(size, cam["origin"], cam["direction"], 4, guide=1, guide_frames=4, **kw)
    assert np.array_equal(plain, w4)
    assert r.guide_stats()[0] > 0
    r.MarkNeedResetGuiding()
    size, spp = (64, 64), 256
    plain = r.Render(size, cam["origin"], cam["direction"], spp, **kw)
    guided = r.Render(size, cam["origin"], cam["direction"], spp, guide=1, guide_frames=16, **kw)
    _, launches_windowed = r.last_render_stats()
    r.MarkNeedResetGuiding()
    r.Render(size, cam["origin"], cam["direction"], spp, guide=1, **kw)
    _, launches_per_frame = r.last_render_stats()
    assert launches_windowed < launches_per_frame / 8
    m_plain, m_guided = plain[..., 1].mean(), guided[..., 1].mean()
    assert abs(m_guided - m_plain) < 0.03 * m_plain, (m_plain, m_guided)
    for mode in (2,):
        r.MarkNeedResetGuiding()
        img = r.Render(size, cam["origin"], cam["direction"], 64, guide=mode, guide_frames=8, **kw)
        assert r.mlp_stats()[0] == 8 * 64  # eight Adam steps per frame, taken after each window
        assert abs(img[..., 1].mean() - m_plain) < 0.05 * m_plain
    assert r.error_word() == 0
