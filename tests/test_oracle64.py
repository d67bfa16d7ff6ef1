"""The FP64 CPU oracle (oracle/pt64.cpp) pinned against the reference's own
integrator (oracle/_ref, float), and its adjoint against its own central
differences.  CPU only."""
import numpy as np
import pytest

from aperturerendererv3_gb300 import configs
from oracle import pt64
from oracle import ref_runner as rr


def per_sample_rel(objs, mesh, cam, size, spp, depth):
    S = pt64.Scene64(objs, mesh)
    m64, p64 = S.render(size, cam["origin"], cam["direction"], spp, fov=cam["fov"], max_depth=depth, per_sample=True)
    mr, pr, _ = rr.render(objs, size, cam["origin"], cam["direction"], spp, fov=cam["fov"], max_depth=depth,
                          per_sample_frames=spp, mesh=mesh)
    pr = pr.astype(np.float64)
    rel = (np.abs(p64 - pr) / np.maximum(np.abs(pr), 1e-6)).max(-1)
    return rel, m64, mr


@pytest.fixture(scope="module")
def ref_available():
    if not rr.available():
        pytest.skip("reference oracle not built in this checkout")


def test_fp64_matches_reference_per_sample_on_the_triangle_cornell_box(ref_available):
    rel, m64, mr = per_sample_rel(configs.cornell_triangles(), None, configs.CORNELL_CAMERA, (24, 24), 4, 8)
    assert (rel < 1e-4).mean() > 0.999, (rel < 1e-4).mean()
    assert abs(m64.mean() - mr.mean()) < 1e-5 * mr.mean()


def test_fp64_matches_reference_per_sample_with_ggx_and_box_lights(ref_available):
    rel, m64, mr = per_sample_rel(configs.reference_cornell(), None, configs.REFERENCE_CORNELL_CAMERA, (24, 24), 4, 16)
    # glossy paths may part ways between float and double
    assert (rel < 1e-3).mean() > 0.95, (rel < 1e-3).mean()


def test_fp64_matches_reference_on_a_small_terrain(ref_available):
    objs, mesh = configs.terrain_scene(res=48, n_spheres=8, seed=7)
    rel, m64, mr = per_sample_rel(objs, mesh, configs.TERRAIN_CAMERA, (16, 12), 2, 16)
    assert (rel < 1e-3).mean() > 0.9, (rel < 1e-3).mean()


def test_fp64_adjoint_is_the_derivative_of_the_fp64_estimator():
    """Central differences inside one LUT cell, NEE off, depth 3 (no roulette)."""
    tex = configs.cornell_textures(4, seed=5)
    objs, mesh, tx = configs.textured_cornell(tex)
    cam = configs.CORNELL_CAMERA
    size, spp, kw = (12, 12), 4, dict(fov=cam["fov"], max_depth=3, use_nee=False)
    S = pt64.Scene64(objs, mesh, tx)
    img = S.render(size, cam["origin"], cam["direction"], spp, **kw)
    target = np.full_like(img, img.mean())
    g = S.adjoint(2.0 * (img - target), size, cam["origin"], cam["direction"], spp, **kw)
    flat = tex.reshape(-1).astype(np.float64)
    gl = flat * 512 - 0.5
    dist = np.abs(gl - np.round(gl)) / 512
    cand = np.flatnonzero((np.abs(g) > 1e-6 * np.abs(g).max()) & (dist > 4e-4))
    rng = np.random.default_rng(0)
    probe = rng.choice(cand, size=min(12, len(cand)), replace=False)
    for i in probe:
        h = 0.45 * dist[i]
        vals = []
        for s in (1.0, -1.0):
            t2 = flat.copy()
            t2[i] += s * h
            S2 = pt64.Scene64(objs, mesh, [t.astype(np.float32) for t in t2.reshape(tex.shape)])
            im = S2.render(size, cam["origin"], cam["direction"], spp, **kw)
            vals.append(((im - target) ** 2).sum())
        # texels travel as float32: difference quotient over the float32 step
        step = float(np.float32(flat[i] + h)) - float(np.float32(flat[i] - h))
        fd = (vals[0] - vals[1]) / step
        assert abs(fd - g[i]) <= 1e-3 * abs(fd) + 1e-12, (i, fd, g[i])


def test_fp64_medium_absorption_known_answer():
    """Albedo 0, no emission: a camera ray sees the sky with probability
    exp(-sigma_t x chord); with the box 1 unit deep along the view axis."""
    from aperturerendererv3_gb300.scene import Medium, SceneObject, Material
    from aperturerendererv3_gb300._lib import OBJECT_SPHERE
    far = SceneObject((50.0, 50.0, 50.0), (0.1, 0.1, 0.1), Material.CreateDiffusePureColor((0.5, 0.5, 0.5)),
                      (0.0, 0.0, 0.0), OBJECT_SPHERE)
    med = Medium((-10.0, -10.0, -1.5), (10.0, 10.0, -0.5), sigma_t=0.7, albedo=0.0, g=0.0, emission=0.0)
    cam = dict(origin=(0.0, 0.0, 0.0), direction=(0.0, 0.0, -1.0), fov=2.0)
    clear = pt64.Scene64([far]).render((2, 2), cam["origin"], cam["direction"], 64, fov=cam["fov"], max_depth=2)
    fog = pt64.Scene64([far], medium=med).render((2, 2), cam["origin"], cam["direction"], 4096, fov=cam["fov"],
                                                  max_depth=2)
    ratio = fog[..., 1].mean() / clear[..., 1].mean()
    assert abs(ratio - np.exp(-0.7)) < 0.03, (ratio, np.exp(-0.7))


def test_fp64_sdf_sphere_matches_analytic_sphere():
    from aperturerendererv3_gb300.scene import Material, SceneObject, SdfUnion
    from aperturerendererv3_gb300._lib import OBJECT_SPHERE, SDF_SPHERE
    objs = configs.cornell_triangles()
    mat = Material.CreateDiffusePureColor((0.3, 0.5, 0.7))
    ball = SceneObject((0.05, -0.3, 0.0), (0.15, 0.15, 0.15), mat, (0.0, 0.0, 0.0), OBJECT_SPHERE)
    sdf = SdfUnion([(SDF_SPHERE, (0.05, -0.3, 0.0), (0.15, 0.0, 0.0))], 1e-3, mat)
    cam = configs.CORNELL_CAMERA
    a = pt64.Scene64(objs + [ball]).render((24, 24), cam["origin"], cam["direction"], 16, fov=cam["fov"], max_depth=4)
    b = pt64.Scene64(objs, sdf=sdf).render((24, 24), cam["origin"], cam["direction"], 16, fov=cam["fov"], max_depth=4)
    assert abs(a.mean() - b.mean()) < 0.01 * a.mean()
    assert np.abs(a - b).mean() < 0.02 * a.mean()


def test_float_sdf_mode_moves_only_samples_that_see_the_sdf():
    """The float-SDF diagnostic mode is off by default, leaves scenes without
    SDF geometry bit for bit, and moves SDF samples by float-sized amounts."""
    from aperturerendererv3_gb300.scene import Material, SdfUnion
    from aperturerendererv3_gb300._lib import SDF_SPHERE, SDF_TORUS
    objs, cam = configs.cornell_triangles(), configs.CORNELL_CAMERA
    kw = dict(fov=cam["fov"], max_depth=2, per_sample=True)
    plain = pt64.Scene64(objs)
    _, a = plain.render((16, 16), cam["origin"], cam["direction"], 2, **kw)
    plain.set_sdf_f32(True)
    _, b = plain.render((16, 16), cam["origin"], cam["direction"], 2, **kw)
    assert np.array_equal(a, b)
    sdf = SdfUnion([(SDF_SPHERE, (0.1, -0.3, 0.0), (0.12, 0, 0)), (SDF_TORUS, (-0.1, -0.2, 0.05), (0.15, 0.04, 0))],
                   0.08, Material.CreateDiffusePureColor((0.6, 0.5, 0.4)))
    S = pt64.Scene64(objs, sdf=sdf)
    _, c = S.render((16, 16), cam["origin"], cam["direction"], 2, **kw)
    _, c2 = S.render((16, 16), cam["origin"], cam["direction"], 2, **kw)
    S.set_sdf_f32(True)
    _, d = S.render((16, 16), cam["origin"], cam["direction"], 2, **kw)
    assert np.array_equal(c, c2)
    rel = (np.abs(d - c) / np.maximum(np.abs(c), 1e-4)).max(-1)
    assert 0.0 < (rel > 0).mean() < 1.0
    assert np.quantile(rel, 0.99) < 1e-2


def test_fp64_medium_adjoint_over_windows_adds_up_to_the_full_image():
    """The crop form of the medium adjoint reads only its window's pixels, with
    the full image's rays and streams: two windows that tile the image sum to
    the full-image adjoint."""
    from aperturerendererv3_gb300.scene import Medium
    objs, cam = configs.cornell_triangles(), configs.CORNELL_CAMERA
    med = Medium((-0.45, -0.5, -0.5), (0.45, 0.2, 0.3), sigma_t=1.5, albedo=0.8, g=0.3, emission=0.1)
    S = pt64.Scene64(objs, medium=med)
    size, kw = (16, 12), dict(fov=cam["fov"], max_depth=6)
    img = S.render(size, cam["origin"], cam["direction"], 2, **kw)
    dl = 2.0 * (img - 0.8 * img.mean())
    full = S.adjoint_medium(dl, size, cam["origin"], cam["direction"], 2, **kw)
    top = S.adjoint_medium(dl, size, cam["origin"], cam["direction"], 2, window=(0, 0, 16, 5), **kw)
    bottom = S.adjoint_medium(dl, size, cam["origin"], cam["direction"], 2, window=(0, 5, 16, 7), **kw)
    for k in range(2):
        assert abs(top[k] + bottom[k] - full[k]) <= 1e-9 * abs(full[k])
    assert abs(top[0]) > 0 and abs(bottom[0]) > 0


def test_fp64_medium_adjoint_is_the_derivative_of_the_fp64_estimator():
    """NEE off, depth 3: the estimator is smooth in the albedo and linear in the emission."""
    from aperturerendererv3_gb300.scene import Medium
    objs = configs.cornell_triangles()
    cam = configs.CORNELL_CAMERA
    size, spp = (12, 12), 8
    kw = dict(fov=cam["fov"], max_depth=3, use_nee=False)

    def med(a, e):
        return Medium((-0.5, -0.5, -0.5), (0.5, 0.5, 0.5), sigma_t=2.0, albedo=a, g=0.3, emission=e)

    S = pt64.Scene64(objs, medium=med(0.7, 0.4))
    img = S.render(size, cam["origin"], cam["direction"], spp, **kw)
    target = np.full_like(img, img.mean() * 0.8)
    ga, ge = S.adjoint_medium(2.0 * (img - target), size, cam["origin"], cam["direction"], spp, **kw)

    def loss(a, e):
        S.set_medium(med(a, e))
        im = S.render(size, cam["origin"], cam["direction"], spp, **kw)
        return ((im - target) ** 2).sum()

    h = 1e-4
    fa = (loss(0.7 + h, 0.4) - loss(0.7 - h, 0.4)) / (2 * h)
    fe = (loss(0.7, 0.4 + h) - loss(0.7, 0.4 - h)) / (2 * h)
    assert abs(fa - ga) < 1e-3 * abs(fa), (fa, ga)
    assert abs(fe - ge) < 1e-3 * abs(fe), (fe, ge)
