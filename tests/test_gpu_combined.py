"""The smooth-union SDF object and the participating medium on the GPU.

* Per-sample radiance matches the FP64 CPU oracle (oracle/pt64.cpp) on the same
  random streams: a Cornell box with an SDF union inside a medium, and a small
  version of the combined workload (terrain, SDF union, medium, sphere lights,
  sun, sky).
* The replay adjoint of the medium's albedo and emission equals central
  differences of the same seeded render (NEE off, depth 3: smooth estimator)
  and the FP64 adjoint with NEE and Russian roulette on.
* Removing the medium restores the plain render exactly.
* The tail of the per-sample comparison is the float arithmetic of the SDF:
  the FP64 oracle with its SDF march and normal run in float departs from the
  FP64 render by the same distribution as the GPU does.
"""
import numpy as np
import pytest

from aperturerendererv3_gb300 import SceneRenderer, configs
from aperturerendererv3_gb300.scene import Material, Medium, SdfUnion
from aperturerendererv3_gb300._lib import SDF_BOX, SDF_SPHERE, SDF_TORUS
from oracle import pt64

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def cornell_sdf():
    sdf = SdfUnion([(SDF_SPHERE, (0.12, -0.3, 0.0), (0.12, 0, 0)), (SDF_BOX, (-0.12, -0.35, -0.1), (0.1, 0.12, 0.08)),
                    (SDF_TORUS, (0.0, -0.1, 0.05), (0.15, 0.04, 0))], 0.08,
                   Material.CreateGGXPureColor((0.8, 0.6, 0.4), 0.3, 0.0, 0.5))
    med = Medium((-0.45, -0.5, -0.5), (0.45, 0.2, 0.3), sigma_t=1.5, albedo=0.8, g=0.3, emission=0.1)
    return configs.cornell_triangles(), None, sdf, med, configs.CORNELL_CAMERA


def small_combined():
    objs, mesh, sdf, med = configs.combined_scene(res=48, n_spheres=8)
    return objs, mesh, sdf, med, configs.COMBINED_CAMERA


@pytest.mark.parametrize("make,size,spp,depth,bar", [(cornell_sdf, (32, 32), 4, 8, 0.97),
                                                     (small_combined, (24, 16), 2, 16, 0.9)])
def test_per_sample_against_fp64_oracle(cuda_device, make, size, spp, depth, bar):
    objs, mesh, sdf, med, cam = make()
    r = SceneRenderer(objs, mesh=mesh, sdf=sdf, medium=med)
    img, ps = r.Render(size, cam["origin"], cam["direction"], spp, fov=cam["fov"], max_depth=depth, per_sample=True)
    assert r.error_word() == 0
    S = pt64.Scene64(objs, mesh, sdf=sdf, medium=med)
    ref, ps64 = S.render(size, cam["origin"], cam["direction"], spp, fov=cam["fov"], max_depth=depth, per_sample=True)
    rel = (np.abs(ps.astype(np.float64) - ps64) / np.maximum(np.abs(ps64), 1e-4)).max(-1)
    assert (rel < 1e-3).mean() > bar, (rel < 1e-3).mean()
    assert abs(img.mean() - ref.mean()) < 0.02 * ref.mean()


def _rel(a, b):
    return (np.abs(a - b) / np.maximum(np.abs(b), 1e-4)).max(-1).ravel()


@pytest.mark.parametrize("make,size,spp", [(cornell_sdf, (32, 32), 4), (small_combined, (24, 16), 2)])
@pytest.mark.parametrize("depth", [1, 8])
def test_tail_is_the_float_arithmetic_of_the_sdf(cuda_device, make, size, spp, depth):
    """The SDF normal is a central difference with h = 1e-4: the field's float
    rounding (about 1e-7 at coordinates of 0.3) divided by 2h moves the normal
    by a few 1e-4, and the march's stopping step can move by one step.  The
    FP64 oracle with the SDF march and field in float (positions rounded to
    float) shows how far that alone moves each sample; the GPU's departures
    from the FP64 render must follow the same distribution: its 99th
    percentile within 2x the oracle's (plus 1e-4, the float level of the rest
    of the path: q99 3.3e-5 and max 1.5e-4 at depth 1 on the Cornell box
    without SDF and medium), as large a share of samples within 1e-3, and
    within 1e-2 up to 0.5 % fewer: past the first bounce float and double also
    send a few paths apart where no SDF is involved (1 of 4096 samples on
    that Cornell box at depth 2).  Depth 1 is the first bounce (camera hit,
    emission and NEE)."""
    objs, mesh, sdf, med, cam = make()
    kw = dict(fov=cam["fov"], max_depth=depth, per_sample=True)
    r = SceneRenderer(objs, mesh=mesh, sdf=sdf, medium=med)
    _, ps = r.Render(size, cam["origin"], cam["direction"], spp, **kw)
    assert r.error_word() == 0
    S = pt64.Scene64(objs, mesh, sdf=sdf, medium=med)
    _, ref = S.render(size, cam["origin"], cam["direction"], spp, **kw)
    S.set_sdf_f32(True)
    _, f32 = S.render(size, cam["origin"], cam["direction"], spp, **kw)
    g, e = _rel(ps.astype(np.float64), ref), _rel(f32, ref)
    qg, qe = np.quantile(g, 0.99), np.quantile(e, 0.99)
    msg = (f"gpu q99 {qg}, float-SDF oracle {qe}; within 1e-3: {(g < 1e-3).mean()} vs {(e < 1e-3).mean()}; "
           f"within 1e-2: {(g < 1e-2).mean()} vs {(e < 1e-2).mean()}")
    assert qg <= 2.0 * qe + 1e-4, msg
    assert (g < 1e-3).mean() >= (e < 1e-3).mean() - 0.01, msg
    assert (g < 1e-2).mean() >= (e < 1e-2).mean() - 0.005, msg


def test_medium_adjoint_at_the_combined_scale_matches_fp64_on_a_window(cuda_device):
    """The combined workload at its stated scale (terrain, 32-primitive smooth
    union, medium; 3840x2160, depth 24, NEE and roulette), 4 spp: the replay
    adjoint of the medium's albedo and emission for a loss that reads one
    64x64 window of the image equals the FP64 oracle's adjoint over that
    window (the same pixels, rays and random streams) within 2e-2, the bar of
    the small-scene comparison."""
    objs, mesh, sdf, med = configs.combined_scene()
    cam = configs.COMBINED_CAMERA
    size, spp, window = (3840, 2160), 4, (1888, 1048, 64, 64)
    kw = dict(fov=cam["fov"], max_depth=24)
    r = SceneRenderer(objs, mesh=mesh, sdf=sdf, medium=med)
    img = r.Render(size, cam["origin"], cam["direction"], spp, **kw)
    assert r.error_word() == 0
    x0, y0, w, h = window
    dl = np.zeros_like(img)
    crop = img[y0:y0 + h, x0:x0 + w]
    dl[y0:y0 + h, x0:x0 + w] = 2.0 * (crop - 0.8 * crop.mean())
    dl = dl.astype(np.float32)
    ga, ge = r.adjoint_medium(torch.as_tensor(dl, device="cuda"), size, cam["origin"], cam["direction"], spp, **kw)
    S = pt64.Scene64(objs, mesh, sdf=sdf, medium=med)
    ra, re = S.adjoint_medium(dl.astype(np.float64), size, cam["origin"], cam["direction"], spp, window=window, **kw)
    assert abs(ra) > 0 and abs(re) > 0
    assert abs(ga - ra) < 2e-2 * abs(ra), (ga, ra)
    assert abs(ge - re) < 2e-2 * abs(re), (ge, re)


def test_removing_the_medium_restores_the_plain_render(cuda_device):
    objs, mesh, sdf, med, cam = cornell_sdf()
    r = SceneRenderer(objs, sdf=sdf)
    a = r.Render((24, 24), cam["origin"], cam["direction"], 4, fov=cam["fov"], max_depth=8)
    r.set_medium(med)
    b = r.Render((24, 24), cam["origin"], cam["direction"], 4, fov=cam["fov"], max_depth=8)
    r.set_medium(None)
    c = r.Render((24, 24), cam["origin"], cam["direction"], 4, fov=cam["fov"], max_depth=8)
    assert np.array_equal(a, c)
    assert not np.array_equal(a, b)


def medium_with(med, a, e):
    return Medium(med.box_lo, med.box_hi, med.sigma_t, a, med.g, e)


def test_medium_adjoint_matches_central_differences(cuda_device):
    objs, mesh, sdf, med, cam = cornell_sdf()
    size, spp = (24, 24), 8
    kw = dict(fov=cam["fov"], max_depth=3, use_nee=False)
    r = SceneRenderer(objs, sdf=sdf, medium=med)
    img = r.Render(size, cam["origin"], cam["direction"], spp, **kw)
    target = np.full_like(img, img.mean() * 0.8)
    dl = torch.as_tensor(2.0 * (img - target), device="cuda").float()
    ga, ge = r.adjoint_medium(dl, size, cam["origin"], cam["direction"], spp, **kw)

    def loss(a, e):
        r.set_medium(medium_with(med, a, e))
        im = r.Render(size, cam["origin"], cam["direction"], spp, **kw)
        return ((im - target) ** 2).sum()

    h = 1e-3
    fa = (loss(med.albedo + h, med.emission) - loss(med.albedo - h, med.emission)) / (2 * h)
    fe = (loss(med.albedo, med.emission + h) - loss(med.albedo, med.emission - h)) / (2 * h)
    assert abs(fa - ga) < 1e-2 * abs(fa), (fa, ga)
    assert abs(fe - ge) < 1e-2 * abs(fe), (fe, ge)


def test_medium_adjoint_matches_fp64_with_nee_and_roulette(cuda_device):
    objs, mesh, sdf, med, cam = cornell_sdf()
    size, spp = (24, 24), 8
    kw = dict(fov=cam["fov"], max_depth=8)
    r = SceneRenderer(objs, sdf=sdf, medium=med)
    img = r.Render(size, cam["origin"], cam["direction"], spp, **kw)
    target = np.full_like(img, img.mean() * 0.8)
    dl = 2.0 * (img - target)
    ga, ge = r.adjoint_medium(torch.as_tensor(dl, device="cuda").float(), size, cam["origin"], cam["direction"], spp,
                              **kw)
    S = pt64.Scene64(objs, sdf=sdf, medium=med)
    ra, re = S.adjoint_medium(dl, size, cam["origin"], cam["direction"], spp, **kw)
    assert abs(ga - ra) < 2e-2 * abs(ra), (ga, ra)
    assert abs(ge - re) < 2e-2 * abs(re), (ge, re)
