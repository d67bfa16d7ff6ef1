"""Albedo textures and the replay adjoint on the GPU.

* A textured Cornell box whose textures hold the plain box's colours renders
  the same samples as the plain box (textures change only where albedo comes
  from).
* ar_adjoint's d(loss)/d(texel) equals central finite differences of the same
  seeded render.  With Russian roulette and NEE off (depth 3) the sampled
  estimator is piecewise linear in each texel channel (trilinear spectral LUT),
  so an in-cell difference quotient matches every probed channel to 1e-2, and
  h = 1e-3 differences match in aggregate; with NEE on, decision flips under a
  perturbation spoil a few channels.
* The torch.autograd.Function returns the same gradient as the direct call,
  and a few gradient steps lower the L2 loss against a target render.
"""
import numpy as np
import pytest

from aperturerendererv3_gb300 import SceneRenderer, configs

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

CAM = configs.CORNELL_CAMERA
GREY, RED, GREEN = configs.GREY, configs.RED, configs.GREEN


def textured_renderer(textures):
    objs, mesh, tex = configs.textured_cornell(textures)
    return SceneRenderer(objs, mesh=mesh, textures=tex)


def render(r, size, spp, **kw):
    return r.Render(size, CAM["origin"], CAM["direction"], spp, fov=CAM["fov"], **kw)


def test_constant_textures_render_like_plain_colours(cuda_device):
    res = 4
    tex = np.empty((8, res, res, 3), np.float32)
    for g, c in enumerate([GREY, GREY, GREY, GREY, RED, GREEN, GREY, GREY]):
        tex[g] = c
    rt = textured_renderer(tex)
    rp = SceneRenderer(configs.cornell_triangles())
    a, sa = render(rt, (48, 48), 4, max_depth=8, per_sample=True)
    b, sb = render(rp, (48, 48), 4, max_depth=8, per_sample=True)
    close = np.isclose(sa, sb, rtol=1e-5, atol=1e-7).all(axis=-1)
    assert close.mean() > 0.999, close.mean()
    assert abs(a.mean() - b.mean()) < 1e-4 * b.mean()


def loss_and_grad(r, target, size, spp, **kw):
    """L2 loss of the render against target and d(loss)/d(texels) from ar_adjoint."""
    dev = torch.device("cuda", 0)
    w, h = size
    img = torch.empty((h, w, 3), dtype=torch.float64, device=dev)
    r.render_into(img, size, CAM["origin"], CAM["direction"], spp, fov=CAM["fov"], **kw)
    t = torch.as_tensor(target, device=dev)
    loss = float(((img - t) ** 2).sum())
    g = torch.empty(r.texel_count(), dtype=torch.float64, device=dev)
    r.adjoint((2.0 * (img - t)).float(), g, size, CAM["origin"], CAM["direction"], spp, fov=CAM["fov"], **kw)
    return loss, g.cpu().numpy(), img


LUT_RES = 512  # RGB -> spectrum lattice: planes at (i + 0.5) / 512 in each channel


def lattice_distance(x):
    g = np.asarray(x, np.float64) * LUT_RES - 0.5
    return np.abs(g - np.round(g)) / LUT_RES


def fd_check(use_nee, max_depth, h=None, n_probe=48, seed=3):
    """Adjoint vs central differences on n_probe texel channels.  h=None picks,
    per channel, a step inside the channel's LUT cell (at most 1e-3): the
    spectral albedo is trilinear in the lattice, so along one channel it is
    linear inside a cell and the difference quotient is the exact derivative of
    the sampled estimator.  A fixed h may straddle a lattice plane and average
    two cells' slopes."""
    res, size, spp = 8, (32, 32), 16
    tex_a = configs.cornell_textures(res, seed=11)
    tex_b = configs.cornell_textures(res, seed=12)
    target = render(textured_renderer(tex_b), size, 64, max_depth=max_depth, use_nee=use_nee)
    r = textured_renderer(tex_a)
    kw = dict(max_depth=max_depth, use_nee=use_nee)
    _, g, _ = loss_and_grad(r, target, size, spp, **kw)
    flat = tex_a.reshape(-1).astype(np.float64)
    rng = np.random.default_rng(seed)
    ok = np.abs(g) > 1e-6 * np.abs(g).max()
    if h is None:
        ok &= lattice_distance(flat) > 4e-4
    cand = np.flatnonzero(ok)
    probe = rng.choice(cand, size=min(n_probe, len(cand)), replace=False)
    fd = np.empty(len(probe))
    for k, i in enumerate(probe):
        step = h if h is not None else min(1e-3, 0.45 * float(lattice_distance(flat[i])))
        vals, at = [], []
        for sgn in (+1.0, -1.0):
            x32 = flat.astype(np.float32)
            x32[i] = np.float32(flat[i] + sgn * step)
            r.update_texels(x32)
            img = render(r, size, spp, **kw)
            vals.append(((img - target) ** 2).sum())
            at.append(float(x32[i]))
        fd[k] = (vals[0] - vals[1]) / (at[0] - at[1])
    r.update_texels(flat.astype(np.float32))
    return g[probe], fd


def test_adjoint_is_the_exact_derivative_of_the_sampled_estimator(cuda_device):
    adj, fd = fd_check(use_nee=False, max_depth=3)
    rel = np.abs(adj - fd) / np.maximum(np.abs(fd), 1e-12)
    assert len(rel) >= 32
    assert np.all(rel < 1e-2), np.sort(rel)[-5:]


def test_adjoint_matches_central_differences_h1e3(cuda_device):
    """h = 1e-3 central differences: aggregate relative error over the probed texels."""
    adj, fd = fd_check(use_nee=False, max_depth=3, h=1e-3)
    agg = np.linalg.norm(adj - fd) / np.linalg.norm(fd)
    assert agg < 1e-2, agg


def test_adjoint_with_nee(cuda_device):
    """NEE on, depth 3: the NEE decision (u < sqrt(mask)) of a path through the
    texel can flip under a perturbation, so most, not all, probed channels
    match the in-cell difference quotient.  (Russian roulette is checked
    against the FP64 adjoint instead: the adjoint holds the survival
    probability fixed, the unbiased choice, while a same-seed difference
    quotient differentiates through 1 / q(texel).)"""
    adj, fd = fd_check(use_nee=True, max_depth=3)
    rel = np.abs(adj - fd) / np.maximum(np.abs(fd), 1e-12)
    assert np.mean(rel < 1e-2) > 0.9, np.sort(rel)[-8:]


def test_untextured_scene_is_rejected(cuda_device):
    r = SceneRenderer(configs.cornell_triangles())
    r.build()
    from aperturerendererv3_gb300._lib import ArError
    dev = torch.device("cuda", 0)
    with pytest.raises(ArError):
        r.adjoint(torch.zeros((8, 8, 3), device=dev), torch.zeros(1, dtype=torch.float64, device=dev), (8, 8),
                  CAM["origin"], CAM["direction"], 1)


def test_autograd_function_and_descent(cuda_device):
    from aperturerendererv3_gb300.torch_render import render_textures
    dev = torch.device("cuda", 0)
    res, size = 16, (32, 32)
    tex_a = configs.cornell_textures(res, seed=21)
    tex_b = configs.cornell_textures(res, seed=22)
    target = torch.as_tensor(render(textured_renderer(tex_b), size, 128, max_depth=3), device=dev)
    r = textured_renderer(tex_a)
    texels = torch.tensor(tex_a, device=dev, requires_grad=True)
    kw = dict(fov=CAM["fov"], max_depth=4)
    img = render_textures(texels, r, size, CAM["origin"], CAM["direction"], 16, **kw)
    loss = ((img - target) ** 2).sum()
    loss.backward()
    direct = torch.empty(texels.numel(), dtype=torch.float64, device=dev)
    r.adjoint((2.0 * (img.detach() - target)).float(), direct, size, CAM["origin"], CAM["direction"], 16, **kw)
    # float32 atomics add in a different order on each call
    scale = float(direct.abs().max())
    assert torch.allclose(texels.grad.reshape(-1).double(), direct, rtol=1e-4, atol=1e-6 * scale)
    # gradient descent on one fixed-seed objective (depth 3: no roulette) lowers it
    kw = dict(fov=CAM["fov"], max_depth=3)
    opt = torch.optim.Adam([texels], lr=0.01)
    losses = []
    for it in range(8):
        opt.zero_grad()
        img = render_textures(texels, r, size, CAM["origin"], CAM["direction"], 16, **kw)
        loss = ((img - target) ** 2).sum()
        loss.backward()
        opt.step()
        with torch.no_grad():
            texels.clamp_(0.0, 1.0)
        losses.append(float(loss.detach()))
    assert losses[-1] < 0.9 * losses[0], losses


def test_adjoint_matches_the_fp64_oracle_with_nee_and_roulette(cuda_device):
    """NEE and Russian roulette on (depth 6): the GPU adjoint against the FP64
    CPU adjoint of the same paths (same random streams, survival
    probabilities held fixed on both sides)."""
    from oracle import pt64
    res, size, spp = 8, (32, 32), 16
    tex_a = configs.cornell_textures(res, seed=11)
    tex_b = configs.cornell_textures(res, seed=12)
    kw = dict(max_depth=6, use_nee=True)
    target = render(textured_renderer(tex_b), size, 64, **kw)
    r = textured_renderer(tex_a)
    _, g_gpu, img = loss_and_grad(r, target, size, spp, **kw)
    dl = (2.0 * (img.cpu().numpy() - target))
    objs, mesh, tx = configs.textured_cornell(tex_a)
    S = pt64.Scene64(objs, mesh, tx)
    img64 = S.render(size, CAM["origin"], CAM["direction"], spp, fov=CAM["fov"], **kw)
    assert abs(img64.mean() - img.cpu().numpy().mean()) < 1e-3 * img64.mean()
    g64 = S.adjoint(dl, size, CAM["origin"], CAM["direction"], spp, fov=CAM["fov"], **kw)
    agg = np.linalg.norm(g_gpu - g64) / np.linalg.norm(g64)
    assert agg < 1e-2, agg
