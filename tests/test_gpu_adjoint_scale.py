"""The differentiable-rendering workload at its stated scale: the textured
Cornell box with 8 albedo textures of 512 x 512 RGB texels (U[0.2, 0.8],
seed 11) as parameters, target rendered from a second texture set (seed 12)
at 256 spp, L2 loss at 64 spp, 256 x 256, NEE on; ar_adjoint's d(loss)/d(texel)
on 256 random texels (among those the render reaches):

* against the FP64 CPU adjoint of the same paths (oracle/pt64), depth 8 with
  Russian roulette: both hold the survival probabilities fixed, the unbiased
  choice;
* against central finite differences with h = 1e-3 of the same seeded render,
  depth 3: no roulette fires there (it starts at the third non-delta vertex,
  core/render/render.cuh:838-859).  With roulette on, a same-seed difference
  quotient differentiates the realisation, in which the survival probability
  q = clamp(throughput) cancels the albedos before an unclamped roulette
  (throughput / q = 1), while the adjoint keeps q fixed; the two then differ
  by design, not by error."""
import numpy as np
import pytest

from aperturerendererv3_gb300 import SceneRenderer, configs

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

CAM = configs.CORNELL_CAMERA
SIZE, SPP, RES = (256, 256), 64, 512


def _renderer(textures):
    objs, mesh, tex = configs.textured_cornell(textures)
    return SceneRenderer(objs, mesh=mesh, textures=tex)


def _setup(depth):
    dev = torch.device("cuda", 0)
    tex_a = configs.cornell_textures(RES, seed=11)
    tex_b = configs.cornell_textures(RES, seed=12)
    kw = dict(fov=CAM["fov"], max_depth=depth, use_nee=True)
    target = _renderer(tex_b).Render(SIZE, CAM["origin"], CAM["direction"], 256, **kw)
    r = _renderer(tex_a)
    img = torch.empty((SIZE[1], SIZE[0], 3), dtype=torch.float64, device=dev)
    r.render_into(img, SIZE, CAM["origin"], CAM["direction"], SPP, **kw)
    t = torch.as_tensor(target, device=dev)
    g = torch.empty(r.texel_count(), dtype=torch.float64, device=dev)
    dl = (2.0 * (img - t)).float()
    r.adjoint(dl, g, SIZE, CAM["origin"], CAM["direction"], SPP, **kw)
    g = g.cpu().numpy()
    nz = np.flatnonzero(np.abs(g) > 1e-3 * np.abs(g).max())
    probe = np.sort(np.random.default_rng(3).choice(nz, 256, replace=False))
    return r, tex_a, target, kw, g, probe, dl.double().cpu().numpy()


def test_adjoint_vs_fp64_adjoint_at_scale(cuda_device):
    from oracle import pt64
    r, tex_a, target, kw, g, probe, dl = _setup(depth=8)
    objs, mesh, tx = configs.textured_cornell(tex_a)
    g64 = pt64.Scene64(objs, mesh, tx).adjoint(dl, SIZE, CAM["origin"], CAM["direction"], SPP, **kw)
    a, b = g[probe], g64[probe]
    agg = np.linalg.norm(a - b) / np.linalg.norm(b)
    rel = np.abs(a - b) / np.abs(b)
    assert agg < 1e-2, agg
    assert np.mean(rel < 1e-2) > 0.9, np.sort(rel)[-8:]
    # the whole gradient (6.3M texel channels, most reached by a handful of paths,
    # some of whose roulette decisions part ways between float and double)
    assert np.linalg.norm(g - g64) / np.linalg.norm(g64) < 5e-2
    assert r.error_word() == 0


def test_adjoint_vs_central_differences_at_scale(cuda_device):
    r, tex_a, target, kw, g, probe, _ = _setup(depth=3)
    flat = tex_a.reshape(-1).astype(np.float64)
    fd = np.empty(len(probe))
    for k, i in enumerate(probe):
        vals, at = [], []
        for sgn in (+1.0, -1.0):
            x32 = flat.astype(np.float32)
            x32[i] = np.float32(flat[i] + sgn * 1e-3)
            r.update_texels(x32)
            im = r.Render(SIZE, CAM["origin"], CAM["direction"], SPP, **kw)
            vals.append(((im - target) ** 2).sum())
            at.append(float(x32[i]))
        fd[k] = (vals[0] - vals[1]) / (at[0] - at[1])
    r.update_texels(flat.astype(np.float32))
    a = g[probe]
    rel = np.abs(a - fd) / np.abs(fd)
    agg = np.linalg.norm(a - fd) / np.linalg.norm(fd)
    # an NEE decision (u < sqrt(throughput)) of a path through the texel can flip
    # under the perturbation: a few texels, each a large jump
    assert np.mean(rel < 1e-2) > 0.9, (np.mean(rel < 1e-2), np.sort(rel)[-8:])
    ok = rel < 0.5
    assert np.linalg.norm((a - fd)[ok]) / np.linalg.norm(fd[ok]) < 1e-2, agg
