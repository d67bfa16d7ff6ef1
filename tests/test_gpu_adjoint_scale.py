"""The differentiable-rendering workload at its stated scale: the textured
Cornell box with 8 albedo textures of 512 x 512 RGB texels (U[0.2, 0.8],
seed 11) as parameters, target rendered from a second texture set (seed 12)
at 256 spp, L2 loss at 64 spp, 256 x 256, NEE on; ar_adjoint's d(loss)/d(texel)
on 256 random texels (among those the render reaches):

* against the FP64 CPU adjoint of the same paths (oracle/pt64), depth 8 with
  Russian roulette: both hold the survival probabilities fixed, the unbiased
  choice;
* against central finite differences of the same seeded render (h = 1e-3,
  and steps inside the spectral LUT cell), depth 3: no roulette fires there (it starts at the third non-delta vertex,
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


LUT_RES = 512  # RGB -> spectrum lattice: planes at (i + 0.5) / 512 per channel


def _lattice_distance(x):
    g = np.asarray(x, np.float64) * LUT_RES - 0.5
    return np.abs(g - np.round(g)) / LUT_RES


def test_adjoint_vs_central_differences_at_scale(cuda_device):
    """Depth 3, NEE on.  Two step sizes per probed channel: h = 1e-3 as the
    workload states, and a step inside the channel's cell of the spectral LUT
    lattice (at most 1e-3).  The lattice cell is 1 / 512 wide, less than 2h, so
    an h = 1e-3 difference averages the slopes of two cells of the trilinear
    spectral albedo; inside a cell the estimator is linear in the channel and
    the difference quotient is its exact derivative.  An NEE decision
    (u < sqrt(throughput)) of a path through the texel can flip under the
    perturbation: a few channels, each a large jump, are left out of the
    aggregates."""
    r, tex_a, target, kw, g, probe, _ = _setup(depth=3)
    flat = tex_a.reshape(-1).astype(np.float64)

    def fd(step_of):
        out = np.empty(len(probe))
        for k, i in enumerate(probe):
            vals, at = [], []
            for sgn in (+1.0, -1.0):
                x32 = flat.astype(np.float32)
                x32[i] = np.float32(flat[i] + sgn * step_of(i))
                r.update_texels(x32)
                im = r.Render(SIZE, CAM["origin"], CAM["direction"], SPP, **kw)
                vals.append(((im - target) ** 2).sum())
                at.append(float(x32[i]))
            out[k] = (vals[0] - vals[1]) / (at[0] - at[1])
        return out

    fd_h = fd(lambda i: 1e-3)
    fd_cell = fd(lambda i: min(1e-3, 0.45 * float(_lattice_distance(flat[i]))))
    r.update_texels(flat.astype(np.float32))
    a = g[probe]
    rel_cell = np.abs(a - fd_cell) / np.abs(fd_cell)
    rel_h = np.abs(a - fd_h) / np.abs(fd_h)
    assert np.mean(rel_cell < 1e-2) > 0.95, (np.mean(rel_cell < 1e-2), np.sort(rel_cell)[-8:])
    ok = rel_cell < 0.1
    assert np.linalg.norm((a - fd_cell)[ok]) / np.linalg.norm(fd_cell[ok]) < 1e-2
    assert np.median(rel_h) < 1e-2 and np.mean(rel_h < 5e-2) > 0.9, (np.median(rel_h), np.mean(rel_h < 5e-2))
    ok = rel_h < 0.1
    assert np.linalg.norm((a - fd_h)[ok]) / np.linalg.norm(fd_h[ok]) < 2e-2
