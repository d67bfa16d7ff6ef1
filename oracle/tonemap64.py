"""FP64 restatement of the reference's display transform (core/tonemap.cuh:6-139):
XYZ -> linear sRGB (D65) -> ACES fit / gamma / linear -> clamp.

TEST INFRASTRUCTURE ONLY (the checker of the GPU tonemap)."""
from __future__ import annotations

import numpy as np

XYZ_2_SRGB = np.array([[3.2406, -1.5372, -0.4986], [-0.9689, 1.8758, 0.0415], [0.0557, -0.204, 1.057]])
SRGB_2_AP0 = np.array([[0.4397010, 0.3829780, 0.1773350], [0.0897923, 0.8134230, 0.0967616],
                       [0.0175440, 0.1115440, 0.8707040]])
AP0_2_AP1 = np.array([[1.4514393161, -0.2365107469, -0.2149285693], [-0.0765537734, 1.1762296998, -0.0996759264],
                      [0.0083161484, -0.0060324498, 0.9977163014]])
AP1_2_XYZ = np.array([[0.6624541811, 0.1340042065, 0.1561876870], [0.2722287168, 0.6740817658, 0.0536895174],
                      [-0.0055746495, 0.0040607335, 1.0103391003]])
XYZ_2_AP1 = np.array([[1.6410233797, -0.3248032942, -0.2364246952], [-0.6636628587, 1.6153315917, 0.0167563477],
                      [0.0117218943, -0.0082844420, 0.9883948585]])
D60_2_D65 = np.array([[0.98722400, -0.00611327, 0.0159533], [-0.00759836, 1.00186000, 0.0053302],
                      [0.00307257, -0.00509595, 1.0816800]])
XYZ_2_REC709 = np.array([[3.2409699419, -1.5373831776, -0.4986107603], [-0.9692436363, 1.8759675015, 0.0415550574],
                         [0.0556300797, -0.2039769589, 1.0569715142]])
Y_W = np.array([0.272229, 0.674082, 0.0536895])


def _gamma(c):
    return np.maximum(c, 0.0) ** (1.0 / 2.2)


def _dim_surround(lin):
    xyz = lin @ AP1_2_XYZ.T
    div = np.maximum(xyz.sum(-1), 1e-4)
    x, y, Y = xyz[..., 0] / div, xyz[..., 1] / div, xyz[..., 1]
    Y = np.clip(Y, 0.0, 65504.0) ** 0.9811
    m = Y / np.maximum(y, 1e-4)
    xyz = np.stack([x * m, Y, (1 - x - y) * m], -1)
    return xyz @ XYZ_2_AP1.T


def aces(rgb):
    acescg = rgb @ SRGB_2_AP0.T @ AP0_2_AP1.T
    t = (acescg @ Y_W)[..., None]
    acescg = t * 0.04 + acescg * 0.96
    a, b, c, d, e = 278.5085, 10.7772, 293.6045, 88.7122, 80.6889
    post = (acescg * (acescg * a + b)) / (acescg * (acescg * c + d) + e)
    lin = _dim_surround(post)
    t = (lin @ Y_W)[..., None]
    lin = t * 0.07 + lin * 0.93
    xyz = lin @ AP1_2_XYZ.T @ D60_2_D65.T
    return _gamma(np.maximum(xyz @ XYZ_2_REC709.T, 0.0))


def tonemap(xyz, exposure=1.0, tone="aces"):
    """(h, w, 4) uint8 display image."""
    rgb = np.maximum(np.asarray(xyz, np.float64) * exposure @ XYZ_2_SRGB.T, 0.0)
    out = {"aces": aces, "gamma": _gamma, "linear": lambda c: c}[tone](rgb)
    out = np.clip(out, 0.0, 1.0)
    u8 = (out * 255.0).astype(np.uint8)
    return np.concatenate([u8, np.full(u8.shape[:-1] + (1,), 255, np.uint8)], -1)
