"""Rays of the BVH stress workload (1M random triangles, centroids U[0,1]^3,
vertices offset by N(0, 0.005^2); 1920x1080 pinhole primary rays plus one
cosine-hemisphere bounce ray per primary hit), built with elementwise IEEE
operations only (no library trigonometry, no vector reductions), so that the
same primary hits give the same float32 bounce rays on every machine.  Shared
by the fixture script (make_bvh_stress_fixture.py) and the GPU test."""
from __future__ import annotations

import hashlib

import numpy as np

N_TRIS = 1_000_000
WIDTH, HEIGHT = 1920, 1080
ORIGIN = (0.5, 0.5, 2.0)
FOV_TAN_HALF = 0.36397023426620234  # tan(20 degrees): the 40-degree vertical field of view
BLOCK = 65536  # rays per hash block


def triangles() -> np.ndarray:
    from aperturerendererv3_gb300 import configs
    return configs.random_triangles(N_TRIS, seed=1)


def _norm3(x, y, z):
    return np.sqrt(x * x + y * y + z * z)


def primary_rays() -> np.ndarray:
    """(W*H, 8) float32: origin, tmin 0, direction towards -z through pixel centres, tmax inf."""
    j, i = np.mgrid[0:HEIGHT, 0:WIDTH]
    sx = ((i + 0.5) / WIDTH * 2.0 - 1.0) * (FOV_TAN_HALF * (WIDTH / HEIGHT))
    sy = ((1.0 - (j + 0.5) / HEIGHT) * 2.0 - 1.0) * FOV_TAN_HALF
    # the reference's camera frame for a view down -z (core/scene.cu:158-160):
    # right = normalize(dir x (0, 1, 0)) = +x, up = normalize(dir x right) = -y
    dx, dy, dz = sx, -sy, -np.ones_like(sx)
    ln = _norm3(dx, dy, dz)
    rays = np.zeros((HEIGHT * WIDTH, 8), np.float32)
    rays[:, 0:3] = ORIGIN
    rays[:, 4] = (dx / ln).reshape(-1)
    rays[:, 5] = (dy / ln).reshape(-1)
    rays[:, 6] = (dz / ln).reshape(-1)
    rays[:, 7] = np.inf
    return rays


def bounce_rays(tris: np.ndarray, rays: np.ndarray, ids: np.ndarray, t: np.ndarray, seed: int = 5) -> np.ndarray:
    """One cosine-hemisphere bounce per hit about the geometric normal facing the
    ray: a uniform point of the unit disk by rejection (seeded PCG64 stream)
    lifted to the hemisphere (Malley's method)."""
    hit = ids >= 0
    r = rays[hit].astype(np.float64)
    o = r[:, 0:3] + r[:, 4:7] * t[hit, None].astype(np.float64)
    v = tris[ids[hit]].reshape(-1, 3, 3).astype(np.float64)
    e1, e2 = v[:, 1] - v[:, 0], v[:, 2] - v[:, 0]
    nx = e1[:, 1] * e2[:, 2] - e1[:, 2] * e2[:, 1]
    ny = e1[:, 2] * e2[:, 0] - e1[:, 0] * e2[:, 2]
    nz = e1[:, 0] * e2[:, 1] - e1[:, 1] * e2[:, 0]
    ln = _norm3(nx, ny, nz)
    nx, ny, nz = nx / ln, ny / ln, nz / ln
    flip = (nx * r[:, 4] + ny * r[:, 5] + nz * r[:, 6]) > 0
    nx, ny, nz = np.where(flip, -nx, nx), np.where(flip, -ny, ny), np.where(flip, -nz, nz)
    # disk samples by rejection: 4 candidates per ray, first inside wins (redraw the rest)
    rng = np.random.default_rng(seed)
    m = len(nx)
    px = np.zeros(m)
    py = np.zeros(m)
    todo = np.arange(m)
    while len(todo):
        cx = rng.random(len(todo)) * 2.0 - 1.0
        cy = rng.random(len(todo)) * 2.0 - 1.0
        ok = cx * cx + cy * cy < 1.0
        px[todo[ok]] = cx[ok]
        py[todo[ok]] = cy[ok]
        todo = todo[~ok]
    pz = np.sqrt(np.maximum(0.0, 1.0 - px * px - py * py))
    # tangent frame: t = normalize(a x n) with a = z unless n is near z
    near_z = np.abs(nz) >= 0.999
    ax, ay, az = np.where(near_z, 1.0, 0.0), 0.0 * nx, np.where(near_z, 0.0, 1.0)
    tx = ay * nz - az * ny
    ty = az * nx - ax * nz
    tz = ax * ny - ay * nx
    lt = _norm3(tx, ty, tz)
    tx, ty, tz = tx / lt, ty / lt, tz / lt
    bx = ny * tz - nz * ty
    by = nz * tx - nx * tz
    bz = nx * ty - ny * tx
    dx = tx * px + bx * py + nx * pz
    dy = ty * px + by * py + ny * pz
    dz = tz * px + bz * py + nz * pz
    ld = _norm3(dx, dy, dz)
    out = np.zeros((m, 8), np.float32)
    out[:, 0:3] = o
    out[:, 3] = 1e-4
    out[:, 4] = dx / ld
    out[:, 5] = dy / ld
    out[:, 6] = dz / ld
    out[:, 7] = np.inf
    return out


def block_hashes(ids: np.ndarray, t: np.ndarray) -> list[str]:
    """SHA-256 (first 16 hex digits) of each BLOCK rays' int32 ids followed by float32 t bits."""
    ids = np.ascontiguousarray(ids, np.int32)
    t = np.ascontiguousarray(t, np.float32)
    out = []
    for a in range(0, len(ids), BLOCK):
        h = hashlib.sha256(ids[a:a + BLOCK].tobytes() + t[a:a + BLOCK].view(np.uint32).tobytes())
        out.append(h.hexdigest()[:16])
    return out
