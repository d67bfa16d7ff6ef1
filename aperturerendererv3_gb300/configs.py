"""Seeded synthetic scenes for the benchmark and test workloads.

  cornell_triangles()   Cornell box from 6 unit quads (12 triangles) and two
                        boxes (0.3^3 and 0.3x0.6x0.3, rotated -18/+18 degrees
                        about y; 12 triangles each), Lambertian albedos, one
                        0.25 x 0.25 ceiling area light (emission 17/12/4), camera
                        inside the box, fov 40: the 256x256 / 16 spp / depth 8
                        workload.  The area light is a thin box so the
                        reference's box-light sampler can sample it.
  reference_cornell()   the reference's own SceneHelper::CreateCornellBox
                        (core/helper/scene_helper.h:10-91): seven thin boxes,
                        GGX floor and metal back wall.
  random_triangles()    n triangles, centroids U[0,1]^3, vertices offset by
                        N(0, 0.005^2) per axis: the 1M-triangle BVH stress scene.
  textured_cornell()    the triangle Cornell box with a 512^2 albedo texture on
                        every wall and box (U[0.2, 0.8] from a seed): the
                        differentiable-rendering workload.
  combined_scene()      the terrain plus 32 smooth-union SDF primitives (spheres,
                        boxes, tori; radii U[0.05, 0.3]) and a homogeneous
                        medium (sigma_t 0.5, albedo 0.8, HG g 0.3) over it: the
                        large combined workload.
  terrain_scene()       2048^2 fBm heightfield (8 octaves, amplitude 0.2), 64
                        emissive spheres, a distant sun sphere, GGX materials
                        with roughness U[0.05, 0.6].
No dataset is involved; every scene is generated from its seed.
"""
from __future__ import annotations

import math

import numpy as np

from .scene import Material, Medium, SceneObject, SdfUnion, TriangleMesh
from ._lib import OBJECT_CUBE, OBJECT_SPHERE, SDF_BOX, SDF_SPHERE, SDF_TORUS

GREY = (0.73, 0.73, 0.73)
RED = (0.63, 0.065, 0.05)
GREEN = (0.14, 0.45, 0.09)


def _quad(a, b, c, d, mat):
    return [SceneObject.Triangle(a, b, c, mat), SceneObject.Triangle(a, c, d, mat)]


def _box_tris(center, half, rot_y_deg, mat):
    """12 triangles of an oriented box (rotation about +y)."""
    cy, sy = math.cos(math.radians(rot_y_deg)), math.sin(math.radians(rot_y_deg))

    def p(x, y, z):
        x, y, z = x * half[0], y * half[1], z * half[2]
        return (float(np.float32(center[0] + cy * x + sy * z)), float(np.float32(center[1] + y)),
                float(np.float32(center[2] - sy * x + cy * z)))

    c = {(i, j, k): p(i, j, k) for i in (-1, 1) for j in (-1, 1) for k in (-1, 1)}
    faces = [((-1, -1, -1), (1, -1, -1), (1, 1, -1), (-1, 1, -1)),
             ((-1, -1, 1), (-1, 1, 1), (1, 1, 1), (1, -1, 1)),
             ((-1, -1, -1), (-1, 1, -1), (-1, 1, 1), (-1, -1, 1)),
             ((1, -1, -1), (1, -1, 1), (1, 1, 1), (1, 1, -1)),
             ((-1, -1, -1), (-1, -1, 1), (1, -1, 1), (1, -1, -1)),
             ((-1, 1, -1), (1, 1, -1), (1, 1, 1), (-1, 1, 1))]
    out = []
    for f in faces:
        out += _quad(c[f[0]], c[f[1]], c[f[2]], c[f[3]], mat)
    return out


CORNELL_CAMERA = dict(origin=(0.0, 0.0, 0.49), direction=(0.0, 0.0, -1.0), fov=40.0)


def cornell_triangles() -> list[SceneObject]:
    grey = Material.CreateDiffusePureColor(GREY)
    red = Material.CreateDiffusePureColor(RED)
    green = Material.CreateDiffusePureColor(GREEN)
    h = 0.5
    objs = []
    objs += _quad((-h, -h, -h), (h, -h, -h), (h, -h, h), (-h, -h, h), grey)      # floor
    objs += _quad((-h, h, -h), (-h, h, h), (h, h, h), (h, h, -h), grey)          # ceiling
    objs += _quad((-h, -h, -h), (-h, h, -h), (h, h, -h), (h, -h, -h), grey)      # back
    objs += _quad((-h, -h, h), (h, -h, h), (h, h, h), (-h, h, h), grey)          # front
    objs += _quad((-h, -h, -h), (-h, -h, h), (-h, h, h), (-h, h, -h), red)       # left
    objs += _quad((h, -h, -h), (h, h, -h), (h, h, h), (h, -h, h), green)         # right
    objs += _box_tris((0.18, -0.35, 0.12), (0.15, 0.15, 0.15), -18.0, grey)      # short box
    objs += _box_tris((-0.17, -0.2, -0.15), (0.15, 0.3, 0.15), 18.0, grey)       # tall box
    objs.append(SceneObject((0.0, 0.5 - 0.005, 0.0), (0.125, 0.005, 0.125), Material.CreateLight((17.0, 12.0, 4.0)),
                            (0.0, 0.0, 0.0), OBJECT_CUBE))
    return objs


def _quad_uv(a, b, c, d):
    """Two triangles (a, b, c), (a, c, d) and their corner uvs (a, b, c, d) -> (0,0) (1,0) (1,1) (0,1)."""
    tris = [a + b + c, a + c + d]
    uvs = [(0.0, 0.0, 1.0, 0.0, 1.0, 1.0), (0.0, 0.0, 1.0, 1.0, 0.0, 1.0)]
    return tris, uvs


def _box_quads(center, half, rot_y_deg):
    cy, sy = math.cos(math.radians(rot_y_deg)), math.sin(math.radians(rot_y_deg))

    def p(x, y, z):
        x, y, z = x * half[0], y * half[1], z * half[2]
        return (float(np.float32(center[0] + cy * x + sy * z)), float(np.float32(center[1] + y)),
                float(np.float32(center[2] - sy * x + cy * z)))

    c = {(i, j, k): p(i, j, k) for i in (-1, 1) for j in (-1, 1) for k in (-1, 1)}
    faces = [((-1, -1, -1), (1, -1, -1), (1, 1, -1), (-1, 1, -1)),
             ((-1, -1, 1), (-1, 1, 1), (1, 1, 1), (1, -1, 1)),
             ((-1, -1, -1), (-1, 1, -1), (-1, 1, 1), (-1, -1, 1)),
             ((1, -1, -1), (1, -1, 1), (1, 1, 1), (1, 1, -1)),
             ((-1, -1, -1), (-1, -1, 1), (1, -1, 1), (1, -1, -1)),
             ((-1, 1, -1), (1, 1, -1), (1, 1, 1), (-1, 1, 1))]
    return [(c[f[0]], c[f[1]], c[f[2]], c[f[3]]) for f in faces]


def cornell_textures(res: int = 512, seed: int = 11, n: int = 8) -> np.ndarray:
    """n albedo textures of res x res RGB texels, U[0.2, 0.8] from `seed`: (n, res, res, 3) float32."""
    rng = np.random.default_rng(seed)
    return rng.uniform(0.2, 0.8, (n, res, res, 3)).astype(np.float32)


def textured_cornell(textures: np.ndarray):
    """The triangle Cornell box with every wall and both boxes carrying an albedo
    texture (the differentiable-rendering workload): 6 walls + 2 boxes = 8
    textures, one per surface group; each wall quad and each box face spans its
    texture's full [0,1]^2.  Returns (objects, mesh, textures): the ceiling light
    (a thin box) is the only object, everything textured is the mesh."""
    h = 0.5
    walls = [((-h, -h, -h), (h, -h, -h), (h, -h, h), (-h, -h, h)),      # floor
             ((-h, h, -h), (-h, h, h), (h, h, h), (h, h, -h)),          # ceiling
             ((-h, -h, -h), (-h, h, -h), (h, h, -h), (h, -h, -h)),      # back
             ((-h, -h, h), (h, -h, h), (h, h, h), (-h, h, h)),          # front
             ((-h, -h, -h), (-h, -h, h), (-h, h, h), (-h, h, -h)),      # left
             ((h, -h, -h), (h, h, -h), (h, h, h), (h, -h, h))]          # right
    groups = [[w] for w in walls]
    groups.append(_box_quads((0.18, -0.35, 0.12), (0.15, 0.15, 0.15), -18.0))
    groups.append(_box_quads((-0.17, -0.2, -0.15), (0.15, 0.3, 0.15), 18.0))
    assert len(textures) == len(groups)
    tris, uvs, mids = [], [], []
    for g, quads in enumerate(groups):
        for q in quads:
            t, u = _quad_uv(*q)
            tris += t
            uvs += u
            mids += [g, g]
    mats = [Material.CreateDiffuseTextured(g) for g in range(len(groups))]
    v = np.asarray(tris, np.float32).reshape(-1, 3)
    mesh = TriangleMesh(v, np.arange(len(v), dtype=np.uint32).reshape(-1, 3), np.asarray(mids, np.int32), mats,
                        uv=np.asarray(uvs, np.float32))
    light = SceneObject((0.0, 0.5 - 0.005, 0.0), (0.125, 0.005, 0.125), Material.CreateLight((17.0, 12.0, 4.0)),
                        (0.0, 0.0, 0.0), OBJECT_CUBE)
    return [light], mesh, [t for t in textures]


REFERENCE_CORNELL_CAMERA = dict(origin=(0.0, 0.0, 1.1), direction=(0.0, 0.0, -1.0), fov=60.0)


def reference_cornell(light=(10.0, 10.0, 10.0)) -> list[SceneObject]:
    """SceneHelper::CreateCornellBox with its default arguments."""
    T = 0.01
    white = (1.0, 1.0, 1.0)
    dark = (0.75, 0.75, 0.75)  # WhiteDarken(0.25)
    objs = [
        SceneObject((0.0, -0.5 - T, 0.0), (0.5, T, 0.5), Material.CreateGGXPureColor(dark, 0.05, 0.0, 0.5)),
        SceneObject((0.0, 0.5 + T, 0.0), (0.5, T, 0.5), Material.CreateDiffusePureColor(white)),
        SceneObject((0.0, 0.5 - T, 0.0), (0.125 * 0.25, T, 0.125 * 0.25), Material.CreateLight(light)),
        SceneObject((0.0, 0.0, -0.5 - T), (0.5, 0.5, T), Material.CreateGGXPureColor(dark, 0.25, 1.0, 0.5)),
        SceneObject((-0.5, 0.0, 0.0), (T, 0.5, 0.5), Material.CreateDiffusePureColor((1.0, 0.0, 0.0))),
        SceneObject((0.5, 0.0, 0.0), (T, 0.5, 0.5), Material.CreateDiffusePureColor((0.0, 1.0, 0.0))),
    ]
    return objs


def _lerp32(a, b, v) -> tuple:
    """lerp(a, b, v) = a (1 - v) + b v in float32, per channel (core/vector.cuh:241-243)."""
    a = np.asarray(a, np.float32)
    b, v = np.float32(b), np.float32(v)
    return tuple(float(x) for x in (a * (np.float32(1.0) - v) + b * v).astype(np.float32))


GLASS_TEST_CAMERA = dict(origin=(0.0, 0.0, 1.1), direction=(0.0, 0.0, -1.0), fov=60.0)


def glass_test_scene(position=(0.0, 0.0, 0.0), ior_strength: float = 1.0, abbe: float = 20.0,
                     tilt: float = 0.0) -> list[SceneObject]:
    """SceneHelper::CreateGlassTestScene (core/helper/scene_helper.h:172-258): five
    glass spheres and three tilted glass slabs (Fresnel, refraction with Abbe
    dispersion, Beer-Lambert absorption, total internal reflection), a small
    spherical light and three GGX slabs; colours as color::* (core/render/color.cuh)."""
    px, py, pz = (float(c) for c in position)

    def at(x, y, z):
        return (float(np.float32(x) + np.float32(px)), float(np.float32(y) + np.float32(py)),
                float(np.float32(z) + np.float32(pz)))

    def ior(b):
        return _lerp32((1.0,), b, ior_strength)[0]

    white, yellow, cyan = (1.0, 1.0, 1.0), (1.0, 1.0, 0.0), (0.0, 1.0, 1.0)
    red, blue, purple = (1.0, 0.0, 0.0), (0.0, 0.0, 1.0), (1.0, 0.0, 1.0)
    azure, orange = (0.25, 0.5, 1.0), (1.0, 0.5, 0.25)
    ball, slab = (0.125, 0.125, 0.125), (0.125, 0.125, 0.01)
    G = Material.CreateGlassPureColor
    S, C = OBJECT_SPHERE, OBJECT_CUBE
    return [
        SceneObject(at(0.0, 0.25, 0.125), ball, G(white, ior(1.6), 1.0, abbe, tilt), (0.0, 0.0, 0.0), S),
        SceneObject(at(0.125, 0.25, -0.125), (0.05, 0.05, 0.05), Material.CreateLight((25.0, 25.0, 25.0)),
                    (0.0, 0.0, 0.0), S),
        SceneObject(at(-0.25, 0.0, -0.125), ball, G(yellow, ior(1.5), 1.0, abbe, tilt), (0.0, 0.0, 0.0), S),
        SceneObject(at(0.25, 0.0, 0.125), ball, G(cyan, ior(1.55), 1.0, abbe, tilt), (0.0, 0.0, 0.0), S),
        SceneObject(at(0.0, 0.0, 0.0), ball, G(_lerp32(red, 1.0, 0.01), ior(1.45), 1.0, abbe, tilt), (0.0, 0.0, 0.0), S),
        SceneObject(at(0.0, -0.25, -0.125), ball, G(_lerp32(blue, 1.0, 0.01), ior(1.5), 1.0, abbe, tilt),
                    (0.0, 0.0, 0.0), S),
        SceneObject(at(0.0, 0.0, 0.25), slab, G(azure, ior(1.5), 25.0, abbe, tilt), (0.0, 0.0, 0.0), C),
        SceneObject(at(0.0, -0.25, 0.3), slab, G(_lerp32(red, 1.0, 0.25), ior(1.5), 25.0, abbe, tilt),
                    (30.0, 0.0, 0.0), C),
        SceneObject(at(0.0, 0.25, 0.3), slab, G(_lerp32(purple, 1.0, 0.25), ior(1.5), 25.0, abbe, tilt),
                    (-30.0, 0.0, 0.0), C),
        SceneObject(at(0.0, 0.0, -0.25), slab, Material.CreateGGXPureColor(orange, 0.1, 1.0, 1.0), (0.0, 0.0, 0.0), C),
        SceneObject(at(0.0, -0.25, -0.3), slab, Material.CreateGGXPureColor(_lerp32(white, 0.0, 0.9), 0.1, 0.0, 0.5),
                    (-30.0, 0.0, 0.0), C),
        SceneObject(at(0.0, 0.25, -0.3), slab, Material.CreateGGXPureColor(_lerp32(white, 0.0, 0.5), 0.5, 1.0, 1.0),
                    (30.0, 0.0, 0.0), C),
    ]


def random_triangles(n: int, seed: int = 1) -> np.ndarray:
    """(n, 9) float32 triangle vertices."""
    rng = np.random.default_rng(seed)
    c = rng.random((n, 1, 3), dtype=np.float64)
    v = c + rng.normal(0.0, 0.005, size=(n, 3, 3))
    return v.astype(np.float32).reshape(n, 9)


def pinhole_rays(width: int, height: int, origin, direction, fov: float) -> np.ndarray:
    """(W*H, 8) float32 rays through pixel centres: (o, tmin=0, d, tmax=inf)."""
    o = np.asarray(origin, np.float64)
    d = np.asarray(direction, np.float64)
    d /= np.linalg.norm(d)
    right = np.cross(d, [0.0, 1.0, 0.0])
    right /= np.linalg.norm(right)
    up = np.cross(d, right)
    up /= np.linalg.norm(up)
    th = math.tan(math.radians(fov) * 0.5)
    aspect = width / max(1.0, height)
    j, i = np.mgrid[0:height, 0:width]
    sx = ((i + 0.5) / width * 2.0 - 1.0) * th * aspect
    sy = ((1.0 - (j + 0.5) / height) * 2.0 - 1.0) * th
    dirs = d[None, None] + right[None, None] * sx[..., None] + up[None, None] * sy[..., None]
    dirs /= np.linalg.norm(dirs, axis=-1, keepdims=True)
    rays = np.zeros((height * width, 8), np.float32)
    rays[:, 0:3] = o
    rays[:, 3] = 0.0
    rays[:, 4:7] = dirs.reshape(-1, 3)
    rays[:, 7] = np.inf
    return rays


BVH_STRESS_CAMERA = dict(origin=(0.5, 0.5, 2.0), direction=(0.0, 0.0, -1.0), fov=40.0)


def _fbm_heightfield(res: int, octaves: int, amplitude: float, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    h = np.zeros((res, res), np.float64)
    amp, total = 1.0, 0.0
    for o in range(octaves):
        cells = 2 ** (o + 2)
        g = rng.random((cells + 1, cells + 1))
        x = np.linspace(0.0, cells, res)
        i0 = np.minimum(x.astype(np.int64), cells - 1)
        f = x - i0
        f = f * f * (3.0 - 2.0 * f)
        a = g[i0][:, i0] * (1 - f)[None, :] + g[i0][:, i0 + 1] * f[None, :]
        b = g[i0 + 1][:, i0] * (1 - f)[None, :] + g[i0 + 1][:, i0 + 1] * f[None, :]
        h += amp * (a * (1 - f)[:, None] + b * f[:, None])
        total += amp
        amp *= 0.5
    return (h / total - 0.5) * amplitude


TERRAIN_CAMERA = dict(origin=(0.5, 0.45, 1.55), direction=(0.0, -0.35, -1.0), fov=40.0)


def terrain_scene(res: int = 2048, n_spheres: int = 64, seed: int = 7):
    """Returns (objects, mesh): spheres + sun as objects, the heightfield as a mesh."""
    rng = np.random.default_rng(seed)
    hf = _fbm_heightfield(res, 8, 0.2, seed)
    xs = np.linspace(0.0, 1.0, res)
    X, Z = np.meshgrid(xs, xs, indexing="xy")
    verts = np.stack([X, hf, Z], -1).reshape(-1, 3).astype(np.float32)
    ii, jj = np.mgrid[0:res - 1, 0:res - 1]
    a = (jj * res + ii).reshape(-1)
    b = a + 1
    c = a + res
    d = c + 1
    idx = np.concatenate([np.stack([a, c, b], 1), np.stack([b, c, d], 1)]).astype(np.uint32)
    n_mat = 16
    mats = [Material.CreateGGXPureColor(tuple(rng.uniform(0.3, 0.8, 3)), float(r), 0.0, 0.5)
            for r in rng.uniform(0.05, 0.6, n_mat)]
    mat_ids = rng.integers(0, n_mat, len(idx)).astype(np.int32)
    mesh = TriangleMesh(verts, idx, mat_ids, mats)
    objs = []
    for _ in range(n_spheres):
        r = float(rng.uniform(0.005, 0.02))
        x, z = rng.uniform(0.05, 0.95, 2)
        gi, gj = int(z * (res - 1)), int(x * (res - 1))
        y = float(hf[gi, gj]) + r + 0.01
        le = float(rng.uniform(5.0, 50.0))
        col = rng.uniform(0.5, 1.0, 3)
        objs.append(SceneObject((float(x), y, float(z)), (r, r, r), Material.CreateLight(tuple(le * col)),
                                (0.0, 0.0, 0.0), OBJECT_SPHERE))
    # small distant sun
    objs.append(SceneObject((-20.0, 40.0, -30.0), (1.0, 1.0, 1.0), Material.CreateLight((400.0, 380.0, 330.0)),
                            (0.0, 0.0, 0.0), OBJECT_SPHERE))
    return objs, mesh


COMBINED_CAMERA = dict(origin=(0.5, 0.55, 1.75), direction=(0.0, -0.3, -1.0), fov=45.0)


def sdf_blobs(n: int = 32, seed: int = 5, k: float = 0.08) -> SdfUnion:
    """n SDF primitives (spheres, boxes, tori; radii U[0.05, 0.3]) above the
    terrain's unit square, in one smooth union."""
    rng = np.random.default_rng(seed)
    prims = []
    for i in range(n):
        kind = (SDF_SPHERE, SDF_BOX, SDF_TORUS)[i % 3]
        r = float(rng.uniform(0.05, 0.3))
        c = (float(rng.uniform(0.15, 0.85)), float(rng.uniform(0.15, 0.45)), float(rng.uniform(0.15, 0.85)))
        if kind == SDF_SPHERE:
            size = (r, 0.0, 0.0)
        elif kind == SDF_BOX:
            size = (r, 0.6 * r, 0.8 * r)
        else:
            size = (r, 0.3 * r, 0.0)
        prims.append((kind, c, size))
    return SdfUnion(prims, k, Material.CreateGGXPureColor((0.8, 0.55, 0.35), 0.3, 0.0, 0.5))


COMBINED_MEDIUM = Medium((-0.05, -0.15, -0.05), (1.05, 0.9, 1.05), sigma_t=0.5, albedo=0.8, g=0.3, emission=0.05)


def combined_scene(res: int = 2048, n_spheres: int = 64, seed: int = 7):
    """(objects, mesh, sdf, medium) of the large combined workload."""
    objs, mesh = terrain_scene(res=res, n_spheres=n_spheres, seed=seed)
    return objs, mesh, sdf_blobs(), COMBINED_MEDIUM
