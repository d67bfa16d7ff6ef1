"""FP64 CPU oracle (oracle/pt64.cpp): the reference integrator restated in
double precision, with the replay adjoint of albedo textures.

TEST INFRASTRUCTURE ONLY: imported by tests/ and bench.py's reference legs,
never by the product package.  Build recipe: one g++ call (build() below,
also run by __graft_entry__.build()); the library lands in oracle/_build/.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
SRC = HERE / "pt64.cpp"
LIB = HERE / "_build" / "libpt64.so"
TABLES = ROOT / "aperturerendererv3_gb300" / "data" / "spectral_tables.npz"

_lib = None


def build(force: bool = False) -> Path:
    if LIB.exists() and not force and LIB.stat().st_mtime >= SRC.stat().st_mtime:
        return LIB
    LIB.parent.mkdir(parents=True, exist_ok=True)
    cmd = ["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-pthread", "-ffp-contract=off", str(SRC), "-o",
           str(LIB)]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return LIB


def load() -> C.CDLL:
    global _lib
    if _lib is None:
        lib = C.CDLL(str(build()))
        vp, i32 = C.c_void_p, C.c_int
        lib.pt64_create.restype = vp
        lib.pt64_create.argtypes = [vp, i32, vp, i32, vp, vp, vp, i32, vp, vp, i32, vp, vp, vp, i32, vp, i32,
                                    vp, i32, C.c_float, i32, C.c_char_p, i32]
        lib.pt64_set_medium.argtypes = [vp, vp]
        lib.pt64_set_sdf_f32.argtypes = [vp, i32]
        lib.pt64_adjoint_medium.restype = i32
        lib.pt64_adjoint_medium.argtypes = [vp, vp, vp, C.c_uint64, vp, vp]
        lib.pt64_destroy.argtypes = [vp]
        lib.pt64_render.restype = i32
        lib.pt64_render.argtypes = [vp, vp, vp, C.c_uint64, vp, vp]
        lib.pt64_render_crop.restype = i32
        lib.pt64_render_crop.argtypes = [vp, vp, vp, C.c_uint64, vp, vp]
        lib.pt64_adjoint_medium_crop.restype = i32
        lib.pt64_adjoint_medium_crop.argtypes = [vp, vp, vp, C.c_uint64, vp, vp, vp]
        lib.pt64_adjoint.restype = i32
        lib.pt64_adjoint.argtypes = [vp, vp, vp, C.c_uint64, vp, vp]
        _lib = lib
    return _lib


def _tables():
    t = np.load(TABLES)
    rgb = [t["RGB_IN_W"], t["RGB_IN_B"]]
    for b in range(7):
        rgb += [t[f"RGB_BLK{b}_W"], t[f"RGB_BLK{b}_B"]]
    rgb.append(t["RGB_OUT_W"])
    lam = []
    for b in range(7):
        lam += [t[f"LAM_BLK{b}_W"], t[f"LAM_BLK{b}_B"]]
    lam.append(t["LAM_OUT_W"])
    f32 = lambda a: np.ascontiguousarray(a, np.float32)
    return (f32(t["CIEXYZ_CMF"]).reshape(-1), f32(t["D65_SPD"]), f32(np.concatenate([x.reshape(-1) for x in rgb])),
            f32(np.concatenate([x.reshape(-1) for x in lam])))


def _material_row(m) -> list:
    tex = 0 if getattr(m, "texture", None) is None else int(m.texture) + 1
    return [m.shading, *m.albedo, *m.emissive, m.roughness, m.metallic, m.specular, m.ior, m.sigma_a, m.abbe, tex]


class Scene64:
    """An FP64 oracle scene built from the product's scene description classes."""

    def __init__(self, objects, mesh=None, textures=None, sdf=None, medium=None):
        lib = load()
        objects = list(objects)
        table: dict = {}
        mats: list = []

        def mid(m):
            if m not in table:
                table[m] = len(mats)
                mats.append(m)
            return table[m]

        orows = []
        for o in objects:
            orows.append([o.type, mid(o.material), *o.center, *o.extent, *o.rotation, *o.v0, *o.v1, *o.v2])
        tri = np.zeros((0, 9), np.float32)
        tri_mat = np.zeros(0, np.int32)
        tri_uv = None
        if mesh is not None:
            tri = mesh.triangle_vertices().astype(np.float32)
            remap = np.array([mid(m) for m in mesh.materials], np.int32)
            tri_mat = remap[np.asarray(mesh.material_ids, np.int64)].astype(np.int32)
            if mesh.uv is not None:
                tri_uv = np.ascontiguousarray(mesh.uv, np.float32).reshape(-1, 6)
        sdf_arr, sdf_mat = None, -1
        if sdf is not None:
            sdf_mat = mid(sdf.material)
            sdf_arr = sdf.array()
        m_arr = np.ascontiguousarray(np.array([_material_row(m) for m in mats], np.float32).reshape(-1, 14))
        o_arr = np.ascontiguousarray(np.array(orows, np.float32).reshape(-1, 20))
        textures = list(textures) if textures is not None else []
        sizes = np.array([[t.shape[1], t.shape[0]] for t in textures], np.int32).reshape(-1)
        texels = (np.concatenate([np.asarray(t, np.float32).reshape(-1) for t in textures]) if textures
                  else np.zeros(1, np.float32))
        self.texel_count = int(sum(t.size for t in textures))
        cmf, d65, rgb, lam = _tables()
        err = C.create_string_buffer(256)
        keep = [m_arr, o_arr, tri, tri_mat, tri_uv, sizes, texels, cmf, d65, rgb, lam, sdf_arr]
        self._keep = keep
        ptr = lambda a: None if a is None or a.size == 0 else a.ctypes.data
        self._h = lib.pt64_create(ptr(m_arr), len(m_arr), ptr(o_arr), len(o_arr), ptr(tri), ptr(tri_mat), ptr(tri_uv),
                                  len(tri), ptr(sizes), texels.ctypes.data, len(textures), cmf.ctypes.data,
                                  d65.ctypes.data, rgb.ctypes.data, rgb.size, lam.ctypes.data, lam.size,
                                  ptr(sdf_arr), 0 if sdf_arr is None else len(sdf_arr),
                                  0.0 if sdf is None else float(sdf.smooth_k), sdf_mat, err, 256)
        if not self._h:
            raise ValueError(f"FP64 oracle: {err.value.decode()}")
        self.set_medium(medium)

    def set_sdf_f32(self, on: bool):
        """Round the SDF march's positions, steps and distances to float (a
        float-sized perturbation of the SDF arithmetic; off by default)."""
        load().pt64_set_sdf_f32(self._h, 1 if on else 0)

    def set_medium(self, medium):
        if medium is None:
            load().pt64_set_medium(self._h, None)
            return
        m = np.array([*medium.box_lo, *medium.box_hi, medium.sigma_t, medium.albedo, medium.g, medium.emission],
                     np.float64)
        load().pt64_set_medium(self._h, m.ctypes.data)

    def __del__(self):
        if getattr(self, "_h", None):
            load().pt64_destroy(self._h)
            self._h = None

    @staticmethod
    def _params(size, origin, direction, spp, fov, max_depth, use_nee, first_frame, threads):
        ip = np.array([size[0], size[1], spp, max_depth, 1 if use_nee else 0, first_frame, threads], np.int32)
        dp = np.array([*origin, *direction, fov], np.float64)
        return ip, dp

    def render(self, size, origin, direction, spp, *, fov=60.0, max_depth=1000, use_nee=True,
               seed=0x9E3779B97F4A7C15, first_frame=0, per_sample=False, threads=0):
        """Per-pixel mean XYZ (h, w, 3) float64, and per-sample XYZ (spp, h, w, 3) when asked."""
        ip, dp = self._params(size, origin, direction, spp, fov, max_depth, use_nee, first_frame,
                              threads or os.cpu_count() or 1)
        w, h = int(size[0]), int(size[1])
        mean = np.zeros((h, w, 3), np.float64)
        ps = np.zeros((spp, h, w, 3), np.float64) if per_sample else None
        rc = load().pt64_render(self._h, ip.ctypes.data, dp.ctypes.data, seed, mean.ctypes.data,
                                ps.ctypes.data if ps is not None else None)
        if rc != 0:
            raise ValueError("FP64 oracle: bad render parameters")
        return (mean, ps) if per_sample else mean

    def render_crop(self, size, window, origin, direction, spp, *, fov=60.0, max_depth=1000, use_nee=True,
                    seed=0x9E3779B97F4A7C15, first_frame=0, threads=0):
        """Per-pixel mean XYZ (h, w, 3) of the window (x0, y0, w, h) of a size[0] x size[1]
        image: the same pixels, camera rays and random streams as in the full render."""
        ip, dp = self._params(size, origin, direction, spp, fov, max_depth, use_nee, first_frame,
                              threads or os.cpu_count() or 1)
        win = np.array(window, np.int32)
        mean = np.zeros((int(win[3]), int(win[2]), 3), np.float64)
        rc = load().pt64_render_crop(self._h, ip.ctypes.data, dp.ctypes.data, seed, win.ctypes.data, mean.ctypes.data)
        if rc != 0:
            raise ValueError("FP64 oracle: bad crop parameters")
        return mean

    def adjoint_medium(self, dl_dxyz, size, origin, direction, spp, *, fov=60.0, max_depth=1000, use_nee=True,
                       seed=0x9E3779B97F4A7C15, first_frame=0, threads=0, window=None):
        """(d loss / d medium albedo, d loss / d medium emission) given d(loss)/d(mean image)
        (h, w, 3).  window (x0, y0, w, h): only that window's pixels (the full
        image's rays and streams), i.e. the gradient of a loss that reads the
        window alone."""
        ip, dp = self._params(size, origin, direction, spp, fov, max_depth, use_nee, first_frame,
                              threads or os.cpu_count() or 1)
        dl = np.ascontiguousarray(dl_dxyz, np.float64)
        g = np.zeros(2, np.float64)
        if window is not None:
            win = np.array(window, np.int32)
            rc = load().pt64_adjoint_medium_crop(self._h, ip.ctypes.data, dp.ctypes.data, seed, win.ctypes.data,
                                                 dl.ctypes.data, g.ctypes.data)
        else:
            rc = load().pt64_adjoint_medium(self._h, ip.ctypes.data, dp.ctypes.data, seed, dl.ctypes.data,
                                            g.ctypes.data)
        if rc != 0:
            raise ValueError("FP64 oracle: bad adjoint parameters")
        return float(g[0]), float(g[1])

    def adjoint(self, dl_dxyz, size, origin, direction, spp, *, fov=60.0, max_depth=1000, use_nee=True,
                seed=0x9E3779B97F4A7C15, first_frame=0, threads=0):
        """d(loss)/d(texels) (texel_count float64) given d(loss)/d(mean image) (h, w, 3)."""
        ip, dp = self._params(size, origin, direction, spp, fov, max_depth, use_nee, first_frame,
                              threads or os.cpu_count() or 1)
        dl = np.ascontiguousarray(dl_dxyz, np.float64)
        grad = np.zeros(max(1, self.texel_count), np.float64)
        rc = load().pt64_adjoint(self._h, ip.ctypes.data, dp.ctypes.data, seed, dl.ctypes.data, grad.ctypes.data)
        if rc != 0:
            raise ValueError("FP64 oracle: bad adjoint parameters")
        return grad[: self.texel_count]
