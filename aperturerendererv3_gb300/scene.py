"""Host-side mirror of the reference's scene interface.

Names, argument meaning and defaults follow the reference so calling code reads
the same:
  Material.Create*                core/render/object.cuh:119-206
  SceneObject(center, extent, material, rotation, type)
                                  core/render/object.cuh:227-316
  SceneRenderer(objects).Render(size, origin, direction, sampleNum)
                                  core/scene.hpp:94-114, core/scene.cu:210-238
  Camera(renderer, name, resX, resY, position, direction).RenderToFile(...)
                                  core/camera.hpp:56-99, core/camera.cu:64-89
Differences, all additive: triangles and triangle meshes (the reference has
none), a field of view argument (the reference fixes 60 degrees), a path-depth
cap, and FP64 accumulation of the returned linear XYZ.  Everything runs through
the C ABI (include/aperture/ar.h); there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import Iterable, Sequence

import numpy as np

from . import _lib
from ._lib import (GLOBAL_SEED, OBJECT_CUBE, OBJECT_SDF, OBJECT_SPHERE, OBJECT_TRIANGLE, SDF_FN_DIAMOND, SDF_FN_TORUS,
                   SDF_OBJECT_TORUS, SDF_OBJECT_VOLUME, SHADING_DIFFUSE, SHADING_GGX, SHADING_GLASS, SHADING_LIGHT,
                   ArMaterial, ArMedium, ArObject, ArRenderParams, check)

Vec3 = Sequence[float]


CUDA_STREAM_LEGACY = 1  # cudaStreamLegacy


def _torch_stream(device) -> int:
    """torch's current stream as a cudaStream_t for the C ABI.  torch's default
    stream has handle 0, which the C ABI reads as "the context's own stream";
    the legacy default stream's own handle keeps the work ordered with torch."""
    import torch
    h = torch.cuda.current_stream(device).cuda_stream
    return h if h else CUDA_STREAM_LEGACY


def _f3(v: Vec3) -> tuple[float, float, float]:
    return (float(v[0]), float(v[1]), float(v[2]))


@dataclass(frozen=True)
class Material:
    shading: int = SHADING_DIFFUSE
    albedo: tuple = (1.0, 1.0, 1.0)
    emissive: tuple = (0.0, 0.0, 0.0)
    roughness: float = 0.0
    metallic: float = 0.0
    specular: float = 0.0
    ior: float = 1.5
    sigma_a: float = 100.0
    abbe: float = 20.0
    tilt: float = 0.0
    texture: int | None = None   # albedo texture index (SceneRenderer textures); None = albedo

    @staticmethod
    def CreateDiffusePureColor(color: Vec3, emissive: Vec3 = (0.0, 0.0, 0.0)) -> "Material":
        return Material(SHADING_DIFFUSE, _f3(color), _f3(emissive))

    @staticmethod
    def CreateLight(emissive: Vec3) -> "Material":
        return Material(SHADING_LIGHT, (0.0, 0.0, 0.0), _f3(emissive))

    @staticmethod
    def CreateGlassPureColor(color: Vec3, IOR: float, sigmaA: float, abbeNumber: float = 20.0,
                             tiltNumber: float = 0.0) -> "Material":
        return Material(SHADING_GLASS, _f3(color), (0.0, 0.0, 0.0), ior=float(IOR), sigma_a=float(sigmaA),
                        abbe=float(abbeNumber), tilt=float(tiltNumber))

    @staticmethod
    def CreateGGXPureColor(baseColor: Vec3, roughness: float, metallic: float, specular: float,
                           emissive: Vec3 = (0.0, 0.0, 0.0)) -> "Material":
        return Material(SHADING_GGX, _f3(baseColor), _f3(emissive), roughness=float(roughness),
                        metallic=float(metallic), specular=float(specular))

    def to_c(self) -> ArMaterial:
        m = ArMaterial()
        m.shading = self.shading
        m.albedo[:] = self.albedo
        m.emissive[:] = self.emissive
        m.roughness, m.metallic, m.specular = self.roughness, self.metallic, self.specular
        m.ior, m.sigma_a, m.abbe, m.tilt = self.ior, self.sigma_a, self.abbe, self.tilt
        m.albedo_texture = 0 if self.texture is None else int(self.texture) + 1
        return m

    @staticmethod
    def CreateDiffuseTextured(texture: int, emissive: Vec3 = (0.0, 0.0, 0.0)) -> "Material":
        """Lambertian surface whose albedo is texture `texture` at the hit's uv."""
        return Material(SHADING_DIFFUSE, (1.0, 1.0, 1.0), _f3(emissive), texture=int(texture))


@dataclass(frozen=True)
class AdditionalObjectInfo:
    """Field of an SDF object (AdditionalObjectInfo, core/render/object.cuh:216-225):
    sdf_type SDF_OBJECT_TORUS (params = (R, r)) or SDF_OBJECT_VOLUME (volume =
    index into the renderer's SDF volume cache)."""
    sdf_type: int = SDF_OBJECT_TORUS
    params: tuple = (0.0, 0.0, 0.0, 0.0)
    volume: int = -1


class sdf:
    """The reference's SDF helpers (namespace sdf, core/object/sdf/*)."""

    @staticmethod
    def CreateTorus(scale: float = 1.0, R: float = 0.375, r: float = 0.125) -> AdditionalObjectInfo:
        return AdditionalObjectInfo(SDF_OBJECT_TORUS, (R * scale, r * scale, 0.0, 0.0))

    @staticmethod
    def CreateSDFVolume(volumeIndex: int) -> AdditionalObjectInfo:
        return AdditionalObjectInfo(SDF_OBJECT_VOLUME, (0.0, 0.0, 0.0, 0.0), int(volumeIndex))

    @staticmethod
    def CreateDiamond(scale: float = 1.0, d: float = 0.94, bias: float = 0.5, tableZ: float = 0.3) -> tuple:
        """Parameters of the diamond functor for SceneRenderer.AddVolumeToCacheManager."""
        return (d, bias, tableZ, scale * 0.5)


@dataclass
class SceneObject:
    center: tuple = (0.0, 0.0, 0.0)
    extent: tuple = (0.0, 0.0, 0.0)
    material: Material = field(default_factory=Material)
    rotation: tuple = (0.0, 0.0, 0.0)  # Euler angles in degrees
    type: int = OBJECT_CUBE
    additionalObjectInfo: AdditionalObjectInfo | None = None  # OBJECT_SDF
    v0: tuple = (0.0, 0.0, 0.0)
    v1: tuple = (0.0, 0.0, 0.0)
    v2: tuple = (0.0, 0.0, 0.0)

    @staticmethod
    def Triangle(v0: Vec3, v1: Vec3, v2: Vec3, material: Material) -> "SceneObject":
        return SceneObject(material=material, type=OBJECT_TRIANGLE, v0=_f3(v0), v1=_f3(v1), v2=_f3(v2))


@dataclass
class TriangleMesh:
    """Indexed triangles sharing a material table (large meshes)."""
    vertices: np.ndarray          # (nv, 3) float32
    indices: np.ndarray           # (nt, 3) uint32
    material_ids: np.ndarray      # (nt,) int32 into `materials`
    materials: list
    uv: np.ndarray | None = None  # (nt, 6) float32: u, v at each corner (textured materials)

    def triangle_vertices(self) -> np.ndarray:
        return np.asarray(self.vertices, np.float32)[np.asarray(self.indices, np.int64)].reshape(-1, 9)


@dataclass
class SdfUnion:
    """Smooth union of SDF primitives: (kind, centre, size) with kind one of
    SDF_SPHERE (size[0] = radius), SDF_BOX (half extents), SDF_TORUS (about +y:
    size[0] major, size[1] minor radius); smooth width k; one material."""
    prims: list
    smooth_k: float
    material: Material

    def array(self) -> np.ndarray:
        rows = [[float(k), *map(float, c), *map(float, sz), 0.0] for k, c, sz in self.prims]
        return np.ascontiguousarray(np.array(rows, np.float32).reshape(-1, 8))


@dataclass
class Medium:
    """Homogeneous participating medium filling an axis-aligned box."""
    box_lo: tuple
    box_hi: tuple
    sigma_t: float
    albedo: float
    g: float = 0.0
    emission: float = 0.0

    def to_c(self) -> ArMedium:
        m = ArMedium()
        m.box_lo[:] = _f3(self.box_lo)
        m.box_hi[:] = _f3(self.box_hi)
        m.sigma_t, m.albedo, m.g, m.emission = self.sigma_t, self.albedo, self.g, self.emission
        return m


def flatten(objects: Iterable[SceneObject], mesh: TriangleMesh | None = None):
    """Material table + C object array + mesh arrays for the C ABI."""
    objects = list(objects)
    table: dict[Material, int] = {}
    mats: list[Material] = []

    def mid(m: Material) -> int:
        if m not in table:
            table[m] = len(mats)
            mats.append(m)
        return table[m]

    arr = (ArObject * max(1, len(objects)))()
    for i, o in enumerate(objects):
        a = arr[i]
        a.type = o.type
        a.material = mid(o.material)
        a.center[:] = _f3(o.center)
        a.extent[:] = _f3(o.extent)
        a.rotation_deg[:] = _f3(o.rotation)
        a.v0[:] = _f3(o.v0)
        a.v1[:] = _f3(o.v1)
        a.v2[:] = _f3(o.v2)
        info = o.additionalObjectInfo if o.additionalObjectInfo is not None else AdditionalObjectInfo()
        a.sdf_type = int(info.sdf_type)
        a.sdf_params[:] = tuple(float(x) for x in info.params)
        a.sdf_volume = int(info.volume)
    mesh_ids = None
    if mesh is not None:
        remap = np.array([mid(m) for m in mesh.materials], np.int32)
        mesh_ids = remap[np.asarray(mesh.material_ids, np.int64)]
    return mats, arr, len(objects), mesh_ids


class SceneRenderer:
    """GPU path tracer for one scene (drop-in for the reference's SceneRenderer)."""

    def __init__(self, sceneObjects: Iterable[SceneObject], device: int = 0, mesh: TriangleMesh | None = None,
                 textures: Sequence[np.ndarray] | None = None, sdf: SdfUnion | None = None,
                 medium: Medium | None = None):
        lib = _lib.load()
        self._lib = lib
        ctx = C.c_void_p()
        code = lib.ar_create(C.byref(ctx), device)
        if code != _lib.AR_OK:
            raise _lib.ArError(code, f"ar_create(device={device}) failed (no usable CUDA device?)")
        self._ctx = ctx
        self.objects = list(sceneObjects)
        self._mesh = mesh
        self._refit_v = None      # vertices of the last refit, folded into `mesh` when it is next read
        self.textures = list(textures) if textures is not None else []
        self.sdf = sdf
        self.medium = medium
        self.device = device
        self.bDirty = True

    def close(self) -> None:
        if getattr(self, "_ctx", None):
            self._lib.ar_destroy(self._ctx)
            self._ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def mesh(self):
        if self._refit_v is not None:
            v = self._refit_v
            v = v.cpu().numpy() if hasattr(v, "cpu") else v
            m = self._mesh
            self._mesh = TriangleMesh(np.asarray(v, np.float32).reshape(-1, 3), m.indices, m.material_ids,
                                      m.materials, m.uv)
            self._refit_v = None
        return self._mesh

    @mesh.setter
    def mesh(self, m) -> None:
        self._mesh = m
        self._refit_v = None

    def MarkAsDirty(self) -> None:
        self.bDirty = True

    def _build(self) -> None:
        if not self.bDirty:
            return
        mats, arr, n, mesh_ids = flatten(self.objects, self.mesh)
        sdf_mat = -1
        if self.sdf is not None:
            if self.sdf.material not in mats:
                mats.append(self.sdf.material)
            sdf_mat = mats.index(self.sdf.material)
        carr = (ArMaterial * max(1, len(mats)))(*[m.to_c() for m in mats])
        check(self._ctx, self._lib.ar_scene_set_materials(self._ctx, carr, len(mats)))
        check(self._ctx, self._lib.ar_scene_set_objects(self._ctx, arr, n))
        if self.mesh is not None:
            v = np.ascontiguousarray(self.mesh.vertices, np.float32)
            idx = np.ascontiguousarray(self.mesh.indices, np.uint32)
            ids = np.ascontiguousarray(mesh_ids, np.int32)
            check(self._ctx, self._lib.ar_scene_set_mesh(self._ctx, v.ctypes.data, len(v), idx.ctypes.data, len(idx),
                                                         ids.ctypes.data))
        else:
            check(self._ctx, self._lib.ar_scene_set_mesh(self._ctx, None, 0, None, 0, None))
        if self.mesh is not None and self.mesh.uv is not None:
            uv = np.ascontiguousarray(self.mesh.uv, np.float32).reshape(-1, 6)
            check(self._ctx, self._lib.ar_scene_set_mesh_uv(self._ctx, uv.ctypes.data, len(uv)))
        else:
            check(self._ctx, self._lib.ar_scene_set_mesh_uv(self._ctx, None, 0))
        if self.textures:
            flat = np.concatenate([np.ascontiguousarray(t, np.float32).reshape(-1) for t in self.textures])
            sizes = np.array([[t.shape[1], t.shape[0]] for t in self.textures], np.int32).reshape(-1)
            check(self._ctx, self._lib.ar_scene_set_textures(self._ctx, flat.ctypes.data, sizes.ctypes.data,
                                                             len(self.textures)))
        else:
            check(self._ctx, self._lib.ar_scene_set_textures(self._ctx, None, None, 0))
        if self.sdf is not None:
            a = self.sdf.array()
            check(self._ctx, self._lib.ar_scene_set_sdf_union(self._ctx, a.ctypes.data, len(a), float(self.sdf.smooth_k),
                                                              sdf_mat))
        else:
            check(self._ctx, self._lib.ar_scene_set_sdf_union(self._ctx, None, 0, 0.0, -1))
        check(self._ctx, self._lib.ar_scene_build(self._ctx))
        self.set_medium(self.medium)
        self.bDirty = False

    def set_medium(self, medium: Medium | None) -> None:
        """Sets (or, with None, removes) the participating medium; no rebuild needed."""
        self.medium = medium
        if medium is None:
            check(self._ctx, self._lib.ar_scene_set_medium(self._ctx, None))
        else:
            m = medium.to_c()
            check(self._ctx, self._lib.ar_scene_set_medium(self._ctx, C.byref(m)))

    def build(self) -> None:
        self._build()

    def set_build_mode(self, mode: str) -> None:
        """Where the next build makes the BVH: "host" (binned SAH, default) or "gpu"
        (Morton-code radix tree collapsed on the GPU; same hits)."""
        code = {"host": _lib.BUILD_HOST, "gpu": _lib.BUILD_GPU}[mode]
        check(self._ctx, self._lib.ar_scene_set_build_mode(self._ctx, code))
        self.bDirty = True

    def refit_mesh(self, vertices) -> None:
        """Moves the mesh's vertices (same count) and refits the BVH on the GPU
        (the tree is kept; hits are exact).  numpy array or CUDA tensor, (nv, 3)."""
        self._build()
        if hasattr(vertices, "data_ptr"):
            import torch
            v = vertices.detach().to(torch.float32).contiguous()
            check(self._ctx, self._lib.ar_scene_refit_mesh(self._ctx, v.data_ptr(), v.numel() // 3, 1,
                                                           _torch_stream(v.device)))
        else:
            v = np.ascontiguousarray(vertices, np.float32)
            check(self._ctx, self._lib.ar_scene_refit_mesh(self._ctx, v.ctypes.data, v.size // 3, 0, None))
        if self._mesh is not None:
            # a private copy (on the device for tensors); the host mesh is made from it only when read
            self._refit_v = v.clone() if hasattr(v, "clone") else v.copy()

    def build_time_ms(self) -> float:
        """Wall time of the last BVH build."""
        ms = C.c_double()
        check(self._ctx, self._lib.ar_scene_build_time(self._ctx, C.byref(ms)))
        return ms.value

    def stats(self) -> dict:
        self._build()
        n, s, d, b = C.c_int64(), C.c_int64(), C.c_int32(), C.c_int64()
        check(self._ctx, self._lib.ar_scene_stats(self._ctx, C.byref(n), C.byref(s), C.byref(d), C.byref(b)))
        return {"nodes": n.value, "slots": s.value, "depth": d.value, "bytes": b.value}

    def params(self, size, cameraOrigin, cameraDirection, sampleNum, fov=60.0, max_depth=1000, use_nee=True,
               seed=GLOBAL_SEED, first_frame=0, wave_paths=0, profile=False, guide=0,
               guide_unit=0.0, guide_train_steps=0, denoise_record=False, guide_frames=0) -> ArRenderParams:
        p = ArRenderParams()
        p.width, p.height = int(size[0]), int(size[1])
        p.spp = int(sampleNum)
        p.max_depth = int(max_depth)
        p.cam_origin[:] = _f3(cameraOrigin)
        p.cam_dir[:] = _f3(cameraDirection)
        p.fov_deg = float(fov)
        p.use_nee = 1 if use_nee else 0
        p.seed = int(seed)
        p.first_frame = int(first_frame)
        p.wave_paths = int(wave_paths)
        p.profile = int(profile)  # 1: stage times, 2: traversal counters, 3: both
        p.guide = int(guide)
        p.guide_unit = float(guide_unit)
        p.guide_train_steps = int(guide_train_steps)
        p.denoise_record = 1 if denoise_record else 0
        p.guide_frames = int(guide_frames)
        return p

    def Render(self, size, cameraOrigin, cameraDirection, sampleNum: int = 1024, *, fov: float = 60.0,
               max_depth: int = 1000, use_nee: bool = True, seed: int = GLOBAL_SEED, first_frame: int = 0,
               per_sample: bool = False, wave_paths: int = 0, profile: bool = False, guide: int = 0,
               guide_unit: float = 0.0, guide_train_steps: int = 0, denoise: bool = False, guide_frames: int = 0):
        """Mean linear XYZ per pixel, shape (height, width, 3), float64.

        With per_sample=True also returns every sample's XYZ, shape
        (sampleNum, height, width, 3), float32.  guide=1 turns on the voxel
        path guide: frames render one sample per pixel each and the probes learn
        after every frame (and persist across calls until MarkNeedResetGuiding);
        guide=2 adds the tensor-core MLP guide, trained online on the same
        records and sampled instead of the probes once it has trained.
        guide_frames=k > 1 updates the guide after every k frames instead of
        every frame (the k frames share waves).
        denoise=True (SceneSetting::bDenoise_) records the denoiser's G-buffer
        and sample moments during the render (starting over at first_frame 0)
        and returns the filtered image instead of the raw mean."""
        self._build()
        p = self.params(size, cameraOrigin, cameraDirection, sampleNum, fov, max_depth, use_nee, seed, first_frame,
                        wave_paths, profile, guide, guide_unit, guide_train_steps, denoise, guide_frames)
        w, h = p.width, p.height
        out = np.zeros((h, w, 3), np.float64)
        ps = np.zeros((p.spp, h, w, 3), np.float32) if per_sample else None
        code = self._lib.ar_render(self._ctx, C.byref(p), out.ctypes.data, 0,
                                   ps.ctypes.data if ps is not None else None, None)
        check(self._ctx, code)
        if denoise:
            out = self.denoise(out)
        return (out, ps) if per_sample else out

    # ---- SDF volume cache (core/object/sdf/sdf_cache_manager.cuh) ----------
    def AddVolumeToCacheManager(self, dims, pMin=(0.0, 0.0, 0.0), pMax=(1.0, 1.0, 1.0), sdfFunctor="diamond",
                                sdfInfo=None) -> int:
        """Adds a dims[0] x dims[1] x dims[2] distance grid over the unit cube
        (SceneRenderer::AddVolumeToCacheManager, core/scene.hpp:120-127; pMin /
        pMax are unused there too) and returns its cache index for
        sdf.CreateSDFVolume.  sdfFunctor: "diamond" or "torus" (filled on the
        GPU from sdfInfo, the functor's four parameters: see sdf.CreateDiamond /
        the torus's (R, r)), or a Python callable f(u) evaluated on the host on
        an (N, 3) array of unit positions in [-0.5, 0.5]^3."""
        d = np.ascontiguousarray([int(x) for x in dims], np.int32)
        idx = C.c_int32()
        if callable(sdfFunctor):
            xs = [np.linspace(0.0, 1.0, n, dtype=np.float32) if n > 1 else np.zeros(1, np.float32) for n in d]
            zz, yy, xx = np.meshgrid(xs[2], xs[1], xs[0], indexing="ij")
            u = np.stack([xx, yy, zz], -1).reshape(-1, 3) - np.float32(0.5)
            vox = np.ascontiguousarray(np.asarray(sdfFunctor(u), np.float32).reshape(-1))
            if vox.size != int(np.prod(d)):
                raise ValueError("the functor must return one distance per position")
            check(self._ctx, self._lib.ar_sdf_volume_add_data(self._ctx, vox.ctypes.data, d.ctypes.data, C.byref(idx)))
        else:
            fn = {"diamond": SDF_FN_DIAMOND, "torus": SDF_FN_TORUS}.get(sdfFunctor, sdfFunctor)
            prm = np.zeros(4, np.float32)
            if sdfInfo is not None:
                vals = sdfInfo.params if isinstance(sdfInfo, AdditionalObjectInfo) else sdfInfo
                prm[: len(vals)] = vals
            check(self._ctx, self._lib.ar_sdf_volume_add(self._ctx, int(fn), prm.ctypes.data, d.ctypes.data,
                                                         C.byref(idx)))
        return idx.value

    def sdf_volume(self, index: int) -> np.ndarray:
        """A cached volume as a (dz, dy, dx) float32 array."""
        dims = np.zeros(3, np.int32)
        check(self._ctx, self._lib.ar_sdf_volume_read(self._ctx, int(index), None, dims.ctypes.data))
        out = np.zeros((dims[2], dims[1], dims[0]), np.float32)
        check(self._ctx, self._lib.ar_sdf_volume_read(self._ctx, int(index), out.ctypes.data, None))
        return out

    def ClearVolumes(self) -> None:
        check(self._ctx, self._lib.ar_sdf_volume_clear(self._ctx))

    # ---- denoiser (core/denoise/*) ----------------------------------------
    def denoise(self, xyz):
        """Bilateral-filters an image of the recorded size with the recorded
        G-buffer and sample moments.  xyz: (height, width, 3) float64 numpy
        array (returns a new array) or CUDA float64 tensor (returns a new tensor)."""
        if hasattr(xyz, "data_ptr"):
            import torch
            x = xyz.detach().to(torch.float64).contiguous()
            out = torch.empty_like(x)
            check(self._ctx, self._lib.ar_denoise(self._ctx, x.data_ptr(), 1, out.data_ptr(), 1,
                                                  _torch_stream(x.device)))
            return out
        a = np.ascontiguousarray(xyz, np.float64)
        w, h = self.denoise_size()
        if a.shape != (h, w, 3):
            raise ValueError(f"image must be ({h}, {w}, 3) to match the recorded buffers")
        out = np.empty_like(a)
        check(self._ctx, self._lib.ar_denoise(self._ctx, a.ctypes.data, 0, out.ctypes.data, 0, None))
        return out

    def denoise_size(self) -> tuple[int, int]:
        """(width, height) of the recorded denoiser buffers, (0, 0) when none."""
        w, h = C.c_int32(), C.c_int32()
        check(self._ctx, self._lib.ar_denoise_read(self._ctx, C.byref(w), C.byref(h), None, None))
        return w.value, h.value

    def denoise_records(self):
        """(gbuffer, moments): structured arrays of shape (height, width) with
        the layouts DENOISE_GBUF_DTYPE / DENOISE_STAT_DTYPE."""
        w, h = self.denoise_size()
        g = np.zeros((h, w), _lib.DENOISE_GBUF_DTYPE)
        m = np.zeros((h, w), _lib.DENOISE_STAT_DTYPE)
        check(self._ctx, self._lib.ar_denoise_read(self._ctx, None, None, g.ctypes.data, m.ctypes.data))
        return g, m

    def set_denoise_records(self, gbuffer, moments) -> None:
        """Replaces the recorded buffers (arrays as denoise_records returns them)."""
        g = np.ascontiguousarray(gbuffer, _lib.DENOISE_GBUF_DTYPE)
        m = np.ascontiguousarray(moments, _lib.DENOISE_STAT_DTYPE)
        if g.shape != m.shape or g.ndim != 2:
            raise ValueError("gbuffer and moments must be (height, width) arrays of the same shape")
        h, w = g.shape
        check(self._ctx, self._lib.ar_denoise_write(self._ctx, w, h, g.ctypes.data, m.ctypes.data))

    # ---- device-side rendering and the replay adjoint (torch tensors) -----
    def texel_count(self) -> int:
        """Texel floats of the built scene (3 per texel, all textures)."""
        self._build()
        n = C.c_int64()
        check(self._ctx, self._lib.ar_scene_texel_count(self._ctx, C.byref(n)))
        return n.value

    def update_texels(self, texels) -> None:
        """Replaces every texel value (CUDA float32 tensor or host array of texel_count() floats)."""
        self._build()
        if hasattr(texels, "data_ptr"):
            import torch
            t = texels.detach().to(torch.float32).contiguous()
            s = _torch_stream(t.device)
            check(self._ctx, self._lib.ar_scene_update_texels(self._ctx, t.data_ptr(), t.numel(), 1, s))
        else:
            a = np.ascontiguousarray(texels, np.float32).reshape(-1)
            check(self._ctx, self._lib.ar_scene_update_texels(self._ctx, a.ctypes.data, a.size, 0, None))

    def render_into(self, out, size, cameraOrigin, cameraDirection, sampleNum: int, **kw) -> None:
        """Renders into a CUDA float64 tensor out of shape (height, width, 3)."""
        import torch
        self._build()
        p = self.params(size, cameraOrigin, cameraDirection, sampleNum, **kw)
        assert out.dtype == torch.float64 and out.is_contiguous() and out.numel() == 3 * p.width * p.height
        s = _torch_stream(out.device)
        check(self._ctx, self._lib.ar_render(self._ctx, C.byref(p), out.data_ptr(), 1, None, s))

    def adjoint(self, dl_dxyz, grad_out, size, cameraOrigin, cameraDirection, sampleNum: int, **kw) -> None:
        """d(loss)/d(texels) into grad_out (CUDA float64, texel_count() elements), given
        dl_dxyz = d(loss)/d(image) (CUDA float32, (height, width, 3)) for the image that
        render_into / Render returns with the same arguments."""
        import torch
        self._build()
        p = self.params(size, cameraOrigin, cameraDirection, sampleNum, **kw)
        g = dl_dxyz.detach().to(torch.float32).contiguous()
        if g.numel() != 3 * p.width * p.height:
            raise ValueError("dl_dxyz must hold 3 floats per pixel")
        n = self.texel_count()
        if n and (grad_out.dtype != torch.float64 or not grad_out.is_contiguous() or grad_out.numel() != n):
            raise ValueError(f"grad_out must be a contiguous float64 tensor of {n} elements")
        s = _torch_stream(g.device)
        check(self._ctx, self._lib.ar_adjoint(self._ctx, C.byref(p), g.data_ptr(), grad_out.data_ptr(), s))

    def adjoint_medium(self, dl_dxyz, size, cameraOrigin, cameraDirection, sampleNum: int, **kw) -> tuple[float, float]:
        """(d loss / d albedo, d loss / d emission) of the medium, given
        dl_dxyz = d(loss)/d(image) (CUDA float32, (height, width, 3))."""
        import torch
        self._build()
        p = self.params(size, cameraOrigin, cameraDirection, sampleNum, **kw)
        g = dl_dxyz.detach().to(torch.float32).contiguous()
        if g.numel() != 3 * p.width * p.height:
            raise ValueError("dl_dxyz must hold 3 floats per pixel")
        out = (C.c_double * 2)()
        check(self._ctx, self._lib.ar_adjoint_medium(self._ctx, C.byref(p), g.data_ptr(), out, _torch_stream(g.device)))
        return out[0], out[1]

    def tonemap(self, xyz: np.ndarray, exposure: float = 1.0, tone: str = "aces") -> np.ndarray:
        """Display image (height, width, 4) uint8 from a linear XYZ image, on the GPU."""
        tones = {"aces": _lib.TONE_ACES, "gamma": _lib.TONE_GAMMA, "linear": _lib.TONE_LINEAR}
        x = np.ascontiguousarray(xyz, np.float64)
        h, w, _ = x.shape
        out = np.zeros((h, w, 4), np.uint8)
        check(self._ctx, self._lib.ar_tonemap(self._ctx, x.ctypes.data, 0, w, h, float(exposure), tones[tone],
                                              out.ctypes.data))
        return out

    def last_render_stats(self) -> tuple[float, int]:
        ms, n = C.c_float(), C.c_int64()
        check(self._ctx, self._lib.ar_last_render_stats(self._ctx, C.byref(ms), C.byref(n)))
        return ms.value, n.value

    def MarkNeedResetGuiding(self) -> int:
        """Forgets the voxel guide's probes; returns how many there were."""
        n = C.c_int32()
        check(self._ctx, self._lib.ar_guide_reset(self._ctx, C.byref(n)))
        return n.value

    def guide_stats(self) -> tuple[int, int]:
        n, cap = C.c_int32(), C.c_int32()
        check(self._ctx, self._lib.ar_guide_stats(self._ctx, C.byref(n), C.byref(cap)))
        return n.value, cap.value

    def SetExposure(self, exp: float) -> None:
        """Exposure of RenderFrame's display image (SceneRenderer::SetExposure, core/scene.hpp:97)."""
        check(self._ctx, self._lib.ar_set_exposure(self._ctx, float(exp)))

    def RenderFrame(self, hdrTarget, ldrTarget, size, cameraOrigin, cameraDirection, frameIndex: int, toneType: int,
                    oddTarget=None, evenTarget=None, *, fov: float = 60.0, max_depth: int = 1000,
                    use_nee: bool = True, seed: int = GLOBAL_SEED, guide: int = 0, guide_unit: float = 0.0,
                    denoise: bool = False, stream=None) -> None:
        """One progressive frame (SceneRenderer::Render(hdrTarget, ldrTarget, size, ...,
        frameIndex, toneType, oddTarget, evenTarget), core/scene.hpp:109-114): renders
        sample frameIndex of every pixel and folds it into hdrTarget (CUDA float32
        (H, W, 3), running mean) and, if given, oddTarget / evenTarget; ldrTarget (CUDA
        int32 (H, W) or None) receives the 0xAARRGGBB display image, toneType 0 linear,
        1 gamma, 2 ACES."""
        self.build()
        p = self.params(size, cameraOrigin, cameraDirection, 1, fov, max_depth, use_nee, seed, int(frameIndex),
                        0, False, guide, guide_unit, 0, denoise)

        def ptr(t):
            if t is None:
                return None
            assert t.is_cuda and t.is_contiguous()
            return t.data_ptr()
        w, h = int(size[0]), int(size[1])
        assert hdrTarget.numel() == 3 * w * h and (ldrTarget is None or ldrTarget.numel() == w * h)
        check(self._ctx, self._lib.ar_render_frame(self._ctx, C.byref(p), int(frameIndex), int(toneType),
                                                   ptr(hdrTarget), ptr(ldrTarget), ptr(oddTarget), ptr(evenTarget),
                                                   stream))

    def guide_probes(self) -> dict:
        """The voxel guide's probes, by probe index: keys (n, 4) int32 (voxel x, y, z,
        face), texels (n, 86, 4) float32 (Texture<4>::data_), counts (n,) uint64."""
        n = C.c_int32()
        check(self._ctx, self._lib.ar_guide_read(self._ctx, C.byref(n), 0, None, None, None))
        k = np.zeros((n.value, 4), np.int32)
        t = np.zeros((n.value, _lib.GUIDE_PROBE_FLOATS // 4, 4), np.float32)
        c = np.zeros(n.value, np.uint64)
        check(self._ctx, self._lib.ar_guide_read(self._ctx, C.byref(n), n.value, k.ctypes.data, t.ctypes.data,
                                                 c.ctypes.data))
        return {"keys": k, "texels": t, "counts": c}

    def set_guide_probes(self, keys, texels, counts, unit: float = 0.0) -> None:
        """Replaces the voxel guide's probes (the layout guide_probes returns)."""
        k = np.ascontiguousarray(keys, np.int32).reshape(-1, 4)
        t = np.ascontiguousarray(texels, np.float32).reshape(len(k), -1)
        c = np.ascontiguousarray(counts, np.uint64).reshape(len(k))
        assert t.shape[1] == _lib.GUIDE_PROBE_FLOATS
        self.build()
        check(self._ctx, self._lib.ar_guide_write(self._ctx, len(k), k.ctypes.data, t.ctypes.data, c.ctypes.data,
                                                  float(unit)))

    def guide_records(self) -> dict:
        """Radiance records of the last guided frame: keys (n, 4) int32, dirs (n, 3),
        radiance (n, 3) XYZ, in the order the kernels emitted them."""
        n = C.c_int32()
        check(self._ctx, self._lib.ar_guide_read_records(self._ctx, C.byref(n), 0, None, None, None))
        k = np.zeros((n.value, 4), np.int32)
        d = np.zeros((n.value, 3), np.float32)
        r = np.zeros((n.value, 3), np.float32)
        check(self._ctx, self._lib.ar_guide_read_records(self._ctx, C.byref(n), n.value, k.ctypes.data,
                                                         d.ctypes.data, r.ctypes.data))
        return {"keys": k, "dirs": d, "radiance": r}

    def mlp_stats(self) -> tuple[int, float]:
        """MLP guide: (training steps taken, loss sum of the last step)."""
        n, loss = C.c_int32(), C.c_float()
        check(self._ctx, self._lib.ar_guide_mlp_stats(self._ctx, C.byref(n), C.byref(loss)))
        return n.value, loss.value

    def render_profile(self) -> dict:
        prof = _lib.ArRenderProfile()
        check(self._ctx, self._lib.ar_last_render_profile(self._ctx, C.byref(prof)))
        return prof.as_dict()

    def error_word(self) -> int:
        w = C.c_uint32()
        check(self._ctx, self._lib.ar_get_error_word(self._ctx, C.byref(w)))
        return w.value

    # ---- raw ray queries (device tensors) --------------------------------
    def trace_closest(self, rays, stream=None):
        """rays: CUDA float32 tensor (n, 8) = (o, tmin, d, tmax).  Returns (prim_id int32, t float32)."""
        import torch
        self._build()
        rays = rays.contiguous()
        n = rays.shape[0]
        ids = torch.empty(n, dtype=torch.int32, device=rays.device)
        t = torch.empty(n, dtype=torch.float32, device=rays.device)
        s = _torch_stream(rays.device) if stream is None else stream
        check(self._ctx, self._lib.ar_trace_closest(self._ctx, rays.data_ptr(), n, ids.data_ptr(), t.data_ptr(), s))
        return ids, t

    def trace_any(self, rays, stream=None):
        import torch
        self._build()
        rays = rays.contiguous()
        n = rays.shape[0]
        hit = torch.empty(n, dtype=torch.int32, device=rays.device)
        s = _torch_stream(rays.device) if stream is None else stream
        check(self._ctx, self._lib.ar_trace_any(self._ctx, rays.data_ptr(), n, hit.data_ptr(), s))
        return hit


class Camera:
    """Headless camera (core/camera.hpp:14-99): renders to a file, no window."""

    def __init__(self, renderer: SceneRenderer, name: str, resolutionX: int, resolutionY: int,
                 position: Vec3, direction: Vec3, fov: float = 60.0):
        self.renderer = renderer
        self.name = name
        self.resolution = (int(resolutionX), int(resolutionY))
        self.position = _f3(position)
        self.direction = _f3(direction)
        self.fov = float(fov)

    def Render(self, sampleNum: int = 1, **kw) -> np.ndarray:
        return self.renderer.Render(self.resolution, self.position, self.direction, sampleNum, fov=self.fov, **kw)

    def RenderToFile(self, path: str, sampleNum: int = 1024, tonemapFunction: str = "aces", exp: float = 1.0,
                     **kw) -> np.ndarray:
        """Renders and writes the image (Camera::RenderToFile, core/camera.cu:64-89).
        The extension picks the format:
          .bmp  tonemapped 8-bit (tonemapFunction "aces" = the reference's
                default, "gamma" or "linear"; exposure `exp`), the reference's
                32-bit top-down BMP;
          .pfm  linear XYZ floats (Portable Float Map), no tonemap;
          other: `<path>.bmp` as the reference names its output.
        Returns the linear XYZ image."""
        img = self.Render(sampleNum, **kw)
        h, w, _ = img.shape
        if path.lower().endswith(".pfm"):
            write_pfm(path, img)
        else:
            if not path.lower().endswith(".bmp"):
                path = path + ".bmp"
            write_bmp(path, self.renderer.tonemap(img, exp, tonemapFunction))
        return img


def write_pfm(path: str, img: np.ndarray) -> None:
    """Colour PFM, little-endian float32, bottom row first."""
    img = np.asarray(img, np.float32)
    h, w, _ = img.shape
    with open(path, "wb") as f:
        f.write(f"PF\n{w} {h}\n-1.0\n".encode())
        f.write(np.ascontiguousarray(img[::-1]).tobytes())


def write_bmp(path: str, rgba: np.ndarray) -> None:
    """32-bit BGRA BMP, top-down (negative height), as SaveBMP (core/camera.cu:10-62) writes it."""
    rgba = np.asarray(rgba, np.uint8)
    h, w, _ = rgba.shape
    bgra = rgba[..., [2, 1, 0, 3]]
    size = 54 + w * h * 4
    header = bytearray(54)
    header[0:2] = b"BM"
    header[2:6] = size.to_bytes(4, "little")
    header[10:14] = (54).to_bytes(4, "little")
    header[14:18] = (40).to_bytes(4, "little")
    header[18:22] = int(w).to_bytes(4, "little", signed=True)
    header[22:26] = int(-h).to_bytes(4, "little", signed=True)
    header[26:28] = (1).to_bytes(2, "little")
    header[28:30] = (32).to_bytes(2, "little")
    header[34:38] = (w * h * 4).to_bytes(4, "little")
    with open(path, "wb") as f:
        f.write(bytes(header))
        f.write(np.ascontiguousarray(bgra).tobytes())


def host_rgb_encode(rgb: np.ndarray) -> np.ndarray:
    lib = _lib.load()
    rgb = np.ascontiguousarray(rgb, np.float32).reshape(-1, 3)
    out = np.zeros((len(rgb), 4), np.float32)
    check(None, lib.ar_host_rgb_encode(rgb.ctypes.data, len(rgb), out.ctypes.data))
    return out


def host_lambda_encode(lam: np.ndarray) -> np.ndarray:
    lib = _lib.load()
    lam = np.ascontiguousarray(lam, np.float32).reshape(-1)
    out = np.zeros((len(lam), 4), np.float32)
    check(None, lib.ar_host_lambda_encode(lam.ctypes.data, len(lam), out.ctypes.data))
    return out


def host_sample_lambda(u3: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    lib = _lib.load()
    u3 = np.ascontiguousarray(u3, np.float32).reshape(-1, 3)
    lam = np.zeros(len(u3), np.float32)
    pdf = np.zeros(len(u3), np.float32)
    check(None, lib.ar_host_sample_lambda(u3.ctypes.data, len(u3), lam.ctypes.data, pdf.ctypes.data))
    return lam, pdf
