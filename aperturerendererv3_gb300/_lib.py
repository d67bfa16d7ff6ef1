"""ctypes binding of the C ABI in include/aperture/ar.h.

The shared library is built in-tree (aperturerendererv3_gb300/build.py); this
module never falls back to anything else: if the library is missing the import
error says how to build it.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as _np

LIB_PATH = Path(__file__).resolve().parent / "libaperture_gb300.so"

AR_OK = 0
AR_ERR_INVALID = -1
AR_ERR_CUDA = -2
AR_ERR_NOMEM = -3
AR_ERR_STATE = -4
AR_ERR_DEVICE = -5

OBJECT_CUBE = 0
OBJECT_SPHERE = 1
OBJECT_SDF = 2
SDF_OBJECT_TORUS, SDF_OBJECT_VOLUME = 0, 1
SDF_FN_TORUS, SDF_FN_DIAMOND = 0, 1
BUILD_HOST, BUILD_GPU = 0, 1
OBJECT_TRIANGLE = 3

SHADING_DIFFUSE = 0
SHADING_LIGHT = 1
SHADING_GLASS = 2
SHADING_GGX = 3

GLOBAL_SEED = 0x9E3779B97F4A7C15

F3 = C.c_float * 3


class ArMaterial(C.Structure):
    _fields_ = [("shading", C.c_int32), ("albedo", F3), ("emissive", F3),
                ("roughness", C.c_float), ("metallic", C.c_float), ("specular", C.c_float),
                ("ior", C.c_float), ("sigma_a", C.c_float), ("abbe", C.c_float), ("tilt", C.c_float),
                ("albedo_texture", C.c_int32)]


class ArObject(C.Structure):
    _fields_ = [("type", C.c_int32), ("material", C.c_int32), ("center", F3), ("extent", F3),
                ("rotation_deg", F3), ("v0", F3), ("v1", F3), ("v2", F3), ("sdf_type", C.c_int32),
                ("sdf_params", C.c_float * 4), ("sdf_volume", C.c_int32)]


class ArMedium(C.Structure):
    _fields_ = [("box_lo", F3), ("box_hi", F3), ("sigma_t", C.c_float), ("albedo", C.c_float), ("g", C.c_float),
                ("emission", C.c_float)]


class ArRenderParams(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("spp", C.c_int32), ("max_depth", C.c_int32),
                ("cam_origin", F3), ("cam_dir", F3), ("fov_deg", C.c_float), ("use_nee", C.c_int32),
                ("seed", C.c_uint64), ("first_frame", C.c_int32), ("wave_paths", C.c_int32),
                ("profile", C.c_int32), ("guide", C.c_int32), ("guide_unit", C.c_float),
                ("guide_train_steps", C.c_int32), ("denoise_record", C.c_int32), ("guide_frames", C.c_int32)]


GUIDE_NONE = 0
GUIDE_VOXEL = 1
GUIDE_MLP = 2
SDF_SPHERE, SDF_BOX, SDF_TORUS = 0, 1, 2
TONE_ACES, TONE_GAMMA, TONE_LINEAR = 0, 1, 2

# denoiser records (ar_denoise_read / ar_denoise_write), 40 bytes per pixel each
DENOISE_GBUF_DTYPE = _np.dtype([("h", "<u2", 14), ("depth", "<f4"), ("valid", "<u4"), ("frames", "<u4")])
DENOISE_STAT_DTYPE = _np.dtype([("num", "<u4"), ("mean", "<f4", 3), ("m2n", "<f4", 3), ("m3n", "<f4", 3)])


class ArRenderProfile(C.Structure):
    _fields_ = [("raygen_ms", C.c_float), ("extend_ms", C.c_float), ("shade_ms", C.c_float),
                ("shadow_ms", C.c_float), ("finalize_ms", C.c_float),
                ("extend_rays", C.c_int64), ("shadow_rays", C.c_int64),
                ("extend_node_visits", C.c_int64), ("extend_prim_tests", C.c_int64),
                ("shadow_node_visits", C.c_int64), ("shadow_prim_tests", C.c_int64),
                ("extend_launches", C.c_int64), ("shadow_launches", C.c_int64), ("shade_launches", C.c_int64)]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


GUIDE_PROBE_FLOATS = 344  # AR_GUIDE_PROBE_FLOATS: Texture<4>::data_ as floats

EXPORTED = [
    "ar_create", "ar_destroy", "ar_scene_set_materials", "ar_scene_set_objects", "ar_scene_set_mesh",
    "ar_scene_build", "ar_scene_stats", "ar_render", "ar_trace_closest", "ar_trace_any", "ar_last_render_stats",
    "ar_last_render_profile", "ar_render_noalloc", "ar_guide_reset", "ar_guide_stats",
    "ar_get_error_word", "ar_clear_error_word", "ar_last_error", "ar_host_rgb_encode", "ar_host_lambda_encode",
    "ar_host_sample_lambda", "ar_host_trace_closest", "ar_host_guide_eval", "ar_abi_version",
    "ar_scene_set_textures", "ar_scene_set_mesh_uv", "ar_scene_update_texels", "ar_scene_texel_count", "ar_adjoint",
    "ar_diag_umma_gemm", "ar_diag_mlp", "ar_guide_mlp_stats", "ar_scene_set_sdf_union", "ar_scene_set_medium",
    "ar_adjoint_medium", "ar_tonemap", "ar_denoise", "ar_denoise_read", "ar_denoise_write",
    "ar_sdf_volume_add", "ar_sdf_volume_add_data", "ar_sdf_volume_read", "ar_sdf_volume_clear",
    "ar_scene_set_build_mode", "ar_scene_build_time", "ar_scene_refit_mesh", "ar_guide_read", "ar_guide_write",
    "ar_guide_read_records", "ar_render_frame", "ar_set_exposure",
]

_lib = None


class ArError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"aperture error {code}: {msg}")
        self.code = code


def load() -> C.CDLL:
    """Loads the in-tree library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise ImportError(f"{LIB_PATH} is missing; build it with `python -m aperturerendererv3_gb300.build` "
                          "or `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(str(LIB_PATH))
    vp = C.c_void_p
    P = C.POINTER
    sig = {
        "ar_create": (C.c_int, [P(vp), C.c_int]),
        "ar_destroy": (C.c_int, [vp]),
        "ar_scene_set_materials": (C.c_int, [vp, P(ArMaterial), C.c_int]),
        "ar_scene_set_objects": (C.c_int, [vp, P(ArObject), C.c_int]),
        "ar_scene_set_mesh": (C.c_int, [vp, vp, C.c_int, vp, C.c_int, vp]),
        "ar_scene_build": (C.c_int, [vp]),
        "ar_scene_stats": (C.c_int, [vp, P(C.c_int64), P(C.c_int64), P(C.c_int32), P(C.c_int64)]),
        "ar_render": (C.c_int, [vp, P(ArRenderParams), vp, C.c_int, vp, vp]),
        "ar_render_noalloc": (C.c_int, [vp, P(ArRenderParams), vp, vp]),
        "ar_trace_closest": (C.c_int, [vp, vp, C.c_int, vp, vp, vp]),
        "ar_trace_any": (C.c_int, [vp, vp, C.c_int, vp, vp]),
        "ar_last_render_stats": (C.c_int, [vp, P(C.c_float), P(C.c_int64)]),
        "ar_last_render_profile": (C.c_int, [vp, P(ArRenderProfile)]),
        "ar_guide_reset": (C.c_int, [vp, P(C.c_int32)]),
        "ar_guide_stats": (C.c_int, [vp, P(C.c_int32), P(C.c_int32)]),
        "ar_get_error_word": (C.c_int, [vp, P(C.c_uint32)]),
        "ar_clear_error_word": (C.c_int, [vp]),
        "ar_last_error": (C.c_char_p, [vp]),
        "ar_host_rgb_encode": (C.c_int, [vp, C.c_int, vp]),
        "ar_host_lambda_encode": (C.c_int, [vp, C.c_int, vp]),
        "ar_host_sample_lambda": (C.c_int, [vp, C.c_int, vp, vp]),
        "ar_host_trace_closest": (C.c_int, [vp, C.c_int, vp, C.c_int, vp, vp, P(C.c_int64)]),
        "ar_host_guide_eval": (C.c_int, [vp, C.c_int, vp]),
        "ar_abi_version": (C.c_int, []),
        "ar_scene_set_textures": (C.c_int, [vp, vp, vp, C.c_int]),
        "ar_scene_set_mesh_uv": (C.c_int, [vp, vp, C.c_int]),
        "ar_scene_update_texels": (C.c_int, [vp, vp, C.c_int64, C.c_int, vp]),
        "ar_scene_texel_count": (C.c_int, [vp, P(C.c_int64)]),
        "ar_adjoint": (C.c_int, [vp, P(ArRenderParams), vp, vp, vp]),
        "ar_diag_umma_gemm": (C.c_int, [C.c_int, vp, vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, vp]),
        "ar_diag_mlp": (C.c_int, [C.c_int, vp, vp, vp, vp, vp, C.c_int, vp, vp, vp]),
        "ar_guide_mlp_stats": (C.c_int, [vp, P(C.c_int32), P(C.c_float)]),
        "ar_scene_set_sdf_union": (C.c_int, [vp, vp, C.c_int, C.c_float, C.c_int32]),
        "ar_scene_set_medium": (C.c_int, [vp, P(ArMedium)]),
        "ar_adjoint_medium": (C.c_int, [vp, P(ArRenderParams), vp, vp, vp]),
        "ar_tonemap": (C.c_int, [vp, vp, C.c_int, C.c_int, C.c_int, C.c_float, C.c_int, vp]),
        "ar_denoise": (C.c_int, [vp, vp, C.c_int, vp, C.c_int, vp]),
        "ar_denoise_read": (C.c_int, [vp, P(C.c_int32), P(C.c_int32), vp, vp]),
        "ar_denoise_write": (C.c_int, [vp, C.c_int32, C.c_int32, vp, vp]),
        "ar_sdf_volume_add": (C.c_int, [vp, C.c_int32, vp, vp, P(C.c_int32)]),
        "ar_sdf_volume_add_data": (C.c_int, [vp, vp, vp, P(C.c_int32)]),
        "ar_sdf_volume_read": (C.c_int, [vp, C.c_int32, vp, vp]),
        "ar_sdf_volume_clear": (C.c_int, [vp]),
        "ar_scene_set_build_mode": (C.c_int, [vp, C.c_int32]),
        "ar_scene_build_time": (C.c_int, [vp, P(C.c_double)]),
        "ar_scene_refit_mesh": (C.c_int, [vp, vp, C.c_int, C.c_int, vp]),
        "ar_guide_read": (C.c_int, [vp, P(C.c_int32), C.c_int32, vp, vp, vp]),
        "ar_guide_write": (C.c_int, [vp, C.c_int32, vp, vp, vp, C.c_float]),
        "ar_guide_read_records": (C.c_int, [vp, P(C.c_int32), C.c_int32, vp, vp, vp]),
        "ar_render_frame": (C.c_int, [vp, P(ArRenderParams), C.c_int32, C.c_int32, vp, vp, vp, vp, vp]),
        "ar_set_exposure": (C.c_int, [vp, C.c_float]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def check(ctx, code: int) -> None:
    if code != AR_OK:
        msg = load().ar_last_error(ctx).decode() if ctx else ""
        raise ArError(code, msg)
