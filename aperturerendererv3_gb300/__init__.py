"""aperture-gb300: GB300-native (sm_103a) spectral path tracing.

Public entry points mirror the reference renderer's host interface
(SceneRenderer, SceneObject, Material, Camera); the work runs in hand-written
CUDA kernels behind the C ABI declared in include/aperture/ar.h.
"""
from ._lib import GLOBAL_SEED, ArError, load as load_library
from .scene import (Camera, Material, SceneObject, SceneRenderer, TriangleMesh, host_lambda_encode,
                    host_rgb_encode, host_sample_lambda)

__all__ = ["Camera", "Material", "SceneObject", "SceneRenderer", "TriangleMesh", "GLOBAL_SEED", "ArError",
           "load_library", "host_rgb_encode", "host_lambda_encode", "host_sample_lambda"]
