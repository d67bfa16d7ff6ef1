"""Recipe that turns the reference's own CUDA C++ path tracer into a CPU oracle.

TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline / reference arm may build or run what this produces; the product
path never touches it.

What it does (every step mechanical, nothing re-implemented):
  1. copies the reference's ``core/`` tree from the reference checkout into
     ``oracle/_ref/src/core`` (git-ignored; the copy is never committed);
  2. applies the patches listed in ``PATCHES`` below so the reference's
     ``__host__ __device__`` integrator (core/render/render.cuh:460-999 and
     everything it calls) compiles and runs on the host under OpenMP:
       * Linux include fixes: case-insensitive ``object/AABB.cuh`` /
         ``object/Sphere.cuh`` (core/render/intersection.cuh:6-7), missing
         ``<cfloat>`` (core/vector.cuh:153), ``cuda::par`` ambiguity
         (core/guiding/guiding.cuh:84-111,148-160,286);
       * device-only helper macros made host+device (core/vector.cuh:35-36) and
         ``__constant__`` scene symbols made host globals
         (core/render/render.cuh:24-56);
       * curand XORWOW replaced by the PCG32 streams of
         aperturerendererv3_gb300/csrc/ar_rng.h (core/random.cuh:31-53), so the
         GPU integrator and this oracle draw identical random numbers;
       * transcendental calls (sincosf, expf, logf, powf, erfcf, rsqrtf, ...)
         renamed to the deterministic versions in
         aperturerendererv3_gb300/csrc/ar_detmath.h, the same functions the GPU
         kernels call, so both sides round identically;
       * 32-bit BVH nodes (core/config.cuh:17-18) so scenes above 32767
         primitives build, and MAX_TRACING_DEPTH (core/config.cuh:8) read from a
         host variable so tests can ask for first-bounce-only paths;
       * a triangle object type (``EObjectType::OBJ_TRIANGLE``) dispatched from
         ``intersection::IntersectBase`` (core/render/intersection.cuh:16-31) to
         oracle/ref_glue.cuh, which calls the same watertight triangle test the
         GPU kernels use.  The reference has no triangles; this is the
         smallest addition that lets it render the triangle scenes.
  3. the driver oracle/ref_driver.cu (our code) is compiled against the patched
     tree by ``build_ref()``.

The patched copy and the binary live under oracle/_ref/ (git-ignored, but it
travels with the working tree so a machine without the reference checkout can
still rebuild the binary from ``oracle/_ref/src``).
"""
from __future__ import annotations

import os
import re
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
REPO = HERE.parent
# The reference checkout: given by the AR_REFERENCE_ROOT environment variable or
# by `--reference PATH` on the command line; there is no default location.
REF_ROOT = Path(os.environ["AR_REFERENCE_ROOT"]) if os.environ.get("AR_REFERENCE_ROOT") else None
OUT = HERE / "_ref"
SRC = OUT / "src"
CORE = SRC / "core"
CSRC = REPO / "aperturerendererv3_gb300" / "csrc"

MATH_FUNCS = ["sincosf", "sinf", "cosf", "tanf", "expf", "logf", "log1pf", "powf",
              "erfcf", "rsqrtf", "atan2f", "asinf", "acosf", "atanf"]
UNSUFFIXED = ["sin", "cos", "exp", "log", "pow"]


def _sub(path: Path, pattern: str, repl: str, count: int = 0, flags: int = 0, must: bool = True) -> None:
    text = path.read_text()
    new, n = re.subn(pattern, repl, text, count=count, flags=flags)
    if must and n == 0:
        raise RuntimeError(f"patch pattern not found in {path}: {pattern!r}")
    path.write_text(new)


def _prepend(path: Path, text: str) -> None:
    path.write_text(text + path.read_text())


def copy_tree() -> None:
    if REF_ROOT is None or not (REF_ROOT / "core").is_dir():
        raise FileNotFoundError(f"reference checkout not found at {REF_ROOT}")
    if SRC.exists():
        shutil.rmtree(SRC)
    SRC.mkdir(parents=True)
    shutil.copytree(REF_ROOT / "core", CORE,
                    ignore=shutil.ignore_patterns("*.pyc", "__pycache__"))
    for p in CORE.rglob("*"):
        if p.is_file():
            p.chmod(0o644)
        else:
            p.chmod(0o755)


def patch_tree() -> None:
    # (1) Linux include fixes: forwarders for the Windows-cased names.
    (CORE / "object" / "AABB.cuh").write_text('#pragma once\n#include "aabb.cuh"\n')
    (CORE / "object" / "Sphere.cuh").write_text('#pragma once\n#include "sphere.cuh"\n')
    _sub(CORE / "guiding" / "guiding.cuh", r"([^:])cuda::par", r"\1thrust::cuda::par")

    # (2) host+device helper macros, <cfloat>, shared deterministic math.
    vec = CORE / "vector.cuh"
    _sub(vec, r"#define FUNCTION_MODIFIER_DEVICE_INLINE __device__ __forceinline__",
         "#define FUNCTION_MODIFIER_DEVICE_INLINE __host__ __device__ __forceinline__")
    _sub(vec, r"#define FUNCTION_MODIFIER_DEVICE __device__\b",
         "#define FUNCTION_MODIFIER_DEVICE __host__ __device__")
    _sub(vec, r'#include "config.cuh"',
         '#include <cfloat>\n#include "config.cuh"\n#include "ar_detmath.h"', count=1)
    # debug-visualisation helpers stay device-only (they read device symbols)
    _sub(CORE / "guiding" / "guiding_debug.cuh", r"FUNCTION_MODIFIER_DEVICE_INLINE",
         "__device__ __forceinline__")

    # (3) scene symbols: __constant__ on the device pass, host globals on the host pass.
    rend = CORE / "render" / "render.cuh"
    _sub(rend, r"__device__ inline __constant__", "REF_GLOBAL")
    _sub(rend, r"#ifndef RENDER_GLOBAL",
         "#ifdef __CUDA_ARCH__\n#define REF_GLOBAL static __device__ __constant__\n"
         "#else\n#define REF_GLOBAL inline\n#endif\n#ifndef RENDER_GLOBAL", count=1)

    # whole-program device pass: definitions instead of extern device symbols
    sdfm = CORE / "object" / "sdf" / "sdf_master.cuh"
    _sub(sdfm, r"extern __device__ SDFVolumeInfo\* cachedSDFInfoPtrs;",
         "static __device__ SDFVolumeInfo* cachedSDFInfoPtrs = nullptr;")
    _sub(sdfm, r"extern __device__ uint32_t cachedSDFInfoPtrsCount;",
         "static __device__ uint32_t cachedSDFInfoPtrsCount = 0;")

    # (4) curand -> PCG32 streams shared with the GPU integrator.
    for p in CORE.rglob("*"):
        if p.suffix in (".cuh", ".h", ".hpp", ".cu"):
            _sub(p, r"#include\s*<curand_kernel\.h>\s*\n", "", must=False)
    rnd = CORE / "random.cuh"
    text = rnd.read_text()
    cut = text.index("FUNCTION_MODIFIER_DEVICE_INLINE void InitRand")
    text = text[:cut]
    text = text.replace("__device__ inline uint64_t TOTAL_FRAME_INDEX", "inline uint64_t TOTAL_FRAME_INDEX")
    text = text.replace("__device__ inline uint64_t GLOBAL_SEED", "inline uint64_t GLOBAL_SEED")
    text = text.replace('#include <cuda_runtime.h>', '#include <cuda_runtime.h>\n#include "ar_rng.h"', 1)
    text += (
        "typedef ar_pcg curandState;\n"
        "FUNCTION_MODIFIER_INLINE float Rand1(curandState* s) { return ar_rand1(s); }\n"
        "FUNCTION_MODIFIER_INLINE float2 Rand2(curandState* s) { const float a = ar_rand1(s); const float b = ar_rand1(s); return {a, b}; }\n"
        "FUNCTION_MODIFIER_INLINE float3 Rand3(curandState* s) { const float a = ar_rand1(s); const float b = ar_rand1(s); const float c = ar_rand1(s); return {a, b, c}; }\n"
    )
    rnd.write_text(text)

    # (5) 32-bit BVH nodes; runtime path-depth cap.
    cfg = CORE / "config.cuh"
    _sub(cfg, r"#define BVH_USE_16_BITS_NODE", "// #define BVH_USE_16_BITS_NODE")
    _sub(cfg, r"#define BVH_PACK_NODE", "// #define BVH_PACK_NODE")
    _sub(cfg, r"#define MAX_TRACING_DEPTH 1000",
         "inline int REF_MAX_TRACING_DEPTH = 1000;\n#define MAX_TRACING_DEPTH (REF_MAX_TRACING_DEPTH)")
    # runtime voxel unit of the guide (the reference compiles in 0.05,
    # core/config.cuh:43, core/guiding/guiding_bin.cuh:102-107)
    _sub(CORE / "guiding" / "guiding_bin.cuh", r"constexpr float invUnit = 1\.0f / PATH_GUIDING_RESOLUTION_UNIT;",
         "const float invUnit = REF_PG_INV_UNIT;")
    _sub(cfg, r"#define PATH_GUIDING_RESOLUTION_UNIT 0\.05\n",
         "#define PATH_GUIDING_RESOLUTION_UNIT 0.05\ninline float REF_PG_INV_UNIT = 1.0f / PATH_GUIDING_RESOLUTION_UNIT;\n")

    # (6) deterministic transcendentals everywhere in the copied tree.
    fn_re = re.compile(r"\b(" + "|".join(MATH_FUNCS) + r")\s*\(")
    un_re = re.compile(r"(?<![\w.:>])(" + "|".join(UNSUFFIXED) + r")\s*\(")
    for p in CORE.rglob("*"):
        if p.suffix not in (".cuh", ".h", ".hpp", ".cu"):
            continue
        text = p.read_text()
        text = fn_re.sub(lambda m: "arm_" + m.group(1) + "(", text)
        text = un_re.sub(lambda m: "arm_" + m.group(1) + "(", text)
        p.write_text(text)

    # (7) triangle object type, dispatched to our glue.
    obj = CORE / "render" / "object.cuh"
    _sub(obj, r"OBJ_SDF = 2,", "OBJ_SDF = 2,\n    OBJ_TRIANGLE = 3,")
    _sub(obj, r"struct SceneObject\s*\{\s*float3 center_;",
         "struct SceneObject\n{\n    float3 triV0_{}, triV1_{}, triV2_{};\n    float3 center_;")
    inter = CORE / "render" / "intersection.cuh"
    _sub(inter, r'#include "object/sdf/sdf_torus.cuh"',
         '#include "object/sdf/sdf_torus.cuh"\n#include "ref_glue.cuh"', count=1)
    _sub(inter,
         r"(else if\(object\.type_ == EObjectType::OBJ_SDF\)\s*\{\s*return sdf::IntersectSDFObject\(depth, rayOrigin, rayDirection, object\);\s*\})",
         r"\1\n        else if(object.type_ == EObjectType::OBJ_TRIANGLE)\n        {\n"
         r"            return ref_glue::IntersectTriangleObject(rayOrigin, rayDirection, object);\n        }",
         count=1)
    # node-visit counter for the traversal roofline's algorithmic bytes
    _sub(inter, r"const int currentNodeIndex = stack\[--sp\];",
         "const int currentNodeIndex = stack[--sp]; REF_NODE_VISIT_HOOK;", count=1)
    shutil.copy(HERE / "ref_glue.cuh", CORE / "render" / "ref_glue.cuh")

    # (8) denoiser: the device code subtracts two halves in half precision
    # (core/denoise/denoise.cuh:213-235, the __CUDA_ARCH__ branches); the host
    # branches subtract in float.  Keep the device arithmetic on the host too.
    den = CORE / "denoise" / "denoise.cuh"
    text = den.read_text()
    text, n = re.subn(r"#ifdef __CUDA_ARCH__\n([^\n]*static_cast<float>\(a\.[^\n]* - b\.[^\n]*\n)#else\n[^\n]*\n#endif\n",
                      r"\1", text)
    if n != 3:
        raise RuntimeError(f"denoise.cuh: expected 3 half-subtraction branches, found {n}")
    den.write_text(text)
    # the t-quantile table compiles into the driver's single translation unit:
    # the (never executed) device copy becomes a local zero table and its
    # separate definition goes; the host table T005QuantilesHost is unchanged
    _sub(CORE / "denoise" / "t_quantile.cuh", r"extern __device__ __constant__ float T005QuantilesDev\[T_QUANTILE_LUT_SIZE\];",
         "static __device__ __constant__ float T005QuantilesDev[T_QUANTILE_LUT_SIZE] = {};")
    _sub(CORE / "denoise" / "t_quantile.cu", r"__device__ __constant__ float T005QuantilesDev\[T_QUANTILE_LUT_SIZE\] = T005_LUT_INIT;",
         "")
    # (9) SDF volume cache on the host: the reference looks volumes up only in
    # device memory (core/object/sdf/sdf_master.cuh:15-39) and returns no volume
    # on the host; here the host branch reads a host table the driver fills.
    sdfm = CORE / "object" / "sdf" / "sdf_master.cuh"
    _sub(sdfm, r"(\s*)FUNCTION_MODIFIER_INLINE SDFVolumeInfo\* GetSDFVolumeInfoPtr\(const int cacheIndex\)",
         r"\1inline SDFVolumeInfo* REF_HOST_SDF_INFOS = nullptr;\1inline uint32_t REF_HOST_SDF_COUNT = 0;"
         r"\1FUNCTION_MODIFIER_INLINE SDFVolumeInfo* GetSDFVolumeInfoPtr(const int cacheIndex)", count=1)
    _sub(sdfm, r"#else\n(\s*)return nullptr;\n#endif",
         r"#else\n\1if (cacheIndex < 0 || cacheIndex >= (int)REF_HOST_SDF_COUNT) return nullptr;\n"
         r"\1return &REF_HOST_SDF_INFOS[cacheIndex];\n#endif", count=1)
    _sub(sdfm, r"#else\n(\s*)return 0u;\n#endif", r"#else\n\1return REF_HOST_SDF_COUNT;\n#endif", count=1)
    (CORE / PATCH_STAMP).write_text(PATCH_VERSION)


# bump when patch_tree() changes, so an existing patched copy is redone
PATCH_VERSION = "5"
PATCH_STAMP = ".ar_patch_version"


def needs_prepare() -> bool:
    """True when the reference checkout is present and the patched copy is
    missing or was made by an older patch_tree()."""
    if REF_ROOT is None or not (REF_ROOT / "core").is_dir():
        return False
    stamp = CORE / PATCH_STAMP
    return not stamp.exists() or stamp.read_text().strip() != PATCH_VERSION


def prepare() -> Path:
    copy_tree()
    patch_tree()
    return CORE


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and Path(c).exists():
            return c
    raise FileNotFoundError("nvcc not found")


def build_ref(jobs_hint: int = 0) -> Path:
    """Compile oracle/ref_driver.cu against the patched tree (host code, OpenMP)."""
    if not CORE.is_dir():
        prepare()
    exe = OUT / "ref_cpu"
    srcs = [HERE / "ref_driver.cu", HERE / "ref_glue.cuh", CSRC / "ar_detmath.h", CSRC / "ar_rng.h", CSRC / "ar_geom.h",
            CORE / PATCH_STAMP]
    if exe.exists() and all(exe.stat().st_mtime > s.stat().st_mtime for s in srcs if s.exists()):
        return exe
    cmd = [nvcc(), "-std=c++17", "-O3", "-DNDEBUG", "-DLINUX=1",
           "-x", "cu", "--extended-lambda", "-rdc=false",
           # the device pass of this TU is never executed; keep it cheap
           "-gencode", "arch=compute_103a,code=compute_103a",
           "-Xcompiler", "-fopenmp,-ffp-contract=off,-fno-fast-math",
           "-fmad=false", "-diag-suppress", "1866,20012,177,550,128,2417",
           "-I", str(CORE), "-I", str(CORE / "render"), "-I", str(CORE / "object"),
           "-I", str(CORE / "object" / "sdf"), "-I", str(CSRC),
           str(HERE / "ref_driver.cu"), "-o", str(exe), "-lgomp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout + r.stderr)
        raise RuntimeError("reference CPU oracle build failed")
    return exe


# ---------------------------------------------------------------- ref_gpu
# The reference's own GPU renderer, for timing beside ours: a copy of the
# core/ tree with the three Linux build fixes (include case forwarders,
# <cfloat>, the thrust::cuda::par qualification) and one launch bound (below),
# compiled with the reference's flags (CMakeLists.txt:111-121: separable
# compilation, -use_fast_math -maxrregcount=168 --extended-lambda) for
# sm_103a, driven by oracle/ref_gpu_driver.cu.
GPU_SRC = OUT / "gpu_src"
GPU_CORE = GPU_SRC / "core"
GPU_STAMP = ".ar_gpu_patch_version"
GPU_PATCH_VERSION = "2"
GPU_TUS = ["scene.cu", "object/sdf/sdf_base.cu", "object/sdf/sdf_cache_manager.cu", "object/sdf/sdf_master.cu",
           "denoise/t_quantile.cu"]


def needs_prepare_gpu() -> bool:
    if REF_ROOT is None or not (REF_ROOT / "core").is_dir():
        return False
    stamp = GPU_CORE / GPU_STAMP
    return not stamp.exists() or stamp.read_text().strip() != GPU_PATCH_VERSION


def prepare_gpu() -> Path:
    if REF_ROOT is None or not (REF_ROOT / "core").is_dir():
        raise FileNotFoundError(f"reference checkout not found at {REF_ROOT}")
    if GPU_SRC.exists():
        shutil.rmtree(GPU_SRC)
    GPU_SRC.mkdir(parents=True)
    shutil.copytree(REF_ROOT / "core", GPU_CORE, ignore=shutil.ignore_patterns("*.pyc", "__pycache__"))
    for q in GPU_CORE.rglob("*"):
        q.chmod(0o644 if q.is_file() else 0o755)
    (GPU_CORE / "object" / "AABB.cuh").write_text('#pragma once\n#include "aabb.cuh"\n')
    (GPU_CORE / "object" / "Sphere.cuh").write_text('#pragma once\n#include "sphere.cuh"\n')
    _sub(GPU_CORE / "guiding" / "guiding.cuh", r"([^:])cuda::par", r"\1thrust::cuda::par")
    _sub(GPU_CORE / "vector.cuh", r'#include "config.cuh"', '#include <cfloat>\n#include "config.cuh"', count=1)
    # the spectral-LUT kernel launches 8 x 8 x 8 threads per block
    # (core/spectrum/spectrum_lut.cuh:68-72); under -maxrregcount=168 this
    # compiler gives it more than 128 registers, so the launch fails with "too
    # many resources requested" and the LUT stays unset.  A launch bound of 512
    # threads on that kernel alone makes it launchable; the render kernels keep
    # the reference's flags.
    _sub(GPU_CORE / "spectrum" / "spectrum_lut.cuh", r"__global__ void PrecomputeRGBLUTKernel",
         "__global__ void __launch_bounds__(512) PrecomputeRGBLUTKernel", count=1)
    (GPU_CORE / GPU_STAMP).write_text(GPU_PATCH_VERSION)
    return GPU_CORE


def build_ref_gpu() -> Path:
    """Compile the reference GPU renderer and its headless driver (parallel TUs)."""
    import concurrent.futures as cf
    if not GPU_CORE.is_dir():
        prepare_gpu()
    exe = OUT / "ref_gpu"
    srcs = [HERE / "ref_gpu_driver.cu", GPU_CORE / GPU_STAMP]
    if exe.exists() and all(exe.stat().st_mtime > s.stat().st_mtime for s in srcs if s.exists()):
        return exe
    objdir = OUT / "gpu_obj"
    objdir.mkdir(exist_ok=True)
    flags = ["-std=c++17", "-O3", "-DNDEBUG", "-DLINUX=1", "-rdc=true", "--extended-lambda", "-use_fast_math",
             "-maxrregcount=168", "-gencode", "arch=compute_103a,code=sm_103a", "-diag-suppress",
             "1866,20012,177,550,128,2417,20011,20014", "-I", str(GPU_CORE), "-I", str(GPU_CORE / "render"),
             "-I", str(GPU_CORE / "object"), "-I", str(GPU_CORE / "object" / "sdf")]
    tus = [GPU_CORE / t for t in GPU_TUS] + [HERE / "ref_gpu_driver.cu"]
    objs = [objdir / (t.name + ".o") for t in tus]

    def one(i):
        return subprocess.run([nvcc(), *flags, "-c", str(tus[i]), "-o", str(objs[i])], capture_output=True, text=True)

    with cf.ThreadPoolExecutor(len(tus)) as ex:
        for r in ex.map(one, range(len(tus))):
            if r.returncode != 0:
                sys.stderr.write(r.stdout + r.stderr)
                raise RuntimeError("reference GPU renderer build failed")
    r = subprocess.run([nvcc(), "-rdc=true", "-gencode", "arch=compute_103a,code=sm_103a", *map(str, objs), "-o",
                        str(exe)], capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout + r.stderr)
        raise RuntimeError("reference GPU renderer link failed")
    return exe


if __name__ == "__main__":
    if "--reference" in sys.argv:
        REF_ROOT = Path(sys.argv[sys.argv.index("--reference") + 1])
    if "--build-only" not in sys.argv:
        prepare()
        print("patched reference tree at", CORE)
    print("built", build_ref())
