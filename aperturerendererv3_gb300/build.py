"""Builds libaperture_gb300.so in-tree for sm_103a.

Every CUDA translation unit is compiled with
    -gencode arch=compute_103a,code=sm_103a -lineinfo -O3 -fmad=false
and host code with -ffp-contract=off: the renderer's parity contract needs
every target to round identically (no implicit FMA contraction anywhere).
Translation units compile in parallel; ptxas resource usage of every kernel is
written to _build/ptxas.log.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
REPO = PKG.parent
CSRC = PKG / "csrc"
BUILD = REPO / "_build"
LIB = PKG / "libaperture_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_SOURCES = ["capi.cu", "render.cu", "trace.cu", "noalloc.cu", "guide.cu", "adjoint.cu", "mlp.cu", "tonemap.cu",
              "denoise.cu", "sdfvol.cu", "bvh_gpu.cu", "frame.cu"]
CPP_SOURCES = ["bvh_build.cpp"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and Path(c).exists():
            return c
    raise FileNotFoundError("nvcc not found")


def _hexf(v: np.float32) -> str:
    return float(v).hex() + "f"


def write_tables(dst: Path) -> None:
    t = np.load(PKG / "data" / "spectral_tables.npz")
    rgb = [t["RGB_IN_W"], t["RGB_IN_B"]]
    for i in range(7):
        rgb += [t[f"RGB_BLK{i}_W"], t[f"RGB_BLK{i}_B"]]
    rgb.append(t["RGB_OUT_W"])
    lam = []
    for i in range(7):
        lam += [t[f"LAM_BLK{i}_W"], t[f"LAM_BLK{i}_B"]]
    lam.append(t["LAM_OUT_W"])
    arrays = {
        "AR_TAB_D65": t["D65_SPD"].astype(np.float32),
        "AR_TAB_CMF": t["CIEXYZ_CMF"].astype(np.float32).reshape(-1),
        "AR_TAB_RGB_MLP": np.concatenate(rgb).astype(np.float32),
        "AR_TAB_LAM_MLP": np.concatenate(lam).astype(np.float32),
    }
    lines = ["// generated by aperturerendererv3_gb300/build.py from data/spectral_tables.npz", "#pragma once"]
    for name, a in arrays.items():
        body = ",".join(_hexf(v) for v in a)
        lines.append(f"alignas(16) static const float {name}[{a.size}] = {{{body}}};")
    text = "\n".join(lines) + "\n"
    if not dst.exists() or dst.read_text() != text:
        dst.write_text(text)


def _stale(obj: Path, deps: list[Path]) -> bool:
    return not obj.exists() or any(d.stat().st_mtime > obj.stat().st_mtime for d in deps)


def _run(cmd: list[str], log: Path | None = None) -> str:
    r = subprocess.run(cmd, capture_output=True, text=True)
    out = r.stdout + r.stderr
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + out)
    return out


def build(force: bool = False, verbose: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    write_tables(BUILD / "spectral_tables.inc")
    nv = nvcc()
    common = ["-std=c++17", "-O3", "-I", str(CSRC), "-I", str(BUILD), "-I", str(REPO / "include")]
    # every header of csrc/ counts: a translation unit is rebuilt when any of them changes
    headers = sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh"))
    deps = headers + [BUILD / "spectral_tables.inc", REPO / "include" / "aperture" / "ar.h", Path(__file__)]
    jobs = []
    for src in CU_SOURCES:
        obj = BUILD / (src + ".o")
        if force or _stale(obj, deps + [CSRC / src]):
            jobs.append([nv, *common, *ARCH, "-lineinfo", "-fmad=false", "-Xptxas", "-v",
                         "-Xcompiler", "-fPIC,-ffp-contract=off", "-c", str(CSRC / src), "-o", str(obj)])
    for src in CPP_SOURCES:
        obj = BUILD / (src + ".o")
        if force or _stale(obj, deps + [CSRC / src]):
            jobs.append(["g++", "-std=c++17", "-O3", "-fPIC", "-ffp-contract=off", "-pthread",
                         "-I", str(CSRC), "-c", str(CSRC / src), "-o", str(obj)])
    logs = []
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=max(2, min(len(jobs), os.cpu_count() or 4))) as ex:
            for out in ex.map(_run, jobs):
                logs.append(out)
        (BUILD / "ptxas.log").write_text("\n".join(logs))
    objs = [str(BUILD / (s + ".o")) for s in CU_SOURCES + CPP_SOURCES]
    if force or jobs or not LIB.exists():
        _run([nv, "-shared", *ARCH, "-o", str(LIB), *objs, "-lcudart", "-Xcompiler", "-pthread"])
    if verbose:
        print("\n".join(logs))
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
