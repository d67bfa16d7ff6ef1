"""Runs the reference CPU oracle (oracle/_ref/ref_cpu) on our scene descriptions.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline / reference arm, never by the product package.
"""
from __future__ import annotations

import json
import os
import subprocess
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
EXE = HERE / "_ref" / "ref_cpu"

OBJ_DTYPE = np.dtype([("type", "<i4"), ("shading", "<i4"), ("center", "<f4", 3), ("extent", "<f4", 3),
                      ("rotation", "<f4", 3), ("v0", "<f4", 3), ("v1", "<f4", 3), ("v2", "<f4", 3),
                      ("albedo", "<f4", 3), ("emissive", "<f4", 3), ("roughness", "<f4"), ("metallic", "<f4"),
                      ("specular", "<f4"), ("ior", "<f4"), ("sigma_a", "<f4"), ("abbe", "<f4"), ("tilt", "<f4"),
                      ("sdf_type", "<i4"), ("sdf_params", "<f4", 4), ("sdf_volume", "<i4")])
# one SDF volume: fn 0 torus / 1 diamond filled by the reference functor, -1: values follow
VOL_DTYPE = np.dtype([("fn", "<i4"), ("params", "<f4", 4), ("dims", "<i4", 3)])
PARAMS_DTYPE = np.dtype([("width", "<i4"), ("height", "<i4"), ("spp", "<i4"), ("max_depth", "<i4"),
                         ("cam_origin", "<f4", 3), ("cam_dir", "<f4", 3), ("fov", "<f4"), ("use_nee", "<i4"),
                         ("seed", "<u8"), ("first_frame", "<i4"), ("per_sample", "<i4"), ("denoise", "<i4"),
                         ("guide", "<i4"), ("guide_inv_unit", "<f4")])
PROBE_FLOATS = 344  # Octahedron::data_ (86 float4) as floats
# one radiance record of the guided integrator: valid, key (voxel xyz, face), direction, XYZ radiance
GREC_DTYPE = np.dtype([("valid", "<i4"), ("key", "<i4", 4), ("dir", "<f4", 3), ("radiance", "<f4", 3)])
# denoiser records in the driver's plain layout (the GPU library's ar_denoise_read layout)
GBUF_DTYPE = np.dtype([("h", "<u2", 14), ("depth", "<f4"), ("valid", "<u4"), ("frames", "<u4")])
STAT_DTYPE = np.dtype([("num", "<u4"), ("mean", "<f4", 3), ("m2n", "<f4", 3), ("m3n", "<f4", 3)])


def available() -> bool:
    return EXE.exists()


def ensure_built() -> Path:
    """Builds the oracle if its patched sources are present (see prepare_ref.py)."""
    if EXE.exists():
        return EXE
    from . import prepare_ref  # noqa: F401  (package-relative when imported as oracle.ref_runner)
    return prepare_ref.build_ref()


def scene_bytes(objects, mesh=None, volumes=None) -> bytes:
    """Objects (and mesh triangles, appended as triangle objects) in the oracle's file format,
    then the SDF volume cache: volumes is a list of (fn, params, dims) to fill with the
    reference's functor, or (None, values (dz, dy, dx), None) for given values."""
    n_mesh = 0 if mesh is None else len(mesh.indices)
    rec = np.zeros(len(objects) + n_mesh, OBJ_DTYPE)
    for i, o in enumerate(objects):
        m = o.material
        info = getattr(o, "additionalObjectInfo", None)
        st, sp, sv = (info.sdf_type, info.params, info.volume) if info is not None else (0, (0.0,) * 4, -1)
        rec[i] = (o.type, m.shading, o.center, o.extent, o.rotation, o.v0, o.v1, o.v2, m.albedo, m.emissive,
                  m.roughness, m.metallic, m.specular, m.ior, m.sigma_a, m.abbe, m.tilt, st, sp, sv)
    if n_mesh:
        tv = mesh.triangle_vertices().reshape(-1, 3, 3)
        base = len(objects)
        r = rec[base:]
        r["type"] = 3
        r["v0"], r["v1"], r["v2"] = tv[:, 0], tv[:, 1], tv[:, 2]
        mids = np.asarray(mesh.material_ids, np.int64)
        for k, m in enumerate(mesh.materials):
            sel = mids == k
            r["shading"][sel] = m.shading
            r["albedo"][sel] = m.albedo
            r["emissive"][sel] = m.emissive
            r["roughness"][sel] = m.roughness
            r["metallic"][sel] = m.metallic
            r["specular"][sel] = m.specular
            r["ior"][sel] = m.ior
            r["sigma_a"][sel] = m.sigma_a
            r["abbe"][sel] = m.abbe
            r["tilt"][sel] = m.tilt
    out = [b"ARS2", np.int32(len(rec)).tobytes(), rec.tobytes(), np.int32(len(volumes or [])).tobytes()]
    for fn, prm, dims in volumes or []:
        v = np.zeros(1, VOL_DTYPE)
        if fn is None:
            vals = np.ascontiguousarray(prm, np.float32)
            v[0] = (-1, (0.0,) * 4, (vals.shape[2], vals.shape[1], vals.shape[0]))
            out += [v.tobytes(), vals.tobytes()]
        else:
            v[0] = (int(fn), tuple(prm), tuple(dims))
            out.append(v.tobytes())
    return b"".join(out)


def sdf_volume(fn: int, params, dims) -> np.ndarray:
    """One volume filled on the host with the reference's functor: (dz, dy, dx) float32."""
    exe = ensure_built()
    v = np.zeros(1, VOL_DTYPE)
    v[0] = (int(fn), tuple(params), tuple(dims))
    with tempfile.TemporaryDirectory() as td:
        td = Path(td)
        (td / "in.bin").write_bytes(v.tobytes())
        r = subprocess.run([str(exe), "sdfvol", str(td / "in.bin"), str(td / "out.bin")], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("reference oracle failed: " + r.stderr)
        return np.frombuffer((td / "out.bin").read_bytes(), np.float32).reshape(dims[2], dims[1], dims[0]).copy()


def probe_bytes(probes: dict) -> bytes:
    """A probe set (keys (n, 4) int32, texels (n, 86, 4) float32, counts (n,) uint64) in the
    oracle's file format."""
    k = np.ascontiguousarray(probes["keys"], np.int32).reshape(-1, 4)
    t = np.ascontiguousarray(probes["texels"], np.float32).reshape(len(k), PROBE_FLOATS)
    c = np.ascontiguousarray(probes["counts"], np.uint64).reshape(len(k))
    return np.int32(len(k)).tobytes() + k.tobytes() + t.tobytes() + c.tobytes()


def _read_probes(raw: bytes) -> dict:
    n = int(np.frombuffer(raw[:4], np.int32)[0])
    at = 4
    k = np.frombuffer(raw[at: at + 16 * n], np.int32).reshape(n, 4).copy()
    at += 16 * n
    t = np.frombuffer(raw[at: at + 4 * PROBE_FLOATS * n], np.float32).reshape(n, PROBE_FLOATS // 4, 4).copy()
    at += 4 * PROBE_FLOATS * n
    c = np.frombuffer(raw[at: at + 8 * n], np.uint64).copy()
    return {"keys": k, "texels": t, "counts": c}


def guide_update(probes: dict, keys, dirs, radiance) -> dict:
    """One probe update of the reference (UpdatePathGuidingSample's accumulate and
    merge) over the given radiance records, from the given probe set."""
    exe = ensure_built()
    k = np.ascontiguousarray(keys, np.int32).reshape(-1, 4)
    rec = np.zeros(len(k), np.dtype([("key", "<i4", 4), ("dir", "<f4", 3), ("rad", "<f4", 3)]))
    rec["key"], rec["dir"], rec["rad"] = k, np.asarray(dirs, np.float32), np.asarray(radiance, np.float32)
    with tempfile.TemporaryDirectory() as td:
        td = Path(td)
        (td / "probes.bin").write_bytes(probe_bytes(probes))
        (td / "rec.bin").write_bytes(np.int32(len(rec)).tobytes() + rec.tobytes())
        r = subprocess.run([str(exe), "pgupdate", str(td / "probes.bin"), str(td / "rec.bin"), str(td / "out.bin")],
                           capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("reference oracle failed: " + r.stderr)
        return _read_probes((td / "out.bin").read_bytes())


def render(objects, size, origin, direction, spp, *, fov=60.0, max_depth=1000, use_nee=True,
           seed=0x9E3779B97F4A7C15, first_frame=0, per_sample_frames=0, mesh=None, threads=None, denoise=False,
           volumes=None, guide_probes=None, guide_unit=0.05):
    """Returns (mean XYZ (H, W, 3) float64, per-sample XYZ or None, stats dict); with
    denoise=True the stats dict also holds the denoiser records under "gbuffer" and
    "moments" ((H, W) arrays of GBUF_DTYPE / STAT_DTYPE).  With guide_probes (a probe
    set as probe_bytes takes it) the reference's guided integrator runs over those
    probes (voxel unit guide_unit) and the stats dict holds the radiance records of
    the per-sample frames under "records" ((frames, H, W, 5) of GREC_DTYPE)."""
    exe = ensure_built()
    w, h = int(size[0]), int(size[1])
    prm = np.zeros(1, PARAMS_DTYPE)
    guided = guide_probes is not None
    prm[0] = (w, h, spp, max_depth, origin, direction, fov, 1 if use_nee else 0, seed, first_frame, per_sample_frames,
              1 if denoise else 0, 1 if guided else 0, np.float32(1.0) / np.float32(guide_unit))
    with tempfile.TemporaryDirectory() as td:
        td = Path(td)
        (td / "scene.bin").write_bytes(scene_bytes(objects, mesh, volumes))
        (td / "params.bin").write_bytes(prm.tobytes())
        args = [str(exe), "render", str(td / "scene.bin"), str(td / "params.bin"), str(td / "out.bin")]
        if guided:
            (td / "probes.bin").write_bytes(probe_bytes(guide_probes))
            args.append(str(td / "probes.bin"))
        env = dict(os.environ)
        if threads:
            env["OMP_NUM_THREADS"] = str(threads)
        env.setdefault("OMP_PROC_BIND", "close")
        r = subprocess.run(args, capture_output=True, text=True, env=env)
        if r.returncode != 0:
            raise RuntimeError("reference oracle failed: " + r.stderr)
        stats = json.loads(r.stdout.strip().splitlines()[-1])
        raw = (td / "out.bin").read_bytes()
    npix = w * h
    sums = np.frombuffer(raw[: npix * 24], np.float64).reshape(h, w, 3)
    at = npix * 24
    per = None
    if per_sample_frames:
        per = np.frombuffer(raw[at: at + npix * 12 * per_sample_frames], np.float32).reshape(per_sample_frames, h, w, 3)
        at += npix * 12 * per_sample_frames
    if guided:
        nrec = per_sample_frames * npix * 5
        stats["records"] = np.frombuffer(raw[at: at + nrec * GREC_DTYPE.itemsize], GREC_DTYPE).reshape(
            per_sample_frames, h, w, 5).copy()
        at += nrec * GREC_DTYPE.itemsize
    if denoise:
        stats["gbuffer"] = np.frombuffer(raw[at: at + npix * GBUF_DTYPE.itemsize], GBUF_DTYPE).reshape(h, w).copy()
        at += npix * GBUF_DTYPE.itemsize
        stats["moments"] = np.frombuffer(raw[at: at + npix * STAT_DTYPE.itemsize], STAT_DTYPE).reshape(h, w).copy()
    return sums / spp, per, stats


def denoise(image, gbuffer, moments, threads=None) -> np.ndarray:
    """The reference's bilateral denoiser on the host: image (H, W, 3) read as
    float32, records as GBUF_DTYPE / STAT_DTYPE (H, W) arrays; returns float32 (H, W, 3)."""
    exe = ensure_built()
    img = np.ascontiguousarray(image, np.float32)
    h, w, _ = img.shape
    g = np.ascontiguousarray(gbuffer, GBUF_DTYPE).reshape(h, w)
    m = np.ascontiguousarray(moments, STAT_DTYPE).reshape(h, w)
    with tempfile.TemporaryDirectory() as td:
        td = Path(td)
        (td / "in.bin").write_bytes(np.array([w, h], np.int32).tobytes() + img.tobytes() + g.tobytes() + m.tobytes())
        env = dict(os.environ)
        if threads:
            env["OMP_NUM_THREADS"] = str(threads)
        r = subprocess.run([str(exe), "denoise", str(td / "in.bin"), str(td / "out.bin")], capture_output=True,
                           text=True, env=env)
        if r.returncode != 0:
            raise RuntimeError("reference oracle failed: " + r.stderr)
        return np.frombuffer((td / "out.bin").read_bytes(), np.float32).reshape(h, w, 3).copy()


def trace(tris: np.ndarray, rays: np.ndarray, brute: bool = False, threads=None):
    """Closest hit through the reference BVH (or brute force): (prim_id int32, t float32, stats)."""
    exe = ensure_built()
    tris = np.ascontiguousarray(tris, np.float32).reshape(-1, 9)
    rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
    with tempfile.TemporaryDirectory() as td:
        td = Path(td)
        (td / "tris.bin").write_bytes(np.int32(len(tris)).tobytes() + tris.tobytes())
        (td / "rays.bin").write_bytes(np.int32(len(rays)).tobytes() + rays.tobytes())
        env = dict(os.environ)
        if threads:
            env["OMP_NUM_THREADS"] = str(threads)
        r = subprocess.run([str(exe), "brute" if brute else "trace", str(td / "tris.bin"), str(td / "rays.bin"),
                            str(td / "out.bin")], capture_output=True, text=True, env=env)
        if r.returncode != 0:
            raise RuntimeError("reference oracle failed: " + r.stderr)
        stats = json.loads(r.stdout.strip().splitlines()[-1])
        raw = (td / "out.bin").read_bytes()
    n = len(rays)
    return np.frombuffer(raw[: 4 * n], np.int32).copy(), np.frombuffer(raw[4 * n:], np.float32).copy(), stats


def guide_eval(payload: bytes, n: int) -> np.ndarray:
    """The reference's probe math on one probe (see ref_driver.cu cmd_guide)."""
    exe = ensure_built()
    with tempfile.TemporaryDirectory() as td:
        td = Path(td)
        (td / "in.bin").write_bytes(np.int32(n).tobytes() + payload)
        subprocess.run([str(exe), "guide", str(td / "in.bin"), str(td / "out.bin")], check=True, capture_output=True)
        return np.frombuffer((td / "out.bin").read_bytes(), np.float32).copy()


def kat() -> dict:
    exe = ensure_built()
    r = subprocess.run([str(exe), "kat"], capture_output=True, text=True, check=True)
    return json.loads(r.stdout)


def luts(lattice: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """(lambda LUT (840, 4), RGBEncode at the given (n, 3) int lattice points)."""
    exe = ensure_built()
    lattice = np.ascontiguousarray(lattice, np.int32).reshape(-1, 3)
    with tempfile.TemporaryDirectory() as td:
        td = Path(td)
        (td / "lat.bin").write_bytes(lattice.tobytes())
        subprocess.run([str(exe), "lut", str(td / "lat.bin"), str(td / "out.bin")], check=True, capture_output=True)
        raw = (td / "out.bin").read_bytes()
    lam = np.frombuffer(raw[: 840 * 16], np.float32).reshape(840, 4)
    rgb = np.frombuffer(raw[840 * 16:], np.float32).reshape(-1, 4)
    return lam, rgb


def tonemap(xyz, exposure: float, tone: str) -> np.ndarray:
    """The reference's display transform (Camera::RenderToFile's pixel loop with
    core/tonemap.cuh's curves) on float32 XYZ (H, W, 3): RGBA8 (H, W, 4)."""
    exe = ensure_built()
    x = np.ascontiguousarray(xyz, np.float32)
    h, w, _ = x.shape
    code = {"aces": 0, "gamma": 1, "linear": 2}[tone]
    with tempfile.TemporaryDirectory() as td:
        td = Path(td)
        (td / "in.bin").write_bytes(np.int32(h * w).tobytes() + np.float32(exposure).tobytes() +
                                    np.int32(code).tobytes() + x.tobytes())
        r = subprocess.run([str(exe), "tonemap", str(td / "in.bin"), str(td / "out.bin")], capture_output=True,
                           text=True)
        if r.returncode != 0:
            raise RuntimeError("reference oracle failed: " + r.stderr)
        return np.frombuffer((td / "out.bin").read_bytes(), np.uint8).reshape(h, w, 4).copy()


def frame_tonemap(hdr, exposure: float, tone_type: int) -> np.ndarray:
    """The display kernel of the reference's progressive Render (core/scene.cu:22-131,
    plain branch) on a float32 XYZ running mean (H, W, 3): uint32 0xAARRGGBB (H, W)."""
    exe = ensure_built()
    x = np.ascontiguousarray(hdr, np.float32)
    h, w, _ = x.shape
    with tempfile.TemporaryDirectory() as td:
        td = Path(td)
        (td / "in.bin").write_bytes(np.int32(h * w).tobytes() + np.float32(exposure).tobytes() +
                                    np.int32(tone_type).tobytes() + x.tobytes())
        r = subprocess.run([str(exe), "frametone", str(td / "in.bin"), str(td / "out.bin")], capture_output=True,
                           text=True)
        if r.returncode != 0:
            raise RuntimeError("reference oracle failed: " + r.stderr)
        return np.frombuffer((td / "out.bin").read_bytes(), np.uint32).reshape(h, w).copy()


def trace_count(tris: np.ndarray, rays: np.ndarray, threads=None):
    """Closest hits through the reference's BuildBVH tree walked with a slab test that
    requires tEnter <= tExit: (prim_id, t, node pops per ray, triangle tests per ray, stats)."""
    exe = ensure_built()
    tris = np.ascontiguousarray(tris, np.float32).reshape(-1, 9)
    rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
    n = len(rays)
    with tempfile.TemporaryDirectory() as td:
        td = Path(td)
        (td / "tris.bin").write_bytes(np.int32(len(tris)).tobytes() + tris.tobytes())
        (td / "rays.bin").write_bytes(np.int32(n).tobytes() + rays.tobytes())
        env = dict(os.environ)
        if threads:
            env["OMP_NUM_THREADS"] = str(threads)
        r = subprocess.run([str(exe), "tracecount", str(td / "tris.bin"), str(td / "rays.bin"), str(td / "out.bin")],
                           capture_output=True, text=True, env=env)
        if r.returncode != 0:
            raise RuntimeError("reference oracle failed: " + r.stderr)
        stats = json.loads(r.stdout.strip().splitlines()[-1])
        raw = (td / "out.bin").read_bytes()
    ids = np.frombuffer(raw[: 4 * n], np.int32).copy()
    t = np.frombuffer(raw[4 * n: 8 * n], np.float32).copy()
    visits = np.frombuffer(raw[8 * n: 12 * n], np.uint32).copy()
    tests = np.frombuffer(raw[12 * n: 16 * n], np.uint32).copy()
    return ids, t, visits, tests, stats
