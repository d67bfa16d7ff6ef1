"""Benchmark: Msamples/s of the spectral path tracer on one GB300 (or N replicas).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload terrain|cornell] [--impl ours|reference]

The default workload is the guided-path-tracing terrain: 2048^2 fBm heightfield
(8.38M triangles), 64 sphere lights and a sun, GGX materials, 1920x1080, 64 spp,
depth 16, NEE + MIS, rendered by the plain method (the drop-in).  Beside the
headline the line carries `extras`: the same workload with the voxel guide
learning online, the replay adjoint's grads/s against central differences on
the textured Cornell box, and closest-hit Mrays/s on 1M random triangles.

A step renders the whole workload once (width x height x spp paths, each a full
path up to max depth) with a fresh block of sample indices, so no work repeats.
`value` is samples / device time (CUDA events on the renderer's stream, scene
resident in HBM); `e2e` is the same metric through SceneRenderer.Render, the
reference-facing call, with host output buffers and the result copied back
inside the timed region.  Path state is ~170 B/path x 33.5M paths in flight, far
above the 129 MB L2, so no L2 flush is needed between steps.

--impl reference runs the reference's own integrator compiled for the CPU
(oracle/_ref, built by __graft_entry__.build()) on every host core, on a bounded
sample of the same workload.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

WORKLOADS = {
    # 256x256, 16 spp, depth 8 Cornell box of triangles
    "cornell": dict(size=(256, 256), spp=16, depth=8),
    # 1920x1080, 64 spp, depth 16 terrain (8.4M triangles), 64 sphere lights + sun
    "terrain": dict(size=(1920, 1080), spp=64, depth=16),
    # the terrain with 32 smooth-union SDF primitives in a participating medium,
    # 3840x2160, 256 spp, depth 24, MLP guide with the voxel guide as fallback
    "combined": dict(size=(3840, 2160), spp=256, depth=24, guide=2),
}


def build_workload(name: str):
    """(objects, mesh, camera, extra SceneRenderer arguments)."""
    from aperturerendererv3_gb300 import configs
    if name == "cornell":
        return configs.cornell_triangles(), None, configs.CORNELL_CAMERA, {}
    if name == "terrain":
        objs, mesh = configs.terrain_scene()
        return objs, mesh, configs.TERRAIN_CAMERA, {}
    if name == "combined":
        objs, mesh, sdf, med = configs.combined_scene()
        return objs, mesh, configs.COMBINED_CAMERA, dict(sdf=sdf, medium=med)
    raise KeyError(name)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons while the timed region runs."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": d["hbm_gbs"], "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def traversal_work(workload: str):
    """Per-ray algorithmic traversal work frozen by oracle/make_traversal_work.py (or None)."""
    p = ROOT / "profiles" / f"traversal_work_{workload}.json"
    return json.loads(p.read_text()) if p.exists() else None


def limiter_summary(workload: str):
    """What bounds the closest-hit kernel, from the committed ncu summary of a small
    case (issue activity, SIMT efficiency, L2 and DRAM throughput), or None."""
    p = ROOT / "profiles" / f"k_extend_limiter_{workload}.json"
    return json.loads(p.read_text()) if p.exists() else None


def profile_traffic(workload: str):
    """k_extend DRAM bytes per camera ray and per bounce ray from the committed
    small-case ncu summary (or None)."""
    p = ROOT / "profiles" / "traffic.json"
    if p.exists():
        d = json.loads(p.read_text())
        return d.get(workload)
    return None


def cpu_reference_run(workload: str, objs, mesh, cam, w: dict, sample_spp: int, sample_size, threads: int):
    from oracle import ref_runner as rr
    rr.ensure_built()
    t0 = time.perf_counter()
    _, _, st = rr.render(objs, sample_size, cam["origin"], cam["direction"], sample_spp, fov=cam["fov"],
                         max_depth=w["depth"], mesh=mesh, threads=threads)
    wall = time.perf_counter() - t0
    return st, wall


def reference_sample(workload: str, size):
    """Bounded sample of the workload for the reference CPU integrator: (size, spp per step).
    The reference renders the terrain at tens of samples per second on the host
    (its slab test does not reject boxes the ray misses, so its traversal visits
    a large share of the BVH), so a step is a 16 x 9 pixel block at 1 spp."""
    if workload == "cornell":
        return size, 2
    return (16, 9), 1


def run_reference(args, w) -> dict:
    """The reference integrator (oracle/_ref, CPU, every host core) on a bounded
    sample of the same workload.  One oracle call renders warmup + steps frames
    of the sample (its BVH is built once per call, outside the timed loop, as
    the reference builds its BVH before rendering)."""
    if args.workload == "combined":
        return {"impl": "reference", "unavailable": "the reference integrator has no participating media and no "
                "smooth-union SDF objects (the combined workload's features)"}
    objs, mesh, cam, _ = build_workload(args.workload)
    threads = os.cpu_count() or 1
    size = w["size"]
    sample_size, sample_spp = reference_sample(args.workload, size)
    st, _ = cpu_reference_run(args.workload, objs, mesh, cam, w, sample_spp * (args.warmup + args.steps),
                              sample_size, threads)
    value = float(st["msamples_per_s"])
    sample = (f"{sample_size[0]}x{sample_size[1]}x{sample_spp} spp of the {args.workload} workload per step, "
              f"{args.warmup + args.steps} steps in one call")
    return {"metric": "Msamples/s", "value": value, "unit": "Msamples/s", "impl": "reference",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": float(np.prod(sample_size) * sample_spp / value / 1e3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": args.workload, "width": size[0], "height": size[1], "spp": w["spp"],
                       "max_depth": w["depth"], "parallelism": "cpu-openmp"},
            "cpu_baseline": {"value": value, "unit": "Msamples/s", "cores": threads, "kind": "reference",
                             "sample": sample},
            "e2e": {"value": value, "unit": "Msamples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def guided_extra(r, w, cam, steps: int, window: int = 16) -> dict:
    """Same workload with the voxel guide learning online: updates after every
    frame (the reference's schedule: one frame per wave) and after every
    `window` frames (the window's frames share waves)."""
    size, spp, depth = w["size"], w["spp"], w["depth"]
    out = {}
    for key, gf in (("per_frame", 1), (f"window_{window}", window)):
        r.MarkNeedResetGuiding()
        r.Render(size, cam["origin"], cam["direction"], spp, fov=cam["fov"], max_depth=depth, guide=1, guide_frames=gf)
        ms = []
        for k in range(steps):
            r.Render(size, cam["origin"], cam["direction"], spp, fov=cam["fov"], max_depth=depth, guide=1,
                     first_frame=(k + 1) * spp, guide_frames=gf)
            ms.append(r.last_render_stats()[0])
        n_probes, _ = r.guide_stats()
        out[key] = {"value": size[0] * size[1] * spp / (float(np.mean(ms)) / 1e3) / 1e6, "unit": "Msamples/s",
                    "ms_per_step": float(np.mean(ms)), "steps": steps, "probes": n_probes, "guide_frames": gf}
    r.MarkNeedResetGuiding()
    out["value"], out["unit"] = out[f"window_{window}"]["value"], "Msamples/s"
    return out


def rel_mse(img, ref) -> float:
    """mean over pixels of sum_c (I - I_ref)^2 / (I_ref^2 + 1e-2)."""
    return float((((img - ref) ** 2) / (ref ** 2 + 1e-2)).sum(-1).mean())


def scene_extent(objs, mesh) -> float:
    """Largest side of the mesh's bounding box (the terrain: its unit square)."""
    v = np.asarray(mesh.vertices, np.float64).reshape(-1, 3)
    return float((v.max(0) - v.min(0)).max())


def guide_compare_extra(r, w, cam, objs, mesh, ref_spp: int = 2048, window: int = 8, crop: int = 64) -> dict:
    """Voxel guide vs MLP guide at equal wall time, each learning from scratch
    (training included), scored by rel-MSE against a converged plain render of
    the same view (ref_spp samples per pixel, FP64 accumulation, disjoint
    sample streams) whose central crop x crop pixels are checked against the
    FP64 CPU oracle (oracle/pt64) rendering the same pixels and streams.  The
    voxel guide uses a 64^3 grid over the scene (voxel = extent / 64).  Guided
    renders update after every `window` frames (calls of `window` frames); the
    voxel guide is also run with the reference's update after every frame.  The
    voxel guide renders the workload's spp; the others as many windows as fit
    in its wall time."""
    size, spp, depth = w["size"], w["spp"], w["depth"]
    kw = dict(fov=cam["fov"], max_depth=depth)
    unit = scene_extent(objs, mesh) / 64.0
    t0 = time.perf_counter()
    ref = r.Render(size, cam["origin"], cam["direction"], ref_spp, first_frame=1 << 20, **kw)
    out = {"reference": {"spp": ref_spp, "ms": r.last_render_stats()[0], "kind": "plain render, FP64 accumulation"},
           "voxel_unit": unit, "window_frames": window}
    # the reference image's crop against the FP64 oracle (same pixels, same random streams)
    x0, y0 = (size[0] - crop) // 2, (size[1] - crop) // 2
    try:
        from oracle import pt64
        t1 = time.perf_counter()
        s64 = pt64.Scene64(objs, mesh)
        ref64 = s64.render_crop(size, (x0, y0, crop, crop), cam["origin"], cam["direction"], ref_spp,
                                first_frame=1 << 20, **kw)
        rc = ref[y0:y0 + crop, x0:x0 + crop]
        rel = np.abs(rc - ref64) / np.maximum(np.abs(ref64), 1e-3)
        out["reference"]["fp64_pin"] = {"crop": [x0, y0, crop, crop], "rel_mse": rel_mse(rc, ref64),
                                        "max_rel_diff": float(rel.max()), "median_rel_diff": float(np.median(rel)),
                                        "s": time.perf_counter() - t1}
    except Exception as e:  # the pin is a check beside the number; report why it is missing
        ref64 = None
        out["reference"]["fp64_pin"] = {"unavailable": str(e)}

    def run(mode, frames=None, budget=None, steps=0, gf=window):
        r.MarkNeedResetGuiding()
        acc, n = None, 0
        t_start = time.perf_counter()
        chunk = gf if mode else window
        while frames is None or n < frames:
            img = r.Render(size, cam["origin"], cam["direction"], chunk, guide=mode, first_frame=n,
                           guide_train_steps=steps, guide_unit=unit, guide_frames=gf, **kw)
            acc = img * chunk if acc is None else acc + img * chunk
            n += chunk
            if budget is not None and time.perf_counter() - t_start >= budget:
                break
        return acc / n, n, time.perf_counter() - t_start

    def score(img):
        d = {"rel_mse": rel_mse(img, ref)}
        if ref64 is not None:
            d["rel_mse_fp64_crop"] = rel_mse(img[y0:y0 + crop, x0:x0 + crop], ref64)
        return d

    # one untimed window of each guide mode first (each timed run still starts
    # from a reset guide): kernel module loads and first-use host work stay out
    # of the equal-time budget, which the first timed run sets
    run(1, frames=window)
    run(2, frames=window, steps=8)
    vox, n_vox, t_vox = run(1, frames=spp)
    out["voxel"] = {"spp": n_vox, "s": t_vox, **score(vox)}
    vox1, n1, t1 = run(1, budget=t_vox, gf=1)
    out["voxel_per_frame"] = {"spp": n1, "s": t1, **score(vox1)}
    for key, steps_per_frame in (("mlp", 8), ("mlp_32_steps", 32)):
        mlp, n_mlp, t_mlp = run(2, budget=t_vox, steps=steps_per_frame)
        steps, loss = r.mlp_stats()
        out[key] = {"spp": n_mlp, "s": t_mlp, **score(mlp), "train_steps": steps,
                    "steps_per_frame": steps_per_frame, "last_loss_sum": loss}
    r.MarkNeedResetGuiding()
    plain, n_plain, t_plain = run(0, budget=t_vox)
    out["plain"] = {"spp": n_plain, "s": t_plain, **score(plain)}
    best_vox = min(out["voxel"]["rel_mse"], out["voxel_per_frame"]["rel_mse"])
    best_mlp = min(out["mlp"]["rel_mse"], out["mlp_32_steps"]["rel_mse"])
    out["mlp_over_voxel"] = out["mlp"]["rel_mse"] / out["voxel"]["rel_mse"]
    out["best_mlp_over_best_voxel"] = best_mlp / best_vox
    out["epsilon"] = 1e-2
    out["s"] = time.perf_counter() - t0
    return out


def ref_gpu_extra(device: int, size=(256, 256), spp: int = 256) -> dict:
    """The reference's own GPU renderer (its RenderCamera megakernel built for
    sm_103a with its own -use_fast_math -maxrregcount=168 flags, oracle/_ref/
    ref_gpu) against ours on the reference's Cornell box (SceneHelper::
    CreateCornellBox; camera (0, 0, 1.1) looking down -z, FOV 60, the
    reference's path depth), plain method (no guide), `spp` frames each:
    Msamples/s of both (the reference: wall time of its per-frame Render calls,
    which synchronise the device; ours: device time of one ar_render) and the
    rel-MSE between the two converged images.  The reference draws from curand
    streams and ours from PCG32 streams, so the images agree statistically;
    the rel-MSE of two of our own renders on disjoint streams is the noise
    floor to compare with."""
    import subprocess
    import tempfile
    from aperturerendererv3_gb300 import SceneRenderer, configs
    exe = ROOT / "oracle" / "_ref" / "ref_gpu"
    if not exe.exists():
        return {"unavailable": "the reference GPU renderer was not built (no reference sources in this checkout)"}
    cam = configs.REFERENCE_CORNELL_CAMERA
    with tempfile.TemporaryDirectory() as td:
        out = Path(td) / "hdr.bin"
        env = dict(os.environ)
        env["CUDA_VISIBLE_DEVICES"] = env.get("CUDA_VISIBLE_DEVICES", str(device))
        r = subprocess.run([str(exe), str(out), str(size[0]), str(size[1]), str(spp), "0"], capture_output=True,
                           text=True, env=env, timeout=600)
        if r.returncode != 0:
            return {"error": f"reference GPU renderer exited {r.returncode}: {r.stderr.strip()[-300:]}"}
        # the reference reports CUDA errors on stdout (CHECK_ERROR, core/vector.cuh:22) and carries on
        if "CUDA ERROR" in r.stdout:
            return {"error": "reference GPU renderer: " + r.stdout[r.stdout.index("CUDA ERROR"):][:200]}
        ref_stats = json.loads(r.stdout.strip().splitlines()[-1])
        ref_img = np.fromfile(out, np.float32).reshape(size[1], size[0], 3).astype(np.float64)
    ours = SceneRenderer(configs.reference_cornell(), device=device)
    kw = dict(fov=cam["fov"], max_depth=1000)
    ours.Render(size, cam["origin"], cam["direction"], 16, first_frame=1 << 22, **kw)  # warm-up
    img = ours.Render(size, cam["origin"], cam["direction"], spp, **kw)
    ms = ours.last_render_stats()[0]
    img2 = ours.Render(size, cam["origin"], cam["direction"], spp, first_frame=1 << 21, **kw)
    ours_rate = size[0] * size[1] * spp / (ms / 1e3) / 1e6
    return {"workload": f"reference Cornell box (SceneHelper::CreateCornellBox) {size[0]}x{size[1]}, {spp} spp, "
                        "depth up to 1000, plain", "reference_gpu": ref_stats, "ours_msamples_per_s": ours_rate,
            "ours_ms": ms, "speedup": ours_rate / ref_stats["msamples_per_s"],
            "rel_mse_ours_vs_reference": rel_mse(img, ref_img), "rel_mse_ours_vs_ours_noise_floor": rel_mse(img, img2),
            "mean_y": {"ours": float(img[..., 1].mean()), "reference": float(ref_img[..., 1].mean())}}


def adjoint_extra(device: int, steps: int) -> dict:
    """Differentiable-rendering workload: the triangle Cornell box with 8 albedo
    textures of 512^2 RGB texels (U[0.2, 0.8], seed 11) as parameters, target
    rendered from a second texture set (seed 12) at 256 spp, L2 loss at 64 spp,
    256x256, depth 8.  grads/s = texel parameters per second of ar_adjoint;
    central finite differences need two renders per parameter."""
    import torch
    from aperturerendererv3_gb300 import SceneRenderer, configs
    cam = configs.CORNELL_CAMERA
    size, kw = (256, 256), dict(fov=cam["fov"], max_depth=8)
    dev = torch.device("cuda", device)
    objs, mesh, tx = configs.textured_cornell(configs.cornell_textures(512, seed=12))
    rb = SceneRenderer(objs, device=device, mesh=mesh, textures=tx)
    target = torch.empty((256, 256, 3), dtype=torch.float64, device=dev)
    rb.render_into(target, size, cam["origin"], cam["direction"], 256, **kw)
    rb.close()
    objs, mesh, tx = configs.textured_cornell(configs.cornell_textures(512, seed=11))
    r = SceneRenderer(objs, device=device, mesh=mesh, textures=tx)
    img = torch.empty_like(target)
    render_ms, adj_ms = [], []
    grad = torch.empty(r.texel_count(), dtype=torch.float64, device=dev)
    for k in range(steps + 1):
        r.render_into(img, size, cam["origin"], cam["direction"], 64, **kw)
        render_ms.append(r.last_render_stats()[0])
        dl = (2.0 * (img - target)).float()
        r.adjoint(dl, grad, size, cam["origin"], cam["direction"], 64, **kw)
        adj_ms.append(r.last_render_stats()[0])
    render_ms, adj_ms = float(np.mean(render_ms[1:])), float(np.mean(adj_ms[1:]))
    n = r.texel_count()
    adj_gps = n / (adj_ms / 1e3)
    fd_gps = 1.0 / (2.0 * render_ms / 1e3)
    return {"params": n, "adjoint_ms": adj_ms, "render_ms": render_ms, "grads_per_s": adj_gps,
            "fd_grads_per_s": fd_gps, "speedup_vs_fd": adj_gps / fd_gps,
            "loss": float(((img - target) ** 2).sum()), "workload": "textured Cornell 256x256, 64 spp, depth 8"}


def combined_extra(device: int, spp: int = 16) -> dict:
    """The combined workload (terrain + 32-primitive smooth-union SDF + medium,
    3840x2160, depth 24, MLP guide over the voxel guide) at `spp` frames per
    render, and the replay adjoint of the medium's albedo and emission."""
    import torch
    from aperturerendererv3_gb300 import SceneRenderer
    objs, mesh, cam, extra = build_workload("combined")
    r = SceneRenderer(objs, device=device, mesh=mesh, **extra)
    r.build()
    size, depth = (3840, 2160), 24
    kw = dict(fov=cam["fov"], max_depth=depth)
    r.Render(size, cam["origin"], cam["direction"], 2, guide=2, **kw)
    img = r.Render(size, cam["origin"], cam["direction"], spp, guide=2, first_frame=2, **kw)
    ms = r.last_render_stats()[0]
    out = {"value": size[0] * size[1] * spp / (ms / 1e3) / 1e6, "unit": "Msamples/s", "ms": ms, "spp": spp,
           "mlp_steps": r.mlp_stats()[0], "error_word": r.error_word()}
    r.MarkNeedResetGuiding()
    # medium adjoint of a plain render (guided rendering is not differentiated), 4 spp
    plain = r.Render(size, cam["origin"], cam["direction"], 4, **kw)
    target = np.full_like(plain, plain.mean())
    dl = torch.as_tensor(2.0 * (plain - target), device=f"cuda:{device}").float()
    ga, ge = r.adjoint_medium(dl, size, cam["origin"], cam["direction"], 4, **kw)
    out["adjoint_medium"] = {"ms": r.last_render_stats()[0], "spp": 4, "d_albedo": ga, "d_emission": ge}
    r.close()
    return out


def bvh_build_extra(device: int, spp: int = 4) -> dict:
    """The terrain's BVH built on the host (binned SAH) and on the GPU (Morton
    radix tree collapsed to the same 8-wide format): build wall time, node
    count, extend-ray node visits, and the device time of a 1920x1080 render
    through each (same image: hits do not depend on the tree)."""
    from aperturerendererv3_gb300 import SceneRenderer
    objs, mesh, cam, _ = build_workload("terrain")
    kw = dict(fov=cam["fov"], max_depth=16)
    out = {"triangles": int(len(mesh.indices))}
    imgs = []
    for mode in ("host", "gpu"):
        r = SceneRenderer(objs, device=device, mesh=mesh)
        if mode == "gpu":
            r.set_build_mode("gpu")
        r.build()
        build_ms = r.build_time_ms()
        r.Render((1920, 1080), cam["origin"], cam["direction"], 1, **kw)
        imgs.append(r.Render((1920, 1080), cam["origin"], cam["direction"], spp, **kw))
        ms = r.last_render_stats()[0]
        r.Render((1920, 1080), cam["origin"], cam["direction"], 1, profile=2, **kw)
        prof = r.render_profile()
        out[mode] = {"build_ms": build_ms, "nodes": r.stats()["nodes"], "render_ms": ms,
                     "msamples_per_s": 1920 * 1080 * spp / (ms / 1e3) / 1e6,
                     "extend_node_visits_per_ray": prof["extend_node_visits"] / max(1, prof["extend_rays"])}
        if mode == "host":
            out["refit"] = refit_measure(r, mesh, cam, kw, spp)
        r.close()
    out["same_image"] = bool(np.array_equal(imgs[0], imgs[1]))
    out["build_speedup"] = out["host"]["build_ms"] / max(1e-9, out["gpu"]["build_ms"])
    return out


def refit_measure(r, mesh, cam, kw, spp: int, steps: int = 5) -> dict:
    """Refit of the built terrain after its heights are scaled by 1.1 (vertices
    given in device memory): wall time of `refit_mesh` (a device copy of the
    vertices, triangle slots, node boxes level by level, one synchronize), and
    the render through the refitted tree."""
    import torch
    dev = torch.device("cuda", r.device)
    v = torch.as_tensor(np.asarray(mesh.vertices, np.float32), device=dev)
    v[:, 1] *= 1.1
    r.refit_mesh(v)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    for _ in range(steps):
        r.refit_mesh(v)
    torch.cuda.synchronize(dev)
    refit_ms = (time.perf_counter() - t0) * 1e3 / steps
    r.Render((1920, 1080), cam["origin"], cam["direction"], spp, **kw)
    ms = r.last_render_stats()[0]
    r.Render((1920, 1080), cam["origin"], cam["direction"], 1, profile=2, **kw)
    prof = r.render_profile()
    return {"vertices": int(v.shape[0]), "refit_ms": refit_ms, "render_ms": ms,
            "msamples_per_s": 1920 * 1080 * spp / (ms / 1e3) / 1e6,
            "extend_node_visits_per_ray": prof["extend_node_visits"] / max(1, prof["extend_rays"])}


def denoise_extra(r, w, cam, spp: int = 8, steps: int = 5) -> dict:
    """The denoiser on the headline workload's image: a render with and without
    the per-sample G-buffer / moment records (device time of ar_render), the
    bilateral filter of the 1920x1080 result (CUDA events on the launching
    stream, mean over `steps` launches) and the reference's own filter loop on
    the host over a 256 x 256 crop of the same image and records."""
    import torch
    size, kw = w["size"], dict(fov=cam["fov"], max_depth=w["depth"])
    r.Render(size, cam["origin"], cam["direction"], spp, **kw)
    plain_ms = r.last_render_stats()[0]
    img = r.Render(size, cam["origin"], cam["direction"], spp, **kw)
    r.Render(size, cam["origin"], cam["direction"], spp, denoise=True, **kw)
    rec_ms = r.last_render_stats()[0]
    dev = torch.device("cuda", r.device)
    t = torch.as_tensor(img, device=dev)
    for _ in range(2):
        r.denoise(t)
    stream = torch.cuda.current_stream(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize(dev)
    e0.record(stream)
    for _ in range(steps):
        r.denoise(t)
    e1.record(stream)
    torch.cuda.synchronize(dev)
    filt_ms = e0.elapsed_time(e1) / steps
    npix = size[0] * size[1]
    out = {"width": size[0], "height": size[1], "spp": spp, "render_ms": plain_ms, "render_with_records_ms": rec_ms,
           "record_overhead": rec_ms / plain_ms - 1.0, "filter_ms": filt_ms,
           "filter_mpix_per_s": npix / (filt_ms / 1e3) / 1e6,
           "filter_pairs_per_s": npix * 225 / (filt_ms / 1e3), "taps": 225}
    try:
        import time
        from oracle import ref_runner as rr
        if rr.available():
            g, m = r.denoise_records()
            y0, x0, n = size[1] // 2 - 128, size[0] // 2 - 128, 256
            crop = (slice(y0, y0 + n), slice(x0, x0 + n))
            t0 = time.perf_counter()
            rr.denoise(img[crop], g[crop], m[crop])
            cpu_s = time.perf_counter() - t0
            out["cpu_reference"] = {"mpix_per_s": n * n / cpu_s / 1e6, "cores": os.cpu_count() or 1,
                                    "sample": "256 x 256 crop of the same image and records",
                                    "kind": "reference"}
    except Exception as e:  # the CPU comparison never hides the GPU numbers
        out["cpu_reference"] = {"error": str(e)}
    return out


def bvh_stress_extra(device: int, steps: int) -> dict:
    """BVH stress workload: 1M random triangles (centroids U[0,1]^3, vertices
    +N(0, 0.005^2)), 1920x1080 primary rays plus one cosine-hemisphere bounce ray
    per hit, closest hit through ar_trace_closest; Mrays/s of device time."""
    import torch
    from aperturerendererv3_gb300 import SceneRenderer, configs
    from aperturerendererv3_gb300.scene import SceneObject, Material, TriangleMesh
    tris = configs.random_triangles(1_000_000, seed=1)
    v = tris.reshape(-1, 3)
    mesh = TriangleMesh(v, np.arange(len(v), dtype=np.uint32).reshape(-1, 3), np.zeros(len(tris), np.int32),
                        [Material.CreateDiffusePureColor((0.5, 0.5, 0.5))])
    r = SceneRenderer([], device=device, mesh=mesh)
    r.build()
    cam = configs.BVH_STRESS_CAMERA
    dev = torch.device("cuda", device)
    prim = torch.as_tensor(configs.pinhole_rays(1920, 1080, cam["origin"], cam["direction"], cam["fov"]), device=dev)
    ids, t = r.trace_closest(prim)
    # one cosine bounce per hit, about the geometric normal facing the ray
    hit = ids >= 0
    tri = torch.as_tensor(tris, device=dev)[ids[hit].long()].view(-1, 3, 3)
    n = torch.linalg.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0])
    n = n / n.norm(dim=1, keepdim=True).clamp_min(1e-30)
    d0 = prim[hit, 4:7]
    n = torch.where((n * d0).sum(1, keepdim=True) > 0, -n, n)
    p = prim[hit, 0:3] + d0 * t[hit, None]
    g = torch.Generator(device=dev).manual_seed(2)
    u1, u2 = torch.rand(len(n), device=dev, generator=g), torch.rand(len(n), device=dev, generator=g)
    a = torch.where(n[:, 2:3].abs() < 0.999, torch.tensor([0.0, 0.0, 1.0], device=dev),
                    torch.tensor([1.0, 0.0, 0.0], device=dev))
    tt = torch.linalg.cross(a, n)
    tt = tt / tt.norm(dim=1, keepdim=True)
    bb = torch.linalg.cross(n, tt)
    rr_, ph = torch.sqrt(u1), 2 * np.pi * u2
    d1 = tt * (rr_ * torch.cos(ph))[:, None] + bb * (rr_ * torch.sin(ph))[:, None] + n * torch.sqrt(1 - u1)[:, None]
    bounce = torch.cat([p, torch.full((len(n), 1), 1e-4, device=dev), d1,
                        torch.full((len(n), 1), float("inf"), device=dev)], 1).float().contiguous()
    stream = torch.cuda.current_stream(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for _ in range(2):
        r.trace_closest(prim)
        r.trace_closest(bounce)
    torch.cuda.synchronize(dev)
    e0.record(stream)
    for _ in range(steps):
        r.trace_closest(prim)
        r.trace_closest(bounce)
    e1.record(stream)
    torch.cuda.synchronize(dev)
    ms = e0.elapsed_time(e1) / steps
    nrays = len(prim) + len(bounce)
    return {"value": nrays / (ms / 1e3) / 1e6, "unit": "Mrays/s", "ms_per_step": ms, "primary_rays": len(prim),
            "bounce_rays": len(bounce), "hit_fraction": float(hit.float().mean())}


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--workload", default="terrain", choices=sorted(WORKLOADS))
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--size", default=None, help="WxH override (small profiling cases)")
    ap.add_argument("--spp", type=int, default=None, help="samples per pixel override")
    ap.add_argument("--guide", type=int, default=0, choices=[0, 1, 2], help="1: voxel path guide, 2: MLP guide")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the guided, adjoint and BVH-stress measurements reported beside the headline")
    ap.add_argument("--extras", default=None,
                    help="comma-separated subset of the extras to run (guided_voxel, guide_compare, ref_gpu, adjoint, "
                         "combined, bvh_stress, denoise, bvh_build); default: all")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    w = dict(WORKLOADS[args.workload])
    if args.size:
        w["size"] = tuple(int(x) for x in args.size.lower().split("x"))
    if args.spp:
        w["spp"] = args.spp
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        if rank == 0:
            try:
                print(json.dumps(run_reference(args, w)))
            except Exception as e:
                print(json.dumps({"impl": "reference", "unavailable": f"reference CPU oracle failed: {e}"}))
        return

    import torch
    import torch.distributed as dist
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    from aperturerendererv3_gb300 import SceneRenderer
    from aperturerendererv3_gb300._lib import ArRenderParams

    objs, mesh, cam, extra_args = build_workload(args.workload)
    r = SceneRenderer(objs, device=local, mesh=mesh, **extra_args)
    if "guide" in w and args.guide == 0:
        args.guide = w["guide"]
    r.build()
    size, spp, depth = w["size"], w["spp"], w["depth"]
    samples = size[0] * size[1] * spp

    def step(k: int):
        return r.Render(size, cam["origin"], cam["direction"], spp, fov=cam["fov"], max_depth=depth,
                        first_frame=(k * world + rank) * spp, guide=args.guide)

    for k in range(args.warmup):
        step(k)
    sampler = ClockSampler(local)
    sampler.start()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    dev_ms, launches = 0.0, 0
    t0 = time.perf_counter()
    for k in range(args.steps):
        step(args.warmup + k)
        ms, L = r.last_render_stats()
        dev_ms += ms
        launches += L
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    wall = time.perf_counter() - t0
    clocks = sampler.stop()
    t = torch.tensor([dev_ms, wall], dtype=torch.float64, device="cuda")
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dev_ms, wall = float(t[0]), float(t[1])
    total = samples * args.steps * world
    value = total / (dev_ms / 1e3) / 1e6
    e2e = total / wall / 1e6

    # profiled renders (outside the timed region) of the same step: stage times
    # from events only, then traversal counters in a second pass (the counters'
    # atomics would distort the times)
    probe_frame = (args.warmup + args.steps) * world * spp
    r.Render(size, cam["origin"], cam["direction"], spp, fov=cam["fov"], max_depth=depth, first_frame=probe_frame,
             profile=1, guide=args.guide)
    prof = r.render_profile()
    r.Render(size, cam["origin"], cam["direction"], spp, fov=cam["fov"], max_depth=depth, first_frame=probe_frame,
             profile=2, guide=args.guide)
    counters = r.render_profile()
    for k in ("extend_rays", "extend_node_visits", "extend_prim_tests", "shadow_rays", "shadow_node_visits",
              "shadow_prim_tests"):
        prof[k] = counters[k]
    # algorithmic bytes of the step's closest-hit traversal: the work a binary SAH
    # BVH needs for the same rays (frozen per ray by the reference oracle:
    # profiles/traversal_work_<workload>.json), so the figure does not move when
    # this project's node layout or traversal changes
    work = traversal_work(args.workload)
    cam_rays = samples
    bounce_rays = max(0, prof["extend_rays"] - cam_rays)
    if work is not None:
        alg_bytes = cam_rays * work["camera"]["bytes"] + bounce_rays * work["bounce"]["bytes"]
        alg_def = ("binary SAH BVH work per ray frozen by the reference oracle (" + work["definition"] + "): camera "
                   f"{work['camera']['bytes']:.1f} B x {cam_rays} rays + bounce {work['bounce']['bytes']:.1f} B x "
                   f"{bounce_rays} rays")
    else:  # workloads without a frozen figure: this BVH's own work
        node_b, slot_b, ray_io_b = 80, 48, 16 + 16 + 4 + 4 + 16 + 4 + 4
        alg_bytes = (prof["extend_node_visits"] * node_b + prof["extend_prim_tests"] * slot_b +
                     prof["extend_rays"] * ray_io_b)
        alg_def = "this BVH: 80 B x node visits + 48 B x primitive slots tested + 64 B ray state per ray"
    launches_ext = max(1, prof["extend_launches"])
    achieved = alg_bytes / (prof["extend_ms"] / 1e3) / 1e9
    peaks = measured_peaks()
    per_ray = profile_traffic(args.workload)
    # DRAM bytes per k_extend launch: the capture's bytes per ray, scaled by the
    # step's rays (an upper bound: a full-size launch shares the BVH among more rays)
    traffic = (None if per_ray is None else
               (cam_rays * per_ray["camera_bytes_per_ray"] + bounce_rays * per_ray["bounce_bytes_per_ray"]) / launches_ext)
    own_bytes = prof["extend_node_visits"] * 80 + prof["extend_prim_tests"] * 48 + prof["extend_rays"] * 64
    out = {
        "metric": "Msamples/s", "value": value, "unit": "Msamples/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dev_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded scene generator)",
        "config": {"workload": args.workload, "width": size[0], "height": size[1], "spp": spp, "max_depth": depth,
                   "guide": ["none", "voxel", "mlp"][args.guide], "paths_per_step": samples, "parallelism": "replicas" if world > 1 else "single-gpu",
                   "l2": "inputs larger than L2 (path state ~170 B x 33.5M paths in flight)"},
        # per step the call reads its render parameters from host memory and copies
        # the FP64 mean image back; the scene stays resident
        "e2e": {"value": e2e, "unit": "Msamples/s", "h2d_bytes_per_step": ctypes.sizeof(ArRenderParams),
                "d2h_bytes_per_step": size[0] * size[1] * 3 * 8},
        "gpu_launches": launches,
        "clocks": clocks,
        "roofline": {"kernel": "k_extend (closest-hit wide-BVH traversal)", "bound": "hbm",
                     "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": achieved / peaks["hbm_gbs"], "peak_source": peaks["source"],
                     "traffic": traffic,
                     "alg_bytes_per_launch": alg_bytes / launches_ext,
                     "alg_bytes_def": alg_def,
                     "this_bvh_bytes_per_launch": own_bytes / launches_ext,
                     "limiter": limiter_summary(args.workload)},
        "stages_ms": {k: prof[k] for k in ("raygen_ms", "extend_ms", "shade_ms", "shadow_ms", "finalize_ms")},
        "traversal": {k: prof[k] for k in ("extend_rays", "extend_node_visits", "extend_prim_tests", "shadow_rays",
                                           "shadow_node_visits", "shadow_prim_tests")},
    }
    if not args.no_extras:
        extras = {}
        for name, fn in (("guided_voxel", lambda: guided_extra(r, w, cam, 3)),
                         ("guide_compare", lambda: guide_compare_extra(r, w, cam, objs, mesh)),
                         ("ref_gpu", lambda: ref_gpu_extra(local)),
                         ("adjoint", lambda: adjoint_extra(local, 3)),
                         ("combined", lambda: combined_extra(local) if args.workload != "combined" else
                          {"note": "the headline is the combined workload"}),
                         ("bvh_stress", lambda: bvh_stress_extra(local, 5)),
                         ("denoise", lambda: denoise_extra(r, w, cam)),
                         ("bvh_build", lambda: bvh_build_extra(local))):
            if args.extras and name not in args.extras.split(","):
                continue
            try:
                extras[name] = fn()
            except Exception as e:  # an extra never hides the headline
                extras[name] = {"error": str(e)}
        out["extras"] = extras
    if rank == 0 and not args.no_cpu_baseline:
        try:
            threads = os.cpu_count() or 1
            sample_size, sample_spp = reference_sample(args.workload, size)
            st, _ = cpu_reference_run(args.workload, objs, mesh, cam, w, sample_spp, sample_size, threads)
            out["cpu_baseline"] = {"value": st["msamples_per_s"], "unit": "Msamples/s", "cores": st["threads"],
                                   "kind": "reference",
                                   "sample": f"{sample_size[0]}x{sample_size[1]}x{sample_spp} spp, same scene"}
        except Exception as e:
            out["cpu_baseline"] = {"value": None, "unit": "Msamples/s", "cores": 0, "kind": "reference",
                                   "sample": f"unavailable: {e}"}
    if rank == 0:
        print(json.dumps(out))
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
