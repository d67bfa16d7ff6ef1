"""Generates the committed golden fixtures from the reference oracle.

Run in a checkout that has the reference tree (oracle/prepare_ref.py builds
oracle/_ref/ref_cpu from it):

    python tests/golden/make_golden.py

Fixtures:
  spectral_kat.json      the reference's 100 spectral known-answer vectors
                         (inputTest / gtTest, core/spectrum/spectrum_basis.cuh:2472-2489)
                         and the reference encoder's own predictions for them
  spectral_luts.npz      the lambda LUT (840 x 4) and RGB-LUT lattice values at
                         seeded lattice points, computed by the reference code
  trace_small.npz        triangles, rays, and closest-hit ids / t from the
                         reference BVH traversal (ties: smallest id)
  render_*.npz           per-sample XYZ of small renders of the reference's own
                         Cornell box, the triangle Cornell box, a small terrain
                         and the reference's glass test scene (first bounce and
                         full depth) from the reference integrator
                         (`--renders NAME ...` regenerates only those)
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))

from aperturerendererv3_gb300 import configs  # noqa: E402
from oracle import ref_runner as rr  # noqa: E402

RENDERS = {
    "render_refcornell_depth1": ("reference_cornell", 24, 24, 2, 1),
    "render_refcornell_full": ("reference_cornell", 24, 24, 2, 1000),
    "render_cornell_depth1": ("cornell_triangles", 24, 24, 2, 1),
    "render_cornell_depth8": ("cornell_triangles", 24, 24, 2, 8),
    "render_terrain_small_depth16": ("terrain_small", 24, 24, 2, 16),
    "render_glass_depth1": ("glass_cornell", 24, 24, 2, 1),
    "render_glass_full": ("glass_cornell", 32, 32, 4, 1000),
    "render_glass_sky_full": ("glass_test", 24, 24, 4, 1000),
}


def scene_by_name(name):
    """(objects, mesh, camera)"""
    if name == "reference_cornell":
        return configs.reference_cornell(), None, configs.REFERENCE_CORNELL_CAMERA
    if name == "cornell_triangles":
        return configs.cornell_triangles(), None, configs.CORNELL_CAMERA
    if name == "glass_cornell":  # the reference's glass test scene inside its Cornell box
        return configs.reference_cornell() + configs.glass_test_scene(), None, configs.GLASS_TEST_CAMERA
    if name == "glass_test":  # the glass test scene alone, under the sky
        return configs.glass_test_scene(), None, configs.GLASS_TEST_CAMERA
    if name == "terrain_small":
        objs, mesh = configs.terrain_scene(res=48, n_spheres=8, seed=7)
        return objs, mesh, configs.TERRAIN_CAMERA
    raise KeyError(name)


def trace_case(seed: int = 3, ntri: int = 6000, nray: int = 4096):
    tris = configs.random_triangles(ntri, seed=seed)
    cam = configs.BVH_STRESS_CAMERA
    rays = configs.pinhole_rays(64, 64, cam["origin"], cam["direction"], cam["fov"])[:nray]
    return tris, rays


def render_fixtures(names) -> None:
    for name in names:
        scene, w, h, spp, depth = RENDERS[name]
        objs, mesh, cam = scene_by_name(scene)
        mean, per, _ = rr.render(objs, (w, h), cam["origin"], cam["direction"], spp, fov=cam["fov"],
                                 max_depth=depth, per_sample_frames=spp, mesh=mesh)
        np.savez(HERE / f"{name}.npz", per_sample=per, mean=mean, scene=scene, size=(w, h), spp=spp, depth=depth)


def main() -> None:
    if "--renders" in sys.argv:  # only the named render fixtures
        render_fixtures(sys.argv[sys.argv.index("--renders") + 1:])
        return
    k = rr.kat()
    (HERE / "spectral_kat.json").write_text(json.dumps(k))
    rng = np.random.default_rng(11)
    lattice = rng.integers(0, 512, (256, 3)).astype(np.int32)
    lattice[:4] = [[0, 0, 0], [511, 511, 511], [0, 511, 0], [255, 256, 257]]
    lam, rgb = rr.luts(lattice)
    np.savez(HERE / "spectral_luts.npz", lambda_lut=lam, lattice=lattice, rgb_values=rgb)
    tris, rays = trace_case()
    ids, t, _ = rr.trace(tris, rays)
    bids, bt, _ = rr.trace(tris, rays, brute=True)
    assert np.array_equal(ids, bids) and np.array_equal(t.view(np.uint32), bt.view(np.uint32))
    np.savez(HERE / "trace_small.npz", tris=tris, rays=rays, ids=ids, t=t)
    import importlib.util
    spec = importlib.util.spec_from_file_location("tgh", HERE.parent / "test_guide_host.py")
    tgh = importlib.util.module_from_spec(spec)
    sys.path.insert(0, str(HERE.parent))
    spec.loader.exec_module(tgh)
    n = 512
    payload = tgh.make_payload(n, seed=4)
    np.savez(HERE / "guide_probe.npz", n=n, payload=np.frombuffer(payload, np.uint8),
             ref_out=rr.guide_eval(payload, n))
    render_fixtures(RENDERS)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
