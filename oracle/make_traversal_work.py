"""Freezes the algorithmic traversal work of the terrain workload:
profiles/traversal_work_terrain.json.

TEST / MEASUREMENT INFRASTRUCTURE: runs the reference oracle (oracle/_ref) once;
bench.py reads only the JSON it writes.

The work is what a binary SAH BVH needs, independent of this project's node
layout: the reference's BuildBVH tree (core/bvh/bvh.cuh:142-422) over the
terrain's 8,380,418 triangles, walked near-first as TraverseBVH does
(core/render/intersection.cuh:148-283) with a slab test that also requires
tEnter <= tExit (ref_runner.trace_count).  Ray sample: the camera rays of every
8th pixel in x and y of the 1920 x 1080 view (pixel centres) and one cosine
bounce ray per camera hit (tests/golden/bvh_stress_rays.bounce_rays).  Bytes
per ray = 32 B x nodes popped + 48 B x triangles tested + 8 B hit record.

    python oracle/make_traversal_work.py
"""
from __future__ import annotations

import json
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests" / "golden"))

NODE_BYTES, TRI_BYTES, HIT_BYTES = 32, 48, 8
STRIDE = 8


def main() -> None:
    from aperturerendererv3_gb300 import configs
    from oracle import ref_runner as rr
    import bvh_stress_rays as bs
    objs, mesh = configs.terrain_scene()
    tris = mesh.triangle_vertices()
    cam = configs.TERRAIN_CAMERA
    W, H = 1920, 1080
    rays = configs.pinhole_rays(W, H, cam["origin"], cam["direction"], cam["fov"]).reshape(H, W, 8)
    cam_rays = np.ascontiguousarray(rays[STRIDE // 2::STRIDE, STRIDE // 2::STRIDE].reshape(-1, 8))
    t0 = time.time()
    ids, t, v, n, st = rr.trace_count(tris, cam_rays)
    bounce = bs.bounce_rays(tris, cam_rays, ids, t, seed=5)
    bids, bt, bv, bn, bst = rr.trace_count(tris, bounce)

    def per_ray(visits, tests, hits):
        return {"rays": int(len(visits)), "node_pops": float(visits.mean()), "tri_tests": float(tests.mean()),
                "hit_fraction": float(hits.mean()),
                "bytes": float(NODE_BYTES * visits.mean() + TRI_BYTES * tests.mean() + HIT_BYTES)}

    out = {
        "workload": "terrain 2048^2 heightfield (8,380,418 triangles; sphere lights and sun left out), camera "
                    "1920x1080 fov %g, every %dth pixel in x and y, one cosine bounce per camera hit" % (cam["fov"], STRIDE),
        "definition": "binary SAH BVH of the reference's BuildBVH (leaf 8, 12 bins), near-first traversal with a "
                      "tEnter <= tExit slab test; bytes per ray = 32 B x nodes popped + 48 B x triangles tested + "
                      "8 B hit record",
        "camera": per_ray(v, n, ids >= 0),
        "bounce": per_ray(bv, bn, bids >= 0),
        "bvh_nodes": st.get("nodes"),
        "oracle_s": round(time.time() - t0, 1),
    }
    dst = ROOT / "profiles" / "traversal_work_terrain.json"
    dst.write_text(json.dumps(out, indent=1) + "\n")
    print("wrote", dst, json.dumps(out))


if __name__ == "__main__":
    main()
