"""Writes tests/golden/bvh_stress_1m.json: the reference BVH's closest hits
(BuildBVH + intersection::TraverseBVH, core/bvh/bvh.cuh:142-422,
core/render/intersection.cuh:148-283, run by the reference oracle oracle/_ref)
for the full BVH stress workload -- 1M random triangles, all 1920x1080 primary
rays and one cosine bounce ray per primary hit (bvh_stress_rays.py) -- as
per-block SHA-256 digests of (ids, t) plus hit counts and a sample of rays
with their hits.  The reference traversal takes about an hour of 8 CPU cores
here, hence a committed digest instead of a live check.

    python tests/golden/make_bvh_stress_fixture.py
"""
from __future__ import annotations

import json
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))
sys.path.insert(0, str(HERE))

import bvh_stress_rays as bs  # noqa: E402
from oracle import ref_runner as rr  # noqa: E402


def main() -> None:
    tris = bs.triangles()
    prim = bs.primary_rays()
    t0 = time.time()
    ids, t, st = rr.trace(tris, prim)
    t1 = time.time()
    bounce = bs.bounce_rays(tris, prim, ids, t)
    bids, bt, bst = rr.trace(tris, bounce)
    t2 = time.time()
    rng = np.random.default_rng(9)
    ps = np.sort(rng.choice(len(prim), 64, replace=False))
    bsel = np.sort(rng.choice(len(bounce), 64, replace=False))
    out = {
        "workload": "1M random triangles (seed 1), 1920x1080 primary rays + one cosine bounce per hit",
        "primary": {"rays": len(prim), "hits": int((ids >= 0).sum()), "blocks": bs.block_hashes(ids, t),
                    "sample_index": ps.tolist(), "sample_ids": ids[ps].tolist(),
                    "sample_t_bits": t[ps].view(np.uint32).tolist()},
        "bounce": {"rays": len(bounce), "hits": int((bids >= 0).sum()), "blocks": bs.block_hashes(bids, bt),
                   "sample_index": bsel.tolist(), "sample_ids": bids[bsel].tolist(),
                   "sample_t_bits": bt[bsel].view(np.uint32).tolist()},
        "oracle": {"primary_s": round(t1 - t0, 1), "bounce_s": round(t2 - t1, 1), "threads": st.get("threads"),
                   "nodes": st.get("nodes"), "primary_node_visits": st.get("node_visits"),
                   "primary_prim_tests": st.get("prim_tests"), "bounce_node_visits": bst.get("node_visits"),
                   "bounce_prim_tests": bst.get("prim_tests")},
    }
    (HERE / "bvh_stress_1m.json").write_text(json.dumps(out, indent=1))
    print("wrote", HERE / "bvh_stress_1m.json", out["oracle"])


if __name__ == "__main__":
    main()
