"""The BVH stress workload at its stated scale: 1M random triangles
(centroids U[0,1]^3, vertices offset by N(0, 0.005^2)), all 1920 x 1080
primary rays and one cosine-hemisphere bounce ray per primary hit.  The
closest-hit primitive ids and distances of the GPU traversal equal, bit for
bit, those of the reference's BuildBVH + TraverseBVH run by the reference
oracle (committed as per-block SHA-256 digests, tests/golden/bvh_stress_1m.json,
made by tests/golden/make_bvh_stress_fixture.py: the reference traversal takes
about an hour of CPU).  The bounce rays are built from the GPU's own primary
hits with elementwise IEEE operations only (tests/golden/bvh_stress_rays.py),
so they equal the fixture's rays exactly when the primary hits do."""
import json
import sys

import numpy as np
import pytest

from conftest import GOLDEN

sys.path.insert(0, str(GOLDEN))
import bvh_stress_rays as bs  # noqa: E402

pytestmark = pytest.mark.gpu

FIXTURE = GOLDEN / "bvh_stress_1m.json"


def _first_mismatch(got, want):
    for k, (a, b) in enumerate(zip(got, want)):
        if a != b:
            return k
    return None


def test_full_scale_closest_hits_equal_the_reference(cuda_device):
    import torch
    if not FIXTURE.exists():
        pytest.skip("full-scale reference digests not generated in this checkout")
    from test_gpu_trace import mesh_renderer
    fx = json.loads(FIXTURE.read_text())
    tris = bs.triangles()
    prim = bs.primary_rays()
    r = mesh_renderer(tris)
    ids, t = r.trace_closest(torch.from_numpy(prim).cuda())
    ids, t = ids.cpu().numpy(), t.cpu().numpy()
    assert int((ids >= 0).sum()) == fx["primary"]["hits"]
    k = np.asarray(fx["primary"]["sample_index"])
    assert np.array_equal(ids[k], fx["primary"]["sample_ids"])
    assert np.array_equal(t[k].view(np.uint32), np.asarray(fx["primary"]["sample_t_bits"], np.uint32))
    blocks = bs.block_hashes(ids, t)
    assert blocks == fx["primary"]["blocks"], f"primary block {_first_mismatch(blocks, fx['primary']['blocks'])} differs"
    bounce = bs.bounce_rays(tris, prim, ids, t)
    assert len(bounce) == fx["bounce"]["rays"]
    bids, bt = r.trace_closest(torch.from_numpy(bounce).cuda())
    bids, bt = bids.cpu().numpy(), bt.cpu().numpy()
    assert int((bids >= 0).sum()) == fx["bounce"]["hits"]
    blocks = bs.block_hashes(bids, bt)
    assert blocks == fx["bounce"]["blocks"], f"bounce block {_first_mismatch(blocks, fx['bounce']['blocks'])} differs"
    assert r.error_word() == 0
