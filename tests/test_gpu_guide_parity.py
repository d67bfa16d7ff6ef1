"""Voxel-guided rendering on the GPU against the reference's own guided
integrator, run by the reference oracle (oracle/_ref) over the same probe set:

* per-sample radiance of a guided frame equals CalculateRadiance<true, NEE,
  true> (core/render/render.cuh:460-999: probe query :434-458, guided mixture
  :553-638, NEE / guide MIS :320-340) within 1e-5 relative, on the same random
  streams and frame index;
* the frame's radiance records (k_shade<1> + k_guide_emit) equal the
  reference's per-path records (CollectRadiance and the record loop,
  core/render/render.cuh:353-432, 909-963) as a multiset;
* the probe update that follows (k_pg_claim / k_pg_accumulate / k_pg_merge)
  equals the reference's UpdatePathGuidingSample arithmetic
  (core/scene.cu:409-570: AccumulateSamplesToOctaLeafKernel, MergeProbeKernel,
  GenerateMipmaps, core/guiding/guiding.cuh:373-517) over the same records, up
  to the order of the float atomic additions into each leaf texel.

The probe set is the one the GPU learned over the first frames; it is read out
with ar_guide_read and handed to the oracle as the reference's index volume and
probe array (SCENE_PROBES / INDIRECT_INDEX_VOLUME)."""
import numpy as np
import pytest

from aperturerendererv3_gb300 import SceneRenderer, configs
from oracle import ref_runner as rr

pytestmark = pytest.mark.gpu

FRAME = 40  # guiding probability ramps with the frame index (core/render/render.cuh:198-203)


@pytest.fixture(scope="module")
def ref_available():
    if not rr.available():
        pytest.skip("reference oracle not built in this checkout")


def scenes():
    objs, mesh = configs.terrain_scene(res=96, n_spheres=8, seed=7)
    return [("reference_cornell", configs.reference_cornell(), None, configs.REFERENCE_CORNELL_CAMERA, (40, 40)),
            ("terrain_small", objs, mesh, configs.TERRAIN_CAMERA, (48, 27))]


def _sorted_records(keys, dirs, rad):
    order = np.lexsort((np.round(dirs[:, 2], 4), np.round(dirs[:, 1], 4), np.round(dirs[:, 0], 4),
                        keys[:, 3], keys[:, 2], keys[:, 1], keys[:, 0]))
    return keys[order], dirs[order], rad[order]


def _by_key(p):
    return {tuple(k): i for i, k in enumerate(p["keys"])}


@pytest.mark.parametrize("name,objs,mesh,cam,size", scenes())
def test_guided_frame_matches_reference_integrator(cuda_device, ref_available, name, objs, mesh, cam, size):
    r = SceneRenderer(objs, mesh=mesh)
    r.Render(size, cam["origin"], cam["direction"], 8, fov=cam["fov"], max_depth=16, guide=1)  # learn
    probes = r.guide_probes()
    assert len(probes["keys"]) > 20
    _, per = r.Render(size, cam["origin"], cam["direction"], 1, fov=cam["fov"], max_depth=16, guide=1,
                      first_frame=FRAME, per_sample=True)
    recs = r.guide_records()
    after = r.guide_probes()
    assert r.error_word() == 0

    _, rper, st = rr.render(objs, size, cam["origin"], cam["direction"], 1, fov=cam["fov"], max_depth=16,
                            first_frame=FRAME, per_sample_frames=1, mesh=mesh, guide_probes=probes)
    # (1) per-sample radiance of the guided frame
    ref = rper.astype(np.float64)
    err = np.abs(per.astype(np.float64) - ref)
    ok = err <= 1e-5 * np.abs(ref) + 1e-6
    assert ok.all(), f"{int((~ok).sum())} of {ok.size} sample channels differ; worst {err.max()}"

    # (2) the frame's radiance records, as a multiset
    rrec = st["records"].reshape(-1)
    rrec = rrec[rrec["valid"] == 1]
    assert len(rrec) == len(recs["keys"]) > 0
    gk, gd, gr = _sorted_records(recs["keys"], recs["dirs"], recs["radiance"])
    rk, rd, rad = _sorted_records(rrec["key"], rrec["dir"], rrec["radiance"])
    assert np.array_equal(gk, rk)
    np.testing.assert_allclose(gd, rd, rtol=0, atol=1e-6)
    np.testing.assert_allclose(gr, rad, rtol=1e-5, atol=1e-9)

    # (3) the probe update after the frame, over the GPU's records
    ref_after = rr.guide_update(probes, recs["keys"], recs["dirs"], recs["radiance"])
    ga, ra = _by_key(after), _by_key(ref_after)
    assert ga.keys() == ra.keys()
    gi = np.array([ga[k] for k in ra])
    ri = np.array(list(ra.values()))
    assert np.array_equal(after["counts"][gi], ref_after["counts"][ri])
    # float atomics add a texel's records in any order: a few ulps of the leaf sums
    np.testing.assert_allclose(after["texels"][gi], ref_after["texels"][ri], rtol=2e-5, atol=1e-12)


def test_probe_set_round_trip(cuda_device):
    """ar_guide_write then ar_guide_read returns the same probes, and a guided
    frame over written probes equals one over the learned originals."""
    objs, cam = configs.reference_cornell(), configs.REFERENCE_CORNELL_CAMERA
    size = (32, 32)
    r = SceneRenderer(objs)
    r.Render(size, cam["origin"], cam["direction"], 4, fov=cam["fov"], max_depth=16, guide=1)
    p = r.guide_probes()
    _, a = r.Render(size, cam["origin"], cam["direction"], 1, fov=cam["fov"], max_depth=16, guide=1,
                    first_frame=FRAME, per_sample=True)
    r2 = SceneRenderer(objs)
    r2.set_guide_probes(p["keys"], p["texels"], p["counts"])
    q = r2.guide_probes()
    assert np.array_equal(q["keys"], p["keys"]) and np.array_equal(q["counts"], p["counts"])
    assert np.array_equal(q["texels"], p["texels"])
    _, b = r2.Render(size, cam["origin"], cam["direction"], 1, fov=cam["fov"], max_depth=16, guide=1,
                     first_frame=FRAME, per_sample=True)
    assert np.array_equal(a, b)
