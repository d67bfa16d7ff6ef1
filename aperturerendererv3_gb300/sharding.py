"""Rendering sharded across processes (one per GPU).

Pixels and samples are independent, so a render splits by sample range: rank r
of W renders a contiguous block of frames (`first_frame` offsets keep every
sample's random stream the one a single process would use) and the ranks'
FP64 per-pixel sums meet in one all-reduce.  The replay adjoint splits the same
way and sums its FP64 gradients.  No other data crosses ranks: the scene, BVH
and LUTs are replicated.

Works with any torch.distributed backend: NCCL over the GPUs' own memory, or
gloo on host tensors.
"""
from __future__ import annotations

import numpy as np


def shard_frames(spp: int, rank: int, world: int) -> tuple[int, int]:
    """(first frame, frame count) of `rank`'s block of `spp` frames."""
    base, extra = divmod(int(spp), int(world))
    first = rank * base + min(rank, extra)
    return first, base + (1 if rank < extra else 0)


def _collective_device(group):
    import torch
    import torch.distributed as dist
    return torch.device("cuda", torch.cuda.current_device()) if dist.get_backend(group) == "nccl" else torch.device("cpu")


def render_sharded(renderer, size, origin, direction, spp: int, group=None, first_frame: int = 0, **kw) -> np.ndarray:
    """Per-pixel mean XYZ of `spp` frames rendered across the group's ranks;
    every rank returns the whole image."""
    import torch
    import torch.distributed as dist
    rank, world = dist.get_rank(group), dist.get_world_size(group)
    first, count = shard_frames(spp, rank, world)
    w, h = int(size[0]), int(size[1])
    sums = np.zeros((h, w, 3), np.float64)
    if count > 0:
        sums = renderer.Render(size, origin, direction, count, first_frame=first_frame + first, **kw) * count
    t = torch.from_numpy(np.ascontiguousarray(sums)).to(_collective_device(group))
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return (t.cpu().numpy() / float(spp)).astype(np.float64)


def adjoint_sharded(renderer, dl_dxyz, size, origin, direction, spp: int, group=None, first_frame: int = 0, **kw):
    """d(loss)/d(texels) for a render of `spp` frames split across the group's
    ranks (float64, on the renderer's device).  dl_dxyz is d(loss)/d(mean image)
    of the whole render; each rank's slice carries weight count / spp."""
    import torch
    import torch.distributed as dist
    rank, world = dist.get_rank(group), dist.get_world_size(group)
    first, count = shard_frames(spp, rank, world)
    n = renderer.texel_count()
    dev = dl_dxyz.device
    grad = torch.zeros(n, dtype=torch.float64, device=dev)
    if count > 0:
        renderer.adjoint(dl_dxyz * (count / spp), grad, size, origin, direction, count,
                         first_frame=first_frame + first, **kw)
    coll = _collective_device(group)
    g = grad.to(coll)
    dist.all_reduce(g, op=dist.ReduceOp.SUM, group=group)
    return g.to(dev)
