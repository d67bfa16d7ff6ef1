"""Sharded rendering across ranks (host logic, CPU): frame blocks cover the
sample range exactly once, and the all-reduced image and adjoint gradients of
a two-rank gloo group equal a single process's.  A deterministic stand-in
renderer replaces the GPU renderer (its frame images and gradients depend only
on the frame indices, like the real one's random streams)."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from aperturerendererv3_gb300.sharding import adjoint_sharded, render_sharded, shard_frames


class FrameRenderer:
    """Image of frame f: a fixed pattern scaled by a function of f; texel
    gradient: sum over frames of the loss gradient times frame weights."""

    def __init__(self, n_texels: int = 7):
        self.n = n_texels

    @staticmethod
    def _frame(f, h, w):
        base = np.arange(h * w * 3, dtype=np.float64).reshape(h, w, 3)
        return np.sin(0.37 * f + 0.011 * base) + 1.5

    def Render(self, size, origin, direction, spp, first_frame=0, **kw):
        w, h = size
        acc = np.zeros((h, w, 3))
        for f in range(first_frame, first_frame + spp):
            acc += self._frame(f, h, w)
        return acc / spp

    def texel_count(self):
        return self.n

    def adjoint(self, dl, grad, size, origin, direction, spp, first_frame=0, **kw):
        w, h = size
        g = torch.zeros(self.n, dtype=torch.float64)
        for f in range(first_frame, first_frame + spp):
            img = torch.from_numpy(self._frame(f, h, w))
            g += (dl.double() * img).sum() * torch.linspace(1.0, 2.0, self.n, dtype=torch.float64) / spp
        grad.copy_(g)


@pytest.mark.parametrize("spp,world", [(16, 2), (7, 2), (5, 3), (1, 2), (64, 4)])
def test_frame_blocks_cover_the_range_once(spp, world):
    seen = []
    for r in range(world):
        first, count = shard_frames(spp, r, world)
        seen += list(range(first, first + count))
    assert seen == list(range(spp))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, spp, out_dir):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r = FrameRenderer()
        size = (6, 4)
        img = render_sharded(r, size, (0, 0, 0), (0, 0, -1), spp, first_frame=3)
        dl = torch.from_numpy(np.cos(np.arange(6 * 4 * 3, dtype=np.float64)).reshape(4, 6, 3))
        g = adjoint_sharded(r, dl, size, (0, 0, 0), (0, 0, -1), spp, first_frame=3)
        np.save(os.path.join(out_dir, f"img{rank}.npy"), img)
        np.save(os.path.join(out_dir, f"grad{rank}.npy"), g.numpy())
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("spp", [9, 16])
def test_two_rank_gloo_group_matches_one_process(tmp_path, spp):
    world = 2
    mp.spawn(_worker, args=(world, _free_port(), spp, str(tmp_path)), nprocs=world, join=True)
    r = FrameRenderer()
    ref = r.Render((6, 4), None, None, spp, first_frame=3)
    dl = torch.from_numpy(np.cos(np.arange(6 * 4 * 3, dtype=np.float64)).reshape(4, 6, 3))
    gref = torch.zeros(r.n, dtype=torch.float64)
    r.adjoint(dl, gref, (6, 4), None, None, spp, first_frame=3)
    for rank in range(world):
        img = np.load(tmp_path / f"img{rank}.npy")
        g = np.load(tmp_path / f"grad{rank}.npy")
        assert np.allclose(img, ref, rtol=1e-12, atol=1e-12)
        assert np.allclose(g, gref.numpy(), rtol=1e-12, atol=1e-12)
