"""FP64 CPU oracle of the MLP path guide's network (forward, loss, backward).

TEST INFRASTRUCTURE ONLY.  The network is the one the GPU trains
(aperturerendererv3_gb300/csrc/ar_mlp.h): a 12-band sin/cos encoding of six
inputs in [0, 1] (144 features), then 144 -> 64 -> 64 -> 64 -> 64 -> 64 with
ReLU between layers; loss per record Y (logsumexp(y) - y_cell), the
radiance-weighted cross-entropy of the record direction's cell under the
softmax of the outputs, averaged over the records.  `cell` is the 8 x 8 cell of the equal-area sphere
map the voxel probes use (core/guiding/octahedron.cuh:87-145, restated here).

With bf16=True the oracle rounds where the tensor-core kernels hold bf16
operands (weights, encoded inputs, hidden activations, layer gradients) and
computes everything else in float64; with bf16=False it is the exact FP64
network.
"""
from __future__ import annotations

import numpy as np

IN, H, OUT, BANDS = 144, 64, 64, 12
DIMS = [IN, H, H, H, H]
PARAMS = 25920


def offsets():
    w, b, o = [], [], 0
    for ind in DIMS:
        w.append(o)
        o += 64 * ind
        b.append(o)
        o += 64
    assert o == PARAMS
    return w, b


W_OFF, B_OFF = offsets()


def bf16(x):
    """Round to bfloat16 (nearest even) and back to float64."""
    f = np.asarray(x, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(params, round_w):
    p = np.asarray(params, np.float64)
    Ws, bs = [], []
    for l, ind in enumerate(DIMS):
        W = p[W_OFF[l]:W_OFF[l] + 64 * ind].reshape(64, ind)
        Ws.append(bf16(W) if round_w else W)
        bs.append(p[B_OFF[l]:B_OFF[l] + 64])
    return Ws, bs


def encode(in6):
    x = np.asarray(in6, np.float64)
    feats = np.empty((len(x), IN))
    for d in range(6):
        for j in range(BANDS):
            a = np.pi * x[:, d] * (1 << j)
            feats[:, d * 2 * BANDS + 2 * j] = np.sin(a)
            feats[:, d * 2 * BANDS + 2 * j + 1] = np.cos(a)
    return feats


def sphere_to_uv(d):
    d = np.asarray(d, np.float64)
    d = d / np.linalg.norm(d, axis=1, keepdims=True)
    phi2 = np.arctan2(d[:, 1], d[:, 0]) * (2.0 / np.pi)
    u = np.empty(len(d))
    v = np.empty(len(d))
    for k in range(len(d)):
        z, p = d[k, 2], phi2[k]
        if z < 0:
            r = np.sqrt(max(0.0, 1 + z))
            if p >= 0:
                if p <= 1:
                    uu = 1 - r * p
                    vv = 2 - r - uu
                else:
                    uu = r * (2 - p) - 1
                    vv = 2 - r + uu
            else:
                if p >= -1:
                    uu = r * p + 1
                    vv = r - 2 + uu
                else:
                    uu = r * (2 + p) - 1
                    vv = r - 2 - uu
        else:
            r = np.sqrt(max(0.0, 1 - z))
            if p >= 0:
                if p < 1:
                    vv = r * p
                    uu = r - vv
                else:
                    vv = r * (2 - p)
                    uu = vv - r
            else:
                if p > -1:
                    vv = r * p
                    uu = r + vv
                else:
                    vv = -r * (2 + p)
                    uu = -(r + vv)
        u[k] = 0.5 * (uu + 1)
        v[k] = 0.5 * (vv + 1)
    return u, v


def cell(dirs):
    u, v = sphere_to_uv(dirs)
    ix = np.clip(np.floor(u * 8).astype(int), 0, 7)
    iy = np.clip(np.floor(v * 8).astype(int), 0, 7)
    return iy * 8 + ix


def forward(params, in6, bf16_ops=True):
    Ws, bs = unpack(params, bf16_ops)
    r = bf16 if bf16_ops else (lambda a: a)
    h = r(encode(in6))
    acts = [h]
    for l in range(5):
        y = h @ Ws[l].T + bs[l]
        if l < 4:
            h = r(np.maximum(y, 0.0))
            acts.append(h)
    return y, acts


def mirrored_cells(dirs, nrm, c):
    """Cell of each direction mirrored below the surface (-1: none, or the same cell)."""
    d = np.asarray(dirs, np.float64)
    d = d / np.linalg.norm(d, axis=1, keepdims=True)
    nn = np.asarray(nrm, np.float64)
    nn = nn / np.linalg.norm(nn, axis=1, keepdims=True)
    dn = (d * nn).sum(1)
    m = d - 2.0 * dn[:, None] * nn
    cm = cell(m)
    cm[(dn <= 0) | (cm == c)] = -1
    return cm


def loss_and_grad(params, in6, dirs, lum, bf16_ops=True, nrm=None):
    """(logits, loss sum, d mean-loss / d params) in float64.  Loss per record:
    the radiance-weighted cross-entropy Y (logsumexp(y) - y_cell) of the record
    direction's cell under the softmax of the 64 outputs.  `nrm` is accepted for
    the kernels' interface and unused (a zero-radiance record adds nothing)."""
    Ws, bs = unpack(params, bf16_ops)
    r = bf16 if bf16_ops else (lambda a: a)
    y, acts = forward(params, in6, bf16_ops)
    n = len(y)
    c = cell(dirs)
    t = np.maximum(np.asarray(lum, np.float64), 0.0)
    mx = y.max(1, keepdims=True)
    e = np.exp(y - mx)
    se = e.sum(1, keepdims=True)
    lse = (mx + np.log(se))[:, 0]
    loss = float((t * (lse - y[np.arange(n), c]))[t > 0].sum())
    dy = e / se
    dy[np.arange(n), c] -= 1.0
    dy *= (t / n)[:, None]
    grad = np.zeros(PARAMS)
    g = dy
    for l in range(4, -1, -1):
        gr = r(g)
        grad[W_OFF[l]:W_OFF[l] + 64 * DIMS[l]] = (gr.T @ acts[l]).reshape(-1)
        grad[B_OFF[l]:B_OFF[l] + 64] = g.sum(0)
        if l > 0:
            dh = gr @ Ws[l]
            g = dh * (acts[l] > 0)
    return y, loss, grad


def init_params(seed=0):
    """He-initialised weights, zero biases; the output layer starts small so the
    first distributions are near uniform (the renderer's own initialisation)."""
    rng = np.random.default_rng(seed)
    p = np.zeros(PARAMS)
    for l, ind in enumerate(DIMS):
        s = np.sqrt(2.0 / ind) * (0.1 if l == 4 else 1.0)
        p[W_OFF[l]:W_OFF[l] + 64 * ind] = rng.standard_normal(64 * ind) * s
    return p.astype(np.float32)
