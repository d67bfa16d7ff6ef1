"""MLP path guide on the tensor cores (tcgen05, BF16 operands, FP32 accumulate).

* The shared-memory descriptors the kernels build give the exact BF16 product
  for every operand arrangement the network uses (K-major / MN-major A and B).
* The inference and training kernels' forward pass, loss and parameter
  gradients match the FP64 CPU oracle (oracle/mlp64.py): tightly when the
  oracle rounds to bf16 where the kernels hold bf16 operands, loosely against
  the exact FP64 network.
"""
import numpy as np
import pytest

from aperturerendererv3_gb300 import _lib
from oracle import mlp64

pytestmark = pytest.mark.gpu


def bf16_bits(x):
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    return ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)


def from_bits(u):
    return (u.astype(np.uint32) << 16).view(np.float32).astype(np.float64)


@pytest.mark.parametrize("a_mn,b_mn,n,k", [(0, 0, 64, 144), (0, 0, 64, 64), (0, 1, 64, 64), (1, 1, 144, 128),
                                           (1, 1, 64, 128)])
def test_tensor_core_descriptors(cuda_device, a_mn, b_mn, n, k):
    rng = np.random.default_rng(n * 1000 + k + 10 * a_mn + b_mn)
    A = bf16_bits(rng.standard_normal((128, k)))
    B = bf16_bits(rng.standard_normal((n, k)))
    ref = from_bits(A) @ from_bits(B).T
    a_in = np.ascontiguousarray(A.T) if a_mn else A
    b_in = np.ascontiguousarray(B.T) if b_mn else B
    d = np.zeros((128, n), np.float32)
    lib = _lib.load()
    assert lib.ar_diag_umma_gemm(0, a_in.ctypes.data, b_in.ctypes.data, a_mn, b_mn, n, k, 0, d.ctypes.data) == 0
    assert np.abs(d - ref).max() <= 1e-5 * np.abs(ref).max()


def run_gpu(params, in6, dirs, lum, nrm=None):
    n = len(in6)
    logits = np.zeros((n, 64), np.float32)
    grad = np.zeros(mlp64.PARAMS, np.float32)
    loss = np.zeros(1, np.float32)
    p = np.ascontiguousarray(params, np.float32)
    x = np.ascontiguousarray(in6, np.float32)
    d = np.ascontiguousarray(dirs, np.float32)
    y = np.ascontiguousarray(lum, np.float32)
    nn = None if nrm is None else np.ascontiguousarray(nrm, np.float32)
    rc = _lib.load().ar_diag_mlp(0, p.ctypes.data, x.ctypes.data, d.ctypes.data, None if nn is None else nn.ctypes.data,
                                 y.ctypes.data, n, logits.ctypes.data, grad.ctypes.data, loss.ctypes.data)
    assert rc == 0
    return logits.astype(np.float64), float(loss[0]), grad.astype(np.float64)


def agg(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)


@pytest.mark.parametrize("n,with_normals", [(300, False), (5000, False), (5000, True)])
def test_forward_backward_against_fp64_oracle(cuda_device, n, with_normals):
    rng = np.random.default_rng(n)
    params = mlp64.init_params(3).astype(np.float64)
    # exercise the biases and a full-scale output layer too
    for l in range(5):
        params[mlp64.B_OFF[l]:mlp64.B_OFF[l] + 64] = rng.normal(0, 0.1, 64)
    w4 = slice(mlp64.W_OFF[4], mlp64.W_OFF[4] + 64 * 64)
    params[w4] *= 10.0
    params = params.astype(np.float32)
    in6 = rng.random((n, 6)).astype(np.float32)
    dirs = rng.standard_normal((n, 3)).astype(np.float32)
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    lum = rng.gamma(0.5, 2.0, n).astype(np.float32)
    nrm = None
    if with_normals:
        # normals on the records' side of the surface, octahedrally quantised as the renderer stores them
        nrm = rng.standard_normal((n, 3))
        nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
        nrm *= np.sign((nrm * dirs).sum(1, keepdims=True) + 1e-12)
        nrm = nrm.astype(np.float32)
    y_gpu, loss_gpu, g_gpu = run_gpu(params, in6, dirs, lum, nrm)
    y_ref, loss_ref, g_ref = mlp64.loss_and_grad(params, in6, dirs, lum, bf16_ops=True, nrm=nrm)
    assert agg(y_gpu, y_ref) < 5e-3, agg(y_gpu, y_ref)
    assert abs(loss_gpu - loss_ref) < 5e-3 * loss_ref
    for l, ind in enumerate(mlp64.DIMS):
        sw = slice(mlp64.W_OFF[l], mlp64.W_OFF[l] + 64 * ind)
        sb = slice(mlp64.B_OFF[l], mlp64.B_OFF[l] + 64)
        assert agg(g_gpu[sw], g_ref[sw]) < 2e-2, (l, agg(g_gpu[sw], g_ref[sw]))
        assert agg(g_gpu[sb], g_ref[sb]) < 2e-2, (l, agg(g_gpu[sb], g_ref[sb]))
    # against the exact FP64 network: bf16 operands cost a few per cent at most
    y64, _, g64 = mlp64.loss_and_grad(params, in6, dirs, lum, bf16_ops=False, nrm=nrm)
    assert agg(y_gpu, y64) < 3e-2
    assert agg(g_gpu, g64) < 1e-1
