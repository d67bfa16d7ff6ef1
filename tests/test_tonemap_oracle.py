"""The reference's display transform compiled into the oracle agrees with the
FP64 restatement (oracle/tonemap64.py) to one 8-bit level: the restatement is
pinned to the reference code it restates."""
import numpy as np
import pytest

from oracle import ref_runner as rr
from oracle import tonemap64


@pytest.mark.parametrize("tone", ["aces", "gamma", "linear"])
def test_reference_tonemap_vs_fp64_restatement(tone):
    if not rr.available():
        pytest.skip("reference oracle not built in this checkout")
    rng = np.random.default_rng(7)
    xyz = rng.gamma(0.7, 0.6, (64, 64, 3)).astype(np.float32)
    xyz[:4] *= 60.0
    ref = rr.tonemap(xyz, 0.8, tone)
    fp64 = tonemap64.tonemap(xyz.astype(np.float64), 0.8, tone)
    d = np.abs(ref.astype(int) - fp64.astype(int))
    assert d.max() <= 1 and (d > 0).mean() < 1e-3
    assert np.all(ref[..., 3] == 255)
