"""Host checks of the per-sample random streams (csrc/ar_rng.h).

The ray generation kernel computes each frame's stream jump once per block
(ar_pcg_jump) and applies it per pixel (ar_pcg_init_jumped).  That must give
the same generator state as ar_pcg_init, which the CPU oracle uses, for every
seed, pixel and frame: checked here with the header compiled by the host
C++ compiler.
"""
import shutil
import subprocess
from pathlib import Path

import pytest

CSRC = Path(__file__).resolve().parents[1] / "aperturerendererv3_gb300" / "csrc"

PROGRAM = r"""
#include <stdio.h>
#include "ar_rng.h"
int main(void)
{
    unsigned long long x = 88172645463325252ull, bad = 0, n = 0;
    for (int i = 0; i < 20000; ++i)
    {
        x ^= x << 13; x ^= x >> 7; x ^= x << 17;
        const uint64_t seed = (i & 1) ? AR_GLOBAL_SEED : x;
        const uint64_t pixel = (x >> 20) % 9000000u;
        const uint64_t frame = (i < 64) ? (uint64_t)i : ((x >> 3) % 70000u);
        uint64_t m, c;
        ar_pcg_jump(frame << 32, &m, &c);
        ar_pcg a = ar_pcg_init(seed, pixel, frame);
        ar_pcg b = ar_pcg_init_jumped(seed, pixel, frame, m, c);
        for (int k = 0; k < 4; ++k)
            if (ar_pcg_next(&a) != ar_pcg_next(&b) || a.state != b.state || a.inc != b.inc) ++bad;
        ++n;
    }
    printf("%llu %llu\n", n, bad);
    return 0;
}
"""


def test_jumped_init_equals_plain_init(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    src = tmp_path / "rng.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "rng"
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", str(CSRC), str(src), "-o", str(exe)], check=True)
    n, bad = map(int, subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split())
    assert n == 20000 and bad == 0
