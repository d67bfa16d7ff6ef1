"""Host check of the order of a frame's pixels among a wave's paths
(slot_pixel, csrc/ar_internal.h): a bijection of [0, W*H) at every size, and,
when the width is a multiple of 8, every aligned run of 32 slots (one warp)
covers an 8 x 4 pixel tile (where the image has 4 rows left).
"""
import os
import shutil
import subprocess
from pathlib import Path

import pytest

CSRC = Path(__file__).resolve().parents[1] / "aperturerendererv3_gb300" / "csrc"

PROGRAM = r"""
#include <cstdio>
#include <vector>
#include "ar_internal.h"
using namespace ar;

int main()
{
    long long sizes = 0, bad_bij = 0, bad_tile = 0;
    const unsigned Ws[] = {1, 2, 3, 7, 8, 9, 15, 16, 31, 33, 64, 100, 255, 1920, 1921};
    const unsigned Hs[] = {1, 2, 3, 4, 5, 7, 8, 13, 64, 101, 1080};
    for (unsigned W : Ws)
        for (unsigned H : Hs)
        {
            if ((unsigned long long)W * H > 3000000ull) continue;
            ++sizes;
            const unsigned n = W * H;
            std::vector<unsigned char> seen(n, 0);
            for (unsigned u = 0; u < n; ++u)
            {
                const unsigned px = slot_pixel(u, W, H);
                if (px >= n || seen[px]) { ++bad_bij; break; }
                seen[px] = 1;
            }
            if (W % 8 != 0) continue;
            for (unsigned w0 = 0; w0 + 32 <= n; w0 += 32)
            {
                const unsigned p0 = slot_pixel(w0, W, H);
                const unsigned x0 = p0 % W, y0 = p0 / W;
                if (y0 + 4 > H) continue;  // the last band is shorter than 4 rows
                for (unsigned i = 0; i < 32; ++i)
                {
                    const unsigned p = slot_pixel(w0 + i, W, H);
                    if (p % W != x0 + i % 8 || p / W != y0 + i / 8) { ++bad_tile; break; }
                }
            }
        }
    std::printf("%lld %lld %lld\n", sizes, bad_bij, bad_tile);
    return 0;
}
"""


def test_slot_pixel_is_a_tiled_bijection(tmp_path):
    cuda = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
    nvcc = cuda / "bin" / "nvcc"
    if not nvcc.exists():
        nvcc = shutil.which("nvcc")
        if nvcc is None:
            pytest.skip("nvcc not found")
    src = tmp_path / "order.cu"
    src.write_text(PROGRAM)
    exe = tmp_path / "order"
    subprocess.run([str(nvcc), "-O2", "-std=c++17", "-I", str(CSRC), str(src), "-o", str(exe)], check=True)
    sizes, bad_bij, bad_tile = map(int, subprocess.run([str(exe)], check=True, capture_output=True,
                                                       text=True).stdout.split())
    assert sizes > 100 and bad_bij == 0 and bad_tile == 0
