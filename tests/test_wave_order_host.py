"""Host checks of the order of a render's paths (csrc/ar_internal.h): the
pixel slots of a frame (slot_pixel: a bijection of [0, W*H) at every size,
and, when the width is a multiple of 8, every aligned run of 32 slots covers
an 8 x 4 pixel tile where the image has 4 rows left), and the order of
(slot, sample) pairs among the render's paths (path_slot / path_index).
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


PATH_ORDER_PROGRAM = r"""
#include <cstdio>
#include <vector>
#include "ar_internal.h"
using namespace ar;

int main()
{
    long long cases = 0, bad_bij = 0, bad_inv = 0, bad_mono = 0, bad_frame_major = 0, bad_first = 0, bad_warp = 0;
    const unsigned npixs[] = {1, 2, 3, 4, 5, 7, 8, 13, 64, 100, 1001, 4096};
    const unsigned spps[] = {1, 2, 3, 7, 8, 9, 16, 17, 64};
    const unsigned blocks[] = {1, 2, 8, AR_SAMPLE_BLOCK};
    for (unsigned npix : npixs)
        for (unsigned spp : spps)
            for (unsigned block : blocks)
            {
                if (block > spp) continue;
                ++cases;
                const PathOrder o{npix, spp, block};
                const unsigned long long total = (unsigned long long)npix * spp;
                std::vector<unsigned char> seen(total, 0);
                for (unsigned long long g = 0; g < total; ++g)
                {
                    uint32_t u, s;
                    path_slot(o, g, &u, &s);
                    if (u >= npix || s >= spp) { ++bad_bij; break; }
                    const unsigned long long cell = (unsigned long long)s * npix + u;
                    if (seen[cell]) { ++bad_bij; break; }
                    seen[cell] = 1;
                    if (path_index(o, u, s) != g) ++bad_inv;
                    if (block == 1 && (u != g % npix || s != g / npix)) ++bad_frame_major;
                }
                for (unsigned u = 0; u < npix; ++u)
                {
                    for (unsigned s = 1; s < spp; ++s)
                        if (path_index(o, u, s) <= path_index(o, u, s - 1)) ++bad_mono;
                    // path_first_sample finds the first sample at or after every index
                    for (unsigned long long g0 = 0; g0 <= total; g0 += 1 + total / 37)
                    {
                        unsigned want = spp;
                        for (unsigned s = 0; s < spp; ++s)
                            if (path_index(o, u, s) >= g0) { want = s; break; }
                        if (path_first_sample(o, u, g0) != want) ++bad_first;
                    }
                }
                // a full block of AR_SAMPLE_BLOCK samples: each aligned warp is all of the
                // block's samples of AR_PATH_GROUP_PX consecutive slots, slot fastest
                if (block == AR_SAMPLE_BLOCK && AR_PATH_GROUP_PX * AR_SAMPLE_BLOCK == 32 && npix % AR_PATH_GROUP_PX == 0)
                    for (unsigned long long w0 = 0; w0 + 32 <= (unsigned long long)npix * block; w0 += 32)
                    {
                        uint32_t u0, s0;
                        path_slot(o, w0, &u0, &s0);
                        for (unsigned i = 0; i < 32; ++i)
                        {
                            uint32_t u, s;
                            path_slot(o, w0 + i, &u, &s);
                            if (u != u0 + i % AR_PATH_GROUP_PX || s != s0 + i / AR_PATH_GROUP_PX) { ++bad_warp; break; }
                        }
                    }
            }
    // renders above 2^32 paths take the 64-bit arithmetic: spot checks of the inverse
    {
        const PathOrder o{100000000u, 64u, AR_SAMPLE_BLOCK};
        const unsigned long long total = (unsigned long long)o.npix * o.spp;
        unsigned long long g = 12345;
        for (int i = 0; i < 200000; ++i)
        {
            uint32_t u, s;
            path_slot(o, g, &u, &s);
            if (u >= o.npix || s >= o.spp || path_index(o, u, s) != g) ++bad_inv;
            g = (g * 6364136223846793005ull + 1442695040888963407ull) % total;
        }
        ++cases;
    }
    std::printf("%lld %lld %lld %lld %lld %lld %lld\n", cases, bad_bij, bad_inv, bad_mono, bad_frame_major, bad_first,
                bad_warp);
    return 0;
}
"""


def test_path_order_is_a_bijection_with_its_inverse(tmp_path):
    """path_slot / path_index (csrc/ar_internal.h): every (slot, sample) of a
    render exactly once, path_index inverts path_slot and rises with the
    sample (the per-pixel sums add samples in order), path_first_sample finds
    a wave's first sample of a slot, block 1 is frame-major order, and with
    full blocks every warp holds all of a block's samples of its slots (32
    samples of one pixel)."""
    cuda = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
    nvcc = cuda / "bin" / "nvcc"
    if not nvcc.exists():
        nvcc = shutil.which("nvcc")
        if nvcc is None:
            pytest.skip("nvcc not found")
    src = tmp_path / "path_order.cu"
    src.write_text(PATH_ORDER_PROGRAM)
    exe = tmp_path / "path_order"
    subprocess.run([str(nvcc), "-O2", "-std=c++17", "-I", str(CSRC), str(src), "-o", str(exe)], check=True)
    out = list(map(int, subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()))
    assert out[0] > 200 and out[1:] == [0, 0, 0, 0, 0, 0], out
