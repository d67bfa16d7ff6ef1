"""Host check of the smooth-union field (csrc/ar_sdf.h).

sdf_union skips primitives whose blend weight is zero: spheres once their
distance is k above the running value, boxes and tori already when a lowered
bounding-sphere distance is.  The skipped fold must equal the plain left fold
smin_poly(... smin_poly(d0, d1) ..., dn) bit for bit: checked here on random
unions (sizes, smoothing widths, offsets far from the origin) at random points,
many of them inside or near the primitives.
"""
import os
import shutil
import subprocess
from pathlib import Path

import pytest

CSRC = Path(__file__).resolve().parents[1] / "aperturerendererv3_gb300" / "csrc"

PROGRAM = r"""
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>
#include <vector_types.h>
#include "ar_sdf.h"
using namespace ar;

static float plain_fold(const std::vector<float4>& pr, int n, float k, V3 p)
{
    float d = sdf_prim(pr[0], pr[1], p);
    for (int i = 1; i < n; ++i) d = smin_poly(d, sdf_prim(pr[2 * i], pr[2 * i + 1], p), k);
    return d;
}

int main()
{
    std::mt19937 rng(1234);
    std::uniform_real_distribution<float> U(0.0f, 1.0f);
    long long checked = 0, bad = 0, skipped_any = 0;
    for (int scene = 0; scene < 400; ++scene)
    {
        const int n = 1 + (int)(U(rng) * 40);
        const float k = (scene % 3 == 0) ? 0.001f + 0.01f * U(rng) : 0.02f + 0.3f * U(rng);
        const float off = (scene % 4 == 0) ? 100.0f * U(rng) : 0.0f;  // unions far from the origin
        std::vector<float4> pr(2 * n);
        for (int i = 0; i < n; ++i)
        {
            const int kind = (int)(U(rng) * 3);
            float4 a, b;
            a.x = (float)kind;
            a.y = off + 2.0f * U(rng) - 1.0f;
            a.z = off + 2.0f * U(rng) - 1.0f;
            a.w = 2.0f * U(rng) - 1.0f;
            b.x = 0.02f + 0.3f * U(rng);
            b.y = 0.01f + 0.2f * U(rng);
            b.z = 0.02f + 0.3f * U(rng);
            b.w = sdf_bounding_radius(a.x, b.x, b.y, b.z);
            pr[2 * i] = a;
            pr[2 * i + 1] = b;
        }
        SdfUnion s;
        s.prims = pr.data();
        s.count = n;
        s.k = k;
        for (int j = 0; j < 3000; ++j)
        {
            V3 p;
            if (j % 2 == 0)
            {
                // near a primitive's surface or inside it
                const int i = (int)(U(rng) * n) % n;
                const float4 a = pr[2 * i], b = pr[2 * i + 1];
                const float r = b.w * (0.2f + 1.6f * U(rng));
                p = v3(a.y + r * (2 * U(rng) - 1), a.z + r * (2 * U(rng) - 1), a.w + r * (2 * U(rng) - 1));
            }
            else
                p = v3(off + 3 * U(rng) - 1.5f, off + 3 * U(rng) - 1.5f, 3 * U(rng) - 1.5f);
            const float x = sdf_union(s, p), y = plain_fold(pr, n, k, p);
            unsigned ux, uy;
            std::memcpy(&ux, &x, 4);
            std::memcpy(&uy, &y, 4);
            if (ux != uy) ++bad;
            ++checked;
        }
    }
    std::printf("%lld %lld\n", checked, bad);
    return 0;
}
"""


def test_skipping_fold_equals_plain_fold(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    cuda_inc = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda")) / "include"
    if not (cuda_inc / "vector_types.h").exists():
        pytest.skip("CUDA headers (vector types) not found")
    src = tmp_path / "sdf.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "sdf"
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I", str(CSRC), "-I", str(cuda_inc), str(src),
                    "-o", str(exe)], check=True)
    checked, bad = map(int, subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split())
    assert checked == 400 * 3000 and bad == 0
