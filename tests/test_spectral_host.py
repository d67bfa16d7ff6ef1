"""Host check of the hero-wavelength sampler (csrc/ar_spectral.h).

sample_cie1931 picks each lane's lobe constants and evaluates one inverse
normal CDF instead of branching into sample_cie_x / _y / _z.  It must return
the branch form's wavelength and pdf bit for bit for every (r0, r1, r2):
checked on random triples and on the lobe and tail boundaries.
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
#include "ar_spectral.h"
using namespace ar;

static LambdaSample branch_form(float r0, float r1, float r2)
{
    const float total = 0.1f + 1.0f + 1.0f + 1.0f;
    const float uniformRatio = 0.1f / total, XRatio = 1.0f / total, YRatio = 1.0f / total, ZRatio = 1.0f / total;
    float lambda;
    if (r0 < uniformRatio) lambda = r1 * (780.0f - 360.0f) + 360.0f;
    else if (r0 < uniformRatio + XRatio) lambda = sample_cie_x(r1, r2);
    else if (r0 < uniformRatio + XRatio + YRatio) lambda = sample_cie_y(r1);
    else lambda = sample_cie_z(r1);
    const float pMix = uniformRatio * 1.0f / (780.0f - 360.0f) + XRatio * pdf_cie_x(lambda) +
                       YRatio * pdf_cie_y(lambda) + ZRatio * pdf_cie_z(lambda);
    LambdaSample s;
    s.lambda = lambda;
    s.pdf = fmaxf(pMix, 1e-16f);
    return s;
}

static bool same(float a, float b)
{
    unsigned x, y;
    std::memcpy(&x, &a, 4);
    std::memcpy(&y, &b, 4);
    return x == y;
}

int main()
{
    std::mt19937 rng(77);
    long long n = 0, bad = 0;
    auto check = [&](float r0, float r1, float r2) {
        const LambdaSample a = sample_cie1931(r0, r1, r2), b = branch_form(r0, r1, r2);
        if (!same(a.lambda, b.lambda) || !same(a.pdf, b.pdf)) ++bad;
        ++n;
    };
    for (int i = 0; i < 3000000; ++i)
    {
        // the renderer's uniforms: 24 random bits, in (0, 1]
        const float r0 = (float)((rng() >> 8) + 1u) * (1.0f / 16777216.0f);
        const float r1 = (float)((rng() >> 8) + 1u) * (1.0f / 16777216.0f);
        const float r2 = (float)((rng() >> 8) + 1u) * (1.0f / 16777216.0f);
        check(r0, r1, r2);
    }
    const float total = 0.1f + 1.0f + 1.0f + 1.0f;
    const float edges[] = {0.1f / total, 0.1f / total + 1.0f / total, 0.1f / total + 2.0f / total,
                           0.8330258723493694f, 0.02425f, 0.97575f, 1.0f, 1.0f / 16777216.0f};
    for (float e : edges)
        for (int k = -4; k <= 4; ++k)
        {
            const float v = std::nextafter(e, k < 0 ? 0.0f : 2.0f) * 0.0f + e + k * 1e-7f;
            for (float w : {0.0000001f, 0.02f, 0.5f, 0.98f, 1.0f})
            {
                check(v, w, 0.5f);
                check(0.5f, v, w);
                check(0.05f, v, w);
                check(0.9f, w, v);
            }
        }
    std::printf("%lld %lld\n", n, bad);
    return 0;
}
"""


def test_lobe_selection_equals_branch_form(tmp_path):
    cuda = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
    nvcc = cuda / "bin" / "nvcc"
    if not nvcc.exists():
        nvcc = shutil.which("nvcc")
        if nvcc is None:
            pytest.skip("nvcc not found")
    # host code only: the header's functions are __host__ __device__ under nvcc
    src = tmp_path / "spec.cu"
    src.write_text(PROGRAM)
    exe = tmp_path / "spec"
    subprocess.run([str(nvcc), "-O2", "-std=c++17", "-fmad=false", "-Xcompiler", "-ffp-contract=off", "-I", str(CSRC),
                    str(src), "-o", str(exe)], check=True)
    n, bad = map(int, subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split())
    assert n > 3000000 and bad == 0
