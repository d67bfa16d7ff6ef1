"""Host check that the traversal's child-box test is conservative (csrc/ar_traverse.cuh).

TravState::step tests the 8 children of a wide node with one fused
multiply-add per plane on per-node terms and an absolute rounding margin.  Hit
ids are exact only if that test never rejects a child box that the ray meets
in [tmin, tlim].  Here the traversal's own step() runs on the host (nvcc host
code) against random quantized nodes and adversarial rays: rays aimed exactly
at points on child box faces, edges and corners with the limit exactly at the
point, random rays, rays with zero direction components and origins far from
the node.  Every child that a double-precision slab test on the exact child
box accepts must be accepted; extra acceptances (boxes the ray misses by less
than the margin) are bounded loosely.
"""
import os
import shutil
import subprocess
from pathlib import Path

import pytest

CSRC = Path(__file__).resolve().parents[1] / "aperturerendererv3_gb300" / "csrc"

PROGRAM = r"""
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include "ar_traverse.cuh"
using namespace ar;

struct Box { double lo[3], hi[3]; };

static bool exact_hit(const Box& b, const double o[3], const double d[3], double tmin, double tlim)
{
    double tn = tmin, tf = tlim;
    for (int k = 0; k < 3; ++k)
    {
        if (d[k] == 0.0)
        {
            if (o[k] < b.lo[k] || o[k] > b.hi[k]) return false;
            continue;
        }
        double t0 = (b.lo[k] - o[k]) / d[k], t1 = (b.hi[k] - o[k]) / d[k];
        if (t0 > t1) std::swap(t0, t1);
        tn = std::max(tn, t0);
        tf = std::min(tf, t1);
    }
    return tn <= tf;
}

int main()
{
    std::mt19937 rng(2024);
    std::uniform_real_distribution<float> U(0.0f, 1.0f);
    long long tested = 0, missed = 0, extra = 0, exact_hits = 0, regular = 0;
    for (int trial = 0; trial < 60000; ++trial)
    {
        // a node: origin, per-axis exponents, 8 internal children with random quantized boxes
        ar_wide_node nd;
        std::memset(&nd, 0, sizeof(nd));
        const float scale_world = (trial % 5 == 0) ? 1000.0f : 1.0f;
        nd.px = scale_world * (2 * U(rng) - 1);
        nd.py = scale_world * (2 * U(rng) - 1);
        nd.pz = scale_world * (2 * U(rng) - 1);
        int e[3];
        for (int k = 0; k < 3; ++k)
        {
            e[k] = -12 + (int)(U(rng) * 10);
            nd.e[k] = (uint8_t)(e[k] + 127);
        }
        nd.imask = 0xff;
        nd.child_base = 1;
        Box box[8];
        const float p[3] = {nd.px, nd.py, nd.pz};
        for (int s = 0; s < 8; ++s)
        {
            nd.meta[s] = (uint8_t)(0x80u | (uint32_t)s);
            for (int k = 0; k < 3; ++k)
            {
                int a = (int)(U(rng) * 256), b = (int)(U(rng) * 256);
                if (a > 255) a = 255;
                if (b > 255) b = 255;
                if (a > b) std::swap(a, b);
                if (trial % 7 == 0) b = a;  // flat boxes (a heightfield's planar leaves)
                nd.qlo[k][s] = (uint8_t)a;
                nd.qhi[k][s] = (uint8_t)b;
                box[s].lo[k] = (double)p[k] + std::ldexp((double)a, e[k]);
                box[s].hi[k] = (double)p[k] + std::ldexp((double)b, e[k]);
            }
        }
        uint4 nodes[5 * 9];
        std::memset(nodes, 0, sizeof(nodes));
        std::memcpy(nodes, &nd, sizeof(nd));
        TravScene sc;
        std::memset(&sc, 0, sizeof(sc));
        sc.nodes = nodes;
        sc.node_count = 9;
        for (int r = 0; r < 8; ++r)
        {
            // a target on a face, edge or corner of a child box, or a random point
            const int s_t = (int)(U(rng) * 8) & 7;
            double tgt[3];
            for (int k = 0; k < 3; ++k)
            {
                const int pick = (int)(U(rng) * 3);
                tgt[k] = pick == 0 ? box[s_t].lo[k] : pick == 1 ? box[s_t].hi[k]
                                                                : box[s_t].lo[k] + U(rng) * (box[s_t].hi[k] - box[s_t].lo[k]);
            }
            float of[3], df[3];
            const float span = std::ldexp(300.0f, e[0]) + 1e-3f;
            const float dist = (r % 4 == 0) ? 1000.0f * span : span * (0.5f + 4 * U(rng));
            for (int k = 0; k < 3; ++k) of[k] = (float)(tgt[k] + dist * (2 * U(rng) - 1));
            double dd[3], len = 0;
            for (int k = 0; k < 3; ++k)
            {
                dd[k] = tgt[k] - (double)of[k];
                len += dd[k] * dd[k];
            }
            len = std::sqrt(len);
            if (len == 0) continue;
            for (int k = 0; k < 3; ++k) df[k] = (float)(dd[k] / len);
            if (r == 5) df[(int)(U(rng) * 3) % 3] = 0.0f;  // axis-parallel component
            if (r == 6) df[(int)(U(rng) * 3) % 3] = -0.0f;
            const double o[3] = {of[0], of[1], of[2]}, d[3] = {df[0], df[1], df[2]};
            // the limit: exactly at the target along the ray (closest-hit so far), or open
            float tlim = (r % 2 == 0) ? (float)len : INFINITY;
            if (r == 7) tlim = std::nextafter((float)len, 0.0f);
            const float tmin = (r % 3 == 0) ? 0.0f : 1e-4f;
            TravState<false> st;
            uint2 stk[AR_TRAV_STACK];
            st.init(sc, v3(of[0], of[1], of[2]), v3(df[0], df[1], df[2]), tmin, tlim, stk);
            st.res.t = tlim;
            st.step(sc, nullptr);
            uint32_t got = 0;
            if (st.node >= 1) got |= 1u << (st.node - 1);
            if (st.sp > 0)
            {
                const uint32_t m = stk[0].y & 0xffu;
                for (int i = 0; i < 8; ++i)
                    if (m & (1u << i)) got |= 1u << (i ^ st.oct);
            }
            for (int s = 0; s < 8; ++s)
            {
                const bool ex = exact_hit(box[s], o, d, (double)tmin, (double)tlim);
                const bool gt = (got >> s) & 1u;
                ++tested;
                exact_hits += ex;
                if (ex && !gt) ++missed;
                // rays with a zero direction component overflow on the permissive side by design
                const bool reg = df[0] != 0.0f && df[1] != 0.0f && df[2] != 0.0f;
                regular += reg;
                if (reg && !ex && gt) ++extra;
            }
        }
    }
    std::printf("%lld %lld %lld %lld %lld\n", tested, exact_hits, missed, regular, extra);
    return 0;
}
"""


def test_child_box_test_is_conservative(tmp_path):
    cuda = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
    nvcc = cuda / "bin" / "nvcc"
    if not nvcc.exists():
        nvcc = shutil.which("nvcc")
        if nvcc is None:
            pytest.skip("nvcc not found")
    src = tmp_path / "trav.cu"
    src.write_text(PROGRAM)
    exe = tmp_path / "trav"
    subprocess.run([str(nvcc), "-O2", "-std=c++17", "-fmad=false", "-Xcompiler", "-ffp-contract=off", "-I", str(CSRC),
                    str(src), "-o", str(exe)], check=True)
    tested, hits, missed, regular, extra = map(int, subprocess.run([str(exe)], check=True, capture_output=True,
                                                                   text=True).stdout.split())
    assert tested > 3_000_000 and hits > tested // 20
    assert missed == 0, f"{missed} child boxes met by the ray were rejected"
    # Extra acceptances (rays with no zero direction component): boxes the ray
    # misses by less than the margin.  One box in eight is aimed at exactly on
    # its boundary with the limit exactly at the target, so double rounding
    # splits those ties; on the terrain the margin adds 0.014 % node visits.
    # The bound only catches a grossly permissive test (accepting everything
    # would give about 90 %).
    assert extra < 0.10 * regular, f"{extra} extra acceptances of {regular}"


PACKET_PROGRAM = r"""
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include "ar_traverse.cuh"
using namespace ar;

struct Box { double lo[3], hi[3]; };

static bool exact_hit(const Box& b, const double o[3], const double d[3], double tmin, double tlim)
{
    double tn = tmin, tf = tlim;
    for (int k = 0; k < 3; ++k)
    {
        double t0 = (b.lo[k] - o[k]) / d[k], t1 = (b.hi[k] - o[k]) / d[k];
        if (t0 > t1) std::swap(t0, t1);
        tn = std::max(tn, t0);
        tf = std::min(tf, t1);
    }
    return tn <= tf;
}

int main()
{
    std::mt19937 rng(77);
    std::uniform_real_distribution<float> U(0.0f, 1.0f);
    long long tested = 0, met = 0, missed = 0, accepted = 0, packets = 0;
    for (int trial = 0; trial < 40000; ++trial)
    {
        ar_wide_node nd;
        std::memset(&nd, 0, sizeof(nd));
        const float scale_world = (trial % 5 == 0) ? 1000.0f : 1.0f;
        nd.px = scale_world * (2 * U(rng) - 1);
        nd.py = scale_world * (2 * U(rng) - 1);
        nd.pz = scale_world * (2 * U(rng) - 1);
        int e[3];
        for (int k = 0; k < 3; ++k)
        {
            e[k] = -12 + (int)(U(rng) * 10);
            nd.e[k] = (uint8_t)(e[k] + 127);
        }
        nd.imask = (uint8_t)(trial % 3 == 0 ? 0x0f : 0xff);  // some leaf children
        nd.child_base = 1;
        Box box[8];
        const float p[3] = {nd.px, nd.py, nd.pz};
        for (int s = 0; s < 8; ++s)
        {
            nd.meta[s] = (uint8_t)(0x20u | (uint32_t)s);  // leaves hold one primitive
            for (int k = 0; k < 3; ++k)
            {
                int a = (int)(U(rng) * 256), b = (int)(U(rng) * 256);
                if (a > 255) a = 255;
                if (b > 255) b = 255;
                if (a > b) std::swap(a, b);
                if (trial % 7 == 0) b = a;
                nd.qlo[k][s] = (uint8_t)a;
                nd.qhi[k][s] = (uint8_t)b;
                box[s].lo[k] = (double)p[k] + std::ldexp((double)a, e[k]);
                box[s].hi[k] = (double)p[k] + std::ldexp((double)b, e[k]);
            }
        }
        uint4 w[5];
        std::memcpy(w, &nd, sizeof(w));
        for (int r = 0; r < 4; ++r)
        {
            // one origin; 32 directions towards points around a face, edge or corner of a child
            const int s_t = (int)(U(rng) * 8) & 7;
            double tgt[3];
            for (int k = 0; k < 3; ++k)
            {
                const int pick = (int)(U(rng) * 3);
                tgt[k] = pick == 0 ? box[s_t].lo[k] : pick == 1 ? box[s_t].hi[k]
                                                                : box[s_t].lo[k] + U(rng) * (box[s_t].hi[k] - box[s_t].lo[k]);
            }
            const float span = std::ldexp(300.0f, e[0]) + 1e-3f;
            const float dist = (r % 2 == 0) ? 1000.0f * span : span * (0.5f + 4 * U(rng));
            float of[3];
            for (int k = 0; k < 3; ++k) of[k] = (float)(tgt[k] + dist * (2 * U(rng) - 1));
            const double spread = (r == 3) ? 0.05 : 1e-4;  // the packet's cone around the target
            float df[32][3];
            bool ok = true;
            for (int l = 0; l < 32 && ok; ++l)
            {
                double dd[3], len = 0;
                for (int k = 0; k < 3; ++k)
                {
                    dd[k] = tgt[k] - (double)of[k] + (l ? spread * dist * (2 * U(rng) - 1) : 0.0);
                    len += dd[k] * dd[k];
                }
                len = std::sqrt(len);
                for (int k = 0; k < 3; ++k) df[l][k] = (float)(dd[k] / len);
                for (int k = 0; k < 3; ++k)
                    if (df[l][k] == 0.0f || ((df[l][k] < 0.0f) != (df[0][k] < 0.0f))) ok = false;
            }
            if (!ok) continue;  // the kernel runs such warps per ray
            ++packets;
            V3 ilo = v3(3e38f, 3e38f, 3e38f), ihi = v3(-3e38f, -3e38f, -3e38f);
            for (int l = 0; l < 32; ++l)
            {
                const V3 iv = v3(inv_safe(df[l][0]), inv_safe(df[l][1]), inv_safe(df[l][2]));
                ilo = v3(std::fmin(ilo.x, iv.x), std::fmin(ilo.y, iv.y), std::fmin(ilo.z, iv.z));
                ihi = v3(std::fmax(ihi.x, iv.x), std::fmax(ihi.y, iv.y), std::fmax(ihi.z, iv.z));
            }
            const V3 iabs = v3(std::fmax(std::fabs(ilo.x), std::fabs(ihi.x)), std::fmax(std::fabs(ilo.y), std::fabs(ihi.y)),
                               std::fmax(std::fabs(ilo.z), std::fabs(ihi.z)));
            const uint32_t oct = (df[0][0] < 0 ? 1u : 0u) | (df[0][1] < 0 ? 2u : 0u) | (df[0][2] < 0 ? 4u : 0u);
            // the limit: at the target distance (a closest hit there), or open
            const float tlim = (r % 2 == 0) ? (float)dist : INFINITY;
            const float tmin = (r == 1) ? 0.0f : 1e-4f;
            for (int s = 0; s < 8; ++s)
            {
                bool any = false;
                for (int l = 0; l < 32 && !any; ++l)
                {
                    const double o[3] = {of[0], of[1], of[2]}, d[3] = {df[l][0], df[l][1], df[l][2]};
                    any = exact_hit(box[s], o, d, (double)tmin, (double)tlim);
                }
                const bool got = packet_child_meets(w[0], w[1], w[2], w[3], w[4], s, v3(of[0], of[1], of[2]), oct, ilo, ihi,
                                                    iabs, tmin, tlim);
                ++tested;
                met += any;
                accepted += got;
                if (any && !got) ++missed;
            }
        }
    }
    std::printf("%lld %lld %lld %lld %lld\n", packets, tested, met, missed, accepted);
    return 0;
}
"""


def test_packet_child_test_is_conservative(tmp_path):
    """packet_child_meets (the camera-ray packet kernel's interval slab test):
    for packets of 32 rays from one origin aimed at faces, edges and corners
    of random quantized child boxes (narrow and wide cones, near and far
    origins, the limit at the target or open), every child that any ray of
    the packet meets in [tmin, tlim] (double-precision slab test on the exact
    box) is accepted."""
    cuda = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
    nvcc = cuda / "bin" / "nvcc"
    if not nvcc.exists():
        nvcc = shutil.which("nvcc")
        if nvcc is None:
            pytest.skip("nvcc not found")
    src = tmp_path / "packet.cu"
    src.write_text(PACKET_PROGRAM)
    exe = tmp_path / "packet"
    subprocess.run([str(nvcc), "-O2", "-std=c++17", "-Xcompiler", "-ffp-contract=off", "-I", str(CSRC), str(src),
                    "-o", str(exe)], check=True)
    packets, tested, met, missed, accepted = map(int, subprocess.run([str(exe)], check=True, capture_output=True,
                                                                     text=True).stdout.split())
    assert packets > 50000 and met > tested // 20
    assert missed == 0, f"{missed} child boxes met by a ray of the packet were rejected"
    assert accepted < tested, "the test accepts everything"
