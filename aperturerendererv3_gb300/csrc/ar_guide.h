// Voxel path guide: per (voxel, icosahedron face) octahedral radiance probes.
// Host + device.  Restates the reference's probe math with the same operation
// order (core/guiding/guiding_bin.cuh:11-114, core/guiding/octahedron.cuh:13-499):
//   * voxel key  = floor(p / unit) and the icosahedron face whose normal is
//                  closest to the reflected ray direction;
//   * probe      = 8x8 equal-area (Clarberg 2008) octahedral map of RGB
//                  radiance x Jacobian, with a mip pyramid 4^2, 2^2, 1;
//   * sampling   = descent through the mips picking children proportionally to
//                  their weight against a per-path RGB query, then uniform in
//                  the leaf texel; hemisphere variant folds the mirrored lobe;
//   * update     = running mean over samples (FP64 blend), count capped at 1e6.
#pragma once
#include "ar_spectral.h"

// PATH_GUIDING_RESOLUTION_LEVEL = 4 (core/config.cuh:40): an 8x8 leaf and
// mips 4x4, 2x2, 1x1 (Texture<4>, core/guiding/octahedron.cuh:203-236)
#define AR_PG_LEVELS 4
#define AR_PG_RES 8
#define AR_PG_RES2 64
#define AR_PG_TEXELS 85               // 64 + 16 + 4 + 1
#define AR_PG_TEXELS_PAD 86
#define AR_PG_FACES 20
#define AR_PG_COLLECT_DEPTH 5
#define AR_PG_COLLECT_MAX 1.0e5f
#define AR_PG_COLLECT_MIN 1.0e-5f
#define AR_PG_PROBE_MIN 1.0e-5f
#define AR_PG_MAX_COUNT 1000000ull
#define AR_PG_MAX_ALPHA 0.5f
#define AR_PG_LERP_FRAMES 64
#define AR_PG_LERP_POW 0.5f
#define AR_PG_QUERY_EPS 1.0e-6

namespace ar
{
// probe layout identical to the reference's Texture<4> with 3-channel texels
struct alignas(16) Probe
{
    float4 data[AR_PG_TEXELS_PAD];
    unsigned long long count;
    unsigned long long pad;
};

// icosahedron face normals (core/guiding/guiding_bin.cuh:40-66)
AR_HD V3 face20_normal(int f)
{
    switch (f)
    {
        case 0: return v3(-0.577350269f, 0.577350269f, 0.577350269f);
        case 1: return v3(0.000000000f, 0.934172359f, 0.356822090f);
        case 2: return v3(0.000000000f, 0.934172359f, -0.356822090f);
        case 3: return v3(-0.577350269f, 0.577350269f, -0.577350269f);
        case 4: return v3(-0.934172359f, 0.356822090f, 0.000000000f);
        case 5: return v3(0.577350269f, 0.577350269f, 0.577350269f);
        case 6: return v3(-0.356822090f, 0.000000000f, 0.934172359f);
        case 7: return v3(-0.934172359f, -0.356822090f, 0.000000000f);
        case 8: return v3(-0.356822090f, 0.000000000f, -0.934172359f);
        case 9: return v3(0.577350269f, 0.577350269f, -0.577350269f);
        case 10: return v3(0.577350269f, -0.577350269f, 0.577350269f);
        case 11: return v3(0.000000000f, -0.934172359f, 0.356822090f);
        case 12: return v3(0.000000000f, -0.934172359f, -0.356822090f);
        case 13: return v3(0.577350269f, -0.577350269f, -0.577350269f);
        case 14: return v3(0.934172359f, -0.356822090f, 0.000000000f);
        case 15: return v3(0.356822090f, 0.000000000f, 0.934172359f);
        case 16: return v3(-0.577350269f, -0.577350269f, 0.577350269f);
        case 17: return v3(-0.577350269f, -0.577350269f, -0.577350269f);
        case 18: return v3(0.356822090f, 0.000000000f, -0.934172359f);
        case 19: return v3(0.934172359f, 0.356822090f, 0.000000000f);
        default: return v3(0.0f, 0.0f, 1.0f);
    }
}

AR_HD int face20_index(V3 n)
{
    const V3 d = normalize(n);
    int best = 0;
    float bestDot = -1e30f;
    for (int f = 0; f < 20; ++f)
    {
        const V3 c = face20_normal(f);
        const float v = d.x * c.x + d.y * c.y + d.z * c.z;
        if (v > bestDot)
        {
            bestDot = v;
            best = f;
        }
    }
    return best;
}

struct VoxelKey
{
    int x, y, z, f;
};

// floor(p / unit) with the unit's reciprocal in float (core/guiding/guiding_bin.cuh:95-100)
AR_HD VoxelKey voxel_key(V3 p, V3 dir, float inv_unit)
{
    VoxelKey k;
    const V3 s = p * inv_unit;
    k.x = (int)floorf(s.x);
    k.y = (int)floorf(s.y);
    k.z = (int)floorf(s.z);
    k.f = face20_index(dir);
    return k;
}

// Clarberg equal-area map [0,1]^2 -> S^2 (core/guiding/octahedron.cuh:13-86)
AR_HD V3 uv_to_sphere(float px, float py)
{
    const float u = 2.0f * px - 1.0f;
    const float v = 2.0f * py - 1.0f;
    const float a = v + u;
    const float b = v - u;
    float r, phi4, zsign;
    if (v >= 0.0f)
    {
        if (u >= 0.0f)
        {
            if (a <= 1.0f) { r = a; zsign = 1.0f; phi4 = (r == 0.0f ? 0.0f : v / r); }
            else { r = 2.0f - a; zsign = -1.0f; phi4 = (1.0f - u) / r; }
        }
        else
        {
            if (b <= 1.0f) { r = b; zsign = 1.0f; phi4 = 1.0f - u / r; }
            else { r = 2.0f - b; zsign = -1.0f; phi4 = 1.0f + (1.0f - v) / r; }
        }
    }
    else
    {
        if (u < 0.0f)
        {
            if (a >= -1.0f) { r = -a; zsign = 1.0f; phi4 = 2.0f - v / r; }
            else { r = 2.0f + a; zsign = -1.0f; phi4 = 2.0f + (1.0f + u) / r; }
        }
        else
        {
            if (b >= -1.0f) { r = -b; zsign = 1.0f; phi4 = 3.0f + u / r; }
            else { r = 2.0f + b; zsign = -1.0f; phi4 = 3.0f + (1.0f + v) / r; }
        }
    }
    if (r == 0.0f) phi4 = 0.0f;
    const float r2 = r * r;
    const float phi = phi4 * (0.5f * AR_PI_F);
    const float sint = r * sqrtf(fmaxf(0.0f, 2.0f - r2));
    const float cost = zsign * (1.0f - r2);
    float s, c;
    arm_sincosf(phi, &s, &c);
    return v3(sint * c, sint * s, cost);
}

// S^2 -> [0,1]^2 (core/guiding/octahedron.cuh:89-143)
AR_HD void sphere_to_uv(V3 d, float* uo, float* vo)
{
    const float phi2 = arm_atan2f(d.y, d.x) * (2.0f / AR_PI_F);
    float u, v;
    if (d.z < 0.0f)
    {
        const float r = sqrtf(fmaxf(0.0f, 1.0f + d.z));
        if (phi2 >= 0.0f)
        {
            if (phi2 <= 1.0f) { u = 1.0f - r * phi2; v = 2.0f - r - u; }
            else { u = r * (2.0f - phi2) - 1.0f; v = 2.0f - r + u; }
        }
        else
        {
            if (phi2 >= -1.0f) { u = r * phi2 + 1.0f; v = r - 2.0f + u; }
            else { u = r * (2.0f + phi2) - 1.0f; v = r - 2.0f - u; }
        }
    }
    else
    {
        const float r = sqrtf(fmaxf(0.0f, 1.0f - d.z));
        if (phi2 >= 0.0f)
        {
            if (phi2 < 1.0f) { v = r * phi2; u = r - v; }
            else { v = r * (2.0f - phi2); u = v - r; }
        }
        else
        {
            if (phi2 > -1.0f) { v = r * phi2; u = r + v; }
            else { v = -r * (2.0f + phi2); u = -(r + v); }
        }
    }
    *uo = 0.5f * (u + 1.0f);
    *vo = 0.5f * (v + 1.0f);
}

AR_HD float clarberg_jacobian() { return 4.0f * AR_PI_F; }

AR_HD int level_offset(int level)
{
    int offset = 0, res = AR_PG_RES;
    for (int i = 0; i < level; ++i)
    {
        offset += res * res;
        res >>= 1;
    }
    return offset;
}

AR_HD float4 texel(const Probe& pr, int x, int y, int level)
{
    const int res = 1 << (AR_PG_LEVELS - 1 - level);
    return pr.data[level_offset(level) + y * res + x];
}

AR_HD float qdot(float4 t, V3 q) { return t.x * q.x + t.y * q.y + t.z * q.z; }

AR_HD V3 reflect_hemisphere(V3 w, V3 n)
{
    return normalize(w) - 2.0f * dot(normalize(n), normalize(w)) * normalize(n);
}

// OctahedronPDF (core/guiding/octahedron.cuh:384-412)
AR_HD float octahedron_pdf(const Probe& pr, V3 d, V3 q)
{
    float u, v;
    sphere_to_uv(d, &u, &v);
    int ix = (int)floorf(u * AR_PG_RES);
    int iy = (int)floorf(v * AR_PG_RES);
    ix = ix < 0 ? 0 : (ix > AR_PG_RES - 1 ? AR_PG_RES - 1 : ix);
    iy = iy < 0 ? 0 : (iy > AR_PG_RES - 1 ? AR_PG_RES - 1 : iy);
    const float wLeaf = qdot(texel(pr, ix, iy, 0), q);
    const float wAvg = qdot(texel(pr, 0, 0, AR_PG_LEVELS - 1), q);
    const float invG = (float)(1.0 / (double)clarberg_jacobian());
    if (!(wAvg > 0.0f)) return invG;
    return fmaxf((wLeaf / wAvg) * invG, 1.0e-12f);
}

AR_HD float octahedron_hemisphere_pdf(const Probe& pr, V3 d, V3 n, V3 q)
{
    if (dot(d, n) <= 0.0f) return 0.0f;
    const V3 m = reflect_hemisphere(d, n);
    return octahedron_pdf(pr, d, q) + octahedron_pdf(pr, m, q);
}

struct GuideSample
{
    V3 dir;
    float pdf;
};

// SampleOctahedron (core/guiding/octahedron.cuh:277-341)
template <typename Rand>
AR_HD GuideSample sample_octahedron(const Probe& pr, Rand& rand, V3 q)
{
    int cx = 0, cy = 0;
    float pTexel = 1.0f;
    for (int level = AR_PG_LEVELS - 1; level > 0; --level)
    {
        const float weightSum = 4.0f * qdot(texel(pr, cx, cy, level), q);
        const int nx = cx << 1, ny = cy << 1;
        const float r = rand();
        if (weightSum <= 0.0f)
        {
            int pick = (int)(r * 4.0f);
            pick = pick < 3 ? pick : 3;
            cx = nx + (pick & 1);
            cy = ny + (pick >> 1);
            pTexel *= 0.25f;
        }
        else
        {
            float cdf = 0.0f;
            bool done = false;
            for (int x = 0; x < 2 && !done; ++x)
                for (int y = 0; y < 2 && !done; ++y)
                {
                    const int chx = nx + x, chy = ny + y;
                    const float w = qdot(texel(pr, chx, chy, level - 1), q) / weightSum;
                    cdf += w;
                    if (r <= cdf || (x == 1 && y == 1))
                    {
                        cx = chx;
                        cy = chy;
                        pTexel *= w;
                        done = true;
                    }
                }
        }
    }
    const float r0 = rand();
    const float r1 = rand();
    const float ux = 1.0f - r0, uy = 1.0f - r1;
    const float su = (cx + ux) / static_cast<float>(AR_PG_RES);
    const float sv = (cy + uy) / static_cast<float>(AR_PG_RES);
    const V3 d = uv_to_sphere(saturate(su), saturate(sv));
    GuideSample s;
    s.dir = d;
    s.pdf = fmaxf(pTexel * AR_PG_RES2 / clarberg_jacobian(), 1.0e-12f);
    return s;
}

template <typename Rand>
AR_HD GuideSample sample_octahedron_hemisphere(const Probe& pr, Rand& rand, V3 n, V3 q)
{
    GuideSample s = sample_octahedron(pr, rand, q);
    const V3 m = reflect_hemisphere(s.dir, n);
    s.pdf += octahedron_pdf(pr, m, q);
    if (dot(s.dir, n) < 0.0f) s.dir = m;
    return s;
}

// GenerateMipmaps (core/guiding/octahedron.cuh:438-499)
AR_HD void generate_mipmaps(Probe& pr)
{
    for (int i = 0; i < AR_PG_RES2; ++i)
    {
        float4& t = pr.data[i];
        t.x = fmaxf(t.x, AR_PG_PROBE_MIN);
        t.y = fmaxf(t.y, AR_PG_PROBE_MIN);
        t.z = fmaxf(t.z, AR_PG_PROBE_MIN);
        t.w = fmaxf(t.w, AR_PG_PROBE_MIN);
    }
    int srcRes = AR_PG_RES, srcOff = 0, nextOff = AR_PG_RES2;
    for (int level = 0; level < AR_PG_LEVELS - 1; ++level)
    {
        const int dr = srcRes >> 1;
        for (int y = 0; y < dr; ++y)
            for (int x = 0; x < dr; ++x)
            {
                const float4 a = pr.data[srcOff + (2 * y) * srcRes + 2 * x];
                const float4 b = pr.data[srcOff + (2 * y) * srcRes + 2 * x + 1];
                const float4 c = pr.data[srcOff + (2 * y + 1) * srcRes + 2 * x];
                const float4 d = pr.data[srcOff + (2 * y + 1) * srcRes + 2 * x + 1];
                float4 o;
                o.x = (a.x + b.x + c.x + d.x) * 0.25f;
                o.y = (a.y + b.y + c.y + d.y) * 0.25f;
                o.z = (a.z + b.z + c.z + d.z) * 0.25f;
                o.w = (a.w + b.w + c.w + d.w) * 0.25f;
                pr.data[nextOff + y * dr + x] = o;
            }
        srcOff = nextOff;
        srcRes = dr;
        nextOff = srcOff + srcRes * srcRes;
    }
    pr.data[AR_PG_TEXELS] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
}

// guide/BSDF mixture probability (core/render/render.cuh:198-203)
AR_HD float guide_probability(int frame)
{
    const float t = fminf(1.0f, static_cast<float>(frame) / AR_PG_LERP_FRAMES);
    return saturate(lerpf(0.0f, AR_PG_MAX_ALPHA, arm_powf(t, AR_PG_LERP_POW)));
}

// leaf texel of a direction (core/guiding/guiding.cuh:336-345)
AR_HD void direction_to_leaf(V3 d, int* px, int* py)
{
    float u, v;
    sphere_to_uv(normalize(d), &u, &v);
    int ix = (int)floorf(u * AR_PG_RES);
    int iy = (int)floorf(v * AR_PG_RES);
    ix = ix < 0 ? 0 : (ix > AR_PG_RES - 1 ? AR_PG_RES - 1 : ix);
    iy = iy < 0 ? 0 : (iy > AR_PG_RES - 1 ? AR_PG_RES - 1 : iy);
    *px = ix;
    *py = iy;
}
} // namespace ar
