// MLP path guide: network shape, input encoding and the directional
// distribution the shading kernel samples.  Host + device.
//
// Network: 12-band frequency encoding of the shading point (position
// normalised to the scene box) and of the reflected view direction (6 inputs x
// 12 bands x sin/cos = 144 features), then 144 -> 64 -> 64 -> 64 -> 64 -> 64
// with ReLU between layers.  The 64 outputs are the logits of a distribution
// over the 8 x 8 cells of the same equal-area (Clarberg) sphere map the voxel
// probes use, trained (cross-entropy weighted by record radiance) towards the
// radiance the records carry into each cell, as a probe's leaf accumulates it;
// the guide samples cells in proportion to exp(output), quantised to 8 bits per
// cell (64 bytes per shading point), and a point uniformly inside the cell,
// folded into the normal's hemisphere as the voxel guide folds its lobe.
#pragma once
#include <string.h>

#include "ar_guide.h"

#define AR_MLP_IN 144
#define AR_MLP_H 64
#define AR_MLP_OUT 64
#define AR_MLP_LAYERS 5
#define AR_MLP_BANDS 12
// parameter block: per layer W[64][in] then b[64], float32 (master) / bf16 (W only)
#ifndef AR_MLP_PARAMS
#define AR_MLP_PARAMS 25920
#endif
static_assert(AR_MLP_PARAMS == 64 * 144 + 64 + 4 * (64 * 64 + 64), "parameter block size");
#define AR_MLP_CELL_FLOOR 0.5f  // added to every quantised cell: no direction has zero density

namespace ar
{
AR_HD int mlp_in_dim(int layer) { return layer == 0 ? AR_MLP_IN : AR_MLP_H; }
AR_HD int mlp_w_offset(int layer) { return layer == 0 ? 0 : (64 * 144 + 64) + (layer - 1) * (64 * 64 + 64); }
AR_HD int mlp_b_offset(int layer) { return mlp_w_offset(layer) + 64 * mlp_in_dim(layer); }

// scene box for position normalisation
struct MlpBox
{
    float lo[3], inv[3];
};

// the six encoded inputs in [0, 1]: position in the box, (reflected direction + 1) / 2
AR_HD void mlp_inputs(const MlpBox& b, V3 p, V3 wr, float in6[6])
{
    in6[0] = saturate((p.x - b.lo[0]) * b.inv[0]);
    in6[1] = saturate((p.y - b.lo[1]) * b.inv[1]);
    in6[2] = saturate((p.z - b.lo[2]) * b.inv[2]);
    in6[3] = saturate(0.5f * (wr.x + 1.0f));
    in6[4] = saturate(0.5f * (wr.y + 1.0f));
    in6[5] = saturate(0.5f * (wr.z + 1.0f));
}

// feature index of (input d, band j, cos?) in the 144-wide encoding
AR_HD int mlp_feature(int d, int j, int c) { return d * 2 * AR_MLP_BANDS + 2 * j + c; }

// unit vector <-> 32 bits (octahedral map, 16-bit signed fixed point per axis)
AR_HD float mlp_pack_normal(V3 n)
{
    const float s = fabsf(n.x) + fabsf(n.y) + fabsf(n.z);
    float u = n.x / fmaxf(s, 1e-20f), v = n.y / fmaxf(s, 1e-20f);
    if (n.z < 0.0f)
    {
        const float pu = (1.0f - fabsf(v)) * (u >= 0.0f ? 1.0f : -1.0f);
        const float pv = (1.0f - fabsf(u)) * (v >= 0.0f ? 1.0f : -1.0f);
        u = pu;
        v = pv;
    }
    const int iu = (int)lrintf(clampf(u, -1.0f, 1.0f) * 32767.0f);
    const int iv = (int)lrintf(clampf(v, -1.0f, 1.0f) * 32767.0f);
    const uint32_t bits = ((uint32_t)(uint16_t)(int16_t)iu) | ((uint32_t)(uint16_t)(int16_t)iv << 16);
    float f;
    memcpy(&f, &bits, 4);
    return f;
}

AR_HD V3 mlp_unpack_normal(float f)
{
    uint32_t bits;
    memcpy(&bits, &f, 4);
    const float u = (float)(int16_t)(uint16_t)(bits & 0xffffu) / 32767.0f;
    const float v = (float)(int16_t)(uint16_t)(bits >> 16) / 32767.0f;
    const float z = 1.0f - fabsf(u) - fabsf(v);
    V3 n = v3(u, v, z);
    if (z < 0.0f)
    {
        n.x = (1.0f - fabsf(v)) * (u >= 0.0f ? 1.0f : -1.0f);
        n.y = (1.0f - fabsf(u)) * (v >= 0.0f ? 1.0f : -1.0f);
    }
    return normalize(n);
}

AR_HD int mlp_cell(V3 d)
{
    int px, py;
    direction_to_leaf(d, &px, &py);
    return py * AR_PG_RES + px;
}

// density (per steradian) of direction d under the quantised cell weights q
AR_HD float mlp_sphere_pdf(const uint8_t* q, float inv_total, V3 d)
{
    const float p = ((float)q[mlp_cell(d)] + AR_MLP_CELL_FLOOR) * inv_total;
    return p * (float)(AR_PG_RES2 / (4.0 * 3.14159265358979323846));
}

AR_HD float mlp_total(const uint8_t* q)
{
    float t = 0.0f;
    for (int i = 0; i < AR_MLP_OUT; ++i) t += (float)q[i] + AR_MLP_CELL_FLOOR;
    return t;
}

AR_HD float mlp_hemisphere_pdf(const uint8_t* q, float inv_total, V3 d, V3 n)
{
    if (dot(d, n) <= 0.0f) return 0.0f;
    return mlp_sphere_pdf(q, inv_total, d) + mlp_sphere_pdf(q, inv_total, reflect_hemisphere(d, n));
}

template <typename Rand>
AR_HD GuideSample mlp_sample_hemisphere(const uint8_t* q, float total, Rand& rand, V3 n)
{
    const float u = rand() * total;
    int cell = AR_MLP_OUT - 1;
    float acc = 0.0f;
    for (int i = 0; i < AR_MLP_OUT; ++i)
    {
        acc += (float)q[i] + AR_MLP_CELL_FLOOR;
        if (u <= acc)
        {
            cell = i;
            break;
        }
    }
    const float px = ((float)(cell % AR_PG_RES) + rand()) * (1.0f / AR_PG_RES);
    const float py = ((float)(cell / AR_PG_RES) + rand()) * (1.0f / AR_PG_RES);
    GuideSample s;
    s.dir = uv_to_sphere(fminf(px, 1.0f), fminf(py, 1.0f));
    const float inv_total = 1.0f / total;
    const V3 m = reflect_hemisphere(s.dir, n);
    s.pdf = mlp_sphere_pdf(q, inv_total, s.dir) + mlp_sphere_pdf(q, inv_total, m);
    if (dot(s.dir, n) < 0.0f) s.dir = m;
    return s;
}
} // namespace ar
