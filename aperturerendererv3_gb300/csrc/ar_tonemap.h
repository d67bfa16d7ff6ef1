// Display transform of the headless output (core/tonemap.cuh:6-139): linear
// CIE XYZ -> linear sRGB (D65), then the reference's ACES fit (RRT + ODT
// approximation with the dim-surround and desaturation steps) or a plain
// gamma, then clamp to [0, 1].  Host + device.  The matrices and curve
// coefficients are colour-science constants and stay as the reference has them.
#pragma once
#include "ar_vec.h"

#define AR_TONE_ACES 0
#define AR_TONE_GAMMA 1
#define AR_TONE_LINEAR 2

namespace ar
{
struct M3r
{
    float m[9];
};

AR_HD V3 mul3(const M3r& a, V3 x)
{
    return v3(a.m[0] * x.x + a.m[1] * x.y + a.m[2] * x.z, a.m[3] * x.x + a.m[4] * x.y + a.m[5] * x.z,
              a.m[6] * x.x + a.m[7] * x.y + a.m[8] * x.z);
}

AR_HD V3 gamma22(V3 c)
{
    return v3(arm_powf(fmaxf(c.x, 0.0f), 1.0f / 2.2f), arm_powf(fmaxf(c.y, 0.0f), 1.0f / 2.2f),
              arm_powf(fmaxf(c.z, 0.0f), 1.0f / 2.2f));
}

// XYZ2SRGBLinearD65 (core/tonemap.cuh:115-125)
AR_HD V3 xyz_to_srgb_linear(V3 xyz)
{
    const M3r m{{3.2406f, -1.5372f, -0.4986f, -0.9689f, 1.8758f, 0.0415f, 0.0557f, -0.204f, 1.057f}};
    return vmax(mul3(m, xyz), 0.0f);
}

// darkSurround_to_dimSurround (core/tonemap.cuh:45-65): xyY luminance to the power 0.9811
AR_HD V3 dim_surround(V3 linearCV)
{
    const M3r ap1_2_xyz{{0.6624541811f, 0.1340042065f, 0.1561876870f, 0.2722287168f, 0.6740817658f, 0.0536895174f,
                         -0.0055746495f, 0.0040607335f, 1.0103391003f}};
    V3 xyz = mul3(ap1_2_xyz, linearCV);
    const float div = fmaxf(xyz.x + xyz.y + xyz.z, 1.0e-4f);
    float x = xyz.x / div, y = xyz.y / div, Y = xyz.y;
    Y = arm_powf(fminf(fmaxf(Y, 0.0f), 65504.0f), 0.9811f);
    const float m = Y / fmaxf(y, 1e-4f);
    xyz = v3(x * m, Y, (1.0f - x - y) * m);
    const M3r xyz_2_ap1{{1.6410233797f, -0.3248032942f, -0.2364246952f, -0.6636628587f, 1.6153315917f, 0.0167563477f,
                         0.0117218943f, -0.0082844420f, 0.9883948585f}};
    return mul3(xyz_2_ap1, xyz);
}

// ACES (core/tonemap.cuh:67-112) on linear sRGB
AR_HD V3 aces(V3 c)
{
    const M3r srgb_2_ap0{{0.4397010f, 0.3829780f, 0.1773350f, 0.0897923f, 0.8134230f, 0.0967616f, 0.0175440f,
                          0.1115440f, 0.8707040f}};
    const M3r ap0_2_ap1{{1.4514393161f, -0.2365107469f, -0.2149285693f, -0.0765537734f, 1.1762296998f, -0.0996759264f,
                         0.0083161484f, -0.0060324498f, 0.9977163014f}};
    const M3r ap1_2_xyz{{0.6624541811f, 0.1340042065f, 0.1561876870f, 0.2722287168f, 0.6740817658f, 0.0536895174f,
                         -0.0055746495f, 0.0040607335f, 1.0103391003f}};
    const M3r d60_2_d65{{0.98722400f, -0.00611327f, 0.0159533f, -0.00759836f, 1.00186000f, 0.0053302f, 0.00307257f,
                         -0.00509595f, 1.0816800f}};
    const M3r xyz_2_rec709{{3.2409699419f, -1.5373831776f, -0.4986107603f, -0.9692436363f, 1.8759675015f,
                            0.0415550574f, 0.0556300797f, -0.2039769589f, 1.0569715142f}};
    const V3 y_w = v3(0.272229f, 0.674082f, 0.0536895f);
    V3 acescg = mul3(ap0_2_ap1, mul3(srgb_2_ap0, c));
    float t = dot(acescg, y_w);
    acescg = v3(lerpf(t, acescg.x, 0.96f), lerpf(t, acescg.y, 0.96f), lerpf(t, acescg.z, 0.96f));
    const float a = 278.5085f, b = 10.7772f, cc = 293.6045f, d = 88.7122f, e = 80.6889f;
    V3 post;
    post.x = (acescg.x * (acescg.x * a + b)) / (acescg.x * (acescg.x * cc + d) + e);
    post.y = (acescg.y * (acescg.y * a + b)) / (acescg.y * (acescg.y * cc + d) + e);
    post.z = (acescg.z * (acescg.z * a + b)) / (acescg.z * (acescg.z * cc + d) + e);
    V3 lin = dim_surround(post);
    t = dot(lin, y_w);
    lin = v3(lerpf(t, lin.x, 0.93f), lerpf(t, lin.y, 0.93f), lerpf(t, lin.z, 0.93f));
    const V3 xyz = mul3(d60_2_d65, mul3(ap1_2_xyz, lin));
    return gamma22(vmax(mul3(xyz_2_rec709, xyz), 0.0f));
}

// one pixel: XYZ x exposure -> display RGB in [0, 1]
AR_HD V3 tonemap_pixel(V3 xyz, float exposure, int tone)
{
    const V3 rgb = xyz_to_srgb_linear(xyz * exposure);
    V3 out;
    if (tone == AR_TONE_ACES) out = aces(rgb);
    else if (tone == AR_TONE_GAMMA) out = gamma22(rgb);
    else out = rgb;
    return v3(saturate(out.x), saturate(out.y), saturate(out.z));
}
} // namespace ar
