// Spectral (hero-wavelength) helpers: wavelength sampling, CIE / D65 lookups,
// RGB -> 4-term basis upsampling through the 512^3 LUT, and the two residual
// MLPs that build the LUTs.  Host + device; every formula keeps the reference's
// operation order so results match it bit for bit:
//   sampling      core/spectrum/sample_ciexyz.cuh:29-326 (ndtrif, SampleCIE1931)
//   CIE / D65     core/spectrum/ciexyz.cuh:67-85, 522-541
//   LUT queries   core/spectrum/spectrum_lut.cuh:93-235
//   encoders      core/spectrum/spectrum_basis.cuh:2262-2469, core/tensor/tensor.cuh:104-183
// Table data (CMFs, D65, MLP weights) comes from data/spectral_tables.npz.
#pragma once
#include "ar_vec.h"

#define AR_LUT_RES 512
#define AR_LAMBDA_LUT_RES 840
#define AR_BASIS 4
#define AR_CIE_COUNT 421

namespace ar
{
// Layout of the MLP weight block (floats):
//   RGB: IN_W[32x32] IN_B[32] {BLKi_W[32x32] BLKi_B[32]} x7 OUT_W[4x32]
//   LAM: {BLKi_W BLKi_B} x7 OUT_W[4x32]
#define AR_RGB_MLP_FLOATS (1024 + 32 + 7 * (1024 + 32) + 128)
#define AR_LAM_MLP_FLOATS (7 * (1024 + 32) + 128)

struct Basis
{
    float k[AR_BASIS];
};

// y = W x + b with W row-major [To][From]; accumulation j = 0..From-1 with fma
template <int From, int To, bool Bias, bool Relu>
AR_HD void linear(const float* x, float* y, const float* W, const float* b)
{
    for (int i = 0; i < To; ++i)
    {
        float acc = Bias ? b[i] : 0.0f;
        for (int j = 0; j < From; ++j) acc = fmaf(x[j], W[i * From + j], acc);
        y[i] = Relu ? fmaxf(acc, 0.0f) : acc;
    }
}

AR_HD void residual_block(float* h, const float* W, const float* b)
{
    float t[32];
    linear<32, 32, true, true>(h, t, W, b);
    for (int i = 0; i < 32; ++i) h[i] = h[i] + t[i];
}

#define AR_PI_F 3.141592654f

// RGB in [0,1]^3 -> basis (the value PrecomputeRGBLUTKernel stores per voxel)
AR_HD void rgb_encode(const float* in3, float* outK, const float* w)
{
    const float scale = fmaxf(fmaxf(in3[0], in3[1]), in3[2]);
    const float scaleEps = scale + 0.001f;
    const float scaleEpsInv = 1.0f / scaleEps;
    float s[32];
    for (int c = 0; c < 3; ++c)
        for (int k = 0; k < 4; ++k)
        {
            const float phase = in3[c] * scaleEpsInv * AR_PI_F * static_cast<float>(k + 1);
            arm_sincosf(phase, &s[k + 8 * c], &s[k + 4 + 8 * c]);
        }
    for (int k = 0; k < 4; ++k)
    {
        const float phase = scale * AR_PI_F * static_cast<float>(k + 1);
        arm_sincosf(phase, &s[k + 24], &s[k + 28]);
    }
    float h[32];
    linear<32, 32, true, true>(s, h, w, w + 1024);
    const float* p = w + 1024 + 32;
    for (int blk = 0; blk < 7; ++blk, p += 1024 + 32) residual_block(h, p, p + 1024);
    linear<32, 4, false, false>(h, outK, p, nullptr);
    for (int i = 0; i < 4; ++i) outK[i] *= scale;
}

// wavelength (nm) -> basis
AR_HD void lambda_encode(float lambda, float* outK, const float* w)
{
    const float x = fminf(fmaxf((lambda - 360.0f) / (780.0f - 360.0f), 0.0f), 1.0f);
    float h[32];
    for (int k = 0; k < 16; ++k)
    {
        const float phase = x * AR_PI_F * static_cast<float>(k + 1);
        arm_sincosf(phase, &h[k], &h[k + 16]);
    }
    const float* p = w;
    for (int blk = 0; blk < 7; ++blk, p += 1024 + 32) residual_block(h, p, p + 1024);
    linear<32, 4, false, false>(h, outK, p, nullptr);
}

AR_HD float spectral_interact(const float* rgbK, const float* lamK)
{
    float acc = 0.0f;
    for (int i = 0; i < AR_BASIS; ++i) acc = fmaf(rgbK[i], lamK[i], acc);
    return fminf(fmaxf(acc, 0.0f), 1.0f);
}

AR_HD void linear_coord(float g, int res, int& i0, int& i1, float& t)
{
    const float fi0 = floorf(g);
    i0 = static_cast<int>(fi0);
    i1 = i0 + 1;
    if (i1 >= res) i1 = res - 1;
    t = g - fi0;
    if (i0 == i1) t = 0.0f;
}

// lattice index of LUT voxel (x, y, z), in float4 units
AR_HD size_t lut_voxel(int x, int y, int z)
{
    return ((size_t)z * AR_LUT_RES + (size_t)y) * AR_LUT_RES + (size_t)x;
}

// Trilinear LUT query; lut is RES^3 float4 (basis per voxel).
template <typename Fetch>
AR_HD Basis query_rgb_basis_f(V3 rgb, const Fetch& fetch)
{
    Basis r;
    for (int i = 0; i < 4; ++i) r.k[i] = 0.0f;
    const float RES = static_cast<float>(AR_LUT_RES);
    float gx = rgb.x * RES - 0.5f;
    float gy = rgb.y * RES - 0.5f;
    float gz = rgb.z * RES - 0.5f;
    const float maxC = RES - 1.0f;
    gx = fminf(fmaxf(gx, 0.0f), maxC);
    gy = fminf(fmaxf(gy, 0.0f), maxC);
    gz = fminf(fmaxf(gz, 0.0f), maxC);
    int x0, x1, y0, y1, z0, z1;
    float tx, ty, tz;
    linear_coord(gx, AR_LUT_RES, x0, x1, tx);
    linear_coord(gy, AR_LUT_RES, y0, y1, ty);
    linear_coord(gz, AR_LUT_RES, z0, z1, tz);
    const float wx0 = 1.0f - tx, wx1 = tx;
    const float wy0 = 1.0f - ty, wy1 = ty;
    const float wz0 = 1.0f - tz, wz1 = tz;
    const float w[8] = {wx0 * wy0 * wz0, wx1 * wy0 * wz0, wx0 * wy1 * wz0, wx1 * wy1 * wz0,
                        wx0 * wy0 * wz1, wx1 * wy0 * wz1, wx0 * wy1 * wz1, wx1 * wy1 * wz1};
    const int xs[8] = {x0, x1, x0, x1, x0, x1, x0, x1};
    const int ys[8] = {y0, y0, y1, y1, y0, y0, y1, y1};
    const int zs[8] = {z0, z0, z0, z0, z1, z1, z1, z1};
    for (int c = 0; c < 8; ++c)
    {
        float v[4];
        fetch(lut_voxel(xs[c], ys[c], zs[c]), v);
        for (int i = 0; i < 4; ++i) r.k[i] = fmaf(w[c], v[i], r.k[i]);
    }
    return r;
}

struct PlainFetch
{
    const float* lut;
    AR_HD void operator()(size_t voxel, float* v) const
    {
        const float* p = lut + voxel * 4;
        v[0] = p[0]; v[1] = p[1]; v[2] = p[2]; v[3] = p[3];
    }
};

AR_HD Basis query_lambda(float lambdaNm, const float* lutLam)
{
    Basis r;
    const float RES = static_cast<float>(AR_LAMBDA_LUT_RES);
    float u = (lambdaNm - 360.0f) / (780.0f - 360.0f);
    u = fminf(fmaxf(u, 0.0f), 1.0f);
    float g = u * RES - 0.5f;
    const float maxG = RES - 1.0f;
    g = fminf(fmaxf(g, 0.0f), maxG);
    int i0, i1;
    float t;
    linear_coord(g, AR_LAMBDA_LUT_RES, i0, i1, t);
    const float w0 = 1.0f - t;
    const float w1 = t;
    const float* a = lutLam + i0 * 4;
    const float* b = lutLam + i1 * 4;
    for (int i = 0; i < 4; ++i) r.k[i] = a[i] * w0 + b[i] * w1;
    return r;
}

// Colour of a material slot prepared for interaction: the basis of rgb (or of
// rgb / max(rgb) when max(rgb) > 1) and the scale max(rgb) (or 1).
struct SpecColor
{
    float k[4];
    float scale;
    int scaled;  // 1 when max(rgb) > 1
};

template <typename Fetch>
AR_HD SpecColor prepare_color(V3 rgb, const Fetch& fetch)
{
    SpecColor c;
    const float lum = max3(rgb);
    Basis b;
    if (lum > 1.0f)
    {
        b = query_rgb_basis_f(rgb / lum, fetch);
        c.scale = lum;
        c.scaled = 1;
    }
    else
    {
        b = query_rgb_basis_f(rgb, fetch);
        c.scale = 1.0f;
        c.scaled = 0;
    }
    for (int i = 0; i < 4; ++i) c.k[i] = b.k[i];
    return c;
}

// spectrum::lut::Interact on a prepared colour
AR_HD float interact(const SpecColor& c, const Basis& lam)
{
    const float q = spectral_interact(c.k, lam.k);
    return c.scaled ? q * c.scale : q;
}

template <typename Fetch>
AR_HD float interact_rgb(const Basis& lam, V3 rgb, const Fetch& fetch)
{
    return interact(prepare_color(rgb, fetch), lam);
}

// Gradient of interact_rgb(lam, rgb) with respect to rgb: the trilinear
// interpolation differentiated inside its cell, zero where a clamp is active
// (the lattice edges, the [0, 1] clamp of the interaction).  When max(rgb) > 1
// the colour is interacted as max(rgb) * q(rgb / max(rgb)), and the chain rule
// runs through both factors.
template <typename Fetch>
AR_HD V3 interact_rgb_grad(const Basis& lam, V3 rgb, const Fetch& fetch)
{
    const float lum = max3(rgb);
    const bool scaled = lum > 1.0f;
    const V3 u = scaled ? rgb / lum : rgb;
    const float RES = static_cast<float>(AR_LUT_RES);
    const float maxC = RES - 1.0f;
    const float g[3] = {u.x * RES - 0.5f, u.y * RES - 0.5f, u.z * RES - 0.5f};
    int lo[3], hi[3];
    float t[3], dg[3];
    for (int a = 0; a < 3; ++a)
    {
        const float gc = fminf(fmaxf(g[a], 0.0f), maxC);
        linear_coord(gc, AR_LUT_RES, lo[a], hi[a], t[a]);
        dg[a] = (g[a] > 0.0f && g[a] < maxC && lo[a] != hi[a]) ? RES : 0.0f;
    }
    float q = 0.0f, dq[3] = {0.0f, 0.0f, 0.0f};
    for (int c = 0; c < 8; ++c)
    {
        const int bx = c & 1, by = (c >> 1) & 1, bz = (c >> 2) & 1;
        float v[4];
        fetch(lut_voxel(bx ? hi[0] : lo[0], by ? hi[1] : lo[1], bz ? hi[2] : lo[2]), v);
        float sc = 0.0f;
        for (int i = 0; i < AR_BASIS; ++i) sc += v[i] * lam.k[i];
        const float wx = bx ? t[0] : 1.0f - t[0];
        const float wy = by ? t[1] : 1.0f - t[1];
        const float wz = bz ? t[2] : 1.0f - t[2];
        q += wx * wy * wz * sc;
        dq[0] += (bx ? 1.0f : -1.0f) * wy * wz * sc;
        dq[1] += (by ? 1.0f : -1.0f) * wx * wz * sc;
        dq[2] += (bz ? 1.0f : -1.0f) * wx * wy * sc;
    }
    const float on = (q > 0.0f && q < 1.0f) ? 1.0f : 0.0f;
    V3 gq = v3(dq[0] * dg[0] * on, dq[1] * dg[1] * on, dq[2] * dg[2] * on);
    if (!scaled) return gq;
    // f = lum * clamp(q(rgb / lum)), lum = rgb[m]
    const float qc = fminf(fmaxf(q, 0.0f), 1.0f);
    const float extra = qc - (gq.x * u.x + gq.y * u.y + gq.z * u.z);
    const int m = (rgb.x >= rgb.y && rgb.x >= rgb.z) ? 0 : (rgb.y >= rgb.z ? 1 : 2);
    if (m == 0) gq.x += extra;
    else if (m == 1) gq.y += extra;
    else gq.z += extra;
    return gq;
}

// ---------------------------------------------------------------- sampling
AR_HD float ndtrif(float u, float (*erfc_fn)(float) = nullptr)
{
    (void)erfc_fn;
    u = clampf(u, 0.0f, 1.0f);
    const float uu = u;
    const float a0 = -3.969683028665376e+01f, a1 = 2.209460984245205e+02f, a2 = -2.759285104469687e+02f,
                a3 = 1.383577518672690e+02f, a4 = -3.066479806614716e+01f, a5 = 2.506628277459239e+00f;
    const float b0 = -5.447609879822406e+01f, b1 = 1.615858368580409e+02f, b2 = -1.556989798598866e+02f,
                b3 = 6.680131188771972e+01f, b4 = -1.328068155288572e+01f;
    const float c0 = -7.784894002430293e-03f, c1 = -3.223964580411365e-01f, c2 = -2.400758277161838e+00f,
                c3 = -2.549732539343734e+00f, c4 = 4.374664141464968e+00f, c5 = 2.938163982698783e+00f;
    const float d0 = 7.784695709041462e-03f, d1 = 3.224671290700398e-01f, d2 = 2.445134137142996e+00f,
                d3 = 3.754408661907416e+00f;
    const float pLow = 0.02425f;
    const float pHigh = 1.0f - pLow;
    float x;
    if (uu < pLow)
    {
        const float q = sqrtf(-2.0f * arm_logf(uu));
        float num = fmaf(c0, q, c1);
        num = fmaf(num, q, c2);
        num = fmaf(num, q, c3);
        num = fmaf(num, q, c4);
        num = fmaf(num, q, c5);
        float den = fmaf(d0, q, d1);
        den = fmaf(den, q, d2);
        den = fmaf(den, q, d3);
        den = fmaf(den, q, 1.0f);
        x = num / den;
    }
    else if (uu > pHigh)
    {
        const float q = sqrtf(-2.0f * arm_log1pf(-uu));
        float num = fmaf(c0, q, c1);
        num = fmaf(num, q, c2);
        num = fmaf(num, q, c3);
        num = fmaf(num, q, c4);
        num = fmaf(num, q, c5);
        float den = fmaf(d0, q, d1);
        den = fmaf(den, q, d2);
        den = fmaf(den, q, d3);
        den = fmaf(den, q, 1.0f);
        x = -num / den;
    }
    else
    {
        const float q = uu - 0.5f;
        const float r = q * q;
        float num = fmaf(a0, r, a1);
        num = fmaf(num, r, a2);
        num = fmaf(num, r, a3);
        num = fmaf(num, r, a4);
        num = fmaf(num, r, a5);
        num *= q;
        float den = fmaf(b0, r, b1);
        den = fmaf(den, r, b2);
        den = fmaf(den, r, b3);
        den = fmaf(den, r, b4);
        den = fmaf(den, r, 1.0f);
        x = num / den;
    }
    // one Newton step on Phi(x) = u
    const float INV_SQRT_2PI = 0.3989422804014327f;
    const float INV_SQRT2 = 0.7071067811865476f;
    const float expo = arm_expf(fmaf(-0.5f, x * x, 0.0f));
    const float pdf = expo * INV_SQRT_2PI;
    const float cdf = 0.5f * arm_erfcf(-x * INV_SQRT2);
    x -= (cdf - uu) / pdf;
    return 1.0f * x;
}

AR_HD float clamp_lambda(float h)
{
    if (h < 360.0f) h = 360.0f;
    if (h > 780.0f) h = 780.0f;
    return h;
}

AR_HD float sample_cie_x(float uComp, float uInvcdf)
{
    const float alpha0 = 0.8330258723493694f;
    const float mu0 = 595.7999999999999545f, sig0 = 33.3299999999999983f;
    const float Fa0 = 7.4884543e-13f, Fb0 = 0.9999999836707862f;
    const float mu1 = 446.8000000000000114f, sig1 = 19.4400000000000013f;
    const float Fa1 = 0.0000040030528583f, Fb1 = 1.0f;
    float h;
    if (uComp < alpha0)
    {
        const float t0 = Fa0 + uInvcdf * (Fb0 - Fa0);
        h = mu0 + sig0 * ndtrif(t0);
    }
    else
    {
        const float t1 = Fa1 + uInvcdf * (Fb1 - Fa1);
        h = mu1 + sig1 * ndtrif(t1);
    }
    return clamp_lambda(h);
}
AR_HD float sample_cie_y(float u)
{
    const float mu_p = 6.3269327170812479f, sig = 0.0750000000000000f;
    const float Fa = 0.0000000020798312f, Fb = 0.9999953206338883f;
    const float t = Fa + u * (Fb - Fa);
    return clamp_lambda(arm_expf(mu_p + sig * ndtrif(t)));
}
AR_HD float sample_cie_z(float u)
{
    const float mu_p = 6.1114040395252154f, sig = 0.0510000000000000f;
    const float Fa = 0.0000049890553249f, Fb = 1.0f;
    const float t = Fa + u * (Fb - Fa);
    return clamp_lambda(arm_expf(mu_p + sig * ndtrif(t)));
}
AR_HD float pdf_cie_x(float l)
{
    const float k1 = (l - 595.8f) / 33.33f;
    const float k2 = (l - 446.8f) / 19.44f;
    return (1.065f * arm_expf(-0.5f * k1 * k1) + 0.366f * arm_expf(-0.5f * k2 * k2)) / 106.81109281f;
}
AR_HD float pdf_cie_y(float l)
{
    const float k = (arm_logf(l) - 6.3213077f) / 0.075f;
    return (1.014f * arm_expf(-0.5f * k * k)) / 106.34513640f;
}
AR_HD float pdf_cie_z(float l)
{
    const float k = (arm_logf(l) - 6.1088030f) / 0.051f;
    return (1.839f * arm_expf(-0.5f * k * k)) / 105.88243587f;
}

struct LambdaSample
{
    float lambda, pdf;
};

// mixture of uniform + three CIE-lobe fits (weights 0.1 : 1 : 1 : 1)
AR_HD LambdaSample sample_cie1931(float r0, float r1, float r2)
{
    const float total = 0.1f + 1.0f + 1.0f + 1.0f;
    const float uniformRatio = 0.1f / total;
    const float XRatio = 1.0f / total;
    const float YRatio = 1.0f / total;
    const float ZRatio = 1.0f / total;
    // Every lobe is lambda = clamp(T(mu + sig * ndtri(Fa + u (Fb - Fa)))) with T
    // the identity (the two x lobes) or exp (y, z): the lane picks its lobe's
    // constants and all lanes share one inverse-CDF evaluation, instead of a
    // warp running up to four lobe branches one after the other.  Each lane
    // performs the same operations on the same values as sample_cie_x / _y / _z.
    const bool uni = r0 < uniformRatio;
    const bool lx = !uni && r0 < uniformRatio + XRatio;
    const bool ly = !uni && !lx && r0 < uniformRatio + XRatio + YRatio;
    const bool lx0 = r1 < 0.8330258723493694f;  // the x lobe's first component
    float Fa, Fb, mu, sig, u;
    if (lx)
    {
        Fa = lx0 ? 7.4884543e-13f : 0.0000040030528583f;
        Fb = lx0 ? 0.9999999836707862f : 1.0f;
        mu = lx0 ? 595.7999999999999545f : 446.8000000000000114f;
        sig = lx0 ? 33.3299999999999983f : 19.4400000000000013f;
        u = r2;
    }
    else
    {
        Fa = ly ? 0.0000000020798312f : 0.0000049890553249f;
        Fb = ly ? 0.9999953206338883f : 1.0f;
        mu = ly ? 6.3269327170812479f : 6.1114040395252154f;
        sig = ly ? 0.0750000000000000f : 0.0510000000000000f;
        u = r1;
    }
    const float t = Fa + u * (Fb - Fa);
    const float g = mu + sig * ndtrif(t);
    const float h = lx ? g : arm_expf(g);
    const float lambda = uni ? r1 * (780.0f - 360.0f) + 360.0f : clamp_lambda(h);
    const float pMix = uniformRatio * 1.0f / (780.0f - 360.0f) + XRatio * pdf_cie_x(lambda) +
                       YRatio * pdf_cie_y(lambda) + ZRatio * pdf_cie_z(lambda);
    LambdaSample s;
    s.lambda = lambda;
    s.pdf = fmaxf(pMix, 1e-16f);
    return s;
}

AR_HD V3 lambda_to_xyz(float lambda, const float* cmf)
{
    if (lambda <= 360.0f) return v3(cmf[0], cmf[1], cmf[2]);
    if (lambda >= 780.0f) return v3(cmf[3 * 420], cmf[3 * 420 + 1], cmf[3 * 420 + 2]);
    const float u = (lambda - 360.0f) * (1.0f / 1.0f);
    const int i = static_cast<int>(u);
    const float t = u - static_cast<float>(i);
    const float* a = cmf + 3 * i;
    const float* b = a + 3;
    return v3(a[0] + (b[0] - a[0]) * t, a[1] + (b[1] - a[1]) * t, a[2] + (b[2] - a[2]) * t);
}

AR_HD float d65_norm(float lambda, const float* d65)
{
    const float k = 1.0f / 10567.065f;
    if (lambda <= 360.0f) return d65[0] * k;
    if (lambda >= 780.0f) return d65[420] * k;
    const float x = lambda - 360.0f;
    const int i = static_cast<int>(floorf(x));
    const float t = x - static_cast<float>(i);
    const float v0 = d65[i];
    const float v1 = d65[i + 1];
    return (v0 + (v1 - v0) * t) * k;
}

// IOR from Abbe number and dispersion tilt of absorption (core/spectrum/spectrum.cuh:8-62)
AR_HD float ior_from_abbe(float lambda_nm, float nd, float Vd)
{
    const float invF = 1.0f / 486.1327f;
    const float invC = 1.0f / 656.2725f;
    const float invD = 1.0f / 587.5618f;
    if (!(lambda_nm > 0.0f)) return nd;
    const float K = (Vd > 0.0f) ? (nd - 1.0f) / (Vd * (invF - invC)) : 0.0f;
    const float invL = 1.0f / lambda_nm;
    return nd + K * (invL - invD);
}
AR_HD float sigma_a_from_tilt(float sigmaA, float lambda_nm, float sigmaTilt)
{
    const float invF = 1.0f / 486.1327f;
    const float invC = 1.0f / 656.2725f;
    const float invD = 1.0f / 587.5618f;
    const float deltaU = (invF - invC);
    const float u = 1.0f / fmaxf(lambda_nm, 1.0e-6f);
    const float du = (u - invD) / deltaU;
    const float sA = sigmaA * (1.0f + 1.0f * sigmaTilt * du);
    return fmaxf(0.0f, sA);
}
} // namespace ar
