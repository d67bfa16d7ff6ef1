// FP64 CPU oracle of the path tracer.  TEST INFRASTRUCTURE ONLY: tests and
// the benchmark's reference legs call it through oracle/pt64.py; the product
// never links it.
//
// It restates, in double precision, the reference integrator
// CalculateRadiance (core/render/render.cuh:460-999) for the workloads whose
// converged images and gradients are judged against an FP64 oracle:
//   geometry   triangles (watertight test), oriented boxes and spheres
//              (core/object/aabb.cuh:9-89, core/object/sphere.cuh:9-70), a
//              binary median-split BVH with closest-hit ties to the smallest
//              primitive id (core/render/intersection.cuh:73 keeps the first)
//   materials  diffuse, GGX (core/render/material.cuh:48-409,
//              core/render/sample.cuh:62-248) and lights; glass is rejected
//   lights     light table and CDF pick (core/scene.cu:677-706,
//              core/nee/nee.cuh:343-357), box facets and sphere caps
//              (core/nee/nee.cuh:36-310), power-heuristic MIS
//              (core/render/render.cuh:185-343, 647-723)
//   spectrum   hero wavelength from the CIE mixture
//              (core/spectrum/sample_ciexyz.cuh:288-326), CIE/D65 lookups
//              (core/spectrum/ciexyz.cuh:67-85, 522-541), the lambda and RGB
//              LUT queries (core/spectrum/spectrum_lut.cuh:124-235) with
//              lattice values from RGBEncode / LambdaEncode
//              (core/spectrum/spectrum_basis.cuh:2262-2469) evaluated in double
//   path       Russian roulette (core/render/render.cuh:829-859), NEE
//              acceptance, sky (core/render/render.cuh:58-73), XYZ clamp (:967)
//   additions  the smooth-union SDF object (sphere tracing as RaymarchLocal,
//              core/object/sdf/sdf_base.cuh:53-105) and the homogeneous medium
//              in a box (free flights, Henyey-Greenstein phase from
//              core/render/sample.cuh:110-145, box-chord transmittance on NEE),
//              with the replay adjoint of the medium's albedo and emission
// Random numbers come from the same per-sample PCG32 streams as the GPU
// integrator (ar_rng.h), so each oracle sample follows the GPU sample's path
// up to floating-point decisions.  The replay adjoint of albedo textures
// records, per textured diffuse vertex, the radiance gathered before it and
// d(albedo)/d(rgb) / albedo, and forms the gradient once the path's total is
// known (the same estimator derivative the GPU adjoint computes by replay).
#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../aperturerendererv3_gb300/csrc/ar_rng.h"

namespace o64
{
using R = double;
constexpr R PI = 3.14159265358979323846;
constexpr int LUT_RES = 512;
constexpr int LAM_RES = 840;

struct V
{
    R x, y, z;
};
static inline V v(R x, R y, R z) { return V{x, y, z}; }
static inline V operator+(V a, V b) { return v(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline V operator-(V a, V b) { return v(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline V operator-(V a) { return v(-a.x, -a.y, -a.z); }
static inline V operator*(V a, R s) { return v(a.x * s, a.y * s, a.z * s); }
static inline V operator*(R s, V a) { return v(a.x * s, a.y * s, a.z * s); }
static inline V operator/(V a, R s) { return v(a.x / s, a.y / s, a.z / s); }
static inline R dot(V a, V b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline V cross(V a, V b) { return v(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
static inline R length(V a) { return std::sqrt(dot(a, a)); }
static inline V normalize(V a)
{
    const R l2 = dot(a, a);
    if (l2 <= 1e-40) return v(0, 0, 0);
    return a / std::sqrt(l2);
}
static inline R comp(V a, int k) { return k == 0 ? a.x : (k == 1 ? a.y : a.z); }
static inline R max3(V a) { return std::max(a.x, std::max(a.y, a.z)); }
static inline R clampd(R x, R a, R b) { return std::isnan(x) ? 0.0 : std::min(std::max(x, a), b); }
static inline R sat(R x) { return clampd(x, 0.0, 1.0); }
static inline R lerp(R a, R b, R t) { return a * (1.0 - t) + b * t; }
static inline R signd(R a) { return a > 0 ? 1.0 : (a < 0 ? -1.0 : 0.0); }
static inline V reflect(V d, V n) { return d - n * (2.0 * dot(d, n)); }
static inline R inv_safe(R x) { return x == 0.0 ? (std::signbit(x) ? -1e300 : 1e300) : 1.0 / x; }

struct M
{
    V r0, r1, r2;
};
static inline V mul(const M& m, V a) { return v(dot(m.r0, a), dot(m.r1, a), dot(m.r2, a)); }
static inline M mulm(const M& a, const M& b)
{
    const V c0 = v(b.r0.x, b.r1.x, b.r2.x), c1 = v(b.r0.y, b.r1.y, b.r2.y), c2 = v(b.r0.z, b.r1.z, b.r2.z);
    return M{v(dot(a.r0, c0), dot(a.r0, c1), dot(a.r0, c2)), v(dot(a.r1, c0), dot(a.r1, c1), dot(a.r1, c2)),
             v(dot(a.r2, c0), dot(a.r2, c1), dot(a.r2, c2))};
}
static inline M transpose(const M& m)
{
    return M{v(m.r0.x, m.r1.x, m.r2.x), v(m.r0.y, m.r1.y, m.r2.y), v(m.r0.z, m.r1.z, m.r2.z)};
}

// ------------------------------------------------------------------ inputs
enum
{
    OBJ_CUBE = 0,
    OBJ_SPHERE = 1,
    OBJ_SDF = 2,
    OBJ_TRIANGLE = 3,
    MAT_DIFFUSE = 0,
    MAT_LIGHT = 1,
    MAT_GLASS = 2,
    MAT_GGX = 3
};

struct Mat
{
    int shading;
    V albedo, emissive;
    R roughness, metallic, specular;
    int tex;  // -1 none
};

struct Obj
{
    int type;
    V center, extent;
    M o2w, w2o;
};

struct Light
{
    int prim, type, material;
    R select_prob, cdf;
};

struct Tables
{
    std::vector<R> cmf, d65;        // 421 x 3, 421
    std::vector<R> rgb_w, lam_w;    // MLP weights (float data, used in double)
    std::vector<std::array<R, 4>> lam_lut;
};

struct Scene
{
    std::vector<Mat> mats;
    std::vector<Obj> objs;               // analytic objects by primitive id (triangles unused)
    std::vector<int> prim_type, prim_mat;
    std::vector<std::array<R, 9>> tri;   // per primitive (triangles)
    std::vector<std::array<R, 6>> uv;    // per primitive
    std::vector<std::array<R, 3>> lo, hi;
    std::vector<Light> lights;
    std::vector<int> tex_off, tex_w, tex_h;
    std::vector<R> texels;
    Tables tab;
    // smooth-union SDF (primitives: kind, centre, size) and the medium
    std::vector<std::array<R, 7>> sdf;
    R sdf_k = 0;
    R sdf_lo[3] = {0, 0, 0}, sdf_hi[3] = {0, 0, 0};
    // sdf_f32: the SDF march and normal run in float, as a float renderer
    // runs them: positions and steps rounded to float, the field evaluated in
    // float arithmetic.  The central-difference normal (h = 1e-4) divides the
    // field's rounding error by 2h and the march's stopping step can move by
    // one step, so renders with it on and off show how far float arithmetic
    // of the SDF alone moves each sample.
    bool sdf_f32 = false;
    bool med_on = false;
    R med_lo[3] = {0, 0, 0}, med_hi[3] = {0, 0, 0};
    R med_sigma = 0, med_albedo = 0, med_g = 0, med_emission = 0;
    // BVH
    struct Node
    {
        R lo[3], hi[3];
        int left, right, first, count;
    };
    std::vector<Node> nodes;
    std::vector<int> order;
};

// ------------------------------------------------------------------ spectral
// y = W x + b, W row-major [To][From] (core/tensor/tensor.cuh:104-183)
static void linear(const R* x, R* y, const R* W, const R* b, int from, int to, bool relu)
{
    for (int i = 0; i < to; ++i)
    {
        R acc = b ? b[i] : 0.0;
        for (int j = 0; j < from; ++j) acc += x[j] * W[i * from + j];
        y[i] = relu ? std::max(acc, 0.0) : acc;
    }
}

static void residual_stack(R* h, const R*& p)
{
    for (int blk = 0; blk < 7; ++blk, p += 1024 + 32)
    {
        R t[32];
        linear(h, t, p, p + 1024, 32, 32, true);
        for (int i = 0; i < 32; ++i) h[i] += t[i];
    }
}

// RGBEncode (core/spectrum/spectrum_basis.cuh:2273-2407): sin/cos features of
// the normalised colour and of its scale, residual MLP, output times scale
static std::array<R, 4> rgb_encode(const Tables& T, const R in3[3])
{
    const R scale = std::max(in3[0], std::max(in3[1], in3[2]));
    const R inv = 1.0 / (scale + 0.001);
    R s[32];
    for (int c = 0; c < 3; ++c)
        for (int k = 0; k < 4; ++k)
        {
            const R ph = in3[c] * inv * PI * (k + 1);
            s[k + 8 * c] = std::sin(ph);
            s[k + 4 + 8 * c] = std::cos(ph);
        }
    for (int k = 0; k < 4; ++k)
    {
        const R ph = scale * PI * (k + 1);
        s[k + 24] = std::sin(ph);
        s[k + 28] = std::cos(ph);
    }
    const R* w = T.rgb_w.data();
    R h[32];
    linear(s, h, w, w + 1024, 32, 32, true);
    const R* p = w + 1024 + 32;
    residual_stack(h, p);
    std::array<R, 4> o;
    linear(h, o.data(), p, nullptr, 32, 4, false);
    for (auto& q : o) q *= scale;
    return o;
}

// LambdaEncode (core/spectrum/spectrum_basis.cuh:2409-2459)
static std::array<R, 4> lambda_encode(const Tables& T, R lambda)
{
    const R x = std::min(std::max((lambda - 360.0) / (780.0 - 360.0), 0.0), 1.0);
    R h[32];
    for (int k = 0; k < 16; ++k)
    {
        const R ph = x * PI * (k + 1);
        h[k] = std::sin(ph);
        h[k + 16] = std::cos(ph);
    }
    const R* p = T.lam_w.data();
    residual_stack(h, p);
    std::array<R, 4> o;
    linear(h, o.data(), p, nullptr, 32, 4, false);
    return o;
}

// lattice corner values of the RGB LUT, computed on demand per thread
struct LutCache
{
    const Tables* T;
    std::unordered_map<uint32_t, std::array<R, 4>> map;
    const std::array<R, 4>& at(int x, int y, int z)
    {
        const uint32_t key = ((uint32_t)z * LUT_RES + (uint32_t)y) * LUT_RES + (uint32_t)x;
        auto it = map.find(key);
        if (it != map.end()) return it->second;
        const R in3[3] = {(x + 0.5) / LUT_RES, (y + 0.5) / LUT_RES, (z + 0.5) / LUT_RES};
        return map.emplace(key, rgb_encode(*T, in3)).first->second;
    }
};

static void cell(R g, int res, int& i0, int& i1, R& t)
{
    const R f = std::floor(g);
    i0 = (int)f;
    i1 = std::min(i0 + 1, res - 1);
    t = (i0 == i1) ? 0.0 : g - f;
}

// QueryRGBBasis (core/spectrum/spectrum_lut.cuh:124-179) and its gradient in rgb
static std::array<R, 4> rgb_basis(LutCache& L, V rgb, std::array<std::array<R, 4>, 3>* grad)
{
    const R RES = LUT_RES, maxC = RES - 1.0;
    const R g[3] = {rgb.x * RES - 0.5, rgb.y * RES - 0.5, rgb.z * RES - 0.5};
    int lo[3], hi[3];
    R t[3], dg[3];
    for (int a = 0; a < 3; ++a)
    {
        cell(std::min(std::max(g[a], 0.0), maxC), LUT_RES, lo[a], hi[a], t[a]);
        dg[a] = (g[a] > 0.0 && g[a] < maxC && lo[a] != hi[a]) ? RES : 0.0;
    }
    std::array<R, 4> b{0, 0, 0, 0};
    if (grad)
        for (auto& r : *grad) r = {0, 0, 0, 0};
    for (int c = 0; c < 8; ++c)
    {
        const int bx = c & 1, by = (c >> 1) & 1, bz = (c >> 2) & 1;
        const auto& val = L.at(bx ? hi[0] : lo[0], by ? hi[1] : lo[1], bz ? hi[2] : lo[2]);
        const R wx = bx ? t[0] : 1 - t[0], wy = by ? t[1] : 1 - t[1], wz = bz ? t[2] : 1 - t[2];
        for (int i = 0; i < 4; ++i) b[i] += wx * wy * wz * val[i];
        if (grad)
            for (int i = 0; i < 4; ++i)
            {
                (*grad)[0][i] += (bx ? 1 : -1) * wy * wz * val[i] * dg[0];
                (*grad)[1][i] += (by ? 1 : -1) * wx * wz * val[i] * dg[1];
                (*grad)[2][i] += (bz ? 1 : -1) * wx * wy * val[i] * dg[2];
            }
    }
    return b;
}

// Interact (core/spectrum/spectrum_lut.cuh:222-235, spectrum_basis.cuh:2461-2469):
// the colour's spectral value at the path's wavelength; optional d/d(rgb)
static R interact(LutCache& L, const std::array<R, 4>& lam, V rgb, V* grad)
{
    const R lum = max3(rgb);
    const bool scaled = lum > 1.0;
    const V u = scaled ? rgb / lum : rgb;
    std::array<std::array<R, 4>, 3> gb;
    const auto b = rgb_basis(L, u, grad ? &gb : nullptr);
    R q = 0;
    for (int i = 0; i < 4; ++i) q += b[i] * lam[i];
    const R qc = std::min(std::max(q, 0.0), 1.0);
    if (grad)
    {
        const R on = (q > 0.0 && q < 1.0) ? 1.0 : 0.0;
        R gq[3];
        for (int a = 0; a < 3; ++a)
        {
            R s = 0;
            for (int i = 0; i < 4; ++i) s += gb[a][i] * lam[i];
            gq[a] = s * on;
        }
        if (scaled)
        {
            const R extra = qc - (gq[0] * u.x + gq[1] * u.y + gq[2] * u.z);
            const int m = (rgb.x >= rgb.y && rgb.x >= rgb.z) ? 0 : (rgb.y >= rgb.z ? 1 : 2);
            gq[m] += extra;
        }
        *grad = v(gq[0], gq[1], gq[2]);
    }
    return scaled ? qc * lum : qc;
}

// QueryLambda (core/spectrum/spectrum_lut.cuh:181-220)
static std::array<R, 4> query_lambda(const Tables& T, R lambda)
{
    R u = std::min(std::max((lambda - 360.0) / (780.0 - 360.0), 0.0), 1.0);
    const R g = std::min(std::max(u * LAM_RES - 0.5, 0.0), (R)(LAM_RES - 1));
    int i0, i1;
    R t;
    cell(g, LAM_RES, i0, i1, t);
    std::array<R, 4> r;
    for (int i = 0; i < 4; ++i) r[i] = T.lam_lut[i0][i] * (1 - t) + T.lam_lut[i1][i] * t;
    return r;
}

static V lambda_to_xyz(const Tables& T, R lambda)
{
    const R* c = T.cmf.data();
    if (lambda <= 360.0) return v(c[0], c[1], c[2]);
    if (lambda >= 780.0) return v(c[3 * 420], c[3 * 420 + 1], c[3 * 420 + 2]);
    const R u = lambda - 360.0;
    const int i = (int)u;
    const R t = u - i;
    const R* a = c + 3 * i;
    const R* b = a + 3;
    return v(a[0] + (b[0] - a[0]) * t, a[1] + (b[1] - a[1]) * t, a[2] + (b[2] - a[2]) * t);
}

static R d65_norm(const Tables& T, R lambda)
{
    const R k = 1.0 / 10567.065;
    if (lambda <= 360.0) return T.d65[0] * k;
    if (lambda >= 780.0) return T.d65[420] * k;
    const R x = lambda - 360.0;
    const int i = (int)std::floor(x);
    const R t = x - i;
    return (T.d65[i] + (T.d65[i + 1] - T.d65[i]) * t) * k;
}

// inverse standard normal CDF: Acklam's rational start, two Halley steps on erfc
static R ndtri(R u)
{
    u = std::min(std::max(u, 1e-300), 1.0 - 1e-16);
    static const R a[6] = {-3.969683028665376e+01, 2.209460984245205e+02, -2.759285104469687e+02,
                           1.383577518672690e+02, -3.066479806614716e+01, 2.506628277459239e+00};
    static const R b[5] = {-5.447609879822406e+01, 1.615858368580409e+02, -1.556989798598866e+02,
                           6.680131188771972e+01, -1.328068155288572e+01};
    static const R c[6] = {-7.784894002430293e-03, -3.223964580411365e-01, -2.400758277161838e+00,
                           -2.549732539343734e+00, 4.374664141464968e+00, 2.938163982698783e+00};
    static const R d[4] = {7.784695709041462e-03, 3.224671290700398e-01, 2.445134137142996e+00,
                           3.754408661907416e+00};
    R x;
    if (u < 0.02425)
    {
        const R q = std::sqrt(-2 * std::log(u));
        x = (((((c[0] * q + c[1]) * q + c[2]) * q + c[3]) * q + c[4]) * q + c[5]) /
            ((((d[0] * q + d[1]) * q + d[2]) * q + d[3]) * q + 1);
    }
    else if (u > 1 - 0.02425)
    {
        const R q = std::sqrt(-2 * std::log(1 - u));
        x = -(((((c[0] * q + c[1]) * q + c[2]) * q + c[3]) * q + c[4]) * q + c[5]) /
            ((((d[0] * q + d[1]) * q + d[2]) * q + d[3]) * q + 1);
    }
    else
    {
        const R q = u - 0.5, r = q * q;
        x = (((((a[0] * r + a[1]) * r + a[2]) * r + a[3]) * r + a[4]) * r + a[5]) * q /
            (((((b[0] * r + b[1]) * r + b[2]) * r + b[3]) * r + b[4]) * r + 1);
    }
    for (int it = 0; it < 2; ++it)
    {
        const R e = 0.5 * std::erfc(-x / std::sqrt(2.0)) - u;
        const R g = e * std::sqrt(2 * PI) * std::exp(x * x / 2);
        x = x - g / (1 + x * g / 2);
    }
    return x;
}

static R clamp_lambda(R h) { return std::min(std::max(h, 360.0), 780.0); }

// SampleCIE1931: 0.1 uniform + three lobe fits (core/spectrum/sample_ciexyz.cuh:198-326)
static void sample_lambda(R r0, R r1, R r2, R* lambda, R* pdf)
{
    const R total = 3.1, uR = 0.1 / total, xR = 1.0 / total, yR = 1.0 / total, zR = 1.0 / total;
    R l;
    if (r0 < uR) l = r1 * (780.0 - 360.0) + 360.0;
    else if (r0 < uR + xR)
    {
        if (r1 < 0.8330258723493694)
        {
            const R Fa = 7.4884543e-13, Fb = 0.9999999836707862;
            l = clamp_lambda(595.8 + 33.33 * ndtri(Fa + r2 * (Fb - Fa)));
        }
        else
        {
            const R Fa = 0.0000040030528583, Fb = 1.0;
            l = clamp_lambda(446.8 + 19.44 * ndtri(Fa + r2 * (Fb - Fa)));
        }
    }
    else if (r0 < uR + xR + yR)
    {
        const R Fa = 0.0000000020798312, Fb = 0.9999953206338883;
        l = clamp_lambda(std::exp(6.3269327170812479 + 0.075 * ndtri(Fa + r1 * (Fb - Fa))));
    }
    else
    {
        const R Fa = 0.0000049890553249, Fb = 1.0;
        l = clamp_lambda(std::exp(6.1114040395252154 + 0.051 * ndtri(Fa + r1 * (Fb - Fa))));
    }
    const R k1 = (l - 595.8) / 33.33, k2 = (l - 446.8) / 19.44;
    const R px = (1.065 * std::exp(-0.5 * k1 * k1) + 0.366 * std::exp(-0.5 * k2 * k2)) / 106.81109281;
    const R ky = (std::log(l) - 6.3213077) / 0.075;
    const R py = (1.014 * std::exp(-0.5 * ky * ky)) / 106.34513640;
    const R kz = (std::log(l) - 6.1088030) / 0.051;
    const R pz = (1.839 * std::exp(-0.5 * kz * kz)) / 105.88243587;
    *lambda = l;
    *pdf = std::max(uR / (780.0 - 360.0) + xR * px + yR * py + zR * pz, 1e-16);
}

// ------------------------------------------------------------------ geometry
struct Hit
{
    bool hit = false;
    int prim = -1;
    R t = 0;
    V pos{0, 0, 0}, nrm{0, 0, 0};
};

// watertight ray/triangle (Woop, Benthin, Wald 2013); t in [tmin, tmax)
static bool tri_hit(const std::array<R, 9>& T, V o, V d, R* tout)
{
    int kz = 0;
    if (std::fabs(d.y) > std::fabs(comp(d, kz))) kz = 1;
    if (std::fabs(d.z) > std::fabs(comp(d, kz))) kz = 2;
    int kx = (kz + 1) % 3, ky = (kx + 1) % 3;
    if (comp(d, kz) < 0) std::swap(kx, ky);
    const R Sx = comp(d, kx) / comp(d, kz), Sy = comp(d, ky) / comp(d, kz), Sz = 1.0 / comp(d, kz);
    const V A = v(T[0], T[1], T[2]) - o, B = v(T[3], T[4], T[5]) - o, C = v(T[6], T[7], T[8]) - o;
    const R Ax = comp(A, kx) - Sx * comp(A, kz), Ay = comp(A, ky) - Sy * comp(A, kz);
    const R Bx = comp(B, kx) - Sx * comp(B, kz), By = comp(B, ky) - Sy * comp(B, kz);
    const R Cx = comp(C, kx) - Sx * comp(C, kz), Cy = comp(C, ky) - Sy * comp(C, kz);
    const R U = Cx * By - Cy * Bx, W0 = Ax * Cy - Ay * Cx, W = Bx * Ay - By * Ax;
    if ((U < 0 || W0 < 0 || W < 0) && (U > 0 || W0 > 0 || W > 0)) return false;
    const R det = U + W0 + W;
    if (det == 0) return false;
    const R Tt = U * Sz * comp(A, kz) + W0 * Sz * comp(B, kz) + W * Sz * comp(C, kz);
    *tout = Tt / det;
    return true;
}

static bool box_hit(V o, V d, const Obj& ob, Hit* h, bool full)
{
    const V lo = mul(ob.w2o, o - ob.center);
    const V ld = normalize(mul(ob.w2o, d));
    const V div = v(inv_safe(ld.x), inv_safe(ld.y), inv_safe(ld.z));
    const V t1 = v((-ob.extent.x - lo.x) * div.x, (-ob.extent.y - lo.y) * div.y, (-ob.extent.z - lo.z) * div.z);
    const V t2 = v((ob.extent.x - lo.x) * div.x, (ob.extent.y - lo.y) * div.y, (ob.extent.z - lo.z) * div.z);
    const R tEnter = std::max(std::max(std::min(t1.x, t2.x), std::min(t1.y, t2.y)), std::min(t1.z, t2.z));
    const R tExit = std::min(std::min(std::max(t1.x, t2.x), std::max(t1.y, t2.y)), std::max(t1.z, t2.z));
    if (tEnter > tExit || tExit <= 0) return false;
    const bool inside = tEnter < 0;
    const R t = inside ? tExit : tEnter;
    h->t = t;
    if (!full) return true;
    const V lp = lo + ld * t;
    h->pos = mul(ob.o2w, lp) + ob.center;
    const R rx = std::fabs(lp.x) / ob.extent.x, ry = std::fabs(lp.y) / ob.extent.y, rz = std::fabs(lp.z) / ob.extent.z;
    V ln;
    if (rx >= ry && rx >= rz) ln = v(lp.x > 0 ? 1 : -1, 0, 0);
    else if (ry >= rz) ln = v(0, lp.y > 0 ? 1 : -1, 0);
    else ln = v(0, 0, lp.z > 0 ? 1 : -1);
    if (inside) ln = -ln;
    h->nrm = normalize(mul(ob.o2w, ln));
    return true;
}

static bool sphere_hit(V o, V d, const Obj& ob, Hit* h, bool full)
{
    const V lo = mul(ob.w2o, o - ob.center);
    const V ld = normalize(mul(ob.w2o, d));
    const R r = max3(ob.extent);
    const R b = dot(lo, ld), c = dot(lo, lo) - r * r, disc = b * b - c;
    if (disc < 0) return false;
    const R s = std::sqrt(disc);
    R t = -b - s;
    bool inside = false;
    if (t <= 0)
    {
        t = -b + s;
        inside = true;
    }
    if (t <= 0) return false;
    h->t = t;
    if (!full) return true;
    const V lp = lo + ld * t;
    h->pos = mul(ob.o2w, lp) + ob.center;
    h->nrm = normalize(mul(ob.o2w, normalize(lp) * (inside ? -1.0 : 1.0)));
    return true;
}

// ---- smooth-union SDF
static R sdf_prim(const std::array<R, 7>& q, V p)
{
    const V c = v(q[1], q[2], q[3]);
    const V x = p - c;
    const int kind = (int)q[0];
    if (kind == 0) return length(x) - q[4];
    if (kind == 1)
    {
        const V d = v(std::fabs(x.x) - q[4], std::fabs(x.y) - q[5], std::fabs(x.z) - q[6]);
        const V dp = v(std::max(d.x, 0.0), std::max(d.y, 0.0), std::max(d.z, 0.0));
        return length(dp) + std::min(std::max(d.x, std::max(d.y, d.z)), 0.0);
    }
    const R rxz = std::sqrt(x.x * x.x + x.z * x.z) - q[4];
    return std::sqrt(rxz * rxz + x.y * x.y) - q[5];
}

static R sdf_eval(const Scene& S, V p)
{
    R d = sdf_prim(S.sdf[0], p);
    for (size_t i = 1; i < S.sdf.size(); ++i)
    {
        const R b = sdf_prim(S.sdf[i], p);
        const R h = std::max(S.sdf_k - std::fabs(d - b), 0.0) / S.sdf_k;
        d = std::min(d, b) - h * h * S.sdf_k * 0.25;
    }
    return d;
}

static R to_f32(R x) { return (R)(float)x; }
static V to_f32(V p) { return v(to_f32(p.x), to_f32(p.y), to_f32(p.z)); }

// sdf_prim and sdf_eval in float arithmetic (same operations and order)
static float sdf_prim_f(const std::array<R, 7>& q, float px, float py, float pz)
{
    const float x = px - (float)q[1], y = py - (float)q[2], z = pz - (float)q[3];
    const int kind = (int)q[0];
    if (kind == 0) return std::sqrt(x * x + y * y + z * z) - (float)q[4];
    if (kind == 1)
    {
        const float dx = std::fabs(x) - (float)q[4], dy = std::fabs(y) - (float)q[5], dz = std::fabs(z) - (float)q[6];
        const float ex = std::max(dx, 0.0f), ey = std::max(dy, 0.0f), ez = std::max(dz, 0.0f);
        return std::sqrt(ex * ex + ey * ey + ez * ez) + std::min(std::max(dx, std::max(dy, dz)), 0.0f);
    }
    const float rxz = std::sqrt(x * x + z * z) - (float)q[4];
    return std::sqrt(rxz * rxz + y * y) - (float)q[5];
}

static float sdf_eval_f(const Scene& S, float px, float py, float pz)
{
    const float k = (float)S.sdf_k;
    float d = sdf_prim_f(S.sdf[0], px, py, pz);
    for (size_t i = 1; i < S.sdf.size(); ++i)
    {
        const float b = sdf_prim_f(S.sdf[i], px, py, pz);
        const float h = std::max(k - std::fabs(d - b), 0.0f) / k;
        d = std::min(d, b) - h * h * k * 0.25f;
    }
    return d;
}

// the SDF at p; under sdf_f32 evaluated in float at p rounded to float
static R sdf_at(const Scene& S, V p)
{
    return S.sdf_f32 ? (R)sdf_eval_f(S, (float)p.x, (float)p.y, (float)p.z) : sdf_eval(S, p);
}

static bool slab(const R lo[3], const R hi[3], V o, V d, R* t0, R* t1)
{
    R a0 = -1e300, a1 = 1e300;
    const R oo[3] = {o.x, o.y, o.z}, dd[3] = {d.x, d.y, d.z};
    for (int k = 0; k < 3; ++k)
    {
        const R inv = inv_safe(dd[k]);
        R x = (lo[k] - oo[k]) * inv, y = (hi[k] - oo[k]) * inv;
        if (x > y) std::swap(x, y);
        a0 = std::max(a0, x);
        a1 = std::min(a1, y);
    }
    *t0 = a0;
    *t1 = a1;
    return a0 <= a1;
}

// first surface crossing in the bounds (the sign at the origin decides which), or -1
static R sdf_march(const Scene& S, V o, V d, R eps)
{
    R t0, t1;
    if (S.sdf.empty() || !slab(S.sdf_lo, S.sdf_hi, o, d, &t0, &t1) || t1 <= 0) return -1.0;
    const bool inside = sdf_at(S, o) <= 0.0;
    R t = std::max(0.0, t0);
    if (S.sdf_f32) t = to_f32(t);
    for (int i = 0; i < 512; ++i)
    {
        const R dist = sdf_at(S, o + d * t);
        if (inside ? (dist > 0 && dist < eps) : (dist < 0 && -dist < eps)) return t;
        t += std::max(std::fabs(dist), eps * 0.5);
        if (S.sdf_f32) t = to_f32(t);
        if (t > t1) break;
    }
    return -1.0;
}

static R prim_t(const Scene& S, int p, V o, V d, R tmin)
{
    Hit h;
    if (S.prim_type[p] == OBJ_SDF) return sdf_march(S, o, d, 0.5 * std::max(tmin, 1e-3));
    if (S.prim_type[p] == OBJ_TRIANGLE)
    {
        R t;
        return tri_hit(S.tri[p], o, d, &t) ? t : -1.0;
    }
    const bool ok = S.prim_type[p] == OBJ_CUBE ? box_hit(o, d, S.objs[p], &h, false) : sphere_hit(o, d, S.objs[p], &h, false);
    return ok ? h.t : -1.0;
}

static void build_bvh(Scene& S)
{
    const int n = (int)S.prim_type.size();
    S.order.resize(n);
    for (int i = 0; i < n; ++i) S.order[i] = i;
    S.nodes.clear();
    S.nodes.reserve(2 * (size_t)n);
    struct Item
    {
        int node, first, count;
    };
    std::vector<Item> st;
    S.nodes.push_back({});
    st.push_back({0, 0, n});
    while (!st.empty())
    {
        const Item it = st.back();
        st.pop_back();
        Scene::Node nd{};
        for (int k = 0; k < 3; ++k)
        {
            nd.lo[k] = 1e300;
            nd.hi[k] = -1e300;
        }
        R clo[3] = {1e300, 1e300, 1e300}, chi[3] = {-1e300, -1e300, -1e300};
        for (int i = it.first; i < it.first + it.count; ++i)
        {
            const int p = S.order[i];
            for (int k = 0; k < 3; ++k)
            {
                nd.lo[k] = std::min(nd.lo[k], S.lo[p][k]);
                nd.hi[k] = std::max(nd.hi[k], S.hi[p][k]);
                const R c = 0.5 * (S.lo[p][k] + S.hi[p][k]);
                clo[k] = std::min(clo[k], c);
                chi[k] = std::max(chi[k], c);
            }
        }
        if (it.count <= 4)
        {
            nd.left = nd.right = -1;
            nd.first = it.first;
            nd.count = it.count;
            S.nodes[it.node] = nd;
            continue;
        }
        int ax = 0;
        for (int k = 1; k < 3; ++k)
            if (chi[k] - clo[k] > chi[ax] - clo[ax]) ax = k;
        const int mid = it.first + it.count / 2;
        std::nth_element(S.order.begin() + it.first, S.order.begin() + mid, S.order.begin() + it.first + it.count,
                         [&](int a, int b) {
                             const R ca = S.lo[a][ax] + S.hi[a][ax], cb = S.lo[b][ax] + S.hi[b][ax];
                             return ca < cb || (ca == cb && a < b);
                         });
        nd.left = (int)S.nodes.size();
        nd.right = nd.left + 1;
        nd.first = nd.count = 0;
        S.nodes[it.node] = nd;
        S.nodes.push_back({});
        S.nodes.push_back({});
        st.push_back({nd.left, it.first, mid - it.first});
        st.push_back({nd.right, mid, it.first + it.count - mid});
    }
}

static bool box_range(const Scene::Node& n, V o, V inv, R tmin, R tmax)
{
    R t0 = tmin, t1 = tmax;
    const R oo[3] = {o.x, o.y, o.z}, ii[3] = {inv.x, inv.y, inv.z};
    for (int k = 0; k < 3; ++k)
    {
        R a = (n.lo[k] - oo[k]) * ii[k], b = (n.hi[k] - oo[k]) * ii[k];
        if (std::isnan(a)) a = -1e300;
        if (std::isnan(b)) b = 1e300;
        if (a > b) std::swap(a, b);
        t0 = std::max(t0, a);
        t1 = std::min(t1, b * (1 + 1e-12));
        if (t0 > t1) return false;
    }
    return true;
}

// closest hit in [tmin, tmax), ties to the smallest primitive id; any hit when any = true
static int trace(const Scene& S, V o, V d, R tmin, R tmax, bool any, R* tout)
{
    const V inv = v(1.0 / d.x, 1.0 / d.y, 1.0 / d.z);
    int best = -1;
    R bt = tmax;
    int stack[128];
    int sp = 0;
    stack[sp++] = 0;
    while (sp)
    {
        const Scene::Node& n = S.nodes[stack[--sp]];
        if (!box_range(n, o, inv, tmin, bt)) continue;
        if (n.left < 0)
        {
            for (int i = n.first; i < n.first + n.count; ++i)
            {
                const int p = S.order[i];
                const R t = prim_t(S, p, o, d, tmin);
                if (!(t >= tmin) || !(t < tmax)) continue;
                if (t < bt || (t == bt && best >= 0 && p < best))
                {
                    bt = t;
                    best = p;
                    if (any)
                    {
                        *tout = t;
                        return p;
                    }
                }
            }
        }
        else
        {
            if (sp + 2 > 128) continue;
            stack[sp++] = n.left;
            stack[sp++] = n.right;
        }
    }
    *tout = bt;
    return best;
}

static void hit_record(const Scene& S, int p, V o, V d, R t, Hit* h)
{
    h->hit = true;
    h->prim = p;
    h->t = t;
    if (S.prim_type[p] == OBJ_TRIANGLE)
    {
        const auto& T = S.tri[p];
        const V a = v(T[0], T[1], T[2]), b = v(T[3], T[4], T[5]), c = v(T[6], T[7], T[8]);
        h->pos = o + d * t;
        V n = normalize(cross(b - a, c - a));
        if (dot(n, d) > 0) n = -n;
        h->nrm = n;
    }
    else if (S.prim_type[p] == OBJ_CUBE) box_hit(o, d, S.objs[p], h, true);
    else if (S.prim_type[p] == OBJ_SDF)
    {
        h->pos = S.sdf_f32 ? to_f32(o + d * t) : o + d * t;
        const R e = 1e-4;
        const V p0 = h->pos;
        h->nrm = normalize(v(sdf_at(S, p0 + v(e, 0, 0)) - sdf_at(S, p0 - v(e, 0, 0)),
                             sdf_at(S, p0 + v(0, e, 0)) - sdf_at(S, p0 - v(0, e, 0)),
                             sdf_at(S, p0 + v(0, 0, e)) - sdf_at(S, p0 - v(0, 0, e))));
    }
    else sphere_hit(o, d, S.objs[p], h, true);
}

// texel index at a triangle hit (nearest, clamped), -1 when not a triangle
static int texel_at(const Scene& S, int tex, int p, V pos)
{
    if (S.prim_type[p] != OBJ_TRIANGLE) return -1;
    const auto& T = S.tri[p];
    const V v0 = v(T[0], T[1], T[2]);
    const V e1 = v(T[3], T[4], T[5]) - v0, e2 = v(T[6], T[7], T[8]) - v0, dd = pos - v0;
    const R d00 = dot(e1, e1), d01 = dot(e1, e2), d11 = dot(e2, e2), d20 = dot(dd, e1), d21 = dot(dd, e2);
    const R den = d00 * d11 - d01 * d01;
    R b1 = 0, b2 = 0;
    if (den > 0)
    {
        b1 = (d11 * d20 - d01 * d21) / den;
        b2 = (d00 * d21 - d01 * d20) / den;
    }
    const R b0 = 1 - b1 - b2;
    const auto& uv = S.uv[p];
    const R u = sat(b0 * uv[0] + b1 * uv[2] + b2 * uv[4]), w = sat(b0 * uv[1] + b1 * uv[3] + b2 * uv[5]);
    const int x = std::min(std::max((int)std::floor(u * S.tex_w[tex]), 0), S.tex_w[tex] - 1);
    const int y = std::min(std::max((int)std::floor(w * S.tex_h[tex]), 0), S.tex_h[tex] - 1);
    return S.tex_off[tex] + y * S.tex_w[tex] + x;
}

// ------------------------------------------------------------------ shading
static void tangent_basis(V n, V* t, V* b)
{
    const V a = std::fabs(n.z) < 0.999 ? v(0, 0, 1) : v(1, 0, 0);
    *t = normalize(cross(a, n));
    *b = cross(n, *t);
}
static void tangent_basis_random(V n, V* t, V* b, R e)
{
    V t0, b0;
    tangent_basis(n, &t0, &b0);
    const R s = std::sin(e * PI * 2), c = std::cos(e * PI * 2);
    *t = c * t0 + s * b0;
    *b = -s * t0 + c * b0;
}

// concentric-disk cosine sampling with a random tangent rotation (core/render/sample.cuh:62-108)
static V cosine_dir(R e0, R e1, R e2, V n, R* pdf)
{
    V T, B;
    tangent_basis_random(n, &T, &B, e2);
    const R sx = 2 * e0 - 1, sy = 2 * e1 - 1;
    R x = 0, y = 0;
    if (!(sx == 0 && sy == 0))
    {
        R r, phi;
        if (std::fabs(sx) > std::fabs(sy))
        {
            r = sx;
            phi = (PI / 4) * (sy / std::max(std::fabs(sx), 1e-20));
        }
        else
        {
            r = sy;
            phi = PI / 2 - (PI / 4) * (sx / std::max(std::fabs(sy), 1e-20));
        }
        x = r * std::cos(phi);
        y = r * std::sin(phi);
    }
    const R z = std::sqrt(std::max(0.0, 1 - x * x - y * y));
    *pdf = z / PI;
    return normalize(x * T + y * B + z * n);
}

static R ggx_d(R alpha, R NoH)
{
    const R a2 = alpha * alpha, d = NoH * NoH * (a2 - 1) + 1;
    return a2 / std::max(PI * d * d, 1e-12);
}
static R ggx_g(R alpha, R NoL, R NoV)
{
    const R a2 = alpha * alpha;
    const R gv = NoL * std::sqrt(a2 + (1 - a2) * NoV * NoV), gl = NoV * std::sqrt(a2 + (1 - a2) * NoL * NoL);
    return gv + gl > 0 ? 2 * NoL * NoV / (gv + gl) : 0.0;
}
static R schlick(R F0, R c)
{
    const R x = clampd(1 - c, 0, 1);
    return F0 + (1 - F0) * x * x * x * x * x;
}

// bounded VNDF sampling (Eto & Tokuyoshi 2023; core/render/sample.cuh:179-248)
static V vndf_dir(V Vw, V N, R alpha, R r0, R r1, R r2, R* pdf)
{
    V X, Y;
    tangent_basis_random(N, &X, &Y, r2);
    const R XoV = dot(X, Vw), YoV = dot(Y, Vw), NoV = dot(N, Vw);
    const V lv = v(XoV, YoV, NoV);
    const R NoV2 = std::min(1.0, NoV * NoV), a2 = alpha * alpha;
    const V ls = v(XoV * alpha, YoV * alpha, NoV) / std::sqrt(a2 + (1 - a2) * NoV2);
    const R phi = 2 * PI * r0;
    const R s = 1 + std::sqrt(1 - NoV2), s2 = s * s;
    const R k = (1 - a2) * s2 / (s2 + a2 * NoV2);
    const R b = NoV > 0 ? k * ls.z : ls.z;
    const R z = (1 - r1) * (1 + b) - b;
    const R st = std::sqrt(sat(1 - z * z));
    const V m = ls + v(st * std::cos(phi), st * std::sin(phi), z);
    const V lh = normalize(v(m.x * alpha, m.y * alpha, m.z));
    const V ll = reflect(-lv, lh);
    const R ndf = ggx_d(alpha, lh.z);
    *pdf = ndf / (2 * (k * NoV + std::sqrt((1 - NoV2) * a2 + NoV2)));
    return ll.x * X + ll.y * Y + ll.z * N;
}
static R vndf_pdf(V Vw, V N, V L, R alpha)
{
    const R NoV = dot(N, Vw), NoL = dot(N, L);
    if (NoV <= 0 || NoL <= 0) return 0.0;
    const V H = normalize(Vw + L);
    const R NoV2 = std::min(1.0, NoV * NoV), a2 = alpha * alpha;
    const R s = 1 + std::sqrt(1 - NoV2), s2 = s * s;
    const R k = (1 - a2) * s2 / (s2 + a2 * NoV2);
    const R ndf = ggx_d(alpha, std::max(0.0, dot(N, H)));
    return std::max(ndf / (2 * (k * NoV + std::sqrt((1 - NoV2) * a2 + NoV2))), 1e-12);
}

struct Shade
{
    const Scene* S;
    LutCache* L;
    std::array<R, 4> lam;
    R lambda;
    Mat m;
    R alb;  // albedo at lambda
};

static R eval_cos(const Shade& s, V rayDir, V L, V N)
{
    const R NoL = std::max(0.0, dot(N, L));
    if (s.m.shading == MAT_DIFFUSE) return s.alb * (NoL / PI);
    if (s.m.shading != MAT_GGX) return 0.0;
    const V Vw = normalize(-rayDir);
    const R NoV = std::max(0.0, dot(N, Vw));
    if (NoV <= 0 || NoL <= 0) return 0.0;
    const R alpha = s.m.roughness * s.m.roughness;
    const R F0 = lerp(0.08 * clampd(s.m.specular, 0, 1), s.alb, s.m.metallic);
    const V H = normalize(Vw + L);
    const R F = schlick(F0, std::max(0.0, dot(L, H)));
    const R spec = F * ggx_d(alpha, std::max(0.0, dot(N, H))) * ggx_g(alpha, NoL, NoV) / std::max(4 * NoV, 1e-7);
    return spec + (1 - s.m.metallic) * (1 - F) * s.alb * (NoL / PI);
}

static R bsdf_pdf(const Shade& s, V N, V rayDir, V L)
{
    const V Vw = -rayDir;
    const R NoL = std::max(0.0, dot(N, L));
    if (s.m.shading == MAT_DIFFUSE) return NoL > 0 ? NoL / PI : 0.0;
    if (s.m.shading != MAT_GGX) return 0.0;
    const R NoV = std::max(0.0, dot(N, Vw));
    if (NoV <= 0 || NoL <= 0) return 0.0;
    const R alpha = s.m.roughness * s.m.roughness;
    const R pSpec = clampd(lerp(0.08 * clampd(s.m.specular, 0, 1), s.alb, s.m.metallic), 0.1, 0.9);
    return std::max(0.0, pSpec * vndf_pdf(Vw, N, L, alpha) + (1 - pSpec) * NoL / PI);
}

struct Sample
{
    V dir{0, 0, 0};
    R pdf = 1, brdf = 0;
    bool terminate = false, delta = false;
};

template <typename Rand>
static Sample sample_bsdf(const Shade& s, Rand& rnd, V rayDir, V N)
{
    Sample r;
    if (s.m.shading == MAT_DIFFUSE)
    {
        const R e0 = rnd(), e1 = rnd(), e2 = rnd();
        r.dir = cosine_dir(e0, e1, e2, N, &r.pdf);
    }
    else if (s.m.shading == MAT_LIGHT)
    {
        r.terminate = true;
    }
    else if (s.m.shading == MAT_GGX)
    {
        const V Vw = -rayDir;
        if (std::max(0.0, dot(N, Vw)) <= 0) r.terminate = true;
        else
        {
            const R alpha = s.m.roughness * s.m.roughness;
            const R pSpec = clampd(lerp(0.08 * clampd(s.m.specular, 0, 1), s.alb, s.m.metallic), 0.1, 0.9);
            const R u = rnd();
            if (u < pSpec)
            {
                const R e0 = rnd(), e1 = rnd(), e2 = rnd();
                R ps;
                const V L = vndf_dir(Vw, N, alpha, e0, e1, e2, &ps);
                const R NoL = std::max(0.0, dot(N, L));
                if (NoL <= 0) r.terminate = true;
                else
                {
                    r.dir = L;
                    r.pdf = pSpec * ps + (1 - pSpec) * NoL / PI;
                }
            }
            else
            {
                const R e0 = rnd(), e1 = rnd(), e2 = rnd();
                R pd;
                const V L = cosine_dir(e0, e1, e2, N, &pd);
                r.dir = L;
                r.pdf = pSpec * vndf_pdf(Vw, N, L, alpha) + (1 - pSpec) * pd;
            }
        }
    }
    r.brdf = eval_cos(s, rayDir, r.dir, N);
    return r;
}

// ------------------------------------------------------------------ lights
struct LightSample
{
    bool valid = false;
    V point{0, 0, 0}, normal{0, 0, 0};
    R p_facet = 0, p_a = 0;
};

struct Facets
{
    V n[6], c[6], t[6], b[6];
    R s1[6], s2[6], area[6];
};

static void box_facets(const Obj& o, Facets* f)
{
    const V ux = normalize(v(o.o2w.r0.x, o.o2w.r1.x, o.o2w.r2.x));
    const V uy = normalize(v(o.o2w.r0.y, o.o2w.r1.y, o.o2w.r2.y));
    const V uz = normalize(v(o.o2w.r0.z, o.o2w.r1.z, o.o2w.r2.z));
    const V c = o.center, e = o.extent;
    const V ns[6] = {ux, -ux, uy, -uy, uz, -uz};
    const V cs[6] = {c + ux * e.x, c - ux * e.x, c + uy * e.y, c - uy * e.y, c + uz * e.z, c - uz * e.z};
    const V ts[6] = {uy, uy, ux, ux, ux, ux}, bs[6] = {uz, uz, uz, uz, uy, uy};
    const R s1[6] = {e.y, e.y, e.x, e.x, e.x, e.x}, s2[6] = {e.z, e.z, e.z, e.z, e.y, e.y};
    for (int i = 0; i < 6; ++i)
    {
        f->n[i] = ns[i];
        f->c[i] = cs[i];
        f->t[i] = ts[i];
        f->b[i] = bs[i];
        f->s1[i] = s1[i];
        f->s2[i] = s2[i];
        f->area[i] = 4 * s1[i] * s2[i];
    }
}

static R facing(V n, V c, V p, R area) { return area * std::max(0.0, dot(n, normalize(p - c))); }

static R area_to_omega(V sp, V lp, V ln, R pA)
{
    const V s2l = lp - sp;
    const R d2 = std::max(dot(s2l, s2l), 1e-20);
    const R cosY = std::max(0.0, dot(ln, -(s2l / std::sqrt(d2))));
    return cosY <= 0 ? 0.0 : pA * (d2 / cosY);
}

template <typename Rand>
static LightSample sample_box(Rand& rnd, const Obj& box, V p)
{
    LightSample ls;
    Facets f;
    box_facets(box, &f);
    int idx[6], cnt = 0;
    R w[6], sum = 0;
    for (int i = 0; i < 6; ++i)
    {
        const R cw = facing(f.n[i], f.c[i], p, f.area[i]);
        if (cw > 0)
        {
            idx[cnt] = i;
            w[cnt] = cw;
            sum += cw;
            ++cnt;
        }
    }
    if (!cnt) return ls;
    int slot = 0, face = idx[0];
    const R r = rnd() * sum;
    R acc = 0;
    for (int k = 0; k < cnt; ++k)
    {
        acc += w[k];
        if (r <= acc)
        {
            slot = k;
            face = idx[k];
            break;
        }
    }
    const R u1 = 2 * rnd() - 1, u2 = 2 * rnd() - 1;
    ls.point = f.c[face] + f.t[face] * (u1 * f.s1[face]) + f.b[face] * (u2 * f.s2[face]);
    ls.normal = f.n[face];
    ls.p_facet = w[slot] / sum;
    ls.p_a = 1.0 / f.area[face];
    ls.valid = true;
    return ls;
}

template <typename Rand>
static LightSample sample_sphere(Rand& rnd, const Obj& s, V p)
{
    LightSample ls;
    const R r = max3(s.extent);
    const V p2c = p - s.center;
    const R d = length(p2c);
    if (d <= r) return ls;
    const V axis = p2c / d;
    const R cosC = clampd(r / d, 0, 1);
    const R areaCap = 2 * PI * r * r * (1 - cosC);
    const R u = rnd(), vphi = rnd();
    const R cosT = lerp(cosC, 1.0, u), sinT = std::sqrt(std::max(0.0, 1 - cosT * cosT)), phi = 2 * PI * vphi;
    V t, b;
    tangent_basis(axis, &t, &b);
    const V n = t * (std::cos(phi) * sinT) + b * (std::sin(phi) * sinT) + axis * cosT;
    ls.point = s.center + n * r;
    ls.normal = n;
    ls.p_facet = 1;
    ls.p_a = 1.0 / areaCap;
    ls.valid = true;
    return ls;
}

static R box_pdf_omega(const Obj& o, R sel, V sp, V lp, V ln)
{
    Facets f;
    box_facets(o, &f);
    int hf = -1;
    for (int i = 0; i < 6 && hf < 0; ++i)
        if (dot(f.n[i], ln) > 0.999) hf = i;
    if (hf < 0)
    {
        R best = 1e300;
        for (int i = 0; i < 6; ++i)
        {
            const R d = std::fabs(dot(f.n[i], lp - f.c[i]));
            if (d < best)
            {
                best = d;
                hf = i;
            }
        }
    }
    R sum = 0, wh = 0, ah = 0;
    for (int i = 0; i < 6; ++i)
    {
        const R w = facing(f.n[i], f.c[i], sp, f.area[i]);
        sum += w;
        if (i == hf)
        {
            wh = w;
            ah = f.area[i];
        }
    }
    if (sum <= 0 || wh <= 0) return 0.0;
    return area_to_omega(sp, lp, ln, sel * (1.0 / ah) * (wh / sum));
}

static R sphere_pdf_omega(const Obj& o, R sel, V sp, V lp, V ln)
{
    const R r = max3(o.extent), d = length(sp - o.center);
    if (d <= r) return 0.0;
    const R areaCap = 2 * PI * r * r * (1 - clampd(r / d, 0, 1));
    if (areaCap <= 1e-20) return 0.0;
    return area_to_omega(sp, lp, ln, sel / areaCap);
}

static R power(R a, R b) { return a * a / std::max(1e-24, a * a + b * b); }

static V sky(V d)
{
    const R t1 = std::pow(std::max(d.y, 0.0), 0.75);
    const V l1 = v(lerp(0.05, 1.0, t1), lerp(0.45, 1.0, t1), lerp(1.0, 1.0, t1));
    const R t2 = std::min(std::max(-d.y * 0.5 + 0.5, 0.0), 1.0);
    const V dn = v(0.2, 0.6, 1.0) * 0.125;
    return 0.5 * v(lerp(l1.x, dn.x, t2), lerp(l1.y, dn.y, t2), lerp(l1.z, dn.z, t2));
}

static R intersect_eps(int depth) { return 1e-3 * std::exp(std::min(depth * 0.5, 4.0)); }

// ---- medium
static R hg_pdf(R c, R g)
{
    const R g2 = g * g;
    const R x = std::max(1 + g2 - 2 * g * c, 1e-20);
    return (1 - g2) / (4 * PI * x * std::sqrt(x));
}

static V hg_sample(R e0, R e1, V vin, R g, R* pdf)
{
    R c;
    if (std::fabs(g) < 0.0001) c = e0 * 2 - 1;
    else
    {
        const R g2 = g * g;
        const R t0 = (1 - g2) / (1 - g + 2 * g * e0);
        c = (1 + g2 - t0 * t0) / (2 * g);
    }
    const R phi = 2 * PI * e1;
    const R s = std::sqrt(std::max(0.0, 1 - c * c));
    const V w = normalize(vin);
    const V a = std::fabs(w.z) > 0.70710678 ? v(0, 1, 0) : v(0, 0, 1);
    const V v2 = normalize(cross(w, a));
    const V v3_ = cross(v2, w);
    *pdf = hg_pdf(c, g);
    return v3_ * (s * std::cos(phi)) + v2 * (s * std::sin(phi)) + w * c;
}

static R med_transmittance(const Scene& S, V o, V d, R dist)
{
    if (!S.med_on) return 1.0;
    R t0, t1;
    if (!slab(S.med_lo, S.med_hi, o, d, &t0, &t1)) return 1.0;
    t0 = std::max(t0, 0.0);
    t1 = std::min(t1, dist);
    return t0 < t1 ? std::exp(-S.med_sigma * (t1 - t0)) : 1.0;
}

// ------------------------------------------------------------------ integrator
struct Params
{
    int width, height, spp, max_depth, use_nee, first_frame, threads;
    int crop_x0 = 0, crop_y0 = 0, crop_w = 0, crop_h = 0;  // crop_w > 0: only this window of pixels
    uint64_t seed;
    R cam_o[3], cam_d[3], fov;
};

struct TexVertex
{
    int texel;
    V dalb;          // d(albedo_lambda)/d(rgb) / albedo_lambda
    R before;        // radiance gathered before this vertex's albedo applies
};

struct MedVertex
{
    R after;  // radiance gathered once this scattering point's emission is added
    R mask;   // throughput arriving at it
    R d65;
};

struct PathOut
{
    R radiance, lambda, pdf;
    std::vector<TexVertex> tv;
    std::vector<MedVertex> mv;
};

struct Cam
{
    V o, d, right, up;
    R tx, ty;
};

static void trace_path(const Scene& S, LutCache& L, const Params& P, const Cam& cam, bool camera_inside, uint32_t pixel,
                       uint32_t frame, bool want_grad, PathOut* out)
{
    ar_pcg g = ar_pcg_init(P.seed, pixel, frame);
    auto rnd = [&g]() -> R { return (R)ar_rand1(&g); };
    const int i = (int)(pixel % (uint32_t)P.width), j = (int)(pixel / (uint32_t)P.width);
    const R u = (i + rnd()) / P.width, vv = (j + rnd()) / P.height;
    const R nx = u * 2 - 1, ny = (1 - vv) * 2 - 1;
    V rayD = normalize(cam.d + cam.right * (nx * cam.tx) + cam.up * (ny * cam.ty));
    V rayO = cam.o;
    R lambda, lpdf;
    {
        const R r0 = rnd(), r1 = rnd(), r2 = rnd();
        sample_lambda(r0, r1, r2, &lambda, &lpdf);
    }
    out->lambda = lambda;
    out->pdf = lpdf;
    out->tv.clear();
    out->mv.clear();
    const auto lam = query_lambda(S.tab, lambda);
    const R d65 = d65_norm(S.tab, lambda);
    R radiance = 0, mask = 1;
    int depth = 0, ndd = 0;
    bool inside = camera_inside;
    int media_obj = -1;
    bool prevNEE = false;
    V prevPos = v(0, 0, 0);
    R prevPdf = 0;
    while (depth < P.max_depth)
    {
        const R tmin = intersect_eps(ndd);
        Hit h;
        R t = 0;
        int prim = -1;
        if (inside && media_obj >= 0)
        {
            const R th = prim_t(S, media_obj, rayO, rayD, tmin);
            if (th >= tmin)
            {
                t = th;
                prim = media_obj;
            }
        }
        else prim = trace(S, rayO, rayD, tmin, 1e300, false, &t);
        if (prim >= 0) hit_record(S, prim, rayO, rayD, t, &h);
        bool scatter = false;
        if (S.med_on)
        {
            R m0, m1;
            if (slab(S.med_lo, S.med_hi, rayO, rayD, &m0, &m1))
            {
                m0 = std::max(m0, 0.0);
                m1 = std::min(m1, h.hit ? h.t : 1e300);
                if (m0 < m1)
                {
                    const R ts = m0 - std::log(rnd()) / S.med_sigma;
                    if (ts < m1)
                    {
                        scatter = true;
                        h.hit = false;
                        prim = -1;
                        h.pos = rayO + rayD * ts;
                        h.nrm = v(0, 0, 0);
                    }
                }
            }
        }
        const R eps = intersect_eps(ndd);
        Shade sh{&S, &L, lam, lambda, Mat{MAT_DIFFUSE, v(1, 1, 1), v(0, 0, 0), 0, 0, 0, -1}, 0};
        Sample smp;
        bool miss_thin = false;
        V emissive = v(0, 0, 0);
        int texel = -1;
        V dalb = v(0, 0, 0);
        if (!h.hit && !scatter && inside)
        {
            miss_thin = true;
            smp.brdf = 1;
            smp.dir = rayD;
            smp.pdf = 1;
            smp.delta = true;
            inside = false;
        }
        if (h.hit)
        {
            sh.m = S.mats[S.prim_mat[prim]];
            V rgb = sh.m.albedo;
            if (sh.m.tex >= 0)
            {
                texel = texel_at(S, sh.m.tex, prim, h.pos);
                if (texel >= 0) rgb = v(S.texels[3 * (size_t)texel], S.texels[3 * (size_t)texel + 1], S.texels[3 * (size_t)texel + 2]);
            }
            sh.alb = interact(L, lam, rgb, (want_grad && texel >= 0) ? &dalb : nullptr);
            smp = sample_bsdf(sh, rnd, rayD, h.nrm);
            emissive = sh.m.emissive;
            inside = inside;  // diffuse / GGX keep the medium flag
        }
        else if (scatter)
        {
            const R e0 = rnd(), e1 = rnd();
            R pd;
            smp.dir = hg_sample(e0, e1, rayD, S.med_g, &pd);
            smp.pdf = pd;
            smp.brdf = S.med_albedo * pd;
        }
        else if (!miss_thin)
        {
            smp.brdf = 1;
            smp.dir = rayD;
            smp.pdf = 1;
            emissive = sky(rayD);
            inside = false;
        }
        {
            const R off = eps * std::max(1.0, length(h.pos));
            h.pos = h.pos + h.nrm * (signd(dot(h.nrm, smp.dir)) * off * (rnd() + 0.5));
        }
        // emission
        if (scatter)
        {
            radiance += mask * (1 - S.med_albedo) * S.med_emission * d65;
            if (want_grad) out->mv.push_back(MedVertex{radiance, mask, d65});
        }
        else if (!h.hit)
        {
            if (!miss_thin) radiance += mask * interact(L, lam, emissive, nullptr) * d65;
        }
        else if (sh.m.shading == MAT_LIGHT)
        {
            R misW = 1;
            if (P.use_nee && depth > 0 && prevNEE)
            {
                const R pB = std::max(prevPdf, 0.0);
                const Light* Lt = nullptr;
                for (const Light& l : S.lights)
                    if (l.prim == prim) Lt = &l;
                R pL = 0;
                if (Lt && Lt->type == OBJ_CUBE) pL = box_pdf_omega(S.objs[prim], Lt->select_prob, prevPos, h.pos, h.nrm);
                else if (Lt && Lt->type == OBJ_SPHERE) pL = sphere_pdf_omega(S.objs[prim], Lt->select_prob, prevPos, h.pos, h.nrm);
                if (pL >= 0 && pB > 0) misW = power(pB, pL);
            }
            radiance += mask * interact(L, lam, sh.m.emissive, nullptr) * d65 * misW;
        }
        if (want_grad && texel >= 0 && sh.m.shading == MAT_DIFFUSE && sh.alb > 1e-8)
            out->tv.push_back(TexVertex{texel, dalb / sh.alb, radiance});
        const bool ended = (!h.hit && !miss_thin && !scatter) || smp.terminate;
        if (ended) break;
        if (!miss_thin)
        {
            const R rate = std::sqrt(sat(mask));
            bool neeValid = false;
            if (P.use_nee && ndd < 10 && !smp.delta && !inside && rnd() < rate)
            {
                LightSample ls;
                int lprim = -1, lmat = -1;
                if (!S.lights.empty())
                {
                    const R r = rnd();
                    size_t pick = S.lights.size() - 1;
                    R pp = 0;
                    for (size_t k = 0; k < S.lights.size(); ++k)
                        if (r < S.lights[k].cdf)
                        {
                            pick = k;
                            pp = S.lights[k].select_prob;
                            break;
                        }
                    const Light& Lt = S.lights[pick];
                    if (Lt.type == OBJ_CUBE) ls = sample_box(rnd, S.objs[Lt.prim], h.pos);
                    else if (Lt.type == OBJ_SPHERE) ls = sample_sphere(rnd, S.objs[Lt.prim], h.pos);
                    if (ls.valid)
                    {
                        lprim = Lt.prim;
                        lmat = Lt.material;
                        ls.p_facet *= pp;
                    }
                }
                (void)lprim;
                if (ls.valid)
                {
                    const R pAT = std::max(1e-20, ls.p_a * ls.p_facet);
                    const V lun = ls.point - h.pos;
                    const R dist2 = std::max(dot(lun, lun), 1e-12);
                    const V Ld = lun / std::sqrt(dist2);
                    const R cosX = scatter ? 1.0 : std::max(0.0, dot(h.nrm, Ld)), cosY = std::max(0.0, dot(ls.normal, -Ld));
                    R vUn = 0;
                    bool validUn = false;
                    if (!(cosX <= 0 || cosY <= 0))
                    {
                        const R f = scatter ? S.med_albedo * hg_pdf(dot(rayD, Ld), S.med_g) : eval_cos(sh, rayD, Ld, h.nrm);
                        const R le = interact(L, lam, S.mats[lmat].emissive, nullptr);
                        const R contribution = f * le * ((cosY / dist2) / pAT);
                        const R pLight = area_to_omega(h.pos, ls.point, ls.normal, ls.p_facet * ls.p_a);
                        const R pBsdf = scatter ? hg_pdf(dot(rayD, Ld), S.med_g) : std::max(bsdf_pdf(sh, h.nrm, rayD, Ld), 0.0);
                        vUn = mask * (contribution * power(pLight, pBsdf)) * d65 * med_transmittance(S, h.pos, Ld, std::sqrt(dist2));
                        validUn = true;
                    }
                    V dirS = ls.point - h.pos;
                    const R dist = length(dirS);
                    bool traced = false;
                    if (dist > 0)
                    {
                        dirS = dirS / dist;
                        const R seps = intersect_eps(depth) * std::max(1.0, std::max(length(h.pos), length(ls.point)));
                        const R tmax = std::max(0.0, dist - seps);
                        if (tmax > 0)
                        {
                            traced = true;
                            R ts;
                            const bool occluded = trace(S, h.pos, dirS, 0.0, tmax, true, &ts) >= 0;
                            radiance += occluded ? 0.0 : vUn;
                            neeValid = occluded ? true : validUn;
                        }
                    }
                    if (!traced)
                    {
                        radiance += vUn;
                        neeValid = validUn;
                    }
                }
            }
            prevNEE = neeValid;
            prevPos = h.pos;
            prevPdf = smp.pdf;
        }
        const R contrib = smp.brdf / std::max(smp.pdf, 1e-12);
        R pSurvive = 1;
        if (ndd >= 3)
        {
            const R basic = clampd(mask * 0.5 + mask * 0.5, 0.05, 0.95);
            pSurvive = lerp(basic, 1.0, inside ? 0.99 : 0.0);
            if (rnd() > pSurvive) break;
        }
        mask = mask * contrib / pSurvive;
        if (!smp.delta) ++ndd;
        ++depth;
        rayO = h.pos;
        rayD = smp.dir;
    }
    out->radiance = std::isfinite(radiance) ? radiance : 0.0;
}

static Cam make_cam(const Params& P)
{
    Cam c;
    c.o = v(P.cam_o[0], P.cam_o[1], P.cam_o[2]);
    c.d = v(P.cam_d[0], P.cam_d[1], P.cam_d[2]);
    const R FOV = P.fov * PI / 180.0;
    c.ty = std::tan(0.5 * FOV);
    c.tx = c.ty * (R)P.width / std::max(1.0, (R)P.height);
    c.right = normalize(cross(c.d, v(0, 1, 0)));
    c.up = normalize(cross(c.d, c.right));
    return c;
}

static bool overlap(V p, const Obj& ob)
{
    const V lp = mul(ob.w2o, p - ob.center);
    if (ob.type == OBJ_CUBE)
        return -ob.extent.x < lp.x && -ob.extent.y < lp.y && -ob.extent.z < lp.z && ob.extent.x > lp.x &&
               ob.extent.y > lp.y && ob.extent.z > lp.z;
    if (ob.type == OBJ_SPHERE) return dot(lp, lp) < max3(ob.extent) * max3(ob.extent);
    return false;
}

static void xyz_of(const Scene& S, const PathOut& po, R out[3], bool on[3])
{
    const V xyz = lambda_to_xyz(S.tab, po.lambda);
    const R c[3] = {xyz.x * po.radiance / po.pdf, xyz.y * po.radiance / po.pdf, xyz.z * po.radiance / po.pdf};
    for (int k = 0; k < 3; ++k)
    {
        on[k] = c[k] > 0 && c[k] < 1e3;
        out[k] = std::max(0.0, std::min(std::max(c[k], 0.0), 1e3));
    }
}

static void run(const Scene& S, const Params& P, double* mean, double* per_sample, const double* dl, double* grad,
                double* grad_med = nullptr)
{
    const Cam cam = make_cam(P);
    bool cam_inside = false;
    for (size_t p = 0; p < S.prim_type.size(); ++p)
        if (S.prim_type[p] != OBJ_TRIANGLE && overlap(cam.o, S.objs[p])) cam_inside = true;
    const long long npix = (long long)P.width * P.height;
    // pixels to render: the whole image, or a crop window (indices local to the window,
    // random streams and camera rays of the full image's pixels)
    const bool crop = P.crop_w > 0;
    const long long nwork = crop ? (long long)P.crop_w * P.crop_h : npix;
    const int nt = std::max(1, P.threads);
    std::atomic<long long> next(0);
    std::vector<std::vector<double>> gpart(grad ? nt : 0);
    std::vector<std::array<double, 2>> mpart(nt, std::array<double, 2>{0.0, 0.0});
    auto work = [&](int tid) {
        LutCache L{&S.tab, {}};
        PathOut po;
        std::vector<double>* G = nullptr;
        if (grad)
        {
            gpart[tid].assign(S.texels.size(), 0.0);
            G = &gpart[tid];
        }
        for (long long q; (q = next.fetch_add(1)) < nwork;)
        {
            const long long pix = crop ? (long long)(P.crop_y0 + q / P.crop_w) * P.width + (P.crop_x0 + q % P.crop_w) : q;
            double acc[3] = {0, 0, 0};
            for (int s = 0; s < P.spp; ++s)
            {
                const uint32_t frame = (uint32_t)(P.first_frame + s);
                trace_path(S, L, P, cam, cam_inside, (uint32_t)pix, frame, grad != nullptr || grad_med != nullptr, &po);
                R c[3];
                bool on[3];
                xyz_of(S, po, c, on);
                for (int k = 0; k < 3; ++k) acc[k] += c[k];
                if (per_sample)
                    for (int k = 0; k < 3; ++k) per_sample[((size_t)s * npix + pix) * 3 + k] = c[k];
                if (G || grad_med)
                {
                    const V xyz = lambda_to_xyz(S.tab, po.lambda);
                    const R xs[3] = {xyz.x, xyz.y, xyz.z};
                    R delta = 0;
                    for (int k = 0; k < 3; ++k)
                        if (on[k]) delta += dl[3 * pix + k] * xs[k] / po.pdf;
                    delta /= P.spp;
                    if (G)
                        for (const TexVertex& tv : po.tv)
                        {
                            const R w = delta * (po.radiance - tv.before);
                            (*G)[3 * (size_t)tv.texel + 0] += w * tv.dalb.x;
                            (*G)[3 * (size_t)tv.texel + 1] += w * tv.dalb.y;
                            (*G)[3 * (size_t)tv.texel + 2] += w * tv.dalb.z;
                        }
                    for (const MedVertex& mv : po.mv)
                    {
                        // what follows carries the albedo once; the emission here carries (1 - albedo)
                        if (S.med_albedo > 1e-8) mpart[tid][0] += delta * (po.radiance - mv.after) / S.med_albedo;
                        mpart[tid][0] -= delta * mv.mask * S.med_emission * mv.d65;
                        mpart[tid][1] += delta * mv.mask * (1 - S.med_albedo) * mv.d65;
                    }
                }
            }
            if (mean)
                for (int k = 0; k < 3; ++k) mean[3 * q + k] = acc[k] / P.spp;
        }
    };
    std::vector<std::thread> th;
    for (int t = 1; t < nt; ++t) th.emplace_back(work, t);
    work(0);
    for (auto& t : th) t.join();
    if (grad)
    {
        std::memset(grad, 0, S.texels.size() * sizeof(double));
        for (auto& g : gpart)
            for (size_t k = 0; k < g.size(); ++k) grad[k] += g[k];
    }
    if (grad_med)
    {
        grad_med[0] = grad_med[1] = 0.0;
        for (auto& m : mpart)
        {
            grad_med[0] += m[0];
            grad_med[1] += m[1];
        }
    }
}

static M euler(V deg)
{
    const R k = PI / 180.0;
    const R ax = deg.x * k, ay = deg.y * k, az = deg.z * k;
    const M rx{v(1, 0, 0), v(0, std::cos(ax), -std::sin(ax)), v(0, std::sin(ax), std::cos(ax))};
    const M ry{v(std::cos(ay), 0, std::sin(ay)), v(0, 1, 0), v(-std::sin(ay), 0, std::cos(ay))};
    const M rz{v(std::cos(az), -std::sin(az), 0), v(std::sin(az), std::cos(az), 0), v(0, 0, 1)};
    return mulm(rz, mulm(ry, rx));
}
} // namespace o64

using namespace o64;

// Flat C interface (ctypes).  Layouts:
//   materials  14 floats: shading, albedo[3], emissive[3], roughness, metallic,
//              specular, ior, sigma_a, abbe, albedo_texture (0 none, k = k-1)
//   objects    20 floats: type, material, center[3], extent[3], rotation_deg[3], v0..v2[9]
//   mesh       tri[9] floats, tri_mat int32, tri_uv[6] floats (may be null)
//   textures   sizes int32 (w, h) per texture, texels RGB floats
//   tables     cmf 421x3, d65 421, rgb MLP, lambda MLP (float32)
//   params     ints: width, height, spp, max_depth, use_nee, first_frame, threads;
//              doubles: cam_o[3], cam_d[3], fov; uint64 seed
struct pt64_scene;

extern "C" {

int pt64_version(void) { return 1; }

pt64_scene* pt64_create(const float* mats, int n_mat, const float* objs, int n_obj, const float* tri, const int32_t* tri_mat,
                        const float* tri_uv, int n_tri, const int32_t* tex_sizes, const float* texels, int n_tex,
                        const float* cmf, const float* d65, const float* rgb_mlp, int rgb_n, const float* lam_mlp, int lam_n,
                        const float* sdf, int n_sdf, float sdf_k, int sdf_mat, char* err, int err_len)
{
    auto fail = [&](const char* m) -> pt64_scene* {
        if (err && err_len > 0)
        {
            std::strncpy(err, m, (size_t)err_len - 1);
            err[err_len - 1] = 0;
        }
        return nullptr;
    };
    Scene* S = new Scene();
    for (int i = 0; i < n_mat; ++i)
    {
        const float* m = mats + 14 * (size_t)i;
        Mat r{};
        r.shading = (int)m[0];
        const V alb = v(m[1], m[2], m[3]), emi = v(m[4], m[5], m[6]);
        r.albedo = v(1, 1, 1);
        r.emissive = v(0, 0, 0);
        r.tex = -1;
        if (r.shading == MAT_LIGHT)
        {
            r.albedo = v(0, 0, 0);
            r.emissive = emi;
        }
        else if (r.shading == MAT_GGX)
        {
            r.albedo = alb;
            r.emissive = emi;
            r.roughness = clampd(m[7], 0.01f, 1.0f);
            r.metallic = clampd(m[8], 0, 1);
            r.specular = clampd(m[9], 0, 1);
        }
        else if (r.shading == MAT_GLASS)
        {
            delete S;
            return fail("the FP64 oracle has no glass");
        }
        else
        {
            r.shading = MAT_DIFFUSE;
            r.albedo = alb;
            r.emissive = emi;
        }
        const int t = (int)m[13];
        if (t > 0 && r.shading != MAT_LIGHT) r.tex = t - 1;
        if (r.tex >= n_tex)
        {
            delete S;
            return fail("texture index out of range");
        }
        S->mats.push_back(r);
    }
    const int np = n_obj + n_tri + (n_sdf > 0 ? 1 : 0);
    if (n_sdf > 0)
    {
        for (int i = 0; i < n_sdf; ++i)
        {
            std::array<R, 7> q;
            for (int k = 0; k < 7; ++k) q[k] = sdf[8 * (size_t)i + k];
            S->sdf.push_back(q);
            R h[3];
            const int kind = (int)q[0];
            if (kind == 0) h[0] = h[1] = h[2] = q[4];
            else if (kind == 1)
            {
                h[0] = q[4];
                h[1] = q[5];
                h[2] = q[6];
            }
            else
            {
                h[0] = h[2] = q[4] + q[5];
                h[1] = q[5];
            }
            for (int k = 0; k < 3; ++k)
            {
                const R pad = 0.25 * sdf_k + 1e-4 * (std::fabs(q[1 + k]) + h[k]) + 1e-6;
                if (i == 0 || q[1 + k] - std::fabs(h[k]) - pad < S->sdf_lo[k]) S->sdf_lo[k] = q[1 + k] - std::fabs(h[k]) - pad;
                if (i == 0 || q[1 + k] + std::fabs(h[k]) + pad > S->sdf_hi[k]) S->sdf_hi[k] = q[1 + k] + std::fabs(h[k]) + pad;
            }
        }
        S->sdf_k = sdf_k;
    }
    S->prim_type.resize(np);
    S->prim_mat.resize(np);
    S->objs.resize(np);
    S->tri.resize(np);
    S->uv.assign(np, std::array<R, 6>{0, 0, 0, 0, 0, 0});
    S->lo.resize(np);
    S->hi.resize(np);
    for (int i = 0; i < np; ++i)
    {
        int type, mat;
        std::array<R, 9> T{};
        if (i >= n_obj + n_tri)
        {
            type = OBJ_SDF;
            mat = sdf_mat;
        }
        else if (i < n_obj)
        {
            const float* o = objs + 20 * (size_t)i;
            type = (int)o[0];
            mat = (int)o[1];
            Obj ob{};
            ob.type = type;
            ob.center = v(o[2], o[3], o[4]);
            ob.extent = v(std::fabs(o[5]), std::fabs(o[6]), std::fabs(o[7]));
            ob.o2w = euler(v(o[8], o[9], o[10]));
            ob.w2o = transpose(ob.o2w);
            S->objs[i] = ob;
            for (int k = 0; k < 9; ++k) T[k] = o[11 + k];
        }
        else
        {
            const int t = i - n_obj;
            type = OBJ_TRIANGLE;
            mat = tri_mat[t];
            for (int k = 0; k < 9; ++k) T[k] = tri[9 * (size_t)t + k];
            if (tri_uv)
                for (int k = 0; k < 6; ++k) S->uv[i][k] = tri_uv[6 * (size_t)t + k];
        }
        if (mat < 0 || mat >= n_mat)
        {
            delete S;
            return fail("material index out of range");
        }
        S->prim_type[i] = type;
        S->prim_mat[i] = mat;
        S->tri[i] = T;
        if (type == OBJ_TRIANGLE)
            for (int k = 0; k < 3; ++k)
            {
                S->lo[i][k] = std::min(T[k], std::min(T[3 + k], T[6 + k]));
                S->hi[i][k] = std::max(T[k], std::max(T[3 + k], T[6 + k]));
            }
        else if (type == OBJ_SDF)
            for (int k = 0; k < 3; ++k)
            {
                S->lo[i][k] = S->sdf_lo[k];
                S->hi[i][k] = S->sdf_hi[k];
            }
        else
        {
            const Obj& ob = S->objs[i];
            V half;
            if (type == OBJ_CUBE)
            {
                const V ax = mul(ob.o2w, v(1, 0, 0)), ay = mul(ob.o2w, v(0, 1, 0)), az = mul(ob.o2w, v(0, 0, 1));
                half = v(std::fabs(ax.x) * ob.extent.x + std::fabs(ay.x) * ob.extent.y + std::fabs(az.x) * ob.extent.z,
                         std::fabs(ax.y) * ob.extent.x + std::fabs(ay.y) * ob.extent.y + std::fabs(az.y) * ob.extent.z,
                         std::fabs(ax.z) * ob.extent.x + std::fabs(ay.z) * ob.extent.y + std::fabs(az.z) * ob.extent.z);
            }
            else
            {
                const R r = max3(ob.extent);
                half = v(r, r, r);
            }
            const R c[3] = {ob.center.x, ob.center.y, ob.center.z}, hh[3] = {half.x, half.y, half.z};
            for (int k = 0; k < 3; ++k)
            {
                S->lo[i][k] = c[k] - hh[k] * (1 + 1e-9) - 1e-12;
                S->hi[i][k] = c[k] + hh[k] * (1 + 1e-9) + 1e-12;
            }
        }
    }
    // light table (core/scene.cu:677-706): area x luminance, sequential CDF
    R total = 0;
    std::vector<R> w;
    for (int i = 0; i < np; ++i)
    {
        const Mat& m = S->mats[S->prim_mat[i]];
        if (m.shading != MAT_LIGHT) continue;
        R area = 0;
        if (S->prim_type[i] == OBJ_CUBE)
        {
            const V e = S->objs[i].extent;
            area = 8 * (e.x * e.y + e.x * e.z + e.y * e.z);
        }
        else if (S->prim_type[i] == OBJ_SPHERE)
            area = 4 * PI * max3(S->objs[i].extent) * max3(S->objs[i].extent);
        const R wt = std::max(area * dot(m.emissive, v(0.2126, 0.7152, 0.0722)), 1e-20);
        total += wt;
        w.push_back(wt);
        S->lights.push_back(Light{i, S->prim_type[i], S->prim_mat[i], 0, 0});
    }
    R acc = 0;
    for (size_t k = 0; k < S->lights.size(); ++k)
    {
        S->lights[k].select_prob = w[k] / total;
        acc += S->lights[k].select_prob;
        S->lights[k].cdf = acc;
    }
    long long off = 0;
    for (int t = 0; t < n_tex; ++t)
    {
        S->tex_off.push_back((int)off);
        S->tex_w.push_back(tex_sizes[2 * t]);
        S->tex_h.push_back(tex_sizes[2 * t + 1]);
        off += (long long)tex_sizes[2 * t] * tex_sizes[2 * t + 1];
    }
    S->texels.assign(texels, texels + 3 * (size_t)off);
    S->tab.cmf.assign(cmf, cmf + 421 * 3);
    S->tab.d65.assign(d65, d65 + 421);
    S->tab.rgb_w.assign(rgb_mlp, rgb_mlp + rgb_n);
    S->tab.lam_w.assign(lam_mlp, lam_mlp + lam_n);
    S->tab.lam_lut.resize(LAM_RES);
    const R step = (780.0 - 360.0) / LAM_RES;
    for (int i = 0; i < LAM_RES; ++i) S->tab.lam_lut[i] = lambda_encode(S->tab, 360.0 + (i + 0.5) * step);
    build_bvh(*S);
    return reinterpret_cast<pt64_scene*>(S);
}

void pt64_destroy(pt64_scene* s) { delete reinterpret_cast<Scene*>(s); }

static Params to_params(const int32_t* ip, const double* dp, uint64_t seed)
{
    Params P{};
    P.width = ip[0];
    P.height = ip[1];
    P.spp = ip[2];
    P.max_depth = ip[3];
    P.use_nee = ip[4];
    P.first_frame = ip[5];
    P.threads = ip[6] > 0 ? ip[6] : (int)std::max(1u, std::thread::hardware_concurrency());
    P.seed = seed;
    for (int k = 0; k < 3; ++k)
    {
        P.cam_o[k] = dp[k];
        P.cam_d[k] = dp[3 + k];
    }
    P.fov = dp[6];
    return P;
}

// mean of the crop window (x0, y0, w, h) of the image the params describe, in window order
int pt64_render_crop(const pt64_scene* s, const int32_t* ip, const double* dp, uint64_t seed, const int32_t* window,
                     double* mean)
{
    if (!s || !ip || !dp || !window || !mean) return -1;
    Params P = to_params(ip, dp, seed);
    if (P.width <= 0 || P.height <= 0 || P.spp <= 0 || P.max_depth <= 0) return -1;
    P.crop_x0 = window[0];
    P.crop_y0 = window[1];
    P.crop_w = window[2];
    P.crop_h = window[3];
    if (P.crop_x0 < 0 || P.crop_y0 < 0 || P.crop_w <= 0 || P.crop_h <= 0 || P.crop_x0 + P.crop_w > P.width ||
        P.crop_y0 + P.crop_h > P.height)
        return -1;
    run(*reinterpret_cast<const Scene*>(s), P, mean, nullptr, nullptr, nullptr);
    return 0;
}

int pt64_render(const pt64_scene* s, const int32_t* ip, const double* dp, uint64_t seed, double* mean, double* per_sample)
{
    if (!s || !ip || !dp) return -1;
    const Params P = to_params(ip, dp, seed);
    if (P.width <= 0 || P.height <= 0 || P.spp <= 0 || P.max_depth <= 0) return -1;
    run(*reinterpret_cast<const Scene*>(s), P, mean, per_sample, nullptr, nullptr);
    return 0;
}

void pt64_set_sdf_f32(pt64_scene* s, int on) { reinterpret_cast<Scene*>(s)->sdf_f32 = on != 0; }

void pt64_set_medium(pt64_scene* s, const double* m)
{
    Scene* S = reinterpret_cast<Scene*>(s);
    if (!m)
    {
        S->med_on = false;
        return;
    }
    S->med_on = true;
    for (int k = 0; k < 3; ++k)
    {
        S->med_lo[k] = m[k];
        S->med_hi[k] = m[3 + k];
    }
    S->med_sigma = m[6];
    S->med_albedo = m[7];
    S->med_g = m[8];
    S->med_emission = m[9];
}

int pt64_adjoint_medium(const pt64_scene* s, const int32_t* ip, const double* dp, uint64_t seed, const double* dl_dxyz,
                        double* grad2)
{
    if (!s || !ip || !dp || !dl_dxyz || !grad2) return -1;
    const Params P = to_params(ip, dp, seed);
    if (P.width <= 0 || P.height <= 0 || P.spp <= 0 || P.max_depth <= 0) return -1;
    run(*reinterpret_cast<const Scene*>(s), P, nullptr, nullptr, dl_dxyz, nullptr, grad2);
    return 0;
}

// the medium adjoint over a window (x0, y0, w, h) of the image: the window's
// pixels with the full image's rays and streams; dl_dxyz covers the full image
int pt64_adjoint_medium_crop(const pt64_scene* s, const int32_t* ip, const double* dp, uint64_t seed,
                             const int32_t* window, const double* dl_dxyz, double* grad2)
{
    if (!s || !ip || !dp || !window || !dl_dxyz || !grad2) return -1;
    Params P = to_params(ip, dp, seed);
    if (P.width <= 0 || P.height <= 0 || P.spp <= 0 || P.max_depth <= 0) return -1;
    P.crop_x0 = window[0];
    P.crop_y0 = window[1];
    P.crop_w = window[2];
    P.crop_h = window[3];
    if (P.crop_x0 < 0 || P.crop_y0 < 0 || P.crop_w <= 0 || P.crop_h <= 0 || P.crop_x0 + P.crop_w > P.width ||
        P.crop_y0 + P.crop_h > P.height)
        return -1;
    run(*reinterpret_cast<const Scene*>(s), P, nullptr, nullptr, dl_dxyz, nullptr, grad2);
    return 0;
}

int pt64_adjoint(const pt64_scene* s, const int32_t* ip, const double* dp, uint64_t seed, const double* dl_dxyz, double* grad)
{
    if (!s || !ip || !dp || !dl_dxyz || !grad) return -1;
    const Params P = to_params(ip, dp, seed);
    if (P.width <= 0 || P.height <= 0 || P.spp <= 0 || P.max_depth <= 0) return -1;
    run(*reinterpret_cast<const Scene*>(s), P, nullptr, nullptr, dl_dxyz, grad);
    return 0;
}
}
