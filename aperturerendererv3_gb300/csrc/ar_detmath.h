// Deterministic single-precision transcendentals shared by the sm_103a kernels
// and by every host build that must agree with them bit for bit.
//
// Why: the path tracer's parity contract is that a path traced on the GPU and
// the same path traced on the CPU produce the same radiance.  CUDA's device
// math library and the host libm round differently in the last ulp, and a
// one-ulp difference in sincosf / rsqrtf flips Russian-roulette or light-pick
// decisions downstream.  Every function here is built only from IEEE
// correctly-rounded operations (+, -, *, /, sqrt, explicit fmaf) with a fixed
// evaluation order, so host (gcc, -ffp-contract=off) and device (nvcc,
// -fmad=false) produce identical bits.
//
// Methods (all textbook, none taken from a vendor library):
//   * sin/cos: Cody-Waite reduction by pi/2 with a three-part constant, then
//     the Taylor series of sin and cos on [-pi/4, pi/4] (terms through x^13 /
//     x^14), Horner form.
//   * exp: reduction x = k ln2 + r, |r| <= ln2/2, Taylor series of e^r through
//     r^9, scaling by 2^k through exponent-field construction.
//   * log: x = m 2^e with m in [sqrt(1/2), sqrt(2)); log m = 2 atanh(s),
//     s = (m-1)/(m+1), odd series through s^15.
//   * erfc: the rational-Chebyshev fit "erfcc" of Press, Teukolsky,
//     Vetterling & Flannery, Numerical Recipes in C (2nd ed.) section 6.2,
//     fractional error below 1.2e-7.
//   * pow: exp(y log x) for x > 0 (the only domain the renderer uses) with the
//     IEEE special cases for x == 0, 1 and y == 0.
// Accuracy is checked against the host libm in the CPU test-suite (a few ulp
// over the ranges the renderer uses); determinism is the contract.
#pragma once

#include <stdint.h>
#include <string.h>
#include <math.h>

#if defined(__CUDACC__)
#define ARM_FN __host__ __device__ __forceinline__
#else
#define ARM_FN static inline
#endif

namespace arm_detail
{
ARM_FN float bits_to_float(uint32_t u)
{
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float f;
    memcpy(&f, &u, 4);
    return f;
#endif
}
ARM_FN uint32_t float_to_bits(float f)
{
#if defined(__CUDA_ARCH__)
    return __float_as_uint(f);
#else
    uint32_t u;
    memcpy(&u, &f, 4);
    return u;
#endif
}
ARM_FN bool is_nan(float x) { return x != x; }
ARM_FN bool is_inf(float x) { return (float_to_bits(x) & 0x7fffffffu) == 0x7f800000u; }
// 2^k for k in [-126, 127] as an exact float
ARM_FN float pow2i(int k) { return bits_to_float((uint32_t)(k + 127) << 23); }

// Taylor coefficients 1/n! rounded to float (pure mathematics).
#define ARM_INV_FACT_2 0.5f
#define ARM_INV_FACT_3 1.66666666666666666667e-1f
#define ARM_INV_FACT_4 4.16666666666666666667e-2f
#define ARM_INV_FACT_5 8.33333333333333333333e-3f
#define ARM_INV_FACT_6 1.38888888888888888889e-3f
#define ARM_INV_FACT_7 1.98412698412698412698e-4f
#define ARM_INV_FACT_8 2.48015873015873015873e-5f
#define ARM_INV_FACT_9 2.75573192239858906526e-6f
#define ARM_INV_FACT_10 2.75573192239858906526e-7f
#define ARM_INV_FACT_11 2.50521083854417187751e-8f
#define ARM_INV_FACT_12 2.08767569878680989792e-9f
#define ARM_INV_FACT_13 1.60590438368216145994e-10f
#define ARM_INV_FACT_14 1.14707455977297247139e-11f

// sin(r), cos(r) for |r| <= pi/4 (slightly beyond is fine)
ARM_FN float sin_poly(float r)
{
    const float r2 = r * r;
    float p = -ARM_INV_FACT_13;
    p = fmaf(p, r2, ARM_INV_FACT_11);
    p = fmaf(p, r2, -ARM_INV_FACT_9);
    p = fmaf(p, r2, ARM_INV_FACT_7);
    p = fmaf(p, r2, -ARM_INV_FACT_5);
    p = fmaf(p, r2, ARM_INV_FACT_3);
    // sin r = r - r^3 * p
    return fmaf(-(r * r2), p, r);
}
ARM_FN float cos_poly(float r)
{
    const float r2 = r * r;
    float p = -ARM_INV_FACT_14;
    p = fmaf(p, r2, ARM_INV_FACT_12);
    p = fmaf(p, r2, -ARM_INV_FACT_10);
    p = fmaf(p, r2, ARM_INV_FACT_8);
    p = fmaf(p, r2, -ARM_INV_FACT_6);
    p = fmaf(p, r2, ARM_INV_FACT_4);
    // cos r = 1 - r^2/2 + r^4 * p
    const float r4 = r2 * r2;
    const float hi = fmaf(-0.5f, r2, 1.0f);
    return fmaf(r4, p, hi);
}

// pi/2 split into three floats whose sum carries ~72 significant bits.
#define ARM_PIO2_1 1.5707963705062866211e+00f   // float(pi/2)
#define ARM_PIO2_2 -4.3711388286737928865e-08f  // float(pi/2 - PIO2_1)
#define ARM_PIO2_3 -1.7151245100059240264e-15f  // float(pi/2 - PIO2_1 - PIO2_2)
#define ARM_2_OVER_PI 6.3661977236758134308e-01f

// Reduce x to r in [-pi/4, pi/4] and quadrant q (x = q pi/2 + r).  Exact
// enough for |x| < 2^17, the range every caller in the renderer uses.
ARM_FN float reduce_pio2(float x, int& q)
{
    const float k = rintf(x * ARM_2_OVER_PI);
    float r = fmaf(-k, ARM_PIO2_1, x);
    r = fmaf(-k, ARM_PIO2_2, r);
    r = fmaf(-k, ARM_PIO2_3, r);
    q = (int)k;
    return r;
}
} // namespace arm_detail

ARM_FN void arm_sincosf(float x, float* s, float* c)
{
    using namespace arm_detail;
    if (is_nan(x) || is_inf(x))
    {
        *s = x - x;
        *c = x - x;
        return;
    }
    int q;
    const float r = reduce_pio2(x, q);
    const float sr = sin_poly(r);
    const float cr = cos_poly(r);
    switch (q & 3)
    {
        case 0: *s = sr;  *c = cr;  break;
        case 1: *s = cr;  *c = -sr; break;
        case 2: *s = -sr; *c = -cr; break;
        default: *s = -cr; *c = sr; break;
    }
}
ARM_FN float arm_sinf(float x) { float s, c; arm_sincosf(x, &s, &c); return s; }
ARM_FN float arm_cosf(float x) { float s, c; arm_sincosf(x, &s, &c); return c; }
ARM_FN float arm_tanf(float x) { float s, c; arm_sincosf(x, &s, &c); return s / c; }

ARM_FN float arm_expf(float x)
{
    using namespace arm_detail;
    if (is_nan(x)) return x;
    if (x > 88.72283935546875f) return bits_to_float(0x7f800000u);
    if (x < -103.972084045410156f) return 0.0f;
    const float LOG2E = 1.44269504088896340736f;
    const float LN2_HI = 6.93145751953125e-1f;        // 12 significant bits: k*LN2_HI exact
    const float LN2_LO = 1.42860682030941723212e-6f;  // ln2 - LN2_HI
    const float k = rintf(x * LOG2E);
    float r = fmaf(-k, LN2_HI, x);
    r = fmaf(-k, LN2_LO, r);
    float p = ARM_INV_FACT_9;
    p = fmaf(p, r, ARM_INV_FACT_8);
    p = fmaf(p, r, ARM_INV_FACT_7);
    p = fmaf(p, r, ARM_INV_FACT_6);
    p = fmaf(p, r, ARM_INV_FACT_5);
    p = fmaf(p, r, ARM_INV_FACT_4);
    p = fmaf(p, r, ARM_INV_FACT_3);
    p = fmaf(p, r, ARM_INV_FACT_2);
    p = fmaf(p, r, 1.0f);
    p = fmaf(p, r, 1.0f);
    int ki = (int)k;
    if (ki > 127)
    {
        p = p * 2.0f;
        ki -= 1;
    }
    if (ki < -126)
    {
        // two exact-or-once-rounded scalings, same order on every target
        p = p * pow2i(-126);
        ki += 126;
    }
    return p * pow2i(ki);
}

ARM_FN float arm_logf(float x)
{
    using namespace arm_detail;
    if (is_nan(x)) return x;
    if (x < 0.0f) return bits_to_float(0x7fc00000u);
    if (x == 0.0f) return bits_to_float(0xff800000u);
    if (is_inf(x)) return x;
    int e = 0;
    uint32_t u = float_to_bits(x);
    if ((u >> 23) == 0)
    {
        // subnormal: scale into the normal range exactly
        x = x * 8388608.0f;  // 2^23
        u = float_to_bits(x);
        e = -23;
    }
    e += (int)(u >> 23) - 127;
    float m = bits_to_float((u & 0x007fffffu) | 0x3f800000u);  // [1, 2)
    if (m > 1.41421356237309504880f)
    {
        m = m * 0.5f;
        e += 1;
    }
    const float s = (m - 1.0f) / (m + 1.0f);
    const float s2 = s * s;
    float p = 1.0f / 15.0f;
    p = fmaf(p, s2, 1.0f / 13.0f);
    p = fmaf(p, s2, 1.0f / 11.0f);
    p = fmaf(p, s2, 1.0f / 9.0f);
    p = fmaf(p, s2, 1.0f / 7.0f);
    p = fmaf(p, s2, 1.0f / 5.0f);
    p = fmaf(p, s2, 1.0f / 3.0f);
    // log m = 2s + 2 s^3 p
    const float lm = fmaf(2.0f * s * s2, p, 2.0f * s);
    const float LN2_HI = 6.93145751953125e-1f;
    const float LN2_LO = 1.42860682030941723212e-6f;
    const float fe = (float)e;
    return fmaf(fe, LN2_HI, fmaf(fe, LN2_LO, lm));
}

ARM_FN float arm_log1pf(float x)
{
    using namespace arm_detail;
    if (is_nan(x)) return x;
    const float u = 1.0f + x;
    if (u == 1.0f) return x;
    // log(u) corrected for the rounding of 1 + x
    const float lu = arm_logf(u);
    if (is_inf(u)) return lu;
    return lu - ((u - 1.0f) - x) / u;
}

ARM_FN float arm_powf(float x, float y)
{
    using namespace arm_detail;
    if (y == 0.0f) return 1.0f;
    if (x == 1.0f) return 1.0f;
    if (is_nan(x) || is_nan(y)) return x + y;
    if (x == 0.0f) return (y > 0.0f) ? 0.0f : bits_to_float(0x7f800000u);
    if (x < 0.0f)
    {
        // integer exponents only; the renderer never raises negatives
        const float yi = rintf(y);
        if (yi != y) return bits_to_float(0x7fc00000u);
        const float a = arm_expf(y * arm_logf(-x));
        const int odd = ((int)fmodf(fabsf(yi), 2.0f)) == 1;
        return odd ? -a : a;
    }
    return arm_expf(y * arm_logf(x));
}

ARM_FN float arm_erfcf(float x)
{
    // Numerical Recipes in C, 2nd ed., section 6.2, function erfcc.
    const float z = fabsf(x);
    const float t = 1.0f / fmaf(0.5f, z, 1.0f);
    float p = 0.17087277f;
    p = fmaf(p, t, -0.82215223f);
    p = fmaf(p, t, 1.48851587f);
    p = fmaf(p, t, -1.13520398f);
    p = fmaf(p, t, 0.27886807f);
    p = fmaf(p, t, -0.18628806f);
    p = fmaf(p, t, 0.09678418f);
    p = fmaf(p, t, 0.37409196f);
    p = fmaf(p, t, 1.00002368f);
    p = fmaf(p, t, -1.26551223f);
    const float ans = t * arm_expf(fmaf(-z, z, p));
    return x >= 0.0f ? ans : 2.0f - ans;
}

ARM_FN float arm_rsqrtf(float x) { return 1.0f / sqrtf(x); }

// atan via argument halving + odd Taylor series; asin/acos/atan2 built on it.
ARM_FN float arm_atanf(float x)
{
    using namespace arm_detail;
    if (is_nan(x)) return x;
    const float ax = fabsf(x);
    const bool inv = ax > 1.0f;
    float t = inv ? 1.0f / ax : ax;  // [0, 1]
    // two halvings: atan t = 2 atan(t / (1 + sqrt(1 + t^2)))
    t = t / (1.0f + sqrtf(fmaf(t, t, 1.0f)));
    t = t / (1.0f + sqrtf(fmaf(t, t, 1.0f)));  // t <= tan(pi/16) ~ 0.199
    const float t2 = t * t;
    float p = -1.0f / 15.0f;
    p = fmaf(p, t2, 1.0f / 13.0f);
    p = fmaf(p, t2, -1.0f / 11.0f);
    p = fmaf(p, t2, 1.0f / 9.0f);
    p = fmaf(p, t2, -1.0f / 7.0f);
    p = fmaf(p, t2, 1.0f / 5.0f);
    p = fmaf(p, t2, -1.0f / 3.0f);
    float a = fmaf(t * t2, p, t) * 4.0f;
    if (inv) a = 1.57079632679489661923f - a;
    return x < 0.0f ? -a : a;
}
ARM_FN float arm_atan2f(float y, float x)
{
    const float PI = 3.14159265358979323846f;
    if (x != x || y != y) return x + y;
    if (x == 0.0f)
    {
        if (y == 0.0f) return 0.0f;
        return y > 0.0f ? 0.5f * PI : -0.5f * PI;
    }
    const float a = arm_atanf(y / x);
    if (x > 0.0f) return a;
    return (y >= 0.0f) ? a + PI : a - PI;
}
ARM_FN float arm_asinf(float x)
{
    if (x > 1.0f || x < -1.0f) return arm_detail::bits_to_float(0x7fc00000u);
    return arm_atan2f(x, sqrtf(fmaf(-x, x, 1.0f)));
}
ARM_FN float arm_acosf(float x)
{
    if (x > 1.0f || x < -1.0f) return arm_detail::bits_to_float(0x7fc00000u);
    return arm_atan2f(sqrtf(fmaf(-x, x, 1.0f)), x);
}
ARM_FN float arm_fmodf(float x, float y) { return fmodf(x, y); }

// Unsuffixed spellings used by code written against <cmath> overloads.
ARM_FN float arm_sin(float x) { return arm_sinf(x); }
ARM_FN float arm_cos(float x) { return arm_cosf(x); }
ARM_FN float arm_exp(float x) { return arm_expf(x); }
ARM_FN float arm_log(float x) { return arm_logf(x); }
ARM_FN float arm_pow(float x, float y) { return arm_powf(x, y); }
#if !defined(__CUDA_ARCH__)
// double overloads only exist for host-side bookkeeping; no kernel calls them
static inline double arm_sin(double x) { return sin(x); }
static inline double arm_cos(double x) { return cos(x); }
static inline double arm_exp(double x) { return exp(x); }
static inline double arm_log(double x) { return log(x); }
static inline double arm_pow(double x, double y) { return pow(x, y); }
#endif
