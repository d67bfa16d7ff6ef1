// Small 3-vector type for the renderer's host and device code.
//
// A distinct type (not CUDA's float3) keeps our operators from colliding with
// any other library's global float3 operators.  Every operation is written out
// in a fixed order (x, y, z; left-to-right sums) because the GPU kernels and
// the CPU oracle must round identically; nothing here may be reassociated, and
// every translation unit that includes it is compiled without FMA contraction.
#pragma once
#include "ar_detmath.h"

#if defined(__CUDACC__)
#define AR_HD __host__ __device__ __forceinline__
#else
#define AR_HD static inline
#endif

namespace ar
{
struct V3
{
    float x, y, z;
};

AR_HD V3 v3(float x, float y, float z) { V3 r; r.x = x; r.y = y; r.z = z; return r; }
AR_HD V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
AR_HD V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
AR_HD V3 operator-(V3 a) { return v3(-a.x, -a.y, -a.z); }
AR_HD V3 operator*(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
AR_HD V3 operator*(float s, V3 a) { return v3(a.x * s, a.y * s, a.z * s); }
AR_HD V3 operator*(V3 a, V3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
AR_HD V3 operator/(V3 a, float s) { return v3(a.x / s, a.y / s, a.z / s); }
AR_HD V3 operator+(V3 a, float s) { return v3(a.x + s, a.y + s, a.z + s); }
AR_HD float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
AR_HD V3 cross(V3 a, V3 b)
{
    return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
AR_HD float length(V3 a) { return sqrtf(dot(a, a)); }
// normalisation with the zero guard used throughout the renderer
AR_HD V3 normalize(V3 v)
{
    const float l2 = dot(v, v);
    if (l2 <= 1e-20f) return v3(0.0f, 0.0f, 0.0f);
    const float inv = arm_rsqrtf(l2);
    return v * inv;
}
AR_HD V3 vmin(V3 a, V3 b) { return v3(fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z)); }
AR_HD V3 vmax(V3 a, V3 b) { return v3(fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z)); }
AR_HD V3 vmax(V3 a, float b) { return v3(fmaxf(a.x, b), fmaxf(a.y, b), fmaxf(a.z, b)); }
AR_HD float max3(V3 a) { return fmaxf(a.x, fmaxf(a.y, a.z)); }
AR_HD float sum3(V3 a) { return a.x + a.y + a.z; }
AR_HD bool all_zero(V3 a) { return a.x == 0.0f && a.y == 0.0f && a.z == 0.0f; }
AR_HD V3 reflect(V3 v, V3 n) { return v - 2.0f * dot(v, n) * n; }
AR_HD float comp(V3 a, int k) { return k == 0 ? a.x : (k == 1 ? a.y : a.z); }
AR_HD float lerpf(float a, float b, float t) { return a * (1.0f - t) + b * t; }
AR_HD float signf(float a) { return a > 0.0f ? 1.0f : (a < 0.0f ? -1.0f : 0.0f); }
AR_HD bool is_nanf(float x) { return x != x; }
AR_HD float clampf(float v, float a, float b) { return is_nanf(v) ? 0.0f : fminf(fmaxf(v, a), b); }
AR_HD float saturate(float v) { return is_nanf(v) ? 0.0f : fminf(fmaxf(v, 0.0f), 1.0f); }
// reciprocal that maps +-0 to +-FLT_MAX instead of infinity
AR_HD float inv_safe(float x) { return (x == 0.0f) ? (x >= 0.0f ? 3.402823466e+38f : -3.402823466e+38f) : 1.0f / x; }

// Row-major 3x3; m * v takes the dot of each row with v.
struct M3
{
    V3 r0, r1, r2;
};
AR_HD V3 mul(const M3& m, V3 v) { return v3(dot(m.r0, v), dot(m.r1, v), dot(m.r2, v)); }
AR_HD M3 mul(const M3& a, const M3& b)
{
    const V3 c0 = v3(b.r0.x, b.r1.x, b.r2.x);
    const V3 c1 = v3(b.r0.y, b.r1.y, b.r2.y);
    const V3 c2 = v3(b.r0.z, b.r1.z, b.r2.z);
    M3 r;
    r.r0 = v3(dot(a.r0, c0), dot(a.r0, c1), dot(a.r0, c2));
    r.r1 = v3(dot(a.r1, c0), dot(a.r1, c1), dot(a.r1, c2));
    r.r2 = v3(dot(a.r2, c0), dot(a.r2, c1), dot(a.r2, c2));
    return r;
}
AR_HD M3 transpose(const M3& m)
{
    M3 r;
    r.r0 = v3(m.r0.x, m.r1.x, m.r2.x);
    r.r1 = v3(m.r0.y, m.r1.y, m.r2.y);
    r.r2 = v3(m.r0.z, m.r1.z, m.r2.z);
    return r;
}
} // namespace ar
