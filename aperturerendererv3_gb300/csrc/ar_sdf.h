// Smooth-union signed-distance object: up to AR_SDF_MAX_PRIMS spheres, boxes
// and tori (torus axis +y) combined with a polynomial smooth minimum of width
// k, marched like the reference's RaymarchLocal (core/object/sdf/sdf_base.cuh:
// 53-105): the start point's sign decides which crossing ends the march, the
// step is the distance (at least eps / 2), and the hit is the last point before
// the crossing.  The reference's own shapes are the torus
// (core/object/sdf/sdf_torus.cuh:14-18) and others; the union is new.
// Host + device.
#pragma once
#include "ar_vec.h"

#define AR_SDF_MAX_PRIMS 64
#define AR_SDF_SPHERE 0
#define AR_SDF_BOX 1
#define AR_SDF_TORUS 2
#define AR_SDF_STEPS 512  // SDF_STEPS (core/config.cuh:75)

namespace ar
{
// primitives: two float4 each, (kind, centre xyz), (size xyz, bounding
// radius: sdf_bounding_radius, filled when the union is uploaded)
struct SdfUnion
{
    const float4* prims;
    int count;
    float k;
    V3 lo, hi;  // bounds of the zero set
};

AR_HD float sdf_prim(float4 a, float4 b, V3 p)
{
    const V3 q = p - v3(a.y, a.z, a.w);
    const int kind = (int)a.x;
    if (kind == AR_SDF_SPHERE) return length(q) - b.x;
    if (kind == AR_SDF_BOX)
    {
        const V3 d = v3(fabsf(q.x) - b.x, fabsf(q.y) - b.y, fabsf(q.z) - b.z);
        const V3 dp = vmax(d, 0.0f);
        return length(dp) + fminf(fmaxf(d.x, fmaxf(d.y, d.z)), 0.0f);
    }
    // torus in the xz plane: (|q.xz| - R, q.y) at distance r
    const float rxz = sqrtf(q.x * q.x + q.z * q.z) - b.x;
    return sqrtf(rxz * rxz + q.y * q.y) - b.y;
}

// polynomial smooth minimum (width k > 0)
AR_HD float smin_poly(float a, float b, float k)
{
    const float h = fmaxf(k - fabsf(a - b), 0.0f) / k;
    return fminf(a, b) - h * h * k * 0.25f;
}

// radius of a sphere about the primitive's centre that holds it
AR_HD float sdf_bounding_radius(float kind, float sx, float sy, float sz)
{
    const int k = (int)kind;
    if (k == AR_SDF_SPHERE) return sx;
    if (k == AR_SDF_BOX) return sqrtf(sx * sx + sy * sy + sz * sz);
    return sx + sy;  // torus: major + minor radius
}

// The smooth union folded left to right.  A primitive whose distance b is at
// least k above the running value d leaves smin_poly(d, b) = d exactly (its
// blend weight is zero), so it is skipped: spheres after their distance, boxes
// and tori already when their bounding sphere's distance, lowered by a margin
// of 2^-20 (|q| + R) that covers the rounding of both evaluations of the same
// q, is k above d.  Every skip returns what the full fold would, bit for bit.
AR_HD float sdf_union(const SdfUnion& s, V3 p)
{
    float d = sdf_prim(s.prims[0], s.prims[1], p);
    for (int i = 1; i < s.count; ++i)
    {
        const float4 a = s.prims[2 * i], b = s.prims[2 * i + 1];
        if ((int)a.x != AR_SDF_SPHERE)
        {
            const V3 q = p - v3(a.y, a.z, a.w);
            const float lq = length(q);
            const float lower = (lq - b.w) - 0x1p-20f * (lq + b.w);
            if (lower - d >= s.k) continue;
        }
        const float di = sdf_prim(a, b, p);
        if (di - d >= s.k) continue;
        d = smin_poly(d, di, s.k);
    }
    return d;
}

// entry / exit distances of the ray through the union's bounds
AR_HD bool sdf_bounds_interval(const SdfUnion& s, V3 o, V3 d, float* t0, float* t1)
{
    const V3 inv = v3(inv_safe(d.x), inv_safe(d.y), inv_safe(d.z));
    const V3 a = (s.lo - o) * inv, b = (s.hi - o) * inv;
    const V3 tn = vmin(a, b), tf = vmax(a, b);
    *t0 = fmaxf(fmaxf(tn.x, tn.y), tn.z);
    *t1 = fminf(fminf(tf.x, tf.y), tf.z);
    return *t0 <= *t1 && *t1 > 0.0f;
}

// The march and the normal are called out of line: inlined into the BVH
// traversal loop they would raise its register count for every ray.
#if defined(__CUDACC__)
#define AR_SDF_CALL static __host__ __device__ __noinline__
#else
#define AR_SDF_CALL inline
#endif

// distance to the first surface crossing in the bounds before tmax, or -1
AR_SDF_CALL float sdf_march(const SdfUnion& s, V3 o, V3 d, float eps, float tmax)
{
    float t0, t1;
    if (s.count <= 0 || !sdf_bounds_interval(s, o, d, &t0, &t1) || t0 >= tmax) return -1.0f;
    t1 = fminf(t1, tmax);
    const bool start_inside = sdf_union(s, o) <= 0.0f;
    const float min_step = eps * 0.5f;
    float t = fmaxf(0.0f, t0);
    for (int i = 0; i < AR_SDF_STEPS; ++i)
    {
        const float t_last = t;
        const float dist = sdf_union(s, o + d * t);
        if (start_inside ? (dist > 0.0f && dist < eps) : (dist < 0.0f && -dist < eps)) return t_last;
        t += fmaxf(fabsf(dist), min_step);
        if (t > t1) break;
    }
    return -1.0f;
}

// outward normal by central differences (sdfNormalUnit, core/object/sdf/sdf_base.cuh:40-51)
AR_SDF_CALL V3 sdf_normal(const SdfUnion& s, V3 p, float h)
{
    const float dx = sdf_union(s, p + v3(h, 0, 0)) - sdf_union(s, p - v3(h, 0, 0));
    const float dy = sdf_union(s, p + v3(0, h, 0)) - sdf_union(s, p - v3(0, h, 0));
    const float dz = sdf_union(s, p + v3(0, 0, h)) - sdf_union(s, p - v3(0, 0, h));
    return normalize(v3(dx, dy, dz));
}
} // namespace ar
