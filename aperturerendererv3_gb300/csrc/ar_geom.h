// Ray-triangle intersection shared by the GPU traversal kernels and the CPU
// oracle, so closest-hit primitive ids and hit distances agree bit for bit.
//
// Method: the watertight test of S. Woop, C. Benthin, I. Wald, "Watertight
// Ray/Triangle Intersection", JCGT 2(1), 2013: shear the triangle into a frame
// where the ray is +z, evaluate the three 2-D edge functions, and fall back to
// double precision when an edge function is exactly zero.  Triangles are
// two-sided.  Hits are accepted for t in (0, inf); the caller applies its own
// [tmin, tmax) window, and ties between primitives at the same t are broken
// by the smallest primitive id (see ar_traverse.cuh).
#pragma once
#include "ar_vec.h"

namespace ar
{
// Per-ray constants of the shear transform.
struct RayShear
{
    int kx, ky, kz;
    float sx, sy, sz;
};

AR_HD RayShear make_shear(V3 d)
{
    RayShear s;
    const float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
    s.kz = (ax > ay) ? ((ax > az) ? 0 : 2) : ((ay > az) ? 1 : 2);
    s.kx = s.kz + 1;
    if (s.kx == 3) s.kx = 0;
    s.ky = s.kx + 1;
    if (s.ky == 3) s.ky = 0;
    if (comp(d, s.kz) < 0.0f)
    {
        const int t = s.kx;
        s.kx = s.ky;
        s.ky = t;
    }
    const float dz = comp(d, s.kz);
    s.sx = comp(d, s.kx) / dz;
    s.sy = comp(d, s.ky) / dz;
    s.sz = 1.0f / dz;
    return s;
}

// Returns true on a hit with t > 0; writes t and the barycentric weights of
// v0, v1, v2 (b0 + b1 + b2 == 1 up to rounding).
AR_HD bool tri_intersect(const RayShear& s, V3 o, V3 v0, V3 v1, V3 v2,
                         float* t_out, float* b0_out, float* b1_out, float* b2_out)
{
    const V3 A = v0 - o;
    const V3 B = v1 - o;
    const V3 C = v2 - o;
    const float Akz = comp(A, s.kz), Bkz = comp(B, s.kz), Ckz = comp(C, s.kz);
    const float Ax = comp(A, s.kx) - s.sx * Akz;
    const float Ay = comp(A, s.ky) - s.sy * Akz;
    const float Bx = comp(B, s.kx) - s.sx * Bkz;
    const float By = comp(B, s.ky) - s.sy * Bkz;
    const float Cx = comp(C, s.kx) - s.sx * Ckz;
    const float Cy = comp(C, s.ky) - s.sy * Ckz;
    float U = Cx * By - Cy * Bx;
    float V = Ax * Cy - Ay * Cx;
    float W = Bx * Ay - By * Ax;
    if (U == 0.0f || V == 0.0f || W == 0.0f)
    {
        const double CxBy = (double)Cx * (double)By;
        const double CyBx = (double)Cy * (double)Bx;
        U = (float)(CxBy - CyBx);
        const double AxCy = (double)Ax * (double)Cy;
        const double AyCx = (double)Ay * (double)Cx;
        V = (float)(AxCy - AyCx);
        const double BxAy = (double)Bx * (double)Ay;
        const double ByAx = (double)By * (double)Ax;
        W = (float)(BxAy - ByAx);
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    const float det = U + V + W;
    if (det == 0.0f) return false;
    const float Az = s.sz * Akz;
    const float Bz = s.sz * Bkz;
    const float Cz = s.sz * Ckz;
    const float T = U * Az + V * Bz + W * Cz;
    // t = T / det must be positive: T and det share a sign
    if ((det > 0.0f && T <= 0.0f) || (det < 0.0f && T >= 0.0f)) return false;
    const float t = T / det;
    if (!(t > 0.0f)) return false;
    *t_out = t;
    *b0_out = U / det;
    *b1_out = V / det;
    *b2_out = W / det;
    return true;
}

// Hit frame for a triangle hit: position along the ray and the geometric
// normal turned to face the incoming ray.
AR_HD void tri_frame(V3 o, V3 d, float t, V3 v0, V3 v1, V3 v2, V3* pos, V3* nrm)
{
    *pos = o + d * t;
    V3 n = normalize(cross(v1 - v0, v2 - v0));
    if (dot(n, d) > 0.0f) n = -n;
    *nrm = n;
}
} // namespace ar
