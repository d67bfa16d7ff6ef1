// Glue compiled into the patched reference tree (oracle only; see
// oracle/prepare_ref.py).  The reference has no triangle primitive; this adds
// one by calling the same watertight test the GPU kernels use
// (aperturerendererv3_gb300/csrc/ar_geom.h), and fills the reference's
// IntersectionContext the way IntersectAABBObject does
// (core/object/aabb.cuh:75-87): world hit position and normal, material
// G-buffer with the hit normal.
#pragma once
#include "ar_geom.h"

namespace ref_glue
{
// per-thread traversal counters (node pops, primitive tests) for the
// algorithmic-bytes figure of the traversal roofline
inline thread_local unsigned long long g_node_visits = 0;
inline thread_local unsigned long long g_prim_tests = 0;
} // namespace ref_glue

#ifdef __CUDA_ARCH__
#define REF_NODE_VISIT_HOOK
#else
#define REF_NODE_VISIT_HOOK (++ref_glue::g_node_visits)
#endif

namespace ref_glue
{

__host__ __device__ inline ar::V3 to_v(const float3 a) { return ar::v3(a.x, a.y, a.z); }
__host__ __device__ inline float3 to_f(const ar::V3 a) { return float3{a.x, a.y, a.z}; }

__host__ __device__ inline IntersectionContext IntersectTriangleObject(const float3 rayOrigin, const float3 rayDirection, const SceneObject& object)
{
    IntersectionContext ctx{};
    const ar::V3 o = to_v(rayOrigin);
    const ar::V3 d = to_v(rayDirection);
    const ar::RayShear s = ar::make_shear(d);
    float t, b0, b1, b2;
    if (!ar::tri_intersect(s, o, to_v(object.triV0_), to_v(object.triV1_), to_v(object.triV2_), &t, &b0, &b1, &b2))
    {
        return ctx;
    }
    ar::V3 p, n;
    ar::tri_frame(o, d, t, to_v(object.triV0_), to_v(object.triV1_), to_v(object.triV2_), &p, &n);
    ctx.bHit_ = true;
    ctx.distance_ = t;
    ctx.hitLocalPosition_ = float3{b0, b1, b2};
    ctx.hitLocalNormal_ = to_f(n);
    ctx.hitPosition_ = to_f(p);
    ctx.hitNormal_ = to_f(n);
    ctx.gbuffer_ = object.material_.texture_.baseTexture_;
    ctx.gbuffer_.normal_ = to_f(n);
    return ctx;
}
} // namespace ref_glue
