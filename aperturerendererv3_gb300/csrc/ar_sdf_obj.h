// SDF scene objects (EObjectType::OBJ_SDF, core/object/sdf/*): an oriented box
// (centre, half extent, rotation) whose inside holds a signed distance field
// in unit coordinates, [-extent, extent] -> [-0.5, 0.5]^3.  Two kinds, as the
// reference dispatches them (core/object/sdf/sdf_master.cuh:40-72):
//   torus   SdfTorus (core/object/sdf/sdf_torus.cuh:9-24), params (R, r)
//   volume  a cached grid of distances (core/object/sdf/sdf_volume.cuh,
//           core/object/sdf/sdf_cache_manager.cuh), sampled nearest when far
//           from the surface and trilinear near it, marched with a 0.9 step
// The march (RaymarchLocal, core/object/sdf/sdf_base.cuh:53-105), the hit
// frame (IntersectSDFObject, :107-163) and the overlap test (:165-176) keep
// the reference's operation order.  Volumes are filled on the GPU from the
// reference's torus or diamond functors (core/object/sdf/sdf_diamond.cuh) or
// from caller data.  Host + device.
#pragma once
#include "ar_vec.h"

#define AR_SDF_OBJ_TORUS 0      // ESDFType::SDF_TORUS
#define AR_SDF_OBJ_VOLUME 1     // ESDFType::SDF_VOLUME
#define AR_SDF_FN_TORUS 0       // volume fill functors
#define AR_SDF_FN_DIAMOND 1
#define AR_SDF_OBJ_STEPS 512                // SDF_STEPS (core/config.cuh:75)
#define AR_SDF_VOLUME_STEP_SCALE 0.9f       // SDF_VOLUME_STEP_SCALE (core/config.cuh:76)
#define AR_SDF_VOLUME_NEAREST_SCALE 2.5f    // SDF_VOLUME_USE_NEAREST_SCALE (core/config.cuh:77)

namespace ar
{
struct SdfVolume
{
    const float* data;  // dx * dy * dz distances, x fastest
    int dx, dy, dz;
    float voxel_size_max;  // the distance above which nearest sampling is used
};

// SDFVolumeInfo::ComputeVoxelSize (core/object/sdf/sdf_volume.cuh:22-42)
AR_HD float sdf_volume_voxel_size_max(int dx, int dy, int dz)
{
    const V3 inv = v3(1.0f / fmaxf((float)dx, 1.0f), 1.0f / fmaxf((float)dy, 1.0f), 1.0f / fmaxf((float)dz, 1.0f));
    return length(inv) * AR_SDF_VOLUME_NEAREST_SCALE;
}

AR_HD size_t sdf_index3(int x, int y, int z, int dx, int dy)
{
    return (size_t)z * dx * dy + (size_t)y * dx + x;
}

AR_HD float sdf_volume_nearest(const SdfVolume& v, V3 p01)
{
    const float gx = p01.x * (float)(v.dx - 1), gy = p01.y * (float)(v.dy - 1), gz = p01.z * (float)(v.dz - 1);
    int xi = (int)floorf(gx + 0.5f), yi = (int)floorf(gy + 0.5f), zi = (int)floorf(gz + 0.5f);
    xi = xi < 0 ? 0 : (xi > v.dx - 1 ? v.dx - 1 : xi);
    yi = yi < 0 ? 0 : (yi > v.dy - 1 ? v.dy - 1 : yi);
    zi = zi < 0 ? 0 : (zi > v.dz - 1 ? v.dz - 1 : zi);
    return v.data[sdf_index3(xi, yi, zi, v.dx, v.dy)];
}

AR_HD int sdf_clampi(int a, int lo, int hi) { return a < lo ? lo : (a > hi ? hi : a); }

AR_HD float sdf_volume_trilinear(const SdfVolume& v, V3 p01)
{
    const float gx = p01.x * (float)(v.dx - 1), gy = p01.y * (float)(v.dy - 1), gz = p01.z * (float)(v.dz - 1);
    int x0 = (int)floorf(gx), y0 = (int)floorf(gy), z0 = (int)floorf(gz);
    const int x1 = sdf_clampi(x0 + 1, 0, v.dx - 1), y1 = sdf_clampi(y0 + 1, 0, v.dy - 1), z1 = sdf_clampi(z0 + 1, 0, v.dz - 1);
    x0 = sdf_clampi(x0, 0, v.dx - 1);
    y0 = sdf_clampi(y0, 0, v.dy - 1);
    z0 = sdf_clampi(z0, 0, v.dz - 1);
    const float fx = fminf(fmaxf(gx - (float)x0, 0.0f), 1.0f);
    const float fy = fminf(fmaxf(gy - (float)y0, 0.0f), 1.0f);
    const float fz = fminf(fmaxf(gz - (float)z0, 0.0f), 1.0f);
    const float* d = v.data;
    const float c000 = d[sdf_index3(x0, y0, z0, v.dx, v.dy)], c100 = d[sdf_index3(x1, y0, z0, v.dx, v.dy)];
    const float c010 = d[sdf_index3(x0, y1, z0, v.dx, v.dy)], c110 = d[sdf_index3(x1, y1, z0, v.dx, v.dy)];
    const float c001 = d[sdf_index3(x0, y0, z1, v.dx, v.dy)], c101 = d[sdf_index3(x1, y0, z1, v.dx, v.dy)];
    const float c011 = d[sdf_index3(x0, y1, z1, v.dx, v.dy)], c111 = d[sdf_index3(x1, y1, z1, v.dx, v.dy)];
    const float c00 = c000 * (1.0f - fx) + c100 * fx;
    const float c10 = c010 * (1.0f - fx) + c110 * fx;
    const float c01 = c001 * (1.0f - fx) + c101 * fx;
    const float c11 = c011 * (1.0f - fx) + c111 * fx;
    const float c0 = c00 * (1.0f - fy) + c10 * fy;
    const float c1 = c01 * (1.0f - fy) + c11 * fy;
    return c0 * (1.0f - fz) + c1 * fz;
}

// SampleSDFAdaptive01 at unit position u (SDFVolumeFunctor queries u + 0.5)
AR_HD float sdf_volume_eval(const SdfVolume& v, V3 u)
{
    if (!v.data || v.dx * v.dy * v.dz == 0) return 1.0e20f;
    const V3 p01 = u + 0.5f;
    const float dn = sdf_volume_nearest(v, p01);
    return (fabsf(dn) > v.voxel_size_max) ? dn : sdf_volume_trilinear(v, p01);
}

AR_HD float sdf_torus_eval(V3 u, float R, float r)
{
    const float qx = sqrtf(u.x * u.x + u.z * u.z) - R;
    return sqrtf(qx * qx + u.y * u.y) - r;
}

// SdfDiamondUnit (core/object/sdf/sdf_diamond.cuh:19-62), the reference's
// volume-fill example shape; params (d, bias, tableZ, scale), zeros -> defaults
AR_HD float sdf_plane(V3 p, V3 n, float d)
{
    const float len = fmaxf(sqrtf(n.x * n.x + n.y * n.y + n.z * n.z), 1e-8f);
    return (p.x * n.x + p.y * n.y + p.z * n.z - d) / len;
}

AR_HD float sdf_diamond_eval(V3 u, float4 prm)
{
    const float d = (prm.x != 0.0f) ? prm.x : 0.94f;
    const float bias = (prm.y != 0.0f) ? prm.y : 0.5f;
    const float tableZ = (prm.z != 0.0f) ? prm.z : 0.3f;
    const float scale = (prm.w != 0.0f) ? prm.w : 1.0f;
    const float scaleInv = 1.0f / scale;
    const V3 p = v3(u.x * scaleInv, u.y * scaleInv, u.z * scaleInv);
    const float af2 = 4.0f / 3.141592654f;
    const float s = arm_atan2f(p.y, p.x);
    const float sf = floorf(s * af2 + bias) / af2;
    const float sf2 = floorf(s * af2) / af2;
    const float csf = arm_cosf(sf), ssf = arm_sinf(sf);
    const float cs = arm_cosf(s), ss = arm_sinf(s);
    const float csf1 = arm_cosf(sf + 0.21f), ssf1 = arm_sinf(sf + 0.21f);
    const float csf2 = arm_cosf(sf - 0.21f), ssf2 = arm_sinf(sf - 0.21f);
    const float csf8 = arm_cosf(sf2 + 0.393f), ssf8 = arm_sinf(sf2 + 0.393f);
    float dMax = -1e20f;
    dMax = fmaxf(dMax, sdf_plane(p, v3(csf, ssf, 1.444f), d));
    dMax = fmaxf(dMax, sdf_plane(p, v3(csf, ssf, -1.072f), d));
    dMax = fmaxf(dMax, sdf_plane(p, v3(0.0f, 0.0f, 1.0f), tableZ));
    dMax = fmaxf(dMax, sdf_plane(p, v3(0.0f, 0.0f, -1.0f), 0.865f));
    dMax = fmaxf(dMax, sdf_plane(p, v3(cs, ss, 0.0f), 0.911f));
    dMax = fmaxf(dMax, sdf_plane(p, v3(csf1, ssf1, -1.02f), 0.9193f));
    dMax = fmaxf(dMax, sdf_plane(p, v3(csf2, ssf2, -1.02f), 0.9193f));
    dMax = fmaxf(dMax, sdf_plane(p, v3(csf2, ssf2, 1.03f), 0.912f));
    dMax = fmaxf(dMax, sdf_plane(p, v3(csf1, ssf1, 1.03f), 0.912f));
    dMax = fmaxf(dMax, sdf_plane(p, v3(csf8, ssf8, 2.21f), 1.131f));
    return dMax * scale;
}

// one voxel of FillSDFVolume (core/object/sdf/sdf_cache_manager.cuh:14-36)
AR_HD float sdf_fill_voxel(int fn, float4 prm, int x, int y, int z, int dx, int dy, int dz)
{
    const float nx = (dx > 1) ? (float)x / (float)(dx - 1) : 0.0f;
    const float ny = (dy > 1) ? (float)y / (float)(dy - 1) : 0.0f;
    const float nz = (dz > 1) ? (float)z / (float)(dz - 1) : 0.0f;
    const V3 u = v3(nx, ny, nz) + (-0.5f);
    return fn == AR_SDF_FN_DIAMOND ? sdf_diamond_eval(u, prm) : sdf_torus_eval(u, prm.x, prm.y);
}

// The SDF of an object at unit position u; kind and volume select the field.
struct SdfObjField
{
    int kind;
    float4 prm;
    const SdfVolume* vol;  // volume kind: the cached grid, or null (no surface)
};

AR_HD float sdf_obj_eval(const SdfObjField& f, V3 u)
{
    if (f.kind == AR_SDF_OBJ_TORUS) return sdf_torus_eval(u, f.prm.x, f.prm.y);
    return f.vol ? sdf_volume_eval(*f.vol, u) : 1.0e20f;
}

AR_HD V3 sdf_to_unit(V3 pl, V3 ext)
{
    const float ex = fmaxf(ext.x, 1e-8f), ey = fmaxf(ext.y, 1e-8f), ez = fmaxf(ext.z, 1e-8f);
    return v3(pl.x / (2.0f * ex), pl.y / (2.0f * ey), pl.z / (2.0f * ez));
}

AR_HD float sdf_local_scale_min(V3 ext) { return 2.0f * fminf(ext.x, fminf(ext.y, ext.z)); }

#if defined(__CUDACC__)
#define AR_SDFOBJ_CALL static __host__ __device__ __noinline__
#else
#define AR_SDFOBJ_CALL static inline
#endif

// IntersectSDFObject: ray (o, d) in world space against an object with frame
// (center, extent, w2o); eps = SDF_EPS of the ray's depth.  Returns the hit
// distance (the march's t) or -1, and the local hit position.
AR_SDFOBJ_CALL float sdf_obj_hit(const SdfObjField& f, V3 center, V3 ext, const M3& w2o, V3 o, V3 d, float eps,
                                 V3* local_pos)
{
    const V3 lo = mul(w2o, o - center);
    const V3 ld = normalize(mul(w2o, d));
    const V3 div = v3(inv_safe(ld.x), inv_safe(ld.y), inv_safe(ld.z));
    const V3 t1 = (-ext - lo) * div;
    const V3 t2 = (ext - lo) * div;
    const V3 tn = vmin(t1, t2), tf = vmax(t1, t2);
    const float tEnter = fmaxf(fmaxf(tn.x, tn.y), tn.z);
    const float tExit = fminf(fminf(tf.x, tf.y), tf.z);
    if (tEnter > tExit || tExit <= 0.0f) return -1.0f;
    // RaymarchLocal
    const float minStep = eps * 0.5f;
    const bool inside = sdf_obj_eval(f, sdf_to_unit(lo, ext)) <= 0.0f;
    float t = fmaxf(0.0f, tEnter);
    const float sMin = sdf_local_scale_min(ext);
    const float stepScale = (f.kind == AR_SDF_OBJ_VOLUME) ? AR_SDF_VOLUME_STEP_SCALE : 1.0f;
    for (int i = 0; i < AR_SDF_OBJ_STEPS; ++i)
    {
        const float tLast = t;
        const V3 pl = lo + ld * t;
        const float dLocal = sdf_obj_eval(f, sdf_to_unit(pl, ext)) * sMin;
        const float real = fabsf(dLocal);
        if (inside ? (dLocal > 0.0f && dLocal < eps) : (dLocal < 0.0f && -dLocal < eps))
        {
            if (local_pos) *local_pos = pl;
            return tLast;
        }
        t += (f.kind == AR_SDF_OBJ_VOLUME) ? fmaxf(real * stepScale, minStep) : fmaxf(real, minStep);
        if (t > tExit) break;
    }
    return -1.0f;
}

// world normal at a local hit position (sdfNormalUnit + UnitNormalToLocal)
AR_SDFOBJ_CALL V3 sdf_obj_normal(const SdfObjField& f, V3 ext, const M3& o2w, V3 local_pos, float eps)
{
    const float sMin = sdf_local_scale_min(ext);
    const float h = eps / fmaxf(sMin, 1e-8f);
    const V3 u = sdf_to_unit(local_pos, ext);
    const float dx = sdf_obj_eval(f, u + v3(h, 0.0f, 0.0f)) - sdf_obj_eval(f, u - v3(h, 0.0f, 0.0f));
    const float dy = sdf_obj_eval(f, u + v3(0.0f, h, 0.0f)) - sdf_obj_eval(f, u - v3(0.0f, h, 0.0f));
    const float dz = sdf_obj_eval(f, u + v3(0.0f, 0.0f, h)) - sdf_obj_eval(f, u - v3(0.0f, 0.0f, h));
    const V3 nu = normalize(v3(dx, dy, dz));
    const float ex = fmaxf(ext.x, 1e-8f), ey = fmaxf(ext.y, 1e-8f), ez = fmaxf(ext.z, 1e-8f);
    const V3 nl = normalize(v3(nu.x / (2.0f * ex), nu.y / (2.0f * ey), nu.z / (2.0f * ez)));
    return normalize(mul(o2w, nl));
}
} // namespace ar
