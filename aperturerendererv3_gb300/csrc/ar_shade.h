// Shading-point math of the path tracer: analytic primitives, BSDFs, light
// sampling and the sky.  Host + device.  Each function restates the reference
// routine named beside it with the same operation order, so the GPU integrator
// and the reference integrator compiled for the CPU produce identical floats.
#pragma once
#include "ar_spectral.h"

#define AR_OBJ_CUBE 0
#define AR_OBJ_SPHERE 1
#define AR_OBJ_SDF 2
#define AR_OBJ_TRIANGLE 3

#define AR_MAT_DIFFUSE 0
#define AR_MAT_LIGHT 1
#define AR_MAT_GLASS 2
// shading models a scene can hold, as bits of the BSDF functions' MATS template
// argument: a kernel built for a scene without some model compiles its code out
#define AR_MATS_DIFFUSE (1 << 0)
#define AR_MATS_LIGHT (1 << 1)
#define AR_MATS_GLASS (1 << 2)
#define AR_MATS_GGX (1 << 3)
#define AR_MATS_ALL 15
#define AR_MAT_GGX 3

#define AR_PERFECT_DELTA_SURFACE 0.99f
#define AR_MAX_DELTA_SURFACE_DEPTH 1024
#define AR_MIN_TRACING_DEPTH 3
#define AR_NEE_MAX_NON_DELTA_DEPTH 10
#define AR_RADIANCE_CLAMP 1.0e3f
#define AR_DELTA_RR_TERMINATE_REDUCE 0.99f

namespace ar
{
// core/config.cuh:3
AR_HD float intersect_eps(int depth)
{
    return 1.0e-3f * arm_expf(fminf(static_cast<float>(depth) * 0.5f, 4.0f));
}

// Analytic object (oriented box or sphere): SceneObject's geometric fields.
struct Object
{
    V3 center, extent;
    M3 w2o, o2w;
    int type;
    int pad[3];
};

// Surface description at a hit (GBuffer + shading model, core/render/object.cuh:59-84)
struct Material
{
    int shading;
    V3 albedo, emissive;
    float specular, metallic, roughness, ior, sigma_a, abbe, tilt;
    SpecColor albedo_c, emissive_c;  // prepared RGB->basis colours
    int albedo_tex;                  // albedo texture index, -1 = none
};

struct Hit
{
    bool hit;
    int obj;
    int light;
    int material;  // material index of the hit primitive (set by the kernels' hit reconstruction)
    float dist;
    V3 pos, nrm;
    V3 local_pos;
};

struct Media
{
    bool inside;
    V3 vertex;
    int obj;
    int depth;
};

AR_HD Media media_default()
{
    Media m;
    m.inside = false;
    m.vertex = v3(0.0f, 0.0f, 0.0f);
    m.obj = -1;
    m.depth = 0;
    return m;
}

// ---------------------------------------------------------------- objects
// core/render/object.cuh:296-315 (Euler degrees -> object frame)
AR_HD void object_frame(V3 rotation_deg, M3* o2w, M3* w2o)
{
    const float k = AR_PI_F / 180.0f;
    const float ax = rotation_deg.x * k, ay = rotation_deg.y * k, az = rotation_deg.z * k;
    M3 rx, ry, rz;
    {
        const float c = arm_cosf(ax), s = arm_sinf(ax);
        rx.r0 = v3(1, 0, 0); rx.r1 = v3(0, c, -s); rx.r2 = v3(0, s, c);
    }
    {
        const float c = arm_cosf(ay), s = arm_sinf(ay);
        ry.r0 = v3(c, 0, s); ry.r1 = v3(0, 1, 0); ry.r2 = v3(-s, 0, c);
    }
    {
        const float c = arm_cosf(az), s = arm_sinf(az);
        rz.r0 = v3(c, -s, 0); rz.r1 = v3(s, c, 0); rz.r2 = v3(0, 0, 1);
    }
    *o2w = mul(rz, mul(ry, rx));
    *w2o = transpose(*o2w);
}

// core/object/aabb.cuh:9-89
AR_HD bool intersect_box(V3 o, V3 d, const Object& ob, Hit* h, bool full)
{
    const V3 lo = mul(ob.w2o, o - ob.center);
    const V3 ld = normalize(mul(ob.w2o, d));
    const V3 bmin = -ob.extent;
    const V3 bmax = ob.extent;
    const V3 div = v3(inv_safe(ld.x), inv_safe(ld.y), inv_safe(ld.z));
    const V3 t1 = (bmin - lo) * div;
    const V3 t2 = (bmax - lo) * div;
    const V3 tn = vmin(t1, t2);
    const V3 tf = vmax(t1, t2);
    const float tEnter = fmaxf(fmaxf(tn.x, tn.y), tn.z);
    const float tExit = fminf(fminf(tf.x, tf.y), tf.z);
    if (tEnter > tExit) return false;
    if (tExit <= 0.0f) return false;
    const bool inside = (tEnter < 0.0f);
    const float tHit = inside ? tExit : tEnter;
    h->dist = tHit;
    if (!full) return true;
    const V3 lp = lo + ld * tHit;
    h->pos = mul(ob.o2w, lp) + ob.center;
    const float rx = fabsf(lp.x) / ob.extent.x;
    const float ry = fabsf(lp.y) / ob.extent.y;
    const float rz = fabsf(lp.z) / ob.extent.z;
    V3 ln;
    if (rx >= ry && rx >= rz) ln = v3((lp.x > 0.0f) ? 1.0f : -1.0f, 0.0f, 0.0f);
    else if (ry >= rz) ln = v3(0.0f, (lp.y > 0.0f) ? 1.0f : -1.0f, 0.0f);
    else ln = v3(0.0f, 0.0f, (lp.z > 0.0f) ? 1.0f : -1.0f);
    if (inside) ln = -ln;
    h->nrm = normalize(mul(ob.o2w, ln));
    h->local_pos = lp;
    return true;
}

// core/object/sphere.cuh:9-70
AR_HD bool intersect_sphere(V3 o, V3 d, const Object& ob, Hit* h, bool full)
{
    const V3 lo = mul(ob.w2o, o - ob.center);
    const V3 ld = normalize(mul(ob.w2o, d));
    const float r = max3(ob.extent);
    const float a = 1;
    const float b = dot(lo, ld);
    const float c = dot(lo, lo) - r * r;
    const float disc = b * b - a * c;
    if (disc < 0.0f) return false;
    const float s = sqrtf(disc);
    float t = -b - s;
    bool inside = false;
    if (t <= 0.0f)
    {
        t = -b + s;
        inside = true;
    }
    if (t <= 0.0f) return false;
    h->dist = t;
    if (!full) return true;
    const V3 lp = lo + ld * t;
    const V3 ln = normalize(lp) * (inside ? -1.0f : 1.0f);
    h->pos = mul(ob.o2w, lp) + ob.center;
    h->nrm = normalize(mul(ob.o2w, ln));
    h->local_pos = lp;
    return true;
}

// core/object/aabb.cuh:92-106, core/object/sphere.cuh:73-85
AR_HD bool overlap_object(V3 p, const Object& ob)
{
    const V3 lp = mul(ob.w2o, p - ob.center);
    if (ob.type == AR_OBJ_CUBE)
    {
        const V3 bmin = -ob.extent, bmax = ob.extent;
        return bmin.x < lp.x && bmin.y < lp.y && bmin.z < lp.z && bmax.x > lp.x && bmax.y > lp.y && bmax.z > lp.z;
    }
    if (ob.type == AR_OBJ_SPHERE)
    {
        const float r = max3(ob.extent);
        return dot(lp, lp) < r * r;
    }
    return false;
}

// ---------------------------------------------------------------- sampling helpers
// core/vector.cuh:390-408
AR_HD void tangent_basis(V3 n, V3* t, V3* b)
{
    const V3 a = (fabsf(n.z) < 0.999f) ? v3(0.0f, 0.0f, 1.0f) : v3(1.0f, 0.0f, 0.0f);
    *t = normalize(cross(a, n));
    *b = cross(n, *t);
}
AR_HD void tangent_basis_random(V3 n, V3* t, V3* b, float e)
{
    const V3 a = (fabsf(n.z) < 0.999f) ? v3(0.0f, 0.0f, 1.0f) : v3(1.0f, 0.0f, 0.0f);
    const V3 t0 = normalize(cross(a, n));
    const V3 b0 = cross(n, t0);
    float s, c;
    arm_sincosf(e * AR_PI_F * 2.0f, &s, &c);
    *t = c * t0 + s * b0;
    *b = -s * t0 + c * b0;
}

// core/vector.cuh:379-387
AR_HD V3 refract(V3 inDir, V3 normal, float eta)
{
    const V3 n = (dot(normal, inDir) > 0.0f) ? -normal : normal;
    const float cosI = -dot(n, inDir);
    const float k = 1.0f - (eta * eta) * fmaxf(0.0f, 1.0f - cosI * cosI);
    const float cosT = sqrtf(fmaxf(0.0f, k));
    return eta * inDir + (eta * cosI - cosT) * n;
}

struct DirSample
{
    V3 dir;
    float pdf;
};

// core/render/sample.cuh:62-108
AR_HD DirSample sample_cosine_hemisphere(float e0, float e1, float e2, V3 normal)
{
    V3 T, B;
    tangent_basis_random(normal, &T, &B, e2);
    const float sx = 2.0f * e0 - 1.0f;
    const float sy = 2.0f * e1 - 1.0f;
    float x = 0.0f, y = 0.0f;
    if (!(sx == 0.0f && sy == 0.0f))
    {
        float r, phi;
        if (fabsf(sx) > fabsf(sy))
        {
            r = sx;
            phi = (AR_PI_F / 4.0f) * (sy / fmaxf(fabsf(sx), 1e-20f));
        }
        else
        {
            r = sy;
            phi = (AR_PI_F / 2.0f) - (AR_PI_F / 4.0f) * (sx / fmaxf(fabsf(sy), 1e-20f));
        }
        const float c = arm_cosf(phi);
        const float s = arm_sinf(phi);
        x = r * c;
        y = r * s;
    }
    const float z = sqrtf(fmaxf(0.0f, 1.0f - x * x - y * y));
    const V3 dir = x * T + y * B + z * normal;
    DirSample out;
    out.pdf = z / AR_PI_F;
    out.dir = normalize(dir);
    return out;
}

// core/render/brdf.cuh:24-88
AR_HD float fresnel_dielectric(float cosI, float cosT, float eta)
{
    const float invE = 1.0f / eta;
    const float rPar = (invE * cosI - cosT) / (invE * cosI + cosT);
    const float rPerp = (cosI - invE * cosT) / (cosI + invE * cosT);
    return 0.5f * (rPar * rPar + rPerp * rPerp);
}
AR_HD float fresnel_schlick(float F0, float cosX)
{
    const float c = clampf(1.0f - cosX, 0.0f, 1.0f);
    const float c5 = c * c * c * c * c;
    return F0 + (1.0f - F0) * c5;
}
AR_HD float ggx_d(float alpha, float NoH)
{
    const float a2 = alpha * alpha;
    const float d = NoH * NoH * (a2 - 1.0f) + 1.0f;
    return a2 / fmaxf(AR_PI_F * d * d, 1e-12f);
}
AR_HD float ggx_g_correlated(float alpha, float NoL, float NoV)
{
    const float a2 = alpha * alpha;
    const float gv = NoL * sqrtf(a2 + (1.0f - a2) * NoV * NoV);
    const float gl = NoV * sqrtf(a2 + (1.0f - a2) * NoL * NoL);
    const float denom = gv + gl;
    return (denom > 0.0f) ? (2.0f * NoL * NoV) / denom : 0.0f;
}
AR_HD float f0_ue(float specular)
{
    const float s = clampf(specular, 0.0f, 1.0f);
    return 0.08f * s;
}
AR_HD float beer_lambert(float distance, float albedoL, float sigmaA)
{
    return arm_expf(distance * sigmaA * arm_logf(fminf(fmaxf(albedoL, 1.0e-12f), 1.0f)));
}

// core/render/sample.cuh:179-248
AR_HD DirSample sample_ggx_bounded_vndf(V3 V, V3 N, float alpha, float r0, float r1, float r2)
{
    V3 X, Y;
    tangent_basis_random(N, &X, &Y, r2);
    const float XoV = dot(X, V);
    const float YoV = dot(Y, V);
    const float NoV = dot(N, V);
    const V3 localV = v3(XoV, YoV, NoV);
    const float NoV2 = fminf(1.0f, NoV * NoV);
    const float a2 = alpha * alpha;
    const V3 localStd = v3(XoV * alpha, YoV * alpha, NoV) / sqrtf(a2 + (1.0f - a2) * NoV2);
    const float phi = 2.0f * AR_PI_F * r0;
    const float s = 1.0f + sqrtf(1.0f - NoV2);
    const float s2 = s * s;
    const float k = (1.0f - a2) * s2 / (s2 + a2 * NoV2);
    const float b = NoV > 0 ? k * localStd.z : localStd.z;
    const float z = fmaf(1.0f - r1, 1.0f + b, -b);
    const float sinTheta = sqrtf(saturate(1.0f - z * z));
    const V3 oStd = v3(sinTheta * arm_cosf(phi), sinTheta * arm_sinf(phi), z);
    const V3 mStd = localStd + oStd;
    const V3 localH = normalize(v3(mStd.x * alpha, mStd.y * alpha, mStd.z));
    const V3 localL = reflect(-localV, localH);
    DirSample out;
    out.dir = localL.x * X + localL.y * Y + localL.z * N;
    const float ndf = ggx_d(alpha, localH.z);
    const float len2 = (1.0f - NoV2) * a2;
    const float t = sqrtf(len2 + NoV2);
    out.pdf = ndf / (2.0f * (k * NoV + t));
    return out;
}
AR_HD float ggx_bounded_vndf_pdf(V3 V, V3 N, V3 L, float alpha)
{
    const float NoV = dot(N, V);
    const float NoL = dot(N, L);
    if (NoV <= 0.0f || NoL <= 0.0f) return 0.0f;
    const V3 H = normalize(V + L);
    const float NoV2 = fminf(1.0f, NoV * NoV);
    const float a2 = alpha * alpha;
    const float s = 1.0f + sqrtf(1.0f - NoV2);
    const float s2 = s * s;
    const float k = (1.0f - a2) * s2 / (s2 + a2 * NoV2);
    const float NoH = fmaxf(0.0f, dot(N, H));
    const float ndf = ggx_d(alpha, NoH);
    const float len2 = (1.0f - NoV2) * a2;
    const float t = sqrtf(len2 + NoV2);
    const float pdf = ndf / (2.0f * (k * NoV + t));
    return fmaxf(pdf, 1e-12f);
}

// ---------------------------------------------------------------- BSDF
// core/render/material.cuh:48-165 (spectral branch)
template <int MATS = AR_MATS_ALL>
AR_HD float eval_bsdf_cos(float lambda, const Basis& lb, const Material& m, V3 rayDir, V3 L, const Hit& h,
                          const Media& media)
{
    const V3 N = h.nrm;
    const float NoL = fmaxf(0.0f, dot(N, L));
    if ((MATS & AR_MATS_DIFFUSE) && m.shading == AR_MAT_DIFFUSE) return interact(m.albedo_c, lb) * (NoL / AR_PI_F);
    if (m.shading == AR_MAT_LIGHT) return 0.0f;
    if ((MATS & AR_MATS_GGX) && m.shading == AR_MAT_GGX)
    {
        const V3 V = normalize(-rayDir);
        const float NoV = fmaxf(0.0f, dot(N, V));
        if (NoV <= 0.0f || NoL <= 0.0f) return 0.0f;
        const float alpha = m.roughness * m.roughness;
        const float F0d = f0_ue(m.specular);
        const float albL = interact(m.albedo_c, lb);
        const float F0 = lerpf(F0d, albL, m.metallic);
        const float kD = (1.0f - m.metallic);
        const V3 Hn = normalize(V + L);
        const float NoH = fmaxf(0.0f, dot(N, Hn));
        const float LoH = fmaxf(0.0f, dot(L, Hn));
        const float F = fresnel_schlick(F0, LoH);
        const float D = ggx_d(alpha, NoH);
        const float G = ggx_g_correlated(alpha, NoL, NoV);
        const float spec = (NoL > 0.0f) ? (F * D * G) / fmaxf(4.0f * NoV, 1e-7f) : 0.0f;
        const float diff = kD * (1.0f - F) * albL * (NoL / AR_PI_F);
        return spec + diff;
    }
    if ((MATS & AR_MATS_GLASS) && m.shading == AR_MAT_GLASS)
    {
        const float IOR = ior_from_abbe(lambda, m.ior, m.abbe);
        float transmittance = 1.0f;
        if (media.inside)
        {
            const float rayDistance = length(media.vertex - h.pos);
            const float albL = interact(m.albedo_c, lb);
            transmittance = beer_lambert(rayDistance, albL, sigma_a_from_tilt(m.sigma_a, lambda, m.tilt));
        }
        const V3 nIn = (dot(N, rayDir) > 0.0f) ? -N : N;
        const float eta = media.inside ? IOR : 1.0f / IOR;
        const float cosI = -dot(nIn, rayDir);
        const float sin2I = fmaxf(0.0f, 1.0f - cosI * cosI);
        const float k = 1.0f - sin2I * (eta * eta);
        if (k <= 0.0f) return transmittance * AR_PERFECT_DELTA_SURFACE;
        const float cosT = sqrtf(k);
        const float Fr = fresnel_dielectric(cosI, cosT, eta);
        const V3 R = reflect(rayDir, nIn);
        const V3 T = refract(rayDir, nIn, eta);
        const float dR = dot(L, R);
        const float dT = dot(L, T);
        if (dR >= dT) return transmittance * Fr;
        const float weight = (eta * eta) * (fabsf(cosT) / fmaxf(1e-6f, cosI));
        return transmittance * (1.0f - Fr) * weight;
    }
    return 0.0f;
}

// core/render/material.cuh:316-371
template <int MATS = AR_MATS_ALL>
AR_HD float bsdf_pdf(const Basis& lb, const Material& m, V3 N, V3 rayDir, V3 L)
{
    const V3 V = -rayDir;
    const float NoL = fmaxf(0.0f, dot(N, L));
    if ((MATS & AR_MATS_DIFFUSE) && m.shading == AR_MAT_DIFFUSE) return NoL > 0.0f ? (NoL * (1.0f / AR_PI_F)) : 0.0f;
    if ((MATS & AR_MATS_GGX) && m.shading == AR_MAT_GGX)
    {
        const float NoV = fmaxf(0.0f, dot(N, V));
        if (NoV <= 0.0f || NoL <= 0.0f) return 0.0f;
        const float alpha = m.roughness * m.roughness;
        const float F0d = f0_ue(m.specular);
        const float albL = interact(m.albedo_c, lb);
        const float F0 = lerpf(F0d, albL, m.metallic);
        const float pSpec = clampf(F0, 0.1f, 0.9f);
        const float pdfSpec = ggx_bounded_vndf_pdf(V, N, L, alpha);
        const float pdfDiff = NoL * (1.0f / AR_PI_F);
        const float pdfMix = pSpec * pdfSpec + (1.0f - pSpec) * pdfDiff;
        return fmaxf(0.0f, pdfMix);
    }
    return 0.0f;
}

struct BsdfSample
{
    V3 next_dir;
    float pdf;
    V3 emissive;  // material emission (rgb)
    float brdf;
    bool terminate, pure_light, delta, miss_thin;
    Media media;
};

AR_HD BsdfSample bsdf_sample_default()
{
    BsdfSample s;
    s.next_dir = v3(0.0f, 0.0f, 0.0f);
    s.pdf = 1.0f;
    s.emissive = v3(0.0f, 0.0f, 0.0f);
    s.brdf = 0.0f;
    s.terminate = s.pure_light = s.delta = s.miss_thin = false;
    s.media = media_default();
    return s;
}

// core/render/material.cuh:167-314 followed by :373-409 (EvaluateMaterial).
// Rand is a callable returning the next uniform in (0, 1].
template <int MATS = AR_MATS_ALL, typename Rand>
AR_HD BsdfSample evaluate_material(float lambda, const Basis& lb, Rand& rand, const Material& m, V3 rayDir,
                                   const Hit& h, const Media& cur)
{
    BsdfSample r = bsdf_sample_default();
    const V3 N = h.nrm;
    const V3 V = -rayDir;
    if ((MATS & AR_MATS_DIFFUSE) && m.shading == AR_MAT_DIFFUSE)
    {
        const float e0 = rand(), e1 = rand(), e2 = rand();
        const DirSample s = sample_cosine_hemisphere(e0, e1, e2, N);
        r.next_dir = s.dir;
        r.pdf = s.pdf;
        r.emissive = m.emissive;
        r.media.inside = cur.inside;
        r.media.vertex = h.pos;
    }
    else if (m.shading == AR_MAT_LIGHT)
    {
        r.pdf = 1.0f;
        r.emissive = m.emissive;
        r.terminate = true;
        r.pure_light = true;
    }
    else if ((MATS & AR_MATS_GLASS) && m.shading == AR_MAT_GLASS)
    {
        const float IOR = ior_from_abbe(lambda, m.ior, m.abbe);
        r.delta = true;
        const bool inside = cur.inside;
        const float eta = inside ? IOR : 1.0f / IOR;
        const V3 nIn = (dot(N, rayDir) > 0.0f) ? -N : N;
        const float cosI = -dot(nIn, rayDir);
        const float sin2I = fmaxf(0.0f, 1.0f - cosI * cosI);
        const float k = 1.0f - sin2I * (eta * eta);
        r.emissive = v3(0.0f, 0.0f, 0.0f);
        if (k <= 0.0f)
        {
            r.next_dir = (cur.depth < AR_MAX_DELTA_SURFACE_DEPTH) ? reflect(rayDir, nIn) : rayDir;
            r.pdf = 1.0f;
            r.media.inside = (cur.depth < AR_MAX_DELTA_SURFACE_DEPTH) ? inside : !inside;
            r.media.vertex = h.pos;
        }
        else
        {
            const float cosT = sqrtf(k);
            const float Fr = fresnel_dielectric(cosI, cosT, eta);
            if (rand() < Fr)
            {
                r.next_dir = reflect(rayDir, nIn);
                r.pdf = Fr;
                r.media.inside = inside;
            }
            else
            {
                r.next_dir = refract(rayDir, nIn, eta);
                r.pdf = 1.0f - Fr;
                r.media.inside = !inside;
            }
            r.media.vertex = h.pos;
        }
    }
    else if ((MATS & AR_MATS_GGX) && m.shading == AR_MAT_GGX)
    {
        r.emissive = m.emissive;
        const float NoV = fmaxf(0.0f, dot(N, V));
        if (NoV <= 0.0f)
        {
            r.terminate = true;
        }
        else
        {
            const float alpha = m.roughness * m.roughness;
            const float F0d = f0_ue(m.specular);
            const float albL = interact(m.albedo_c, lb);
            const float F0 = lerpf(F0d, albL, m.metallic);
            const float pSpec = clampf(F0, 0.1f, 0.9f);
            const float u = rand();
            bool ok = true;
            if (u < pSpec)
            {
                const float e0 = rand(), e1 = rand(), e2 = rand();
                const DirSample s = sample_ggx_bounded_vndf(V, N, alpha, e0, e1, e2);
                const V3 L = s.dir;
                const float NoL = fmaxf(0.0f, dot(N, L));
                if (NoL <= 0.0f)
                {
                    r.terminate = true;
                    ok = false;
                }
                else
                {
                    const float pdfSpec = s.pdf;
                    const float pdfDiff = NoL / AR_PI_F;
                    r.next_dir = L;
                    r.pdf = pSpec * pdfSpec + (1.0f - pSpec) * pdfDiff;
                }
            }
            else
            {
                const float e0 = rand(), e1 = rand(), e2 = rand();
                const DirSample s = sample_cosine_hemisphere(e0, e1, e2, N);
                const V3 L = s.dir;
                const float pdfDiff = s.pdf;
                const float pdfSpec = ggx_bounded_vndf_pdf(V, N, L, alpha);
                r.next_dir = L;
                r.pdf = pSpec * pdfSpec + (1.0f - pSpec) * pdfDiff;
            }
            if (ok)
            {
                r.media.inside = cur.inside;
                r.media.vertex = h.pos;
            }
        }
    }
    r.media.obj = h.obj;
    r.media.depth = cur.depth + 1;
    r.brdf = eval_bsdf_cos<MATS>(lambda, lb, m, rayDir, r.next_dir, h, cur);
    return r;
}

// ---------------------------------------------------------------- lights
// light-table entry: the light object and its selection probability; the
// prefix sum reproduces the sequential CDF scan of NEESampleLight exactly
struct Light
{
    int obj;          // object / primitive index
    int type;         // AR_OBJ_*
    int material;
    float select_prob;
    float cdf;        // running sum of select_prob through this light
};

struct LightSample
{
    bool valid;
    int obj;
    V3 point, normal;
    float p_facet, p_a;
    int material;
};

AR_HD float power_heuristic(float pA, float pB)
{
    const float a = pA * pA;
    const float b = pB * pB;
    return a / fmaxf(1e-24f, a + b);
}

AR_HD void obb_axes(const Object& o, V3* ux, V3* uy, V3* uz)
{
    *ux = normalize(v3(o.o2w.r0.x, o.o2w.r1.x, o.o2w.r2.x));
    *uy = normalize(v3(o.o2w.r0.y, o.o2w.r1.y, o.o2w.r2.y));
    *uz = normalize(v3(o.o2w.r0.z, o.o2w.r1.z, o.o2w.r2.z));
}

// Facet i of an oriented box light (core/nee/nee.cuh:153-251 lists them in
// this order): outward normal, centre, the two in-plane axes and half sizes.
// Computed per facet on demand, so no six-facet table has to live in memory.
AR_HD void box_facet(V3 ux, V3 uy, V3 uz, V3 c, V3 e, int i, V3* n, V3* ctr, V3* t, V3* b, float* s1, float* s2)
{
    switch (i)
    {
    case 0: *n = ux; *ctr = c + ux * e.x; *t = uy; *b = uz; *s1 = e.y; *s2 = e.z; break;
    case 1: *n = -ux; *ctr = c - ux * e.x; *t = uy; *b = uz; *s1 = e.y; *s2 = e.z; break;
    case 2: *n = uy; *ctr = c + uy * e.y; *t = ux; *b = uz; *s1 = e.x; *s2 = e.z; break;
    case 3: *n = -uy; *ctr = c - uy * e.y; *t = ux; *b = uz; *s1 = e.x; *s2 = e.z; break;
    case 4: *n = uz; *ctr = c + uz * e.z; *t = ux; *b = uy; *s1 = e.x; *s2 = e.y; break;
    default: *n = -uz; *ctr = c - uz * e.z; *t = ux; *b = uy; *s1 = e.x; *s2 = e.y; break;
    }
}

// core/nee/nee.cuh:56-62
AR_HD float facing_weight(V3 n, V3 c, V3 p, float area)
{
    const V3 l2s = normalize(p - c);
    const float cs = fmaxf(0.0f, dot(n, l2s));
    return area * cs;
}

// core/nee/nee.cuh:36-54
AR_HD float area_to_solid_angle_pdf(V3 sp, V3 lp, V3 ln, float pA)
{
    const V3 s2l = lp - sp;
    const float d2 = fmaxf(dot(s2l, s2l), 1e-20f);
    const V3 dir = s2l * arm_rsqrtf(d2);
    const float cosY = fmaxf(0.0f, dot(ln, -dir));
    if (cosY <= 0.0f) return 0.0f;
    return pA * (d2 / cosY);
}

// core/nee/nee.cuh:153-251.  The facets with a positive facing weight, in facet
// order, form the selection list; the loops run over all six facets and skip
// the others, and the chosen facet's geometry is computed again from its index.
template <typename Rand>
AR_HD LightSample sample_box_light(Rand& rand, const Object& box, V3 p)
{
    LightSample ls;
    ls.valid = false;
    V3 ux, uy, uz;
    obb_axes(box, &ux, &uy, &uz);
    const V3 c = box.center, e = box.extent;
    float w[6];
    int cnt = 0;
    int first = -1;
    float sum = 0;
#pragma unroll
    for (int i = 0; i < 6; ++i)
    {
        V3 n, ctr, t, b;
        float s1, s2;
        box_facet(ux, uy, uz, c, e, i, &n, &ctr, &t, &b, &s1, &s2);
        w[i] = facing_weight(n, ctr, p, 4.0f * s1 * s2);
        if (w[i] > 0.0f)
        {
            if (first < 0) first = i;
            sum += w[i];
            ++cnt;
        }
    }
    if (cnt == 0) return ls;
    int face = first;
    {
        const float r = rand() * sum;
        float acc = 0;
        bool found = false;
#pragma unroll
        for (int i = 0; i < 6; ++i)
        {
            if (!found && w[i] > 0.0f)
            {
                acc += w[i];
                if (r <= acc)
                {
                    face = i;
                    found = true;
                }
            }
        }
    }
    float fw = w[0];
#pragma unroll
    for (int i = 1; i < 6; ++i)
        if (face == i) fw = w[i];
    V3 fn, fc, ft, fb;
    float fs1, fs2;
    box_facet(ux, uy, uz, c, e, face, &fn, &fc, &ft, &fb, &fs1, &fs2);
    const float u1 = 2.0f * rand() - 1.0f;
    const float u2 = 2.0f * rand() - 1.0f;
    ls.point = fc + ft * (u1 * fs1) + fb * (u2 * fs2);
    ls.normal = fn;
    ls.p_facet = 1.0f * (fw / sum);
    ls.p_a = 1.0f / (4.0f * fs1 * fs2);
    ls.valid = true;
    return ls;
}

// core/nee/nee.cuh:272-310
template <typename Rand>
AR_HD LightSample sample_sphere_light(Rand& rand, const Object& sph, V3 p)
{
    LightSample ls;
    ls.valid = false;
    const V3 c = sph.center;
    const float r = max3(sph.extent);
    const V3 p2c = p - c;
    const float d = length(p2c);
    if (d <= r) return ls;
    const V3 axis = p2c / d;
    const float cosC = clampf(r / d, 0.0f, 1.0f);
    const float areaCap = 2.0f * AR_PI_F * r * r * (1.0f - cosC);
    const float u = rand();
    const float vphi = rand();
    const float cosT = lerpf(cosC, 1.0f, u);
    const float sinT = sqrtf(fmaxf(0.0f, 1.0f - cosT * cosT));
    const float phi = 2.0f * AR_PI_F * vphi;
    V3 t, b;
    tangent_basis(axis, &t, &b);
    const V3 n = t * (arm_cosf(phi) * sinT) + b * (arm_sinf(phi) * sinT) + axis * cosT;
    ls.point = c + n * r;
    ls.normal = n;
    ls.p_facet = 1.0f;
    ls.p_a = 1.0f / areaCap;
    ls.valid = true;
    return ls;
}

// core/nee/nee.cuh:64-151
AR_HD float box_light_pdf_omega(const Object& o, float selectProb, V3 sp, V3 lp, V3 ln)
{
    V3 ux, uy, uz;
    obb_axes(o, &ux, &uy, &uz);
    const V3 c = o.center, e = o.extent;
    int hitFacet = -1;
#pragma unroll
    for (int i = 0; i < 6; ++i)
    {
        V3 n, ctr, t, b;
        float s1, s2;
        box_facet(ux, uy, uz, c, e, i, &n, &ctr, &t, &b, &s1, &s2);
        if (hitFacet < 0 && dot(n, ln) > 0.999f) hitFacet = i;
    }
    if (hitFacet < 0)
    {
        float best = 1e30f;
#pragma unroll
        for (int i = 0; i < 6; ++i)
        {
            V3 n, ctr, t, b;
            float s1, s2;
            box_facet(ux, uy, uz, c, e, i, &n, &ctr, &t, &b, &s1, &s2);
            const float d = fabsf(dot(n, lp - ctr));
            if (d < best)
            {
                best = d;
                hitFacet = i;
            }
        }
    }
    float sum = 0.0f, wHit = 0.0f, aHit = 0.0f;
#pragma unroll
    for (int i = 0; i < 6; ++i)
    {
        V3 n, ctr, t, b;
        float s1, s2;
        box_facet(ux, uy, uz, c, e, i, &n, &ctr, &t, &b, &s1, &s2);
        const float area = 4.0f * s1 * s2;
        const float w = facing_weight(n, ctr, sp, area);
        sum += w;
        if (i == hitFacet)
        {
            wHit = w;
            aHit = area;
        }
    }
    if (sum <= 0.0f || wHit <= 0.0f) return 0.0f;
    const float pATotal = selectProb * (1.0f / aHit) * (wHit / sum);
    return area_to_solid_angle_pdf(sp, lp, ln, pATotal);
}

// core/nee/nee.cuh:253-270
AR_HD float sphere_light_pdf_omega(const Object& o, float selectProb, V3 sp, V3 lp, V3 ln)
{
    const float r = max3(o.extent);
    const float d = length(sp - o.center);
    if (d <= r) return 0.0f;
    const float cosC = clampf(r / d, 0.0f, 1.0f);
    const float areaCap = 2.0f * AR_PI_F * r * r * (1.0f - cosC);
    if (areaCap <= 1e-20f) return 0.0f;
    const float pATotal = selectProb / areaCap;
    return area_to_solid_angle_pdf(sp, lp, ln, pATotal);
}

// ---------------------------------------------------------------- participating medium
// Homogeneous medium filling an axis-aligned box (no reference counterpart):
// extinction sigma_t, single-scattering albedo, Henyey-Greenstein phase g, and
// an emission radiance released where light is absorbed (white, scaled like
// emitters by D65).  Free flights are sampled in the box; shadow rays carry the
// box chord's transmittance.
struct BoxMedium
{
    int on;
    V3 lo, hi;
    float sigma_t, albedo, g, emission;
};

// the part [t0, t1] of the ray's [tmin, tmax] inside the box
AR_HD bool medium_segment(const BoxMedium& m, V3 o, V3 d, float tmin, float tmax, float* t0, float* t1)
{
    const V3 inv = v3(inv_safe(d.x), inv_safe(d.y), inv_safe(d.z));
    const V3 a = (m.lo - o) * inv, b = (m.hi - o) * inv;
    const V3 tn = vmin(a, b), tf = vmax(a, b);
    *t0 = fmaxf(fmaxf(fmaxf(tn.x, tn.y), tn.z), tmin);
    *t1 = fminf(fminf(fminf(tf.x, tf.y), tf.z), tmax);
    return *t0 < *t1;
}

AR_HD float medium_transmittance(const BoxMedium& m, V3 o, V3 d, float dist)
{
    if (!m.on) return 1.0f;
    float t0, t1;
    if (!medium_segment(m, o, d, 0.0f, dist, &t0, &t1)) return 1.0f;
    return arm_expf(-m.sigma_t * (t1 - t0));
}

// HenyeyGreensteinPDF, SampleHenyeyGreensteinBase, SampleHenyeyGreenstein (core/render/sample.cuh:110-145)
AR_HD float hg_pdf(float cosTheta, float g)
{
    const float g2 = g * g;
    const float x = fmaxf(1.0f + g2 - 2.0f * g * cosTheta, 1e-20f);
    return (1.0f - g2) / (4.0f * AR_PI_F * x * sqrtf(x));
}

AR_HD float hg_sample_cos(float e, float g)
{
    if (fabsf(g) < 0.0001f) return e * 2.0f - 1.0f;
    const float g2 = g * g;
    const float t0 = (1.0f - g2) / (1.0f - g + 2.0f * g * e);
    return (1.0f + g2 - t0 * t0) / (2.0f * g);
}

AR_HD DirSample hg_sample(float e0, float e1, V3 v, float g)
{
    const float cosTheta = hg_sample_cos(e0, g);
    const float phi = 2.0f * AR_PI_F * e1;
    const float sinTheta = sqrtf(fmaxf(0.0f, 1.0f - cosTheta * cosTheta));
    const V3 w = normalize(v);
    const V3 a = (fabsf(w.z) > 0.70710678f) ? v3(0.0f, 1.0f, 0.0f) : v3(0.0f, 0.0f, 1.0f);
    const V3 v2 = normalize(cross(w, a));
    const V3 v3_ = cross(v2, w);
    float sp, cp;
    arm_sincosf(phi, &sp, &cp);
    DirSample out;
    out.dir = v3_ * (sinTheta * cp) + v2 * (sinTheta * sp) + w * cosTheta;
    out.pdf = hg_pdf(cosTheta, g);
    return out;
}

// ---------------------------------------------------------------- sky
// core/render/render.cuh:58-73
AR_HD V3 sky_lighting(V3 d)
{
    const V3 skyWhite = v3(1.0f, 1.0f, 1.0f);
    const V3 skyBlue = v3(0.05f, 0.45f, 1.0f);
    const V3 skyDown = v3(0.2f, 0.6f, 1.0f) * 0.125f;
    const float t1 = arm_powf(fmaxf(d.y, 0.0f), 0.75f);
    const V3 l1 = v3(lerpf(skyBlue.x, skyWhite.x, t1), lerpf(skyBlue.y, skyWhite.y, t1), lerpf(skyBlue.z, skyWhite.z, t1));
    const float t2 = fminf(fmaxf(-d.y * 0.5f + 0.5f, 0.0f), 1.0f);
    const V3 l2 = v3(lerpf(l1.x, skyDown.x, t2), lerpf(l1.y, skyDown.y, t2), lerpf(l1.z, skyDown.z, t2));
    return 0.5f * l2;
}
} // namespace ar
