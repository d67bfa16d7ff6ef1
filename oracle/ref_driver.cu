// Host driver that runs the reference's own integrator and BVH on the CPU.
//
// TEST INFRASTRUCTURE ONLY (see oracle/prepare_ref.py).  Compiled against the
// patched reference tree in oracle/_ref/src/core; every computation below is a
// call into reference code:
//   kat     spectrum::query::RGBEncode / LambdaEncode / SpectralInteract on the
//           reference's golden vectors (core/spectrum/spectrum_basis.cuh:2472-2513)
//   lut     the lambda LUT as PrecomputeLambdaLUTKernel builds it, and RGB LUT
//           lattice values as PrecomputeRGBLUTKernel builds them
//           (core/spectrum/spectrum_lut.cuh:12-60)
//   trace   BuildBVH + intersection::TraverseBVH<false> over triangles
//           (core/bvh/bvh.cuh:142-422, core/render/intersection.cuh:148-283),
//           or brute force
//   tracecount the reference's BuildBVH tree walked near-first with a slab test
//           that also requires tEnter <= tExit: node pops and triangle tests
//           per ray (the traversal roofline's algorithmic work)
//   render  CalculateRadiance<true, NEE, false> per pixel sample
//           (core/render/render.cuh:460-999) behind the camera model of
//           RenderCamera (core/scene.cu:135-189), OpenMP over pixels;
//           optionally with the denoiser's per-pixel records
//           (denoise::RecordScreenGBuffer / RecordScreenStatisticBuffer)
//   render  with params.guide: CalculateRadiance<true, NEE, true> over a given
//           voxel-guide probe set, also returning its radiance records
//           (core/render/render.cuh:553-638, 909-963)
//   pgupdate one probe update over given records (core/scene.cu:409-570,
//           core/guiding/guiding.cuh:373-517), kernel loop bodies restated
//           around the reference's own probe functions
//   tonemap the per-pixel display transform of Camera::RenderToFile with the
//           reference's tone curves (core/camera.cu:64-89, core/tonemap.cuh)
//   frametone the display kernel of the progressive Render (core/scene.cu:22-131)
//   denoise the loop of denoise::Bilateral16x16<7> (core/denoise/denoise.cuh:
//           360-443) per output pixel, calling the reference's weight,
//           t-test and sample transforms
// The scene / light-table setup mirrors SceneRenderer::UpdateSceneToDeviceIfDirty
// (core/scene.cu:656-732) on host memory.
#include <cfloat>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cstdint>
#include <vector>
#include <string>
#include <set>
#include <chrono>
#include <algorithm>
#include <omp.h>

#include "scene.hpp"
#include "render/render.cuh"
#include "spectrum/spectrum_lut.cuh"
#include "denoise/denoise.cuh"
#include "tonemap.cuh"
// the t-quantile table the denoiser's t-test reads
#include "denoise/t_quantile.cu"
// explicit SDF instantiations the intersection dispatch links against
#include "object/sdf/sdf_base.cu"

#ifndef __CUDA_ARCH__

static void die(const char* msg)
{
    fprintf(stderr, "ref_cpu: %s\n", msg);
    exit(2);
}

static std::vector<char> read_file(const char* path)
{
    FILE* f = fopen(path, "rb");
    if (!f) die("cannot open input");
    fseek(f, 0, SEEK_END);
    const long n = ftell(f);
    fseek(f, 0, SEEK_SET);
    std::vector<char> buf(n);
    if (n && fread(buf.data(), 1, n, f) != (size_t)n) die("short read");
    fclose(f);
    return buf;
}

static void write_file(const char* path, const void* data, size_t n, bool append = false)
{
    FILE* f = fopen(path, append ? "ab" : "wb");
    if (!f) die("cannot open output");
    if (n && fwrite(data, 1, n, f) != n) die("short write");
    fclose(f);
}

// ---------------------------------------------------------------- kat
static int cmd_kat()
{
    using namespace spectrum::query;
    printf("{\"input\": [");
    for (int i = 0; i < 100; ++i)
    {
        printf("%s[%.9g, %.9g, %.9g, %.9g]", i ? ", " : "", inputTest[0][i], inputTest[1][i], inputTest[2][i], inputTest[3][i]);
    }
    printf("], \"gt\": [");
    for (int i = 0; i < 100; ++i) printf("%s%.9g", i ? ", " : "", gtTest[i]);
    printf("], \"ref_pred\": [");
    for (int i = 0; i < 100; ++i)
    {
        const float rgb3[3] = {inputTest[0][i], inputTest[1][i], inputTest[2][i]};
        const float lam1[1] = {inputTest[3][i]};
        float k1[KERNEL], k2[KERNEL];
        RGBEncode(rgb3, k1);
        LambdaEncode(lam1, k2);
        printf("%s%.9g", i ? ", " : "", SpectralInteract(k1, k2));
    }
    printf("]}\n");
    return 0;
}

// ---------------------------------------------------------------- lut
// out: lambda LUT (840 x 4 f32), then RGBEncode at each requested lattice point
static int cmd_lut(const char* lattice_path, const char* out_path)
{
    using namespace spectrum::query;
    constexpr int LRES = SPECTRUM_LAMBDA_LUT_RES;
    std::vector<float> lam((size_t)LRES * KERNEL);
    const float step = (780.0f - 360.0f) / static_cast<float>(LRES);
    for (int i = 0; i < LRES; ++i)
    {
        const float lambda = 360.0f + (i + 0.5f) * step;
        const float in1[1] = {lambda};
        LambdaEncode(in1, &lam[(size_t)i * KERNEL]);
    }
    write_file(out_path, lam.data(), lam.size() * 4);
    std::vector<char> lat = read_file(lattice_path);
    const int n = (int)(lat.size() / 12);
    const int32_t* idx = reinterpret_cast<const int32_t*>(lat.data());
    std::vector<float> vals((size_t)n * KERNEL);
    constexpr int RES = SPECTRUM_RGB_LUT_RES;
    constexpr float invRes = 1.0f / static_cast<float>(RES);
#pragma omp parallel for
    for (int i = 0; i < n; ++i)
    {
        float in3[3] = {(idx[3 * i] + 0.5f) * invRes, (idx[3 * i + 1] + 0.5f) * invRes, (idx[3 * i + 2] + 0.5f) * invRes};
        RGBEncode(in3, &vals[(size_t)i * KERNEL]);
    }
    write_file(out_path, vals.data(), vals.size() * 4, true);
    return 0;
}

// ---------------------------------------------------------------- trace
// Triangle intersector for TraverseBVH: same watertight test as the GPU, ties at
// equal t resolved to the smallest primitive id.
struct TriIntersector
{
    const float* tris;  // 9 floats per triangle
    int sceneCount_;
    __host__ __device__ bool operator()(const int, const int id, const float3 o, const float3 d,
                                        const float tMin, const float tMax, IntersectionContext* out) const
    {
#ifndef __CUDA_ARCH__
        ++ref_glue::g_prim_tests;
#endif
        const float* v = tris + (size_t)id * 9;
        const ar::RayShear s = ar::make_shear(ref_glue::to_v(d));
        float t, b0, b1, b2;
        if (!ar::tri_intersect(s, ref_glue::to_v(o), ar::v3(v[0], v[1], v[2]), ar::v3(v[3], v[4], v[5]), ar::v3(v[6], v[7], v[8]), &t, &b0, &b1, &b2))
            return false;
        if (t < tMin) return false;
        if (t > tMax) return false;
        if (t == tMax && !(out && out->bHit_ && id < out->objectIndex_)) return false;
        if (out)
        {
            out->bHit_ = true;
            out->distance_ = t;
            out->objectIndex_ = id;
        }
        return true;
    }
};

static int cmd_trace(const char* tri_path, const char* ray_path, const char* out_path, bool brute)
{
    std::vector<char> tb = read_file(tri_path);
    std::vector<char> rb = read_file(ray_path);
    const int ntri = *reinterpret_cast<const int32_t*>(tb.data());
    const float* tris = reinterpret_cast<const float*>(tb.data() + 4);
    const int nray = *reinterpret_cast<const int32_t*>(rb.data());
    const float* rays = reinterpret_cast<const float*>(rb.data() + 4);
    auto t0 = std::chrono::steady_clock::now();
    std::vector<PrimitiveProxy> proxy(ntri);
    for (int i = 0; i < ntri; ++i)
    {
        const float* v = tris + (size_t)i * 9;
        PrimitiveProxy p;
        p.boundMin_ = float3{fminf(v[0], fminf(v[3], v[6])), fminf(v[1], fminf(v[4], v[7])), fminf(v[2], fminf(v[5], v[8]))};
        p.boundMax_ = float3{fmaxf(v[0], fmaxf(v[3], v[6])), fmaxf(v[1], fmaxf(v[4], v[7])), fmaxf(v[2], fmaxf(v[5], v[8]))};
        p.center_ = float3{(p.boundMin_.x + p.boundMax_.x) * 0.5f, (p.boundMin_.y + p.boundMax_.y) * 0.5f, (p.boundMin_.z + p.boundMax_.z) * 0.5f};
        proxy[i] = p;
    }
    BVHHost bvh;
    if (!brute) bvh = BuildBVH(proxy);
    auto t1 = std::chrono::steady_clock::now();
    std::vector<int32_t> ids(nray);
    std::vector<float> ts(nray);
    unsigned long long visits = 0, tests = 0;
    const TriIntersector isect{tris, ntri};
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : visits, tests)
    for (int r = 0; r < nray; ++r)
    {
        ref_glue::g_node_visits = 0;
        ref_glue::g_prim_tests = 0;
        // ray layout: origin, tmin, direction, tmax
        const float* q = rays + (size_t)r * 8;
        const float3 o{q[0], q[1], q[2]}, d{q[4], q[5], q[6]};
        const float tmin = q[3], tmax = q[7];
        IntersectionContext res{};
        if (brute)
        {
            res.distance_ = tmax;
            for (int i = 0; i < ntri; ++i) isect(0, i, o, d, tmin, res.distance_, &res);
        }
        else
        {
            res = intersection::TraverseBVH<false>(0, o, d, isect, bvh.nodes_.data(), (int)bvh.nodes_.size(),
                                                  bvh.objectIndices_.data(), tmin, tmax);
        }
        ids[r] = res.bHit_ ? res.objectIndex_ : -1;
        ts[r] = res.bHit_ ? res.distance_ : -1.0f;
        visits += ref_glue::g_node_visits;
        tests += ref_glue::g_prim_tests;
    }
    auto t2 = std::chrono::steady_clock::now();
    write_file(out_path, ids.data(), ids.size() * 4);
    write_file(out_path, ts.data(), ts.size() * 4, true);
    printf("{\"build_s\": %.4f, \"trace_s\": %.4f, \"nodes\": %zu, \"node_visits\": %llu, \"prim_tests\": %llu, \"threads\": %d}\n",
           std::chrono::duration<double>(t1 - t0).count(), std::chrono::duration<double>(t2 - t1).count(),
           bvh.nodes_.size(), visits, tests, omp_get_max_threads());
    return 0;
}

// ---------------------------------------------------------------- tracecount
// The traversal work a binary SAH BVH needs for a ray set: the reference's
// BuildBVH tree (core/bvh/bvh.cuh:142-422) walked near-first as TraverseBVH
// does (core/render/intersection.cuh:148-283), but with the slab test also
// requiring tEnter <= tExit (the reference's FastAABBHit, core/bvh/bvh.cuh:
// 424-444, omits it and so visits every box in front of the ray).  Counts the
// nodes popped and the triangles tested; the hits equal TraverseBVH's.
static bool slab_hit(const float3 o, const float3 inv, const float3 lo, const float3 hi, float tmin, float tmax, float* tenter)
{
    const float3 t0 = (lo - o) * inv;
    const float3 t1 = (hi - o) * inv;
    const float3 tn = min(t0, t1);
    const float3 tf = max(t0, t1);
    const float te = fmaxf(fmaxf(tn.x, tn.y), tn.z);
    const float tx = fminf(fminf(tf.x, tf.y), tf.z);
    *tenter = te;
    return te <= tx && tx >= fmaxf(0.0f, tmin) && te <= tmax;
}

static int cmd_tracecount(const char* tri_path, const char* ray_path, const char* out_path)
{
    std::vector<char> tb = read_file(tri_path);
    std::vector<char> rb = read_file(ray_path);
    const int ntri = *reinterpret_cast<const int32_t*>(tb.data());
    const float* tris = reinterpret_cast<const float*>(tb.data() + 4);
    const int nray = *reinterpret_cast<const int32_t*>(rb.data());
    const float* rays = reinterpret_cast<const float*>(rb.data() + 4);
    std::vector<PrimitiveProxy> proxy(ntri);
    for (int i = 0; i < ntri; ++i)
    {
        const float* v = tris + (size_t)i * 9;
        PrimitiveProxy pp;
        pp.boundMin_ = float3{fminf(v[0], fminf(v[3], v[6])), fminf(v[1], fminf(v[4], v[7])), fminf(v[2], fminf(v[5], v[8]))};
        pp.boundMax_ = float3{fmaxf(v[0], fmaxf(v[3], v[6])), fmaxf(v[1], fmaxf(v[4], v[7])), fmaxf(v[2], fmaxf(v[5], v[8]))};
        pp.center_ = float3{(pp.boundMin_.x + pp.boundMax_.x) * 0.5f, (pp.boundMin_.y + pp.boundMax_.y) * 0.5f, (pp.boundMin_.z + pp.boundMax_.z) * 0.5f};
        proxy[i] = pp;
    }
    auto t0 = std::chrono::steady_clock::now();
    const BVHHost bvh = BuildBVH(proxy);
    auto t1 = std::chrono::steady_clock::now();
    const BVHNode* nodes = bvh.nodes_.data();
    const int* idx = bvh.objectIndices_.data();
    std::vector<int32_t> ids(nray);
    std::vector<float> ts(nray);
    std::vector<uint32_t> visits(nray), tests(nray);
    const TriIntersector isect{tris, ntri};
#pragma omp parallel for schedule(dynamic, 256)
    for (int r = 0; r < nray; ++r)
    {
        const float* q = rays + (size_t)r * 8;
        const float3 o{q[0], q[1], q[2]}, d{q[4], q[5], q[6]};
        const float tmin = q[3];
        IntersectionContext res{};
        res.distance_ = q[7];
        const float3 inv = invSafe(d);
        int stack[128];
        int sp = 0;
        stack[sp++] = 0;
        uint32_t nv = 0, nt = 0;
        while (sp)
        {
            const BVHNode& n = nodes[stack[--sp]];
            ++nv;
            float te;
            if (!slab_hit(o, inv, n.boundMin_, n.boundMax_, tmin, res.distance_, &te)) continue;
            if (n.count_ > 0)
            {
                for (int i = 0; i < n.count_; ++i)
                {
                    ++nt;
                    isect(0, idx[n.first_ + i], o, d, tmin, res.distance_, &res);
                }
                continue;
            }
            float tl = 0.0f, tr = 0.0f;
            const bool hl = slab_hit(o, inv, nodes[n.left_].boundMin_, nodes[n.left_].boundMax_, tmin, res.distance_, &tl);
            const bool hr = slab_hit(o, inv, nodes[n.right_].boundMin_, nodes[n.right_].boundMax_, tmin, res.distance_, &tr);
            if (hl && hr && sp + 2 <= 128)
            {
                stack[sp++] = tl > tr ? n.left_ : n.right_;
                stack[sp++] = tl > tr ? n.right_ : n.left_;
            }
            else if (hl && sp < 128) stack[sp++] = n.left_;
            else if (hr && sp < 128) stack[sp++] = n.right_;
        }
        ids[r] = res.bHit_ ? res.objectIndex_ : -1;
        ts[r] = res.bHit_ ? res.distance_ : -1.0f;
        visits[r] = nv;
        tests[r] = nt;
    }
    auto t2 = std::chrono::steady_clock::now();
    unsigned long long sv = 0, st = 0;
    for (int r = 0; r < nray; ++r)
    {
        sv += visits[r];
        st += tests[r];
    }
    write_file(out_path, ids.data(), ids.size() * 4);
    write_file(out_path, ts.data(), ts.size() * 4, true);
    write_file(out_path, visits.data(), visits.size() * 4, true);
    write_file(out_path, tests.data(), tests.size() * 4, true);
    printf("{\"build_s\": %.4f, \"trace_s\": %.4f, \"nodes\": %zu, \"node_visits\": %llu, \"prim_tests\": %llu, \"threads\": %d}\n",
           std::chrono::duration<double>(t1 - t0).count(), std::chrono::duration<double>(t2 - t1).count(),
           bvh.nodes_.size(), sv, st, omp_get_max_threads());
    return 0;
}

// ---------------------------------------------------------------- render
#pragma pack(push, 1)
struct FileObject
{
    int32_t type, shading;
    float center[3], extent[3], rotation[3];
    float v0[3], v1[3], v2[3];
    float albedo[3], emissive[3];
    float roughness, metallic, specular, ior, sigma_a, abbe, tilt;
    int32_t sdf_type;       // OBJ_SDF: ESDFType
    float sdf_params[4];    // SDFInfo::sdfInfo0_
    int32_t sdf_volume;     // SDFInfo::cachedVolumeIndex_
};
struct RenderParams
{
    int32_t width, height, spp, max_depth;
    float cam_origin[3], cam_dir[3];
    float fov_deg;
    int32_t use_nee;
    uint64_t seed;
    int32_t first_frame, per_sample_frames;
    int32_t denoise;  // 1: record the denoiser's G-buffer and sample moments and append them
    int32_t guide;    // 1: CalculateRadiance<true, NEE, true> over the probe set given as a 4th file
    float guide_inv_unit;  // 1 / voxel unit of pg::GetVoxelLocation (the reference's 1 / 0.05 = 20)
};
// Plain per-pixel layouts of the denoiser records (40 bytes each), shared with
// the GPU library's ar_denoise_read / ar_denoise_write.
struct PlainGBuf
{
    uint16_t h[14];  // albedo xyz, normal xyz, metallic, roughness, shading model[5], pad
    float depth;
    uint32_t valid, frames;
};
struct PlainStat
{
    uint32_t num;
    float mean[3], m2n[3], m3n[3];
};
// one SDF volume of the scene file: fn >= 0 fills from the reference functor
// (0 torus, 1 diamond) with params; fn < 0 is followed by the voxel values
struct FileVolume
{
    int32_t fn;
    float params[4];
    int32_t dims[3];
};
#pragma pack(pop)

// FillSDFVolume's loop (core/object/sdf/sdf_cache_manager.cuh:14-36) on the host,
// calling the reference's functors
static void fill_volume(int fn, const float* prm, const int32_t* dims, float* out)
{
    SDFInfo info{};
    info.sdfInfo0_ = float4{prm[0], prm[1], prm[2], prm[3]};
    const int3 d{dims[0], dims[1], dims[2]};
#pragma omp parallel for
    for (int z = 0; z < d.z; ++z)
        for (int y = 0; y < d.y; ++y)
            for (int x = 0; x < d.x; ++x)
            {
                const float nx = (d.x > 1) ? static_cast<float>(x) / static_cast<float>(d.x - 1) : 0.0f;
                const float ny = (d.y > 1) ? static_cast<float>(y) / static_cast<float>(d.y - 1) : 0.0f;
                const float nz = (d.z > 1) ? static_cast<float>(z) / static_cast<float>(d.z - 1) : 0.0f;
                const float3 pos01 = make_float3(nx, ny, nz);
                const size_t idx = static_cast<size_t>(z) * d.x * d.y + static_cast<size_t>(y) * d.x + x;
                out[idx] = fn == 1 ? sdf::SDFDiamondFunctor{}(pos01 - 0.5f, info) : sdf::SDFTorusFunctor{}(pos01 - 0.5f, info);
            }
}

// sdfvol: one volume as ar_sdf_volume_add fills it.  in: FileVolume; out: floats
static int cmd_sdfvol(const char* in_path, const char* out_path)
{
    std::vector<char> buf = read_file(in_path);
    if (buf.size() < sizeof(FileVolume)) die("bad sdfvol input");
    const FileVolume* fv = reinterpret_cast<const FileVolume*>(buf.data());
    std::vector<float> data((size_t)fv->dims[0] * fv->dims[1] * fv->dims[2]);
    fill_volume(fv->fn, fv->params, fv->dims, data.data());
    write_file(out_path, data.data(), data.size() * 4);
    return 0;
}

static float3 f3(const float* v) { return float3{v[0], v[1], v[2]}; }

static uint16_t half_bits(const half& h)
{
    uint16_t u;
    memcpy(&u, &h, 2);
    return u;
}
static half bits_half(uint16_t u)
{
    half h;
    memcpy(&h, &u, 2);
    return h;
}

static void to_plain(const denoise::ScreenGBuffer& g, const denoise::ScreenStatisticsBuffer& s, PlainGBuf* pg,
                     PlainStat* ps)
{
    const half hs[8] = {g.albedoX_, g.albedoY_, g.albedoZ_, g.normalX_, g.normalY_, g.normalZ_, g.metallic_, g.roughness_};
    for (int i = 0; i < 8; ++i) pg->h[i] = half_bits(hs[i]);
    for (int i = 0; i < 5; ++i) pg->h[8 + i] = half_bits(g.shadingModel_[i]);
    pg->h[13] = 0;
    pg->depth = g.depth_;
    pg->valid = (uint32_t)g.validFrameIndex_;
    pg->frames = (uint32_t)g.frameIndex_;
    ps->num = s.num_;
    const float3 v[3] = {s.mean_, s.M2DivNum_, s.M3DivNum_};
    float* dst[3] = {ps->mean, ps->m2n, ps->m3n};
    for (int k = 0; k < 3; ++k)
    {
        dst[k][0] = v[k].x;
        dst[k][1] = v[k].y;
        dst[k][2] = v[k].z;
    }
}

static void from_plain(const PlainGBuf& pg, const PlainStat& ps, denoise::ScreenGBuffer* g,
                       denoise::ScreenStatisticsBuffer* s)
{
    memset(static_cast<void*>(g), 0, sizeof(*g));
    memset(static_cast<void*>(s), 0, sizeof(*s));
    half* hs[8] = {&g->albedoX_, &g->albedoY_, &g->albedoZ_, &g->normalX_, &g->normalY_, &g->normalZ_, &g->metallic_,
                   &g->roughness_};
    for (int i = 0; i < 8; ++i) *hs[i] = bits_half(pg.h[i]);
    for (int i = 0; i < 5; ++i) g->shadingModel_[i] = bits_half(pg.h[8 + i]);
    g->depth_ = pg.depth;
    g->validFrameIndex_ = pg.valid;
    g->frameIndex_ = pg.frames;
    s->num_ = ps.num;
    s->mean_ = float3{ps.mean[0], ps.mean[1], ps.mean[2]};
    s->M2DivNum_ = float3{ps.m2n[0], ps.m2n[1], ps.m2n[2]};
    s->M3DivNum_ = float3{ps.m3n[0], ps.m3n[1], ps.m3n[2]};
}

static Material make_material(const FileObject& o)
{
    switch (o.shading)
    {
        case 1: return Material::CreateLight(f3(o.emissive));
        case 2: return Material::CreateGlassPureColor(f3(o.albedo), o.ior, o.sigma_a, o.abbe, o.tilt);
        case 3: return Material::CreateGGXPureColor(f3(o.albedo), o.roughness, o.metallic, o.specular, f3(o.emissive));
        default: return Material::CreateDiffusePureColor(f3(o.albedo), f3(o.emissive));
    }
}

// RGB LUT lattice points a render can touch: material colours and the sky
// gradient (SkyLighting depends on the ray's y only).  Only these are filled.
static void collect_cells(float3 rgb, std::set<uint64_t>& pts)
{
    const float lum = max3(rgb);
    if (lum > 1.0f) rgb = rgb / lum;
    constexpr int RES = SPECTRUM_RGB_LUT_RES;
    const float c[3] = {rgb.x, rgb.y, rgb.z};
    int lo[3], hi[3];
    for (int k = 0; k < 3; ++k)
    {
        float g = c[k] * static_cast<float>(RES) - 0.5f;
        g = fminf(fmaxf(g, 0.0f), static_cast<float>(RES) - 1.0f);
        lo[k] = (int)floorf(g);
        hi[k] = lo[k] + 1 >= RES ? RES - 1 : lo[k] + 1;
    }
    for (int a = 0; a < 2; ++a)
        for (int b = 0; b < 2; ++b)
            for (int e = 0; e < 2; ++e)
            {
                const uint64_t x = a ? hi[0] : lo[0], y = b ? hi[1] : lo[1], z = e ? hi[2] : lo[2];
                pts.insert((z * RES + y) * RES + x);
            }
}

// ---------------------------------------------------------------- probes
// Probe-set file: int32 n; n x int4 key (pg::GetVoxelGrid: voxel xyz, face);
// n x Octahedron::data_ (totalPixelCountWithPad_ x float4); n x uint64 count_.
struct ProbeSet
{
    std::vector<int4> keys;
    std::vector<Octahedron> probes;
};

static ProbeSet read_probes(const std::vector<char>& b, size_t* at_io)
{
    constexpr int ALL = Octahedron::totalPixelCountWithPad_;
    size_t at = *at_io;
    if (b.size() < at + 4) die("bad probe file");
    const int n = *reinterpret_cast<const int32_t*>(b.data() + at);
    at += 4;
    if (n < 0 || b.size() < at + (size_t)n * (16 + ALL * 16 + 8)) die("bad probe file (size)");
    ProbeSet ps;
    ps.keys.resize(n);
    ps.probes.resize(n);
    memcpy(ps.keys.data(), b.data() + at, (size_t)n * 16);
    at += (size_t)n * 16;
    for (int i = 0; i < n; ++i)
    {
        memcpy(ps.probes[i].data_, b.data() + at, ALL * 16);
        at += ALL * 16;
    }
    for (int i = 0; i < n; ++i)
    {
        memcpy(&ps.probes[i].count_, b.data() + at, 8);
        at += 8;
    }
    *at_io = at;
    return ps;
}

static void write_probes(const char* path, const ProbeSet& ps)
{
    constexpr int ALL = Octahedron::totalPixelCountWithPad_;
    const int32_t n = (int32_t)ps.keys.size();
    write_file(path, &n, 4);
    write_file(path, ps.keys.data(), (size_t)n * 16, true);
    for (int i = 0; i < n; ++i) write_file(path, ps.probes[i].data_, ALL * 16, true);
    for (int i = 0; i < n; ++i) write_file(path, &ps.probes[i].count_, 8, true);
}

// The index volume QueryProbe reads (core/render/render.cuh:434-458): a dense
// box over the keys' voxels, PATH_GUIDING_FACE_COUNT entries per voxel,
// SIZE_T_MAX where no probe is allocated -- what UpdatePathGuidingSample grows
// (core/scene.cu:440-500).
static std::vector<size_t> index_volume(const ProbeSet& ps, int3* start, int3* end, int3* size)
{
    if (ps.keys.empty())
    {
        *start = *end = *size = int3{0, 0, 0};
        return {};
    }
    int3 lo{INT32_MAX, INT32_MAX, INT32_MAX}, hi{INT32_MIN, INT32_MIN, INT32_MIN};
    for (const int4& k : ps.keys)
    {
        lo = int3{std::min(lo.x, k.x), std::min(lo.y, k.y), std::min(lo.z, k.z)};
        hi = int3{std::max(hi.x, k.x), std::max(hi.y, k.y), std::max(hi.z, k.z)};
    }
    *start = lo;
    *end = hi;
    *size = pg::DimsFromBoundsInclusive(lo, hi);
    std::vector<size_t> vol((size_t)size->x * size->y * size->z * PATH_GUIDING_FACE_COUNT, SIZE_T_MAX);
    for (size_t i = 0; i < ps.keys.size(); ++i)
    {
        const int4 k = ps.keys[i];
        if (k.w < 0 || k.w >= PATH_GUIDING_FACE_COUNT) die("probe key with a bad face");
        const size_t lin = (size_t)(k.x - lo.x) + (size_t)size->x * ((size_t)(k.y - lo.y) + (size_t)size->y * (size_t)(k.z - lo.z));
        vol[lin * PATH_GUIDING_FACE_COUNT + (size_t)k.w] = i;
    }
    return vol;
}

// One probe update as SceneRenderer::UpdatePathGuidingSample runs it
// (core/scene.cu:409-570): every record's key gets a probe (new probes start
// zeroed), AccumulateSamplesToOctaLeafKernel's body per record in record
// order, then MergeProbeKernel's body for every probe the frame touched
// (core/guiding/guiding.cuh:373-517), which ends in Texture::GenerateMipmaps.
// in: probe-set file; records file int32 n + n x {int4 key, float3 dir,
// float3 radiance}.  out: the updated probe set (new probes after the old, in
// key order as the reference's sorted unique grids).
static int cmd_pgupdate(const char* probe_path, const char* rec_path, const char* out_path)
{
    std::vector<char> pb = read_file(probe_path);
    size_t at = 0;
    ProbeSet ps = read_probes(pb, &at);
    std::vector<char> rb = read_file(rec_path);
    const int nrec = *reinterpret_cast<const int32_t*>(rb.data());
    struct Rec { int32_t key[4]; float dir[3]; float rad[3]; };
    static_assert(sizeof(Rec) == 40, "record layout");
    if (rb.size() < 4 + (size_t)nrec * sizeof(Rec)) die("bad record file");
    std::vector<Rec> recs(nrec);
    memcpy(recs.data(), rb.data() + 4, (size_t)nrec * sizeof(Rec));
    // keys without a probe, sorted and unique, take the next indices
    auto less = [](const int4& a, const int4& b) {
        if (a.x != b.x) return a.x < b.x;
        if (a.y != b.y) return a.y < b.y;
        if (a.z != b.z) return a.z < b.z;
        return a.w < b.w;
    };
    std::vector<int4> fresh;
    {
        std::vector<int4> known = ps.keys;
        std::sort(known.begin(), known.end(), less);
        for (const Rec& r : recs)
        {
            const int4 k{r.key[0], r.key[1], r.key[2], r.key[3]};
            if (!std::binary_search(known.begin(), known.end(), k, less)) fresh.push_back(k);
        }
        std::sort(fresh.begin(), fresh.end(), less);
        fresh.erase(std::unique(fresh.begin(), fresh.end(), [&](const int4& a, const int4& b) { return !less(a, b) && !less(b, a); }), fresh.end());
    }
    for (const int4& k : fresh)
    {
        ps.keys.push_back(k);
        ps.probes.emplace_back();
        memset(static_cast<void*>(&ps.probes.back()), 0, sizeof(Octahedron));
    }
    int3 vs, ve, vd;
    std::vector<size_t> vol = index_volume(ps, &vs, &ve, &vd);
    const pg::ProbeIndexLookup lookup{vol.data(), vs, vd};
    std::vector<Octahedron> temp(ps.probes.size());
    for (auto& t : temp) memset(static_cast<void*>(&t), 0, sizeof(Octahedron));
    constexpr int res = Octahedron::resolution_;
    for (const Rec& r : recs)
    {
        const size_t realIndex = lookup(int4{r.key[0], r.key[1], r.key[2], r.key[3]});
        if (realIndex == SIZE_T_MAX) continue;
        const float3 dir = normalize(float3{r.dir[0], r.dir[1], r.dir[2]});
        const int2 pix = pg::DirectionToLeafPixel(dir);
        Octahedron& cp = temp[realIndex];
        float4* leaf = &cp.data_[0];
        const int idx = pix.y * res + pix.x;
        const float J = pg::JacobianUVToOctahedronSphereDirection(dir);
        const float3 rj = float3{r.rad[0], r.rad[1], r.rad[2]} * J;
        leaf[idx].x += rj.x;
        leaf[idx].y += rj.y;
        leaf[idx].z += rj.z;
        cp.count_ += 1ull;
    }
    constexpr int N = Octahedron::resolution2_;
    for (size_t p = 0; p < ps.probes.size(); ++p)
    {
        const Octahedron& probeNew = temp[p];
        const unsigned long long countNew = probeNew.count_;
        if (countNew == 0ull) continue;
        Octahedron& probeOld = ps.probes[p];
        const unsigned long long countOld = probeOld.count_;
        const double invDen = 1.0 / static_cast<double>(countOld + countNew);
        const double alpha = static_cast<double>(countOld) * invDen;
        for (int k = 0; k < N; ++k)
        {
            float4 oldValue = probeOld.data_[k];
            const float4 newValue = probeNew.data_[k];
            oldValue.x = static_cast<float>(static_cast<double>(oldValue.x) * alpha + static_cast<double>(newValue.x) * invDen);
            oldValue.y = static_cast<float>(static_cast<double>(oldValue.y) * alpha + static_cast<double>(newValue.y) * invDen);
            oldValue.z = static_cast<float>(static_cast<double>(oldValue.z) * alpha + static_cast<double>(newValue.z) * invDen);
            probeOld.data_[k] = oldValue;
        }
        probeOld.count_ = std::min(PATH_GUIDING_PROBE_MAX_STORE_COUNT, countOld + countNew);
        probeOld.GenerateMipmaps();
    }
    write_probes(out_path, ps);
    printf("{\"probes\": %zu, \"new\": %zu, \"records\": %d}\n", ps.probes.size(), fresh.size(), nrec);
    return 0;
}

static int cmd_render(const char* scene_path, const char* params_path, const char* out_path,
                      const char* probe_path)
{
    std::vector<char> sb = read_file(scene_path);
    std::vector<char> pb = read_file(params_path);
    if (sb.size() < 8 || memcmp(sb.data(), "ARS2", 4) != 0) die("bad scene file");
    const int nobj = *reinterpret_cast<const int32_t*>(sb.data() + 4);
    const FileObject* fo = reinterpret_cast<const FileObject*>(sb.data() + 8);
    // SDF volume cache after the objects
    std::vector<std::vector<float>> vol_data;
    std::vector<sdf::SDFVolumeInfo> vol_info;
    {
        size_t at = 8 + (size_t)nobj * sizeof(FileObject);
        if (sb.size() < at + 4) die("bad scene file (volumes)");
        const int nvol = *reinterpret_cast<const int32_t*>(sb.data() + at);
        at += 4;
        for (int v = 0; v < nvol; ++v)
        {
            const FileVolume* fv = reinterpret_cast<const FileVolume*>(sb.data() + at);
            at += sizeof(FileVolume);
            const size_t n = (size_t)fv->dims[0] * fv->dims[1] * fv->dims[2];
            std::vector<float> data(n);
            if (fv->fn < 0)
            {
                memcpy(data.data(), sb.data() + at, n * sizeof(float));
                at += n * sizeof(float);
            }
            else
            {
                fill_volume(fv->fn, fv->params, fv->dims, data.data());
            }
            vol_data.push_back(std::move(data));
            sdf::SDFVolumeInfo info{};
            info.dim_ = int3{fv->dims[0], fv->dims[1], fv->dims[2]};
            info.ComputeVoxelSize();
            vol_info.push_back(info);
        }
        for (size_t v = 0; v < vol_info.size(); ++v) vol_info[v].volumePtr_ = vol_data[v].data();
        sdf::REF_HOST_SDF_INFOS = vol_info.empty() ? nullptr : vol_info.data();
        sdf::REF_HOST_SDF_COUNT = (uint32_t)vol_info.size();
    }
    RenderParams prm;
    memset(&prm, 0, sizeof(prm));
    memcpy(&prm, pb.data(), std::min(pb.size(), sizeof(prm)));
    if (!(prm.guide_inv_unit > 0.0f)) prm.guide_inv_unit = REF_PG_INV_UNIT;

    // scene objects through the reference's own constructors
    std::vector<SceneObject> objs;
    objs.reserve(nobj);
    for (int i = 0; i < nobj; ++i)
    {
        const FileObject& o = fo[i];
        if (o.type == 3)
        {
            SceneObject so;
            so.type_ = EObjectType::OBJ_TRIANGLE;
            so.material_ = make_material(o);
            so.triV0_ = f3(o.v0);
            so.triV1_ = f3(o.v1);
            so.triV2_ = f3(o.v2);
            so.proxy_.boundMin_ = float3{fminf(o.v0[0], fminf(o.v1[0], o.v2[0])), fminf(o.v0[1], fminf(o.v1[1], o.v2[1])), fminf(o.v0[2], fminf(o.v1[2], o.v2[2]))};
            so.proxy_.boundMax_ = float3{fmaxf(o.v0[0], fmaxf(o.v1[0], o.v2[0])), fmaxf(o.v0[1], fmaxf(o.v1[1], o.v2[1])), fmaxf(o.v0[2], fmaxf(o.v1[2], o.v2[2]))};
            so.proxy_.center_ = (so.proxy_.boundMin_ + so.proxy_.boundMax_) * 0.5f;
            objs.push_back(so);
        }
        else if (o.type == 2)
        {
            AdditionalObjectInfo info{};
            info.sdfType_ = static_cast<ESDFType>(o.sdf_type);
            info.sdfInfo_.sdfInfo0_ = float4{o.sdf_params[0], o.sdf_params[1], o.sdf_params[2], o.sdf_params[3]};
            info.sdfInfo_.cachedVolumeIndex_ = o.sdf_volume;
            objs.emplace_back(f3(o.center), f3(o.extent), make_material(o), f3(o.rotation), EObjectType::OBJ_SDF, info);
        }
        else
        {
            objs.emplace_back(f3(o.center), f3(o.extent), make_material(o), f3(o.rotation),
                              o.type == 1 ? EObjectType::OBJ_SPHERE : EObjectType::OBJ_CUBE);
        }
    }
    // BVH + light table (core/scene.cu:666-706)
    std::vector<PrimitiveProxy> proxys;
    for (auto& so : objs) proxys.push_back(so.proxy_);
    BVHHost bvh = BuildBVH(proxys);
    std::vector<AdditionalLightInfo> lights;
    float total = 0.0f;
    for (int i = 0; i < (int)objs.size(); ++i)
    {
        objs[i].objectIndex_ = i;
        if (objs[i].material_.shadingModel_ == EShadingModel::MAT_LIGHT)
        {
            objs[i].lightIndex_ = (int)lights.size();
            AdditionalLightInfo li;
            li.objectIndex_ = i;
            li.importanceWeight_ = fmaxf(objs[i].GetArea() * objs[i].GetEmissivePower(), 1.0e-20f);
            total += li.importanceWeight_;
            lights.push_back(li);
        }
        else
        {
            objs[i].lightIndex_ = -1;
        }
    }
    for (auto& li : lights) li.selectProb_ = li.importanceWeight_ / total;

    // spectral LUTs: full lambda LUT, RGB lattice points the scene can touch
    using namespace spectrum::query;
    constexpr int RES = SPECTRUM_RGB_LUT_RES;
    constexpr int LRES = SPECTRUM_LAMBDA_LUT_RES;
    std::vector<float> lam((size_t)LRES * KERNEL);
    {
        const float step = (780.0f - 360.0f) / static_cast<float>(LRES);
        for (int i = 0; i < LRES; ++i)
        {
            const float in1[1] = {360.0f + (i + 0.5f) * step};
            LambdaEncode(in1, &lam[(size_t)i * KERNEL]);
        }
    }
    float* lut = static_cast<float*>(calloc((size_t)RES * RES * RES * KERNEL, sizeof(float)));
    if (!lut) die("LUT allocation failed");
    {
        std::set<uint64_t> pts;
        for (auto& so : objs)
        {
            collect_cells(so.material_.texture_.baseTexture_.albedo_, pts);
            collect_cells(so.material_.texture_.baseTexture_.emissive_, pts);
        }
        const int NS = 1 << 22;
        for (int i = 0; i <= NS; ++i)
        {
            const float y = -1.0f + 2.0f * (float)i / (float)NS;
            collect_cells(SkyLighting(float3{0.0f, y, 0.0f}), pts);
        }
        std::vector<uint64_t> v(pts.begin(), pts.end());
        constexpr float invRes = 1.0f / static_cast<float>(RES);
#pragma omp parallel for
        for (int i = 0; i < (int)v.size(); ++i)
        {
            const uint64_t p = v[i];
            const int x = (int)(p % RES), y = (int)((p / RES) % RES), z = (int)(p / ((uint64_t)RES * RES));
            float in3[3] = {(x + 0.5f) * invRes, (y + 0.5f) * invRes, (z + 0.5f) * invRes};
            RGBEncode(in3, &lut[p * KERNEL]);
        }
    }

    SCENE_OBJECTS = objs.data();
    SCENE_OBJECT_COUNTS = (int)objs.size();
    SCENE_LIGHTS_INFO = lights.data();
    SCENE_LIGHTS_COUNTS = (int)lights.size();
    BVH_NODES = bvh.nodes_.data();
    BVH_NODES_COUNTS = (int)bvh.nodes_.size();
    BVH_OBJECT_INDICES = bvh.objectIndices_.data();
    SPECTRUM_LUT_RGB = lut;
    SPECTRUM_LUT_LAMBDA = lam.data();
    REF_MAX_TRACING_DEPTH = prm.max_depth;
    SCENE_PROBES_COUNTS = 0;
    // voxel guide: the given probe set behind the index volume QueryProbe reads
    ProbeSet guide_set;
    std::vector<size_t> guide_vol;
    if (prm.guide)
    {
        if (!probe_path) die("guided render without a probe file");
        std::vector<char> gb = read_file(probe_path);
        size_t at = 0;
        guide_set = read_probes(gb, &at);
        int3 vs, ve, vd;
        guide_vol = index_volume(guide_set, &vs, &ve, &vd);
        SCENE_PROBES = guide_set.probes.data();
        SCENE_PROBES_COUNTS = guide_set.probes.size();
        INDIRECT_VOLUME_START = vs;
        INDIRECT_VOLUME_END = ve;
        INDIRECT_VOLUME_SIZE = vd;
        INDIRECT_INDEX_VOLUME = guide_vol.data();
        REF_PG_INV_UNIT = prm.guide_inv_unit;
    }
    // radiance records of the per-sample frames: PATH_GUIDING_COLLECT_DEPTH per pixel sample

    const int W = prm.width, H = prm.height;
    const size_t npix = (size_t)W * H;
    std::vector<double> sums(npix * 3, 0.0);
    std::vector<float> per_sample((size_t)prm.per_sample_frames * npix * 3, 0.0f);
    std::vector<pg::PathGuidingSample> records(prm.guide ? (size_t)prm.per_sample_frames * npix * PATH_GUIDING_COLLECT_DEPTH : 0);
    std::vector<pg::PathGuidingSample> scratch_records(prm.guide ? (size_t)npix * PATH_GUIDING_COLLECT_DEPTH : 0);
    const float3 camO = f3(prm.cam_origin), camD = f3(prm.cam_dir);
    const float FOV = prm.fov_deg * 3.1415926f / 180.0f;
    const float aspect = static_cast<float>(W) / fmaxf(1.0f, static_cast<float>(H));
    const float tanHalfY = arm_tanf(0.5f * FOV);
    const float tanHalfX = tanHalfY * aspect;
    const float3 right = normalize(cross(camD, float3{0.0, 1.0, 0.0}));
    const float3 up = normalize(cross(camD, right));

    // the reference zeroes its device-side records (ResetScreenGBuffer, core/GUI.hpp:202-230)
    std::vector<denoise::ScreenGBuffer> gbuf(prm.denoise ? npix : 0);
    std::vector<denoise::ScreenStatisticsBuffer> stats(prm.denoise ? npix : 0);
    if (prm.denoise)
    {
        memset(static_cast<void*>(gbuf.data()), 0, npix * sizeof(denoise::ScreenGBuffer));
        memset(static_cast<void*>(stats.data()), 0, npix * sizeof(denoise::ScreenStatisticsBuffer));
    }
    auto t0 = std::chrono::steady_clock::now();
    for (int s = 0; s < prm.spp; ++s)
    {
        const int frame = prm.first_frame + s;
        FRAME_INDEX = frame;
        TOTAL_FRAME_INDEX = (uint64_t)frame;
#pragma omp parallel for schedule(dynamic, 64)
        for (long long p = 0; p < (long long)npix; ++p)
        {
            const int i = (int)(p % W), j = (int)(p / W);
            curandState seed = ar_pcg_init(prm.seed, (uint64_t)p, (uint64_t)frame);
            const float u = (i + Rand1(&seed)) / static_cast<float>(W);
            const float v = (j + Rand1(&seed)) / static_cast<float>(H);
            const float2 ndc = make_float2(u * 2.f - 1.f, (1.0 - v) * 2.f - 1.f);
            const float sx = ndc.x * tanHalfX;
            const float sy = ndc.y * tanHalfY;
            const float3 rayDirection = normalize(camD + right * sx + up * sy);
            float4 r;
            denoise::ScreenGBuffer* gbp = prm.denoise ? &gbuf[p] : nullptr;
            denoise::ScreenStatisticsBuffer* stp = prm.denoise ? &stats[p] : nullptr;
            if (prm.guide)
            {
                pg::PathGuidingSample* rec = s < prm.per_sample_frames
                                                 ? &records[((size_t)s * npix + p) * PATH_GUIDING_COLLECT_DEPTH]
                                                 : &scratch_records[(size_t)p * PATH_GUIDING_COLLECT_DEPTH];
                if (prm.use_nee) r = CalculateRadiance<true, true, true>(&seed, camO, rayDirection, rec, gbp, stp);
                else r = CalculateRadiance<true, false, true>(&seed, camO, rayDirection, rec, gbp, stp);
            }
            else if (prm.use_nee) r = CalculateRadiance<true, true, false>(&seed, camO, rayDirection, nullptr, gbp, stp);
            else r = CalculateRadiance<true, false, false>(&seed, camO, rayDirection, nullptr, gbp, stp);
            float3 result = make_f3(r);
            result = max(float3{0}, result);
            sums[3 * p + 0] += (double)result.x;
            sums[3 * p + 1] += (double)result.y;
            sums[3 * p + 2] += (double)result.z;
            if (s < prm.per_sample_frames)
            {
                float* q = &per_sample[((size_t)s * npix + p) * 3];
                q[0] = result.x;
                q[1] = result.y;
                q[2] = result.z;
            }
        }
    }
    auto t1 = std::chrono::steady_clock::now();
    write_file(out_path, sums.data(), sums.size() * 8);
    if (prm.per_sample_frames) write_file(out_path, per_sample.data(), per_sample.size() * 4, true);
    if (prm.guide)
    {
        // per pixel sample, PATH_GUIDING_COLLECT_DEPTH x {int32 valid, int4 key, float3 dir, float3 radiance}
        std::vector<int32_t> flat(records.size() * 11);
        for (size_t i = 0; i < records.size(); ++i)
        {
            const pg::PathGuidingSample& g = records[i];
            int32_t* o = &flat[i * 11];
            o[0] = g.valid_ ? 1 : 0;
            o[1] = g.voxelGrid_.x;
            o[2] = g.voxelGrid_.y;
            o[3] = g.voxelGrid_.z;
            o[4] = g.voxelGrid_.w;
            memcpy(&o[5], &g.radianceDirection_, 12);
            memcpy(&o[8], &g.radiance_, 12);
        }
        write_file(out_path, flat.data(), flat.size() * 4, true);
    }
    if (prm.denoise)
    {
        std::vector<PlainGBuf> pg(npix);
        std::vector<PlainStat> ps(npix);
        for (size_t i = 0; i < npix; ++i) to_plain(gbuf[i], stats[i], &pg[i], &ps[i]);
        write_file(out_path, pg.data(), pg.size() * sizeof(PlainGBuf), true);
        write_file(out_path, ps.data(), ps.size() * sizeof(PlainStat), true);
    }
    free(lut);
    const double secs = std::chrono::duration<double>(t1 - t0).count();
    printf("{\"render_s\": %.6f, \"samples\": %llu, \"msamples_per_s\": %.6f, \"threads\": %d, \"bvh_nodes\": %zu}\n",
           secs, (unsigned long long)npix * prm.spp, (double)npix * prm.spp / secs / 1e6, omp_get_max_threads(), bvh.nodes_.size());
    return 0;
}

// ---------------------------------------------------------------- denoise
// in: int32 width, height; float XYZ image (3 per pixel); PlainGBuf and
// PlainStat per pixel.  out: float XYZ (3 per pixel).  Per output pixel the
// loop of Bilateral16x16<7>: neighbours at clamped image coordinates, centre
// term with weight 1e-6, weights ComputeSVGFWeight x spatial Gaussian x
// ComputeTStatisticFinal, SeparateSample before and CompositeSample after.
static int cmd_denoise(const char* in_path, const char* out_path)
{
    std::vector<char> buf = read_file(in_path);
    if (buf.size() < 8) die("bad denoise input");
    const int W = *reinterpret_cast<const int32_t*>(buf.data());
    const int H = *reinterpret_cast<const int32_t*>(buf.data() + 4);
    const size_t npix = (size_t)W * H;
    if (W <= 0 || H <= 0 || buf.size() != 8 + npix * (12 + sizeof(PlainGBuf) + sizeof(PlainStat))) die("bad denoise input size");
    const float* img = reinterpret_cast<const float*>(buf.data() + 8);
    const PlainGBuf* pg = reinterpret_cast<const PlainGBuf*>(buf.data() + 8 + npix * 12);
    const PlainStat* pst = reinterpret_cast<const PlainStat*>(buf.data() + 8 + npix * (12 + sizeof(PlainGBuf)));
    std::vector<denoise::ScreenGBuffer> g(npix);
    std::vector<denoise::ScreenStatisticsBuffer> st(npix);
    for (size_t i = 0; i < npix; ++i) from_plain(pg[i], pst[i], &g[i], &st[i]);
    std::vector<float> out(npix * 3);
    constexpr int R = 7;
#pragma omp parallel for schedule(dynamic, 16)
    for (int oy = 0; oy < H; ++oy)
    {
        for (int ox = 0; ox < W; ++ox)
        {
            const size_t c = (size_t)oy * W + ox;
            const float3 cc{img[3 * c], img[3 * c + 1], img[3 * c + 2]};
            float3 acc = make_float3(0, 0, 0);
            float accW = 0.0f;
            constexpr float CENTER_PIXEL_EPS = 1.0e-6f;
            acc = acc + denoise::SeparateSample(g[c], cc) * CENTER_PIXEL_EPS;
            accW = accW + CENTER_PIXEL_EPS;
            for (int j = -R; j <= R; ++j)
            {
                const int ny = clampi(oy + j, 0, H - 1);
                for (int i = -R; i <= R; ++i)
                {
                    const int nx = clampi(ox + i, 0, W - 1);
                    const size_t q = (size_t)ny * W + nx;
                    const float3 qc{img[3 * q], img[3 * q + 1], img[3 * q + 2]};
                    const float weight = denoise::ComputeSVGFWeight(g[c], g[q]) *
                                         arm_expf(-(i * i + j * j) * denoise::FilterParams::inv2Sigma2Spatial_) *
                                         denoise::ComputeTStatisticFinal(st[c], st[q]);
                    acc = acc + denoise::SeparateSample(g[q], qc) * weight;
                    accW = accW + weight;
                }
            }
            const float3 r = denoise::CompositeSample(g[c], acc / accW);
            out[3 * c] = r.x;
            out[3 * c + 1] = r.y;
            out[3 * c + 2] = r.z;
        }
    }
    write_file(out_path, out.data(), out.size() * 4);
    return 0;
}

// ---------------------------------------------------------------- guide
// Probe math of the reference's voxel guide on one probe: in = header
// {int32 n} + leaf (Octahedron::resolution2_ x float4) + n x {dir 3, normal 3,
// query 3, pos 3, uv 2, seed u64 as 2 floats}; out = all texels
// (Octahedron::totalPixelCountWithPad_ x float4) + n x 14 floats:
// face, voxel xyz, uv(dir) 2, sphere(uv) 3, hemisphere pdf, sampled dir 3 + pdf.
static int cmd_guide(const char* in_path, const char* out_path)
{
    std::vector<char> buf = read_file(in_path);
    const int n = *reinterpret_cast<const int32_t*>(buf.data());
    const float* leaf = reinterpret_cast<const float*>(buf.data() + 4);
    constexpr int LEAF = Octahedron::resolution2_;
    constexpr int ALL = Octahedron::totalPixelCountWithPad_;
    const float* rec = leaf + LEAF * 4;
    Octahedron* probe = new Octahedron();
    for (int i = 0; i < LEAF; ++i)
        probe->data_[i] = float4{leaf[4 * i], leaf[4 * i + 1], leaf[4 * i + 2], leaf[4 * i + 3]};
    probe->GenerateMipmaps();
    std::vector<float> out(ALL * 4 + (size_t)n * 14);
    for (int i = 0; i < ALL; ++i)
    {
        out[4 * i] = probe->data_[i].x;
        out[4 * i + 1] = probe->data_[i].y;
        out[4 * i + 2] = probe->data_[i].z;
        out[4 * i + 3] = probe->data_[i].w;
    }
    for (int i = 0; i < n; ++i)
    {
        const float* r = rec + (size_t)i * 16;
        const float3 dir{r[0], r[1], r[2]}, nrm{r[3], r[4], r[5]}, q{r[6], r[7], r[8]}, pos{r[9], r[10], r[11]};
        const float2 uv{r[12], r[13]};
        uint64_t seed;
        memcpy(&seed, r + 14, 8);
        float* o = &out[ALL * 4 + (size_t)i * 14];
        const int4 key = pg::GetVoxelGrid(pos, dir);
        o[0] = (float)key.w;
        o[1] = (float)key.x;
        o[2] = (float)key.y;
        o[3] = (float)key.z;
        const float2 uvd = pg::SphereToUV(dir);
        o[4] = uvd.x;
        o[5] = uvd.y;
        const float3 s = pg::UVtoSphere(uv);
        o[6] = s.x;
        o[7] = s.y;
        o[8] = s.z;
        o[9] = probe->OctahedronHemispherePDF(dir, nrm, q);
        curandState st = ar_pcg_init(seed, (uint64_t)i, 0);
        const Sample smp = probe->SampleOctahedronHemisphere(&st, nrm, q);
        o[10] = smp.direction_.x;
        o[11] = smp.direction_.y;
        o[12] = smp.direction_.z;
        o[13] = smp.pdf_;
    }
    delete probe;
    write_file(out_path, out.data(), out.size() * 4);
    return 0;
}

// ---------------------------------------------------------------- tonemap
// in: int32 n, float exposure, int32 tone (0 ACES, 1 Gamma, 2 linear), n x float3 XYZ.
// out: n x RGBA8, the per-pixel body of Camera::RenderToFile (core/camera.cu:
// 64-89): tonemapFunction(XYZ2SRGBLinearD65(value * exp)), saturate, x 255
// truncated, alpha 255; the tone curves are core/tonemap.cuh's.
static int cmd_tonemap(const char* in_path, const char* out_path)
{
    std::vector<char> b = read_file(in_path);
    if (b.size() < 12) die("bad tonemap input");
    const int n = *reinterpret_cast<const int32_t*>(b.data());
    const float exposure = *reinterpret_cast<const float*>(b.data() + 4);
    const int tone = *reinterpret_cast<const int32_t*>(b.data() + 8);
    if (n < 0 || b.size() < 12 + (size_t)n * 12) die("bad tonemap input (size)");
    const float* xyz = reinterpret_cast<const float*>(b.data() + 12);
    std::vector<unsigned char> out((size_t)n * 4);
    for (int i = 0; i < n; ++i)
    {
        const float3 value = float3{xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]} * exposure;
        const float3 lin = XYZ2SRGBLinearD65(value);
        float3 res = tone == 0 ? ACES(lin) : (tone == 1 ? Gamma(lin) : lin);
        res = saturate(res);
        out[4 * (size_t)i] = static_cast<unsigned char>(res.x * 255);
        out[4 * (size_t)i + 1] = static_cast<unsigned char>(res.y * 255);
        out[4 * (size_t)i + 2] = static_cast<unsigned char>(res.z * 255);
        out[4 * (size_t)i + 3] = static_cast<unsigned char>(255);
    }
    write_file(out_path, out.data(), out.size());
    return 0;
}

// ---------------------------------------------------------------- frametone
// in: int32 n, float exposure, int32 toneType, n x float3 XYZ (the HDR running
// mean).  out: n x uint32, the Tonemap kernel's plain branch (core/scene.cu:
// 113-131): XYZ2SRGBLinearD65, x exposure, toneType 1 Gamma / 2 ACES, then
// 0xff000000 | r << 16 | g << 8 | b of 255 x saturate_.
static int cmd_frametone(const char* in_path, const char* out_path)
{
    std::vector<char> b = read_file(in_path);
    if (b.size() < 12) die("bad frametone input");
    const int n = *reinterpret_cast<const int32_t*>(b.data());
    const float exposure_ = *reinterpret_cast<const float*>(b.data() + 4);
    const int toneType = *reinterpret_cast<const int32_t*>(b.data() + 8);
    if (n < 0 || b.size() < 12 + (size_t)n * 12) die("bad frametone input (size)");
    const float* xyz = reinterpret_cast<const float*>(b.data() + 12);
    std::vector<uint32_t> out(n);
    for (int id = 0; id < n; ++id)
    {
        const float3 result = XYZ2SRGBLinearD65(float3{xyz[3 * id], xyz[3 * id + 1], xyz[3 * id + 2]});
        float3 value = result * exposure_;
        if (toneType == 1) value = Gamma(value);
        else if (toneType == 2) value = ACES(value);
        const unsigned int red = static_cast<unsigned int>(255.0f * saturate_(value.x));
        const unsigned int green = static_cast<unsigned int>(255.0f * saturate_(value.y));
        const unsigned int blue = static_cast<unsigned int>(255.0f * saturate_(value.z));
        out[id] = 0xff000000 | (red << 16) | (green << 8) | blue;
    }
    write_file(out_path, out.data(), out.size() * 4);
    return 0;
}

int main(int argc, char** argv)
{
    if (argc < 2) die("usage: ref_cpu kat | lut <lattice> <out> | trace|brute <tris> <rays> <out> | render <scene> <params> <out>");
    const std::string cmd = argv[1];
    if (cmd == "kat") return cmd_kat();
    if (cmd == "lut" && argc == 4) return cmd_lut(argv[2], argv[3]);
    if ((cmd == "trace" || cmd == "brute") && argc == 5) return cmd_trace(argv[2], argv[3], argv[4], cmd == "brute");
    if (cmd == "render" && argc == 5) return cmd_render(argv[2], argv[3], argv[4], nullptr);
    if (cmd == "render" && argc == 6) return cmd_render(argv[2], argv[3], argv[4], argv[5]);
    if (cmd == "tracecount" && argc == 5) return cmd_tracecount(argv[2], argv[3], argv[4]);
    if (cmd == "tonemap" && argc == 4) return cmd_tonemap(argv[2], argv[3]);
    if (cmd == "frametone" && argc == 4) return cmd_frametone(argv[2], argv[3]);
    if (cmd == "pgupdate" && argc == 5) return cmd_pgupdate(argv[2], argv[3], argv[4]);
    if (cmd == "guide" && argc == 4) return cmd_guide(argv[2], argv[3]);
    if (cmd == "denoise" && argc == 4) return cmd_denoise(argv[2], argv[3]);
    if (cmd == "sdfvol" && argc == 4) return cmd_sdfvol(argv[2], argv[3]);
    die("bad arguments");
    return 2;
}
#else
int main() { return 0; }
#endif
