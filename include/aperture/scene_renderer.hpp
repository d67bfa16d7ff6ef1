// Header-only C++ layer with the reference's class names over the C ABI.
//
// Mirrors SceneRenderer (core/scene.hpp:18-135), SceneObject and Material
// (core/render/object.cuh:119-316) and Camera (core/camera.hpp:14-99) for the
// headless path: construct from a vector of objects, Render(size, origin,
// direction, sampleNum) returns the per-pixel linear XYZ image.  Errors throw
// aperture::Error (the reference only prints, core/vector.cuh:22).
//
// Beyond the reference's surface: a triangle mesh with per-triangle materials
// and uv, albedo textures, the smooth-union SDF object, a homogeneous medium,
// the voxel / MLP path guide, the replay adjoints (device pointers, as the C
// ABI takes them) and Camera::RenderToFile writing the reference's BMP or a
// linear PFM.
#pragma once
#include <cctype>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "ar.h"

namespace aperture
{
struct float3
{
    float x, y, z;
};
struct int2
{
    int x, y;
};

struct Error : std::runtime_error
{
    ar_status code;
    Error(ar_status c, const std::string& m) : std::runtime_error(m), code(c) {}
};

enum class EObjectType
{
    OBJ_CUBE = AR_OBJECT_CUBE,
    OBJ_SPHERE = AR_OBJECT_SPHERE,
    OBJ_SDF = AR_OBJECT_SDF,
    OBJ_TRIANGLE = AR_OBJECT_TRIANGLE,
};

struct int3
{
    int x, y, z;
};

// field of an SDF object (AdditionalObjectInfo, core/render/object.cuh:216-225)
struct AdditionalObjectInfo
{
    int sdfType = AR_SDF_OBJECT_TORUS;
    float params[4] = {0, 0, 0, 0};  // SDFInfo::sdfInfo0_
    int volume = -1;                 // SDFInfo::cachedVolumeIndex_
};

// the reference's SDF helpers (namespace sdf, core/object/sdf/*)
namespace sdf
{
inline AdditionalObjectInfo CreateTorus(float scale = 1.0f, float R = 0.375f, float r = 0.125f)
{
    AdditionalObjectInfo a;
    a.sdfType = AR_SDF_OBJECT_TORUS;
    a.params[0] = R * scale;
    a.params[1] = r * scale;
    return a;
}
inline AdditionalObjectInfo CreateSDFVolume(int volumeIndex)
{
    AdditionalObjectInfo a;
    a.sdfType = AR_SDF_OBJECT_VOLUME;
    a.volume = volumeIndex;
    return a;
}
// parameters of the diamond volume functor (SDFInfo::sdfInfo0_ of sdf::CreateDiamond)
inline AdditionalObjectInfo CreateDiamond(float scale = 1.0f, float d = 0.94f, float bias = 0.5f, float tableZ = 0.3f)
{
    AdditionalObjectInfo a;
    a.params[0] = d;
    a.params[1] = bias;
    a.params[2] = tableZ;
    a.params[3] = scale * 0.5f;
    return a;
}
} // namespace sdf

enum class EShadingModel
{
    MAT_DIFFUSE = AR_SHADING_DIFFUSE,
    MAT_LIGHT = AR_SHADING_LIGHT,
    MAT_GLASS = AR_SHADING_GLASS,
    MAT_GGX = AR_SHADING_GGX,
};

struct Material
{
    ar_material m{};
    Material()
    {
        m.shading = AR_SHADING_DIFFUSE;
        m.albedo[0] = m.albedo[1] = m.albedo[2] = 1.0f;
        m.ior = 1.5f;
        m.sigma_a = 100.0f;
        m.abbe = 20.0f;
    }
    static void set3(float* d, float3 v) { d[0] = v.x; d[1] = v.y; d[2] = v.z; }
    static Material CreateDiffusePureColor(float3 color, float3 emissive = {0, 0, 0})
    {
        Material r;
        set3(r.m.albedo, color);
        set3(r.m.emissive, emissive);
        return r;
    }
    // diffuse albedo read from texture `texture` (0-based) at the mesh uv
    static Material CreateDiffuseTextured(int texture, float3 emissive = {0, 0, 0})
    {
        Material r;
        r.m.albedo_texture = texture + 1;
        set3(r.m.emissive, emissive);
        return r;
    }
    static Material CreateLight(float3 emissive)
    {
        Material r;
        r.m.shading = AR_SHADING_LIGHT;
        set3(r.m.albedo, {0, 0, 0});
        set3(r.m.emissive, emissive);
        return r;
    }
    static Material CreateGlassPureColor(float3 color, float IOR, float sigmaA, float abbeNumber = 20.0f,
                                         float tiltNumber = 0.0f)
    {
        Material r;
        r.m.shading = AR_SHADING_GLASS;
        set3(r.m.albedo, color);
        r.m.ior = IOR;
        r.m.sigma_a = sigmaA;
        r.m.abbe = abbeNumber;
        r.m.tilt = tiltNumber;
        return r;
    }
    static Material CreateGGXPureColor(float3 baseColor, float roughness, float metallic, float specular,
                                       float3 emissive = {0, 0, 0})
    {
        Material r;
        r.m.shading = AR_SHADING_GGX;
        set3(r.m.albedo, baseColor);
        set3(r.m.emissive, emissive);
        r.m.roughness = roughness;
        r.m.metallic = metallic;
        r.m.specular = specular;
        return r;
    }
};

struct SceneObject
{
    float3 center_{0, 0, 0}, extent_{0, 0, 0}, rotation_{0, 0, 0};
    float3 v0_{0, 0, 0}, v1_{0, 0, 0}, v2_{0, 0, 0};
    Material material_;
    EObjectType type_ = EObjectType::OBJ_CUBE;
    AdditionalObjectInfo additionalObjectInfo_;
    SceneObject() = default;
    SceneObject(float3 center, float3 extent, const Material& material, float3 rotation,
                EObjectType type = EObjectType::OBJ_CUBE, const AdditionalObjectInfo& additionalObjectInfo = {})
        : center_(center), extent_(extent), rotation_(rotation), material_(material), type_(type),
          additionalObjectInfo_(additionalObjectInfo)
    {
    }
    static SceneObject Triangle(float3 a, float3 b, float3 c, const Material& material)
    {
        SceneObject o;
        o.v0_ = a;
        o.v1_ = b;
        o.v2_ = c;
        o.material_ = material;
        o.type_ = EObjectType::OBJ_TRIANGLE;
        return o;
    }
};

class SceneRenderer
{
  public:
    explicit SceneRenderer(const std::vector<SceneObject>& sceneObjects, int device = 0) : objects_(sceneObjects)
    {
        check(ar_create(&ctx_, device), "ar_create");
    }
    ~SceneRenderer()
    {
        if (ctx_) ar_destroy(ctx_);
    }
    SceneRenderer(const SceneRenderer&) = delete;
    SceneRenderer& operator=(const SceneRenderer&) = delete;

    void MarkAsDirty() { dirty_ = true; }
    // SceneRenderer::MarkNeedResetGuiding (core/scene.hpp:102-105)
    void MarkNeedResetGuiding() { check(ar_guide_reset(ctx_, nullptr), "ar_guide_reset"); }
    float fov_deg = 60.0f;          // the reference's fixed FOV
    int max_depth = 1000;           // the reference's MAX_TRACING_DEPTH
    bool use_nee = true;            // SceneSetting::bUseNEE_
    int guide = AR_GUIDE_NONE;      // SceneSetting::bUsePathGuiding_ (AR_GUIDE_VOXEL), or AR_GUIDE_MLP
    bool denoise = false;           // SceneSetting::bDenoise_: Render returns the bilateral-filtered image
    uint64_t seed = 0x9e3779b97f4a7c15ULL;

    // Triangle mesh: n_vertices x 3 floats, 3 indices per triangle, one material per triangle.
    void SetMesh(const std::vector<float3>& vertices, const std::vector<uint32_t>& indices,
                 const std::vector<Material>& triangleMaterials)
    {
        mesh_vertices_ = vertices;
        mesh_indices_ = indices;
        mesh_materials_ = triangleMaterials;
        dirty_ = true;
    }
    // 6 floats per mesh triangle: (u, v) at each vertex
    void SetMeshUV(const std::vector<float>& uv)
    {
        mesh_uv_ = uv;
        dirty_ = true;
    }
    // RGB float textures, texels row-major (width x height x 3 each)
    void SetTextures(const std::vector<std::vector<float>>& texels, const std::vector<int2>& sizes)
    {
        textures_ = texels;
        texture_sizes_ = sizes;
        dirty_ = true;
    }
    // Replaces the texel values of the built scene (device or host floats, all textures concatenated).
    void UpdateTexels(const float* texels, int64_t nFloats, bool isDevice, void* stream = nullptr)
    {
        build();
        check(ar_scene_update_texels(ctx_, texels, nFloats, isDevice ? 1 : 0, stream), "ar_scene_update_texels");
    }
    // Smooth-union SDF object: primitives of 8 floats (kind, centre xyz, size xyz, 0).
    void SetSdfUnion(const std::vector<float>& prims, float smoothK, const Material& material)
    {
        sdf_prims_ = prims;
        sdf_k_ = smoothK;
        sdf_material_ = material;
        dirty_ = true;
    }
    // SDF volume cache (SceneRenderer::AddVolumeToCacheManager, core/scene.hpp:120-127):
    // a dims grid over the unit cube filled on the GPU from a built-in functor
    // (AR_SDF_FN_DIAMOND / AR_SDF_FN_TORUS, parameters in sdfInfo.params;
    // pMin / pMax are unused, as in the reference); returns the cache index.
    int AddVolumeToCacheManager(int3 dims, float3 pMin, float3 pMax, int functor, const AdditionalObjectInfo& sdfInfo)
    {
        (void)pMin;
        (void)pMax;
        const int32_t d[3] = {dims.x, dims.y, dims.z};
        int32_t index = -1;
        check(ar_sdf_volume_add(ctx_, functor, sdfInfo.params, d, &index), "ar_sdf_volume_add");
        return index;
    }
    // the same with caller values (dims.x fastest)
    int AddVolumeToCacheManager(int3 dims, const std::vector<float>& distances)
    {
        const int32_t d[3] = {dims.x, dims.y, dims.z};
        if (distances.size() != (size_t)dims.x * dims.y * dims.z) throw Error(AR_ERR_INVALID, "volume size mismatch");
        int32_t index = -1;
        check(ar_sdf_volume_add_data(ctx_, distances.data(), d, &index), "ar_sdf_volume_add_data");
        return index;
    }

    // Homogeneous medium in a box (takes effect on the next render); ClearMedium removes it.
    void SetMedium(float3 boxLo, float3 boxHi, float sigmaT, float albedo, float g, float emission)
    {
        ar_medium m{};
        Material::set3(m.box_lo, boxLo);
        Material::set3(m.box_hi, boxHi);
        m.sigma_t = sigmaT;
        m.albedo = albedo;
        m.g = g;
        m.emission = emission;
        check(ar_scene_set_medium(ctx_, &m), "ar_scene_set_medium");
    }
    void ClearMedium() { check(ar_scene_set_medium(ctx_, nullptr), "ar_scene_set_medium"); }

    ar_render_params Params(int2 size, float3 cameraOrigin, float3 cameraDirection, int sampleNum) const
    {
        ar_render_params p{};
        p.width = size.x;
        p.height = size.y;
        p.spp = sampleNum;
        p.max_depth = max_depth;
        Material::set3(p.cam_origin, cameraOrigin);
        Material::set3(p.cam_dir, cameraDirection);
        p.fov_deg = fov_deg;
        p.use_nee = use_nee ? 1 : 0;
        p.seed = seed;
        p.guide = guide;
        return p;
    }

    // Per-pixel mean linear XYZ, FP64 (3 doubles per pixel, top row first).
    std::vector<double> RenderXYZ(int2 size, float3 cameraOrigin, float3 cameraDirection, int sampleNum = 1024)
    {
        build();
        ar_render_params p = Params(size, cameraOrigin, cameraDirection, sampleNum);
        p.denoise_record = denoise ? 1 : 0;
        std::vector<double> xyz((size_t)size.x * size.y * 3);
        check(ar_render(ctx_, &p, xyz.data(), 0, nullptr, nullptr), "ar_render");
        if (!denoise) return xyz;
        std::vector<double> filtered(xyz.size());
        check(ar_denoise(ctx_, xyz.data(), 0, filtered.data(), 0, nullptr), "ar_denoise");
        return filtered;
    }

    // Where the next build makes the BVH: AR_BUILD_HOST (binned SAH, the
    // default) or AR_BUILD_GPU (same node format, same hits).
    void SetBuildMode(int mode)
    {
        check(ar_scene_set_build_mode(ctx_, mode), "ar_scene_set_build_mode");
        dirty_ = true;
    }
    // wall time of the last BVH build
    double BuildTimeMs()
    {
        build();
        double ms = 0.0;
        check(ar_scene_build_time(ctx_, &ms), "ar_scene_build_time");
        return ms;
    }
    // Moves the mesh's vertices (same count) and refits the BVH on the GPU:
    // the tree is kept, hits are exact for the moved mesh.
    void RefitMesh(const std::vector<float3>& vertices)
    {
        build();
        check(ar_scene_refit_mesh(ctx_, vertices.empty() ? nullptr : &vertices[0].x, (int)vertices.size(), 0, nullptr),
              "ar_scene_refit_mesh");
        mesh_vertices_ = vertices;
    }

    std::vector<float3> Render(int2 size, float3 cameraOrigin, float3 cameraDirection, int sampleNum = 1024)
    {
        const std::vector<double> xyz = RenderXYZ(size, cameraOrigin, cameraDirection, sampleNum);
        std::vector<float3> out((size_t)size.x * size.y);
        for (size_t i = 0; i < out.size(); ++i)
            out[i] = float3{(float)xyz[3 * i], (float)xyz[3 * i + 1], (float)xyz[3 * i + 2]};
        return out;
    }

    // One progressive frame (SceneRenderer::Render(hdrTarget, ldrTarget, size,
    // origin, direction, frameIndex, toneType, oddTarget, evenTarget,
    // radianceSampleBuffer, screenGBuffer, screenStatisticsBuffer),
    // core/scene.hpp:109-114): device buffers owned by the caller, hdrTarget the
    // float32 running mean of XYZ, ldrTarget 0xAARRGGBB (toneType 0 linear,
    // 1 gamma, 2 ACES).  The guide's radiance records and the denoiser's
    // G-buffer and moments live in the context, so the last three arguments are
    // accepted for the reference's signature and must be null.
    void Render(float3* hdrTarget, unsigned int* ldrTarget, int2 size, float3 cameraOrigin, float3 cameraDirection,
                int frameIndex, int toneType, float3* oddTarget = nullptr, float3* evenTarget = nullptr,
                void* radianceSampleBuffer = nullptr, void* screenGBuffer = nullptr,
                void* screenStatisticsBuffer = nullptr)
    {
        if (radianceSampleBuffer || screenGBuffer || screenStatisticsBuffer)
            throw Error(AR_ERR_INVALID, "record buffers are kept by the context; pass null");
        build();
        ar_render_params p = Params(size, cameraOrigin, cameraDirection, 1);
        p.denoise_record = denoise ? 1 : 0;
        check(ar_render_frame(ctx_, &p, frameIndex, toneType, &hdrTarget->x, ldrTarget,
                              oddTarget ? &oddTarget->x : nullptr, evenTarget ? &evenTarget->x : nullptr, nullptr),
              "ar_render_frame");
    }
    // SceneRenderer::SetExposure (core/scene.hpp:97): exposure of the frame's display image
    void SetExposure(float exp) { check(ar_set_exposure(ctx_, exp), "ar_set_exposure"); }

    // d(loss)/d(texels) into gradTexelsDevice (float64, TexelCount()) from
    // dLossDXyzDevice (float32, 3 per pixel), for the render with the same arguments.
    void Adjoint(const float* dLossDXyzDevice, double* gradTexelsDevice, int2 size, float3 cameraOrigin,
                 float3 cameraDirection, int sampleNum, void* stream = nullptr)
    {
        build();
        const ar_render_params p = Params(size, cameraOrigin, cameraDirection, sampleNum);
        check(ar_adjoint(ctx_, &p, dLossDXyzDevice, gradTexelsDevice, stream), "ar_adjoint");
    }
    // (d loss / d medium albedo, d loss / d medium emission)
    std::pair<double, double> AdjointMedium(const float* dLossDXyzDevice, int2 size, float3 cameraOrigin,
                                            float3 cameraDirection, int sampleNum, void* stream = nullptr)
    {
        build();
        const ar_render_params p = Params(size, cameraOrigin, cameraDirection, sampleNum);
        double g[2] = {0, 0};
        check(ar_adjoint_medium(ctx_, &p, dLossDXyzDevice, g, stream), "ar_adjoint_medium");
        return {g[0], g[1]};
    }
    int64_t TexelCount()
    {
        build();
        int64_t n = 0;
        check(ar_scene_texel_count(ctx_, &n), "ar_scene_texel_count");
        return n;
    }

    // XYZ (host, 3 doubles per pixel) -> 8-bit RGBA on the GPU (core/tonemap.cuh)
    std::vector<uint8_t> Tonemap(const std::vector<double>& xyz, int2 size, float exposure = 1.0f,
                                 int tone = AR_TONE_ACES)
    {
        std::vector<uint8_t> rgba((size_t)size.x * size.y * 4);
        check(ar_tonemap(ctx_, xyz.data(), 0, size.x, size.y, exposure, tone, rgba.data()), "ar_tonemap");
        return rgba;
    }

    ar_ctx* handle() const { return ctx_; }

  private:
    void check(ar_status s, const char* what)
    {
        if (s != AR_OK) throw Error(s, std::string(what) + ": " + (ctx_ ? ar_last_error(ctx_) : "no context"));
    }
    void build()
    {
        if (!dirty_) return;
        std::vector<ar_material> mats;
        auto mat_id = [&mats](const Material& m) {
            for (size_t i = 0; i < mats.size(); ++i)
                if (std::memcmp(&mats[i], &m.m, sizeof(ar_material)) == 0) return (int32_t)i;
            mats.push_back(m.m);
            return (int32_t)(mats.size() - 1);
        };
        std::vector<ar_object> objs(objects_.size());
        for (size_t i = 0; i < objects_.size(); ++i)
        {
            const SceneObject& s = objects_[i];
            ar_object& o = objs[i];
            std::memset(&o, 0, sizeof(o));
            o.type = (int32_t)s.type_;
            o.material = mat_id(s.material_);
            Material::set3(o.center, s.center_);
            Material::set3(o.extent, s.extent_);
            Material::set3(o.rotation_deg, s.rotation_);
            Material::set3(o.v0, s.v0_);
            Material::set3(o.v1, s.v1_);
            Material::set3(o.v2, s.v2_);
            o.sdf_type = s.additionalObjectInfo_.sdfType;
            for (int k = 0; k < 4; ++k) o.sdf_params[k] = s.additionalObjectInfo_.params[k];
            o.sdf_volume = s.additionalObjectInfo_.volume;
        }
        std::vector<int32_t> tri_mat(mesh_materials_.size());
        for (size_t i = 0; i < tri_mat.size(); ++i) tri_mat[i] = mat_id(mesh_materials_[i]);
        const int32_t sdf_mat = sdf_prims_.empty() ? -1 : mat_id(sdf_material_);
        check(ar_scene_set_materials(ctx_, mats.data(), (int)mats.size()), "ar_scene_set_materials");
        check(ar_scene_set_objects(ctx_, objs.data(), (int)objs.size()), "ar_scene_set_objects");
        const int ntri = (int)(mesh_indices_.size() / 3);
        check(ar_scene_set_mesh(ctx_, ntri ? &mesh_vertices_[0].x : nullptr, (int)mesh_vertices_.size(),
                                ntri ? mesh_indices_.data() : nullptr, ntri, ntri ? tri_mat.data() : nullptr),
              "ar_scene_set_mesh");
        if (!mesh_uv_.empty()) check(ar_scene_set_mesh_uv(ctx_, mesh_uv_.data(), ntri), "ar_scene_set_mesh_uv");
        if (!textures_.empty())
        {
            std::vector<float> all;
            std::vector<int32_t> sizes;
            for (size_t k = 0; k < textures_.size(); ++k)
            {
                all.insert(all.end(), textures_[k].begin(), textures_[k].end());
                sizes.push_back(texture_sizes_[k].x);
                sizes.push_back(texture_sizes_[k].y);
            }
            check(ar_scene_set_textures(ctx_, all.data(), sizes.data(), (int)textures_.size()),
                  "ar_scene_set_textures");
        }
        check(ar_scene_set_sdf_union(ctx_, sdf_prims_.empty() ? nullptr : sdf_prims_.data(),
                                     (int)(sdf_prims_.size() / 8), sdf_k_, sdf_mat),
              "ar_scene_set_sdf_union");
        check(ar_scene_build(ctx_), "ar_scene_build");
        dirty_ = false;
    }
    static_assert(sizeof(float3) == 3 * sizeof(float), "float3 is three packed floats");
    std::vector<SceneObject> objects_;
    std::vector<float3> mesh_vertices_;
    std::vector<uint32_t> mesh_indices_;
    std::vector<Material> mesh_materials_;
    std::vector<float> mesh_uv_;
    std::vector<std::vector<float>> textures_;
    std::vector<int2> texture_sizes_;
    std::vector<float> sdf_prims_;
    float sdf_k_ = 0.0f;
    Material sdf_material_;
    ar_ctx* ctx_ = nullptr;
    bool dirty_ = true;
};

class Camera
{
  public:
    Camera(SceneRenderer& renderer, std::string name, int resolutionX, int resolutionY, float3 position,
           float3 direction)
        : renderer_(renderer), name_(std::move(name)), res_{resolutionX, resolutionY}, pos_(position), dir_(direction)
    {
    }
    std::vector<float3> Render(int sampleNum = 1) { return renderer_.Render(res_, pos_, dir_, sampleNum); }

    // Camera::RenderToFile (core/camera.cu:64-89): ".pfm" writes linear XYZ
    // floats (bottom row first); otherwise the tonemapped 32-bit top-down BMP
    // the reference writes, at `path` if it ends in ".bmp", else `path`.bmp.
    // tone: AR_TONE_ACES (the reference's default), AR_TONE_GAMMA, AR_TONE_LINEAR.
    std::vector<double> RenderToFile(const std::string& path, int sampleNum = 1024, int tone = AR_TONE_ACES,
                                     float exposure = 1.0f)
    {
        std::vector<double> xyz = renderer_.RenderXYZ(res_, pos_, dir_, sampleNum);
        auto ends = [&path](const char* ext) {
            const size_t n = std::strlen(ext);
            if (path.size() < n) return false;
            for (size_t i = 0; i < n; ++i)
                if (std::tolower((unsigned char)path[path.size() - n + i]) != ext[i]) return false;
            return true;
        };
        if (ends(".pfm"))
            write_pfm(path, xyz);
        else
            write_bmp(ends(".bmp") ? path : path + ".bmp", renderer_.Tonemap(xyz, res_, exposure, tone));
        return xyz;
    }

  private:
    void write_pfm(const std::string& path, const std::vector<double>& xyz) const
    {
        FILE* f = std::fopen(path.c_str(), "wb");
        if (!f) throw Error(AR_ERR_INVALID, "cannot open " + path);
        std::fprintf(f, "PF\n%d %d\n-1.0\n", res_.x, res_.y);
        std::vector<float> row((size_t)res_.x * 3);
        for (int y = res_.y - 1; y >= 0; --y)
        {
            for (size_t i = 0; i < row.size(); ++i) row[i] = (float)xyz[(size_t)y * res_.x * 3 + i];
            std::fwrite(row.data(), sizeof(float), row.size(), f);
        }
        std::fclose(f);
    }
    void write_bmp(const std::string& path, const std::vector<uint8_t>& rgba) const
    {
        FILE* f = std::fopen(path.c_str(), "wb");
        if (!f) throw Error(AR_ERR_INVALID, "cannot open " + path);
        const uint32_t px = (uint32_t)res_.x * (uint32_t)res_.y * 4u;
        uint8_t h[54] = {};
        auto put32 = [&h](int at, uint32_t v) {
            for (int i = 0; i < 4; ++i) h[at + i] = (uint8_t)(v >> (8 * i));
        };
        h[0] = 'B';
        h[1] = 'M';
        put32(2, 54u + px);
        put32(10, 54u);
        put32(14, 40u);
        put32(18, (uint32_t)res_.x);
        put32(22, (uint32_t)(-res_.y));  // negative height: top row first
        h[26] = 1;
        h[28] = 32;
        put32(34, px);
        std::fwrite(h, 1, 54, f);
        std::vector<uint8_t> bgra(rgba.size());
        for (size_t i = 0; i < rgba.size(); i += 4)
        {
            bgra[i] = rgba[i + 2];
            bgra[i + 1] = rgba[i + 1];
            bgra[i + 2] = rgba[i];
            bgra[i + 3] = rgba[i + 3];
        }
        std::fwrite(bgra.data(), 1, bgra.size(), f);
        std::fclose(f);
    }

    SceneRenderer& renderer_;
    std::string name_;
    int2 res_;
    float3 pos_, dir_;
};
} // namespace aperture
