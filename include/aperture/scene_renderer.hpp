// Header-only C++ layer with the reference's class names over the C ABI.
//
// Mirrors SceneRenderer (core/scene.hpp:18-135), SceneObject and Material
// (core/render/object.cuh:119-316) and Camera (core/camera.hpp:14-99) for the
// headless path: construct from a vector of objects, Render(size, origin,
// direction, sampleNum) returns the per-pixel linear XYZ image.  Errors throw
// aperture::Error (the reference only prints, core/vector.cuh:22).
#pragma once
#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
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
    OBJ_TRIANGLE = AR_OBJECT_TRIANGLE,
};

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
    SceneObject() = default;
    SceneObject(float3 center, float3 extent, const Material& material, float3 rotation,
                EObjectType type = EObjectType::OBJ_CUBE)
        : center_(center), extent_(extent), rotation_(rotation), material_(material), type_(type)
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
    float fov_deg = 60.0f;          // the reference's fixed FOV
    int max_depth = 1000;           // the reference's MAX_TRACING_DEPTH
    bool use_nee = true;            // SceneSetting::bUseNEE_
    uint64_t seed = 0x9e3779b97f4a7c15ULL;

    std::vector<float3> Render(int2 size, float3 cameraOrigin, float3 cameraDirection, int sampleNum = 1024)
    {
        build();
        ar_render_params p{};
        p.width = size.x;
        p.height = size.y;
        p.spp = sampleNum;
        p.max_depth = max_depth;
        p.cam_origin[0] = cameraOrigin.x; p.cam_origin[1] = cameraOrigin.y; p.cam_origin[2] = cameraOrigin.z;
        p.cam_dir[0] = cameraDirection.x; p.cam_dir[1] = cameraDirection.y; p.cam_dir[2] = cameraDirection.z;
        p.fov_deg = fov_deg;
        p.use_nee = use_nee ? 1 : 0;
        p.seed = seed;
        std::vector<double> xyz((size_t)size.x * size.y * 3);
        check(ar_render(ctx_, &p, xyz.data(), 0, nullptr, nullptr), "ar_render");
        std::vector<float3> out((size_t)size.x * size.y);
        for (size_t i = 0; i < out.size(); ++i)
            out[i] = float3{(float)xyz[3 * i], (float)xyz[3 * i + 1], (float)xyz[3 * i + 2]};
        return out;
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
        std::vector<ar_object> objs(objects_.size());
        for (size_t i = 0; i < objects_.size(); ++i)
        {
            const SceneObject& s = objects_[i];
            ar_object& o = objs[i];
            std::memset(&o, 0, sizeof(o));
            o.type = (int32_t)s.type_;
            o.material = (int32_t)mats.size();
            mats.push_back(s.material_.m);
            Material::set3(o.center, s.center_);
            Material::set3(o.extent, s.extent_);
            Material::set3(o.rotation_deg, s.rotation_);
            Material::set3(o.v0, s.v0_);
            Material::set3(o.v1, s.v1_);
            Material::set3(o.v2, s.v2_);
        }
        check(ar_scene_set_materials(ctx_, mats.data(), (int)mats.size()), "ar_scene_set_materials");
        check(ar_scene_set_objects(ctx_, objs.data(), (int)objs.size()), "ar_scene_set_objects");
        check(ar_scene_build(ctx_), "ar_scene_build");
        dirty_ = false;
    }
    std::vector<SceneObject> objects_;
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

  private:
    SceneRenderer& renderer_;
    std::string name_;
    int2 res_;
    float3 pos_, dir_;
};
} // namespace aperture
