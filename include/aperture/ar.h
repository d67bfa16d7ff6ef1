/*
 * aperture-gb300 C ABI: GB300 (sm_103a) path tracing behind plain pointers.
 *
 * This is the drop-in boundary for the reference's host entry points:
 *   SceneRenderer(const std::vector<SceneObject>&)        core/scene.hpp:94, core/scene.cu:734-743
 *   std::vector<float3> SceneRenderer::Render(size, origin, dir, sampleNum)
 *                                                          core/scene.hpp:107, core/scene.cu:210-238
 *   SceneObject / Material::Create* / SceneSetting          core/render/object.cuh:10-27, 119-206, 227-316
 *   BuildBVH + TraverseBVH (closest / any hit)             core/bvh/bvh.cuh:142-422, core/render/intersection.cuh:148-310
 * A header-only C++ layer with the reference's class names sits on top of it
 * (include/aperture/scene_renderer.hpp).
 *
 * Conventions: every call returns an ar_status (0 = ok, negative = error; the
 * message is available from ar_last_error).  No call aborts or traps.  Device
 * kernels report recoverable faults (traversal stack or queue overflow) in a
 * sticky error word read with ar_get_error_word.  All state lives in the
 * context; several contexts may coexist in one process.  `stream` arguments
 * are cudaStream_t values (NULL = the context's own stream).
 */
#ifndef APERTURE_AR_H
#define APERTURE_AR_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int ar_status;
#define AR_OK 0
#define AR_ERR_INVALID -1   /* bad argument */
#define AR_ERR_CUDA -2      /* CUDA runtime error (no device, launch failure, ...) */
#define AR_ERR_NOMEM -3     /* device or host allocation failed */
#define AR_ERR_STATE -4     /* call out of order (e.g. render before build) */
#define AR_ERR_DEVICE -5    /* a kernel raised its error word */

/* object kinds (EObjectType, core/render/object.cuh:29-34, plus triangles) */
#define AR_OBJECT_CUBE 0
#define AR_OBJECT_SPHERE 1
#define AR_OBJECT_SDF 2        /* EObjectType::OBJ_SDF: a signed distance field inside an oriented box */
#define AR_OBJECT_TRIANGLE 3

/* Fields of SDF objects (ESDFType, core/render/object.cuh:36-42) */
#define AR_SDF_OBJECT_TORUS 0  /* sdf_params = (R, r) in unit coordinates (sdf::CreateTorus: 0.375, 0.125 x scale) */
#define AR_SDF_OBJECT_VOLUME 1 /* sdf_volume = index into the SDF volume cache */

/* shading models (EShadingModel, core/render/object.cuh:44-51) */
#define AR_SHADING_DIFFUSE 0
#define AR_SHADING_LIGHT 1
#define AR_SHADING_GLASS 2
#define AR_SHADING_GGX 3

/* device error word bits */
#define AR_DEVERR_TRAVERSAL_STACK 1u
#define AR_DEVERR_QUEUE 2u
#define AR_DEVERR_MLP 4u    /* a tensor-core wait of the MLP guide ran out (work skipped) */

typedef struct ar_ctx ar_ctx;

/* Material fields of GBuffer (core/render/object.cuh:59-71).  Values are
 * clamped exactly as the Material::Create* factories do. */
typedef struct ar_material
{
    int32_t shading;
    float albedo[3];
    float emissive[3];
    float roughness, metallic, specular;
    float ior, sigma_a, abbe, tilt;
    /* Albedo texture (no counterpart in the reference): 0 = none (use albedo),
     * k > 0 = texture k-1 of ar_scene_set_textures, sampled at the mesh
     * triangle's interpolated uv (nearest texel, clamped to the edge). */
    int32_t albedo_texture;
} ar_material;

/* One SceneObject: an oriented box (centre, half extent, Euler rotation in
 * degrees), a sphere (radius = max extent), a triangle (v0, v1, v2), or an SDF
 * object: the oriented box's inside mapped to the unit cube [-0.5, 0.5]^3,
 * where the field (sdf_type, sdf_params / sdf_volume; the reference's
 * AdditionalObjectInfo) is marched as IntersectSDFObject does
 * (core/object/sdf/sdf_base.cuh:107-163).  SDF objects with a light material
 * are in the light table but, as in the reference's NEESampleLight, are never
 * picked for next-event estimation. */
typedef struct ar_object
{
    int32_t type;
    int32_t material;        /* index into the material table */
    float center[3];
    float extent[3];
    float rotation_deg[3];
    float v0[3], v1[3], v2[3];
    int32_t sdf_type;        /* AR_OBJECT_SDF: AR_SDF_OBJECT_TORUS or AR_SDF_OBJECT_VOLUME */
    float sdf_params[4];     /* SDFInfo::sdfInfo0_ */
    int32_t sdf_volume;      /* SDFInfo::cachedVolumeIndex_ */
} ar_object;

/* Parameters of one render call (SceneRenderer::Render). */
typedef struct ar_render_params
{
    int32_t width, height;
    int32_t spp;             /* samples per pixel = frames */
    int32_t max_depth;       /* path vertices; the reference's MAX_TRACING_DEPTH */
    float cam_origin[3];
    float cam_dir[3];
    float fov_deg;           /* vertical field of view (the reference fixes 60) */
    int32_t use_nee;         /* next-event estimation with MIS (SceneSetting::bUseNEE_) */
    uint64_t seed;           /* global seed (GLOBAL_SEED = 0x9e3779b97f4a7c15) */
    int32_t first_frame;     /* frame index of the first sample */
    int32_t wave_paths;      /* paths in flight per wave, 0 = automatic (ar_render: up to 2^25,
                                about 8 GB of device state; ar_adjoint: up to 2^21) */
    int32_t profile;         /* 1 = per-stage device times, 2 = traversal counters, 3 = both */
    int32_t guide;           /* AR_GUIDE_NONE, AR_GUIDE_VOXEL (SceneSetting::bUsePathGuiding_) or AR_GUIDE_MLP */
    float guide_unit;        /* voxel size of the guide (0 = 0.05, PATH_GUIDING_RESOLUTION_UNIT) */
    int32_t guide_train_steps; /* AR_GUIDE_MLP: Adam steps after each frame (0 = 8) */
    int32_t denoise_record;  /* 1: record the denoiser's per-pixel G-buffer and sample moments (ar_denoise) */
    int32_t guide_frames;    /* guided rendering: frames between two guide updates (0 = 1, the reference's
                                update after every frame); the frames of one update window share waves */
} ar_render_params;

/* Path guiding modes.  With AR_GUIDE_VOXEL, ar_render renders one frame (one
 * sample per pixel) at a time and, after each frame, folds its radiance records
 * into the context's voxel probes (core/scene.cu:240-273, 409-570); the probes
 * persist across ar_render calls until ar_guide_reset or a scene rebuild.
 * With params->guide_frames = k > 1 the update comes after every k frames
 * instead, over all their records (the same count-weighted running mean the
 * per-frame updates build, so only the probes the k frames sample from are
 * older); the k frames then run together in waves of up to k x pixels paths. */
#define AR_GUIDE_NONE 0
#define AR_GUIDE_VOXEL 1
/* AR_GUIDE_MLP (no reference counterpart): the voxel probes learn as with
 * AR_GUIDE_VOXEL and, after every frame, a small network (12-band encoding of
 * position and reflected direction, 5 layers of width 64, BF16 tensor-core
 * kernels with FP32 accumulation) trains alongside: guide_train_steps Adam
 * steps at lr 1e-3, each on 16,384 of the frame's radiance records.  Once it
 * has taken 16 steps, vertices of the first three diffuse bounces sample the
 * network's 64-cell directional distribution; later bounces keep the probes. */
#define AR_GUIDE_MLP 2

/* Per-stage profile of the last ar_render with params->profile = 1. */
typedef struct ar_render_profile
{
    float raygen_ms, extend_ms, shade_ms, shadow_ms, finalize_ms;
    int64_t extend_rays, shadow_rays;
    int64_t extend_node_visits, extend_prim_tests;
    int64_t shadow_node_visits, shadow_prim_tests;
    int64_t extend_launches, shadow_launches, shade_launches;
} ar_render_profile;

ar_status ar_create(ar_ctx** out, int device);
ar_status ar_destroy(ar_ctx* ctx);

/* Scene description.  Replaces the previous description; takes effect at
 * ar_scene_build.  Primitive ids: objects first (0..n_objects-1), then mesh
 * triangles (n_objects + i). */
ar_status ar_scene_set_materials(ar_ctx* ctx, const ar_material* materials, int n);
ar_status ar_scene_set_objects(ar_ctx* ctx, const ar_object* objects, int n);
ar_status ar_scene_set_mesh(ar_ctx* ctx, const float* vertices, int n_vertices, const uint32_t* indices, int n_triangles,
                            const int32_t* material_ids);
/* Albedo textures (no counterpart in the reference; the differentiable
 * rendering workload's parameters).  texels: host, n_textures textures of
 * sizes[2k] x sizes[2k+1] (width x height) RGB float32 texels, row-major,
 * concatenated.  uv: host, 6 floats per mesh triangle (u, v at each vertex);
 * texture row 0 is v = 0.  Both take effect at ar_scene_build. */
ar_status ar_scene_set_textures(ar_ctx* ctx, const float* texels, const int32_t* sizes, int n_textures);
ar_status ar_scene_set_mesh_uv(ar_ctx* ctx, const float* uv, int n_triangles);
/* Replaces the texel values of a built scene without rebuilding it (same
 * count as given to ar_scene_set_textures).  texels is device memory when
 * is_device != 0, host memory otherwise; ordered on `stream`. */
ar_status ar_scene_update_texels(ar_ctx* ctx, const float* texels, int64_t n_floats, int is_device, void* stream);
/* Texel floats of the built scene (3 per texel, all textures). */
ar_status ar_scene_texel_count(ar_ctx* ctx, int64_t* n_floats);

/* Smooth-union SDF object (no reference counterpart; the reference's OBJ_SDF
 * marches one analytic shape per object, core/object/sdf/sdf_base.cuh:53-163):
 * the surface where the polynomial smooth minimum (width smooth_k) of the
 * primitives' signed distances is zero, in world space, one primitive of the
 * scene with id n_objects + n_mesh_triangles.  prims: n x 8 floats (kind,
 * centre xyz, size xyz, 0): sphere (size.x = radius), box (half extents),
 * torus about +y (size.x = major, size.y = minor radius).  n = 0 removes it.
 * Takes effect at ar_scene_build. */
#define AR_SDF_SPHERE 0
#define AR_SDF_BOX 1
#define AR_SDF_TORUS 2
ar_status ar_scene_set_sdf_union(ar_ctx* ctx, const float* prims, int n, float smooth_k, int32_t material);

/* SDF volume cache (SDFCacheManager, core/object/sdf/sdf_cache_manager.cuh;
 * SceneRenderer::AddVolumeToCacheManager, core/scene.hpp:120-127).  A volume
 * is a dims[0] x dims[1] x dims[2] grid of signed distances (x fastest) over
 * the unit cube, sampled nearest far from the surface and trilinearly near it
 * (SampleSDFAdaptive01, core/object/sdf/sdf_volume.cuh:138-149).
 * ar_sdf_volume_add fills it on the GPU from a built-in functor (FillSDFVolume:
 * voxel (x, y, z) holds f(x / (dx - 1) - 0.5, ...)): AR_SDF_FN_TORUS with
 * params (R, r), AR_SDF_FN_DIAMOND with params (d, bias, tableZ, scale), zeros
 * meaning the reference's defaults (sdf::CreateDiamond: 0.94, 0.5, 0.3, 0.5).
 * ar_sdf_volume_add_data takes caller values (host memory).  *index receives
 * the cache index for ar_object.sdf_volume.  Volumes persist across scene
 * builds until ar_sdf_volume_clear.  ar_sdf_volume_read copies a volume out
 * (voxels may be NULL to query dims). */
#define AR_SDF_FN_TORUS 0
#define AR_SDF_FN_DIAMOND 1
ar_status ar_sdf_volume_add(ar_ctx* ctx, int32_t fn, const float* params, const int32_t* dims, int32_t* index);
ar_status ar_sdf_volume_add_data(ar_ctx* ctx, const float* voxels, const int32_t* dims, int32_t* index);
ar_status ar_sdf_volume_read(ar_ctx* ctx, int32_t index, float* voxels, int32_t* dims);
ar_status ar_sdf_volume_clear(ar_ctx* ctx);

/* Homogeneous participating medium filling an axis-aligned box (no reference
 * counterpart): extinction sigma_t, single-scattering albedo, Henyey-Greenstein
 * g (core/render/sample.cuh:110-145), and an emission radiance released where
 * light is absorbed (white, scaled like emitters by D65).  Free flights are
 * sampled inside the box, NEE shadow rays carry the box chord's transmittance.
 * Takes effect immediately (no rebuild); NULL removes it. */
typedef struct ar_medium
{
    float box_lo[3], box_hi[3];
    float sigma_t, albedo, g, emission;
} ar_medium;
ar_status ar_scene_set_medium(ar_ctx* ctx, const ar_medium* medium);
/* Builds the BVH, the light table and the spectral LUTs; uploads the scene. */
ar_status ar_scene_build(ar_ctx* ctx);
/* Where ar_scene_build builds the main BVH (the reference builds on the host,
 * BuildBVH, core/bvh/bvh.cuh:142-422): AR_BUILD_HOST (default) is a binned-SAH
 * build on the host threads; AR_BUILD_GPU sorts the primitives' centroid
 * Morton codes, builds a binary radix tree (Karras 2012) and collapses it to
 * the same 8-wide node format on the GPU: much faster for large meshes, a
 * tree of lower SAH quality, identical hit results.  Takes effect at the next
 * ar_scene_build; ar_scene_build_time reports the last build's wall time. */
#define AR_BUILD_HOST 0
#define AR_BUILD_GPU 1
ar_status ar_scene_set_build_mode(ar_ctx* ctx, int32_t mode);
ar_status ar_scene_build_time(ar_ctx* ctx, double* ms);
/* Refit after the mesh's vertices moved (same triangles, same vertex count as
 * ar_scene_set_mesh; 3 floats per vertex, host or device memory): the BVH keeps
 * its tree, triangle slots take the new vertices and every node's quantized
 * child boxes are recomputed from the leaves up, on the GPU.  Hits are exact
 * for the moved mesh; traversal cost grows with how far the tree's original
 * grouping no longer fits (rebuild with ar_scene_build then). */
ar_status ar_scene_refit_mesh(ar_ctx* ctx, const float* vertices, int n_vertices, int is_device, void* stream);
/* BVH statistics: nodes, primitive slots, depth, bytes on the device. */
ar_status ar_scene_stats(ar_ctx* ctx, int64_t* n_nodes, int64_t* n_slots, int32_t* depth, int64_t* device_bytes);

/* Renders params->spp samples per pixel and writes the per-pixel mean linear
 * CIE XYZ (3 doubles per pixel, row-major, FP64 accumulation in sample order).
 * out_xyz is host memory when out_is_device == 0, device memory otherwise.
 * per_sample_xyz (optional, host, 3 floats per pixel per sample in sample-major
 * order) receives every sample's XYZ. */
ar_status ar_render(ar_ctx* ctx, const ar_render_params* params, double* out_xyz, int out_is_device,
                    float* per_sample_xyz, void* stream);

/* Progressive rendering, one frame per call: SceneRenderer::Render(hdrTarget,
 * ldrTarget, size, cameraOrigin, cameraDirection, frameIndex, toneType,
 * oddTarget, evenTarget, radianceSampleBuffer, screenGBuffer,
 * screenStatisticsBuffer) (core/scene.hpp:109-114, core/scene.cu:240-366).
 * Renders one sample per pixel with frame index frame_index (the same paths as
 * sample frame_index of ar_render; params->spp and first_frame are ignored)
 * and folds it into the caller's DEVICE buffers:
 *   hdr   3 floats per pixel, the float32 running mean of linear XYZ:
 *         hdr = hdr (1 - r) + sample r with r = 1 / (1 + frame_index)
 *         (RenderCamera, core/scene.cu:178-180), so frame 0 replaces any
 *         finite contents (NaN or inf stay, as in the reference);
 *   odd / even (both or neither) the same over odd / even frames at rate
 *         1 / (1 + frame_index / 2) (core/scene.cu:181-191);
 *   ldr   (optional) one uint32 per pixel, 0xAARRGGBB: XYZ -> linear sRGB,
 *         times the exposure (ar_set_exposure), then tone_type
 *         AR_FRAME_TONE_LINEAR / _GAMMA / _ACES (the reference's toneType
 *         0 / 1 / 2, core/scene.cu:113-131), clamped, x 255 truncated.
 * With params->guide the voxel / MLP guide learns from the frame, as the
 * reference updates its probes after every frame; its radiance records and
 * G-buffer live in the context (the reference's caller-owned
 * radianceSampleBuffer / screenGBuffer / screenStatisticsBuffer).  With
 * params->denoise_record the display image is made from the running mean
 * filtered by ar_denoise (SceneSetting::bDenoise_, core/scene.cu:324-348).
 * Returns after the frame is finished (the reference synchronises the device);
 * `stream` (optional) is synchronised first. */
#define AR_FRAME_TONE_LINEAR 0
#define AR_FRAME_TONE_GAMMA 1
#define AR_FRAME_TONE_ACES 2
ar_status ar_render_frame(ar_ctx* ctx, const ar_render_params* params, int32_t frame_index, int32_t tone_type,
                          float* hdr, uint32_t* ldr, float* odd, float* even, void* stream);
/* Display exposure of ar_render_frame's ldr image (SceneRenderer::SetExposure,
 * core/scene.hpp:97, core/scene.cu:752-755; default 1). */
ar_status ar_set_exposure(ar_ctx* ctx, float exposure);

/* Closest / any hit for n rays.  rays: device pointer, 8 floats per ray
 * (ox, oy, oz, tmin, dx, dy, dz, tmax), direction normalised by the caller.
 * prim_id: device int32[n] (-1 = miss).  t: device float[n] (closest only,
 * may be NULL). */
ar_status ar_trace_closest(ar_ctx* ctx, const float* rays, int n, int32_t* prim_id, float* t, void* stream);
ar_status ar_trace_any(ar_ctx* ctx, const float* rays, int n, int32_t* hit, void* stream);

/* Allocation-free rendering.  No counterpart in the reference: it exists for
 * callers that must not allocate device memory (a frame loop that cannot
 * afford the device-wide synchronisation of cudaFree, an application whose
 * memory pool owns every allocation).  Same result as ar_render, written as
 * per-pixel mean XYZ (3 doubles per pixel) into the caller's DEVICE buffer
 * out_xyz_device, which also serves as the FP64 accumulator.  The wavefront
 * working set comes from one fixed 8 MiB array in the library image
 * (AR_NOALLOC_SCRATCH_BYTES, held by every GPU that loads the library until
 * exit), so at most AR_NOALLOC_MAX_PATHS paths are in flight per wave;
 * params->wave_paths above that is rejected with AR_ERR_INVALID (0 = the
 * maximum).  The first call on a device looks the array up with
 * cudaGetSymbolAddress and must happen before any stream capture; the address
 * is kept for the rest of the process.  cudaDeviceReset ends every ar_ctx of
 * that device and unloads the array with the library's module, so after a
 * reset this entry point must not be called again in that process.  Calls share
 * the array: calls that overlap on the GPU race, so serialise them.  When
 * `stream` is not the context's own stream, the call first makes it wait for
 * the work the context has queued (e.g. ar_scene_update_texels with a NULL
 * stream).  No cudaMalloc / cudaFree is made; profiling (params->profile) is
 * rejected. */
#define AR_NOALLOC_SCRATCH_BYTES (8u << 20)
#define AR_NOALLOC_MAX_PATHS 40704
ar_status ar_render_noalloc(ar_ctx* ctx, const ar_render_params* params, double* out_xyz_device, void* stream);

/* Replay adjoint (no counterpart in the reference).  Gradient of a scalar loss
 * with respect to every albedo texel, given dl_dxyz = d(loss)/d(image), where
 * image is what ar_render returns for the same params (per-pixel mean XYZ):
 * device float32, 3 per pixel.  grad_texels: device float64, one per texel
 * float (ar_scene_texel_count), overwritten.  The paths of the render are
 * replayed from their random streams (nothing is stored per vertex): each wave
 * is traced once for its radiance and once more to scatter
 * d(loss)/d(radiance) x (radiance still to come) x d(albedo)/d(texel) / albedo
 * at every textured diffuse vertex.  Russian-roulette and NEE decisions are
 * held fixed (their probabilities are not differentiated).  Gradients gather
 * in float32 per wave and fold into grad_texels in float64.  Guided rendering
 * is rejected. */
ar_status ar_adjoint(ar_ctx* ctx, const ar_render_params* params, const float* dl_dxyz, double* grad_texels,
                     void* stream);

/* Replay adjoint of the medium's scalar parameters (no reference counterpart):
 * grad2 (host) = d(loss)/d(albedo), d(loss)/d(emission), from dl_dxyz as for
 * ar_adjoint.  Every scattering event multiplies what follows by the albedo
 * and releases (1 - albedo) x emission; roulette and NEE decisions are held
 * fixed. */
ar_status ar_adjoint_medium(ar_ctx* ctx, const ar_render_params* params, const float* dl_dxyz, double* grad2,
                            void* stream);

/* Display transform (Camera::RenderToFile, core/camera.cu:64-89, and
 * core/tonemap.cuh): per-pixel XYZ x exposure -> linear sRGB (D65) -> tone
 * curve -> clamp -> 8-bit RGBA (alpha 255), on the GPU.  xyz: 3 doubles per
 * pixel (what ar_render writes), host or device memory; rgba: host, 4 bytes
 * per pixel, top row first. */
#define AR_TONE_ACES 0      /* the reference's ACES fit (its default) */
#define AR_TONE_GAMMA 1     /* gamma 1/2.2 */
#define AR_TONE_LINEAR 2    /* linear sRGB */
ar_status ar_tonemap(ar_ctx* ctx, const double* xyz, int xyz_is_device, int width, int height, float exposure, int tone,
                     uint8_t* rgba);

/* Denoiser (SceneRenderer::Render with SceneSetting::bDenoise_,
 * core/scene.cu:324-348; core/denoise/denoise.cuh).  An ar_render with
 * params->denoise_record = 1 records, for every sample in sample order, the
 * camera ray's first hit into per-pixel running means (albedo, normal,
 * metallic, roughness as halves; hit distance; shading-model histogram) and
 * the moments of BoxCox(sample XYZ); the records start over when
 * params->first_frame is 0 or the image size changes, and accumulate across
 * calls otherwise.  ar_denoise then filters an image of that size (3 doubles
 * per pixel, as ar_render writes it, read as float) with the reference's
 * bilateral filter: radius 7, weights from the G-buffer differences, a
 * Gaussian in pixel distance, and a per-pair Welch t-test (0.5 % two-sided) on
 * the sample moments; filtering happens on log(1 + XYZ).  Output: 3 doubles
 * per pixel.  Host or device buffers; ordered on `stream`. */
ar_status ar_denoise(ar_ctx* ctx, const double* xyz_in, int in_is_device, double* xyz_out, int out_is_device,
                     void* stream);
/* The recorded buffers (host copies): 40 bytes per pixel each.
 * gbuffer: uint16 halves[14] (albedo xyz, normal xyz, metallic, roughness,
 * shading-model histogram [diffuse, light, glass, GGX, no hit], pad), float
 * distance, uint32 samples that hit, uint32 samples.  moments: uint32 count,
 * float mean[3], M2/n[3], M3/n[3] of BoxCox(XYZ) = 2 (sqrt(XYZ) - 1).
 * width / height (optional) receive the image size (0 when nothing is
 * recorded); pass NULL buffers to query it. */
ar_status ar_denoise_read(ar_ctx* ctx, int32_t* width, int32_t* height, void* gbuffer, void* moments);
/* Replaces the recorded buffers (same layout), e.g. to filter with records
 * made elsewhere. */
ar_status ar_denoise_write(ar_ctx* ctx, int32_t width, int32_t height, const void* gbuffer, const void* moments);

/* Device time (ms) of the last ar_render and the number of kernels it launched. */
ar_status ar_last_render_stats(ar_ctx* ctx, float* device_ms, int64_t* kernel_launches);
/* Stage times and traversal counters of the last profiled ar_render. */
ar_status ar_last_render_profile(ar_ctx* ctx, ar_render_profile* out);

/* Forgets the learned voxel probes (SceneRenderer::MarkNeedResetGuiding,
 * core/scene.hpp:102-105).  n_probes (optional) receives the probe count first. */
ar_status ar_guide_reset(ar_ctx* ctx, int32_t* n_probes);
/* Number of probes the voxel guide holds. */
ar_status ar_guide_stats(ar_ctx* ctx, int32_t* n_probes, int32_t* capacity);
/* MLP guide: training steps taken and the loss sum of the last one. */
ar_status ar_guide_mlp_stats(ar_ctx* ctx, int32_t* steps, float* last_loss);

/* The voxel guide's probe set (the reference keeps it in the SCENE_PROBES /
 * INDIRECT_INDEX_VOLUME device symbols, core/render/render.cuh:43-50, that
 * SceneRenderer::UpdatePathGuidingSample fills, core/scene.cu:409-570).
 * Probes are ordered by probe index.  keys: 4 int32 per probe, the
 * (voxel x, y, z, face) that pg::GetVoxelGrid returns
 * (core/guiding/guiding_bin.cuh:109-114); texels: AR_GUIDE_PROBE_FLOATS floats
 * per probe, Texture<4>::data_ (86 float4: 8x8 leaf, 4x4, 2x2, 1x1 mips, pad,
 * core/guiding/octahedron.cuh:203-240); counts: Texture<4>::count_.
 * ar_guide_read: *n receives the probe count; NULL buffers query it only.
 * ar_guide_write: replaces the probe set and the voxel unit (0 = 0.05); a
 * guided ar_render with the same guide_unit then samples these probes and
 * keeps learning into them. */
#define AR_GUIDE_PROBE_FLOATS 344
ar_status ar_guide_read(ar_ctx* ctx, int32_t* n, int32_t capacity, int32_t* keys, float* texels, uint64_t* counts);
ar_status ar_guide_write(ar_ctx* ctx, int32_t n, const int32_t* keys, const float* texels, const uint64_t* counts,
                         float unit);
/* Radiance records of the last guided frame (pg::PathGuidingSample,
 * core/guiding/guiding.cuh:22-32, as CalculateRadiance writes them,
 * core/render/render.cuh:909-963), in the order the kernels emitted them:
 * key (4 int32, as above), direction (3 floats), XYZ radiance (3 floats). */
ar_status ar_guide_read_records(ar_ctx* ctx, int32_t* n, int32_t capacity, int32_t* keys, float* dirs,
                                float* radiance);

ar_status ar_get_error_word(ar_ctx* ctx, uint32_t* word);
ar_status ar_clear_error_word(ar_ctx* ctx);
const char* ar_last_error(ar_ctx* ctx);

/* Host-side helpers (no GPU needed): the spectral encoders and the BVH builder
 * as the kernels use them, for checks against the reference. */
ar_status ar_host_rgb_encode(const float* rgb, int n, float* basis_out);
ar_status ar_host_lambda_encode(const float* lambda_nm, int n, float* basis_out);
ar_status ar_host_sample_lambda(const float* u3, int n, float* lambda_out, float* pdf_out);
/* Builds the wide BVH over n triangles (9 floats each) on the host and runs the
 * kernels' closest-hit traversal on the CPU; same outputs as ar_trace_closest. */
ar_status ar_host_trace_closest(const float* tris, int ntri, const float* rays, int nray, int32_t* prim_id, float* t,
                                int64_t* node_visits);
/* Voxel-guide probe math on the host (mips, voxel keys, equal-area map, pdf,
 * sampling) for one probe: the functions the guided kernels run. */
ar_status ar_host_guide_eval(const float* in, int n, float* out);
int ar_abi_version(void);

/* Diagnostic (no reference counterpart): one 128 x n x k BF16 tensor-core
 * product through the shared-memory descriptors the MLP guide uses, D = A B^T
 * with FP32 accumulation.  a: 128 x k row-major (a_mn = 0) or k x 128
 * (a_mn = 1); b: n x k (b_mn = 0) or k x n (b_mn = 1); bf16 bit patterns, host
 * memory; d: 128 x n floats, host.  swap exchanges the descriptors' two stride
 * fields (for checking the layout convention).  n, k in {64, 128, 144}. */
/* Diagnostic (no reference counterpart): the MLP guide's tensor-core forward
 * and backward passes on given inputs.  params: AR_MLP_PARAMS floats (per
 * layer W[64][in] row-major then b[64]; in = 144 for layer 0, 64 after).
 * in6: n x 6 encoded inputs in [0, 1] (position in the scene box, then
 * (reflected direction + 1) / 2); dirs: n x 3 record directions; nrm: n x 3
 * surface normals (may be NULL; the loss does not use them); lum: n record
 * radiances (CIE Y).  Outputs (host): logits n x 64, grad AR_MLP_PARAMS
 * (d mean loss / d params), loss (sum over records of Y (logsumexp(y) -
 * y_cell): the radiance-weighted cross-entropy of the record direction's cell
 * under the softmax of the 64 outputs). */
#define AR_MLP_PARAMS 25920
ar_status ar_diag_mlp(int device, const float* params, const float* in6, const float* dirs, const float* nrm,
                      const float* lum, int n, float* logits, float* grad, float* loss);
ar_status ar_diag_umma_gemm(int device, const uint16_t* a, const uint16_t* b, int a_mn, int b_mn, int n, int k,
                            int swap, float* d);

#ifdef __cplusplus
}
#endif
#endif /* APERTURE_AR_H */
