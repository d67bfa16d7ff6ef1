// Internal state shared by the C-ABI layer (capi.cu) and the kernel
// translation units.  Not part of the public interface.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "ar_bvh_build.h"
#include "ar_guide.h"
#include "ar_mlp.h"
#include "ar_denoise.h"
#include "ar_shade.h"
#include "ar_traverse.cuh"

namespace ar
{
#define AR_WAVE_PATHS_AUTO (1 << 25)      // ar_render's automatic wave size
#define AR_BOUNCE_LOOKAHEAD 4             // depths the host queues ahead of the queue lengths it has read
#define AR_WAVE_PATHS_ADJOINT (1 << 21)   // ar_adjoint's

// Order of a frame's pixels among the paths of a wave: bands of 4 rows, each
// cut into chunks 8 pixels wide taken left to right, row by row inside a
// chunk.  When the width is a multiple of 8, 32 consecutive paths (one warp)
// cover an 8 x 4 tile of the image, whose camera rays stay closer together
// through the BVH than a 32 x 1 strip's.  A bijection of [0, W*H); each path's
// random stream is keyed by its pixel and frame, so results do not depend on
// this order.
#define AR_TILE_W 8u
#define AR_TILE_H 4u
AR_HD uint32_t slot_pixel(uint32_t u, uint32_t W, uint32_t H)
{
    const uint32_t band_px = AR_TILE_H * W;
    const uint32_t b = u / band_px;
    uint32_t rem = u - b * band_px;
    const uint32_t hb = (H - AR_TILE_H * b) < AR_TILE_H ? (H - AR_TILE_H * b) : AR_TILE_H;
    const uint32_t chunk_px = AR_TILE_W * hb;
    const uint32_t c = rem / chunk_px;
    rem -= c * chunk_px;
    const uint32_t wc = (W - AR_TILE_W * c) < AR_TILE_W ? (W - AR_TILE_W * c) : AR_TILE_W;
    const uint32_t r = rem / wc;
    const uint32_t x = rem - r * wc;
    return (AR_TILE_H * b + r) * W + AR_TILE_W * c + x;
}

// Order of a render's paths.  Path g of an spp-sample render over npix pixel
// slots (slot_pixel order) is sample s of slot u.  Samples come in blocks of
// `block` consecutive samples; inside a block, groups of AR_PATH_GROUP_PX
// consecutive slots take all of the block's samples of those slots (slot
// fastest).  With blocks of AR_SAMPLE_BLOCK samples a warp's 32 paths are 32
// samples of one pixel, whose camera rays nearly coincide and whose first
// hits lie close together (measured on the 64-sample terrain step: 85.3 ms
// against 86.4 for 16 samples of 2 pixels, 87.8 for 8 of 4, 89.8 for 4 of 8
// and 93.1 for one sample of an 8x4 tile); block 1 is frame-major order.  A
// path's (pixel, sample) picks its random stream and its place in the
// per-pixel sums (added in sample order), so the order changes no result.
#define AR_PATH_GROUP_PX 1u
#define AR_SAMPLE_BLOCK 32
struct PathOrder
{
    uint32_t npix, spp, block;
};

AR_HD uint32_t path_block_samples(const PathOrder& o, uint32_t fb)
{
    const uint32_t left = o.spp - fb * o.block;
    return o.block < left ? o.block : left;
}

// (slot, sample) of path g, 0 <= g < npix * spp
AR_HD void path_slot(const PathOrder& o, unsigned long long g, uint32_t* u, uint32_t* s)
{
    const unsigned long long per_block = (unsigned long long)o.npix * o.block;
    if (((g | per_block) >> 32) == 0)
    {
        // the same arithmetic in 32 bits (renders below 2^32 paths): integer
        // division of 64-bit values is a long software sequence on the GPU
        const uint32_t pb = (uint32_t)per_block, g32 = (uint32_t)g;
        const uint32_t fb = g32 / pb;
        const uint32_t r = g32 - fb * pb;
        const uint32_t sb = path_block_samples(o, fb);
        const uint32_t group = AR_PATH_GROUP_PX * sb;
        const uint32_t ub = r / group;
        const uint32_t w = r - ub * group;
        const uint32_t left = o.npix - ub * AR_PATH_GROUP_PX;
        const uint32_t q = left < AR_PATH_GROUP_PX ? left : AR_PATH_GROUP_PX;
        *u = ub * AR_PATH_GROUP_PX + w % q;
        *s = fb * o.block + w / q;
        return;
    }
    const uint32_t fb = (uint32_t)(g / per_block);
    const unsigned long long r = g - (unsigned long long)fb * per_block;
    const uint32_t sb = path_block_samples(o, fb);
    const unsigned long long group = (unsigned long long)AR_PATH_GROUP_PX * sb;
    const uint32_t ub = (uint32_t)(r / group);
    const uint32_t w = (uint32_t)(r - (unsigned long long)ub * group);
    const uint32_t left = o.npix - ub * AR_PATH_GROUP_PX;
    const uint32_t q = left < AR_PATH_GROUP_PX ? left : AR_PATH_GROUP_PX;  // the last group may be short
    *u = ub * AR_PATH_GROUP_PX + w % q;
    *s = fb * o.block + w / q;
}

// path index of (slot u, sample s): the inverse of path_slot, rising with s
AR_HD unsigned long long path_index(const PathOrder& o, uint32_t u, uint32_t s)
{
    const uint32_t fb = s / o.block;
    const uint32_t sb = path_block_samples(o, fb);
    const uint32_t ub = u / AR_PATH_GROUP_PX;
    const uint32_t left = o.npix - ub * AR_PATH_GROUP_PX;
    const uint32_t q = left < AR_PATH_GROUP_PX ? left : AR_PATH_GROUP_PX;
    return (unsigned long long)fb * o.npix * o.block + (unsigned long long)ub * AR_PATH_GROUP_PX * sb +
           (unsigned long long)(s - fb * o.block) * q + (u - ub * AR_PATH_GROUP_PX);
}

// first sample of slot u whose path index is at least g0 (spp if none)
AR_HD uint32_t path_first_sample(const PathOrder& o, uint32_t u, unsigned long long g0)
{
    uint32_t lo = 0, hi = o.spp;
    while (lo < hi)
    {
        const uint32_t mid = lo + (hi - lo) / 2;
        if (path_index(o, u, mid) < g0) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// Voxel guide as the kernels see it: a sparse open-addressing hash from the
// packed (voxel, face) key to a probe index, and the probe pool.  The
// reference keeps the same sparse key set as a sorted unique array
// (core/guiding/guiding.cuh:84-160); a hash gives O(1) lookups and inserts
// without a sort, and any scene extent works.
constexpr unsigned long long AR_PG_KEY_EMPTY = ~0ull;
constexpr int AR_PG_HASH_PROBES = 64;  // linear-probe limit; a key that finds no slot stays unguided
constexpr int AR_PG_KEY_BITS = 19;     // per axis, signed: +-262144 voxels

struct DevGuide
{
    const unsigned long long* keys;
    const int* vals;     // probe index; -3 = key known but the pool was full
    const Probe* probes;
    int probe_count;     // > 0 once any probe exists
    unsigned mask;       // hash slots - 1 (power of two)
    float inv_unit;
};

// packed key: face (5 bits) | z | y | x (19 bits each, biased); EMPTY if out of range
AR_HD unsigned long long guide_pack(VoxelKey k)
{
    const int lim = 1 << (AR_PG_KEY_BITS - 1);
    if (k.f < 0 || k.f >= AR_PG_FACES) return AR_PG_KEY_EMPTY;
    if (k.x < -lim || k.x >= lim || k.y < -lim || k.y >= lim || k.z < -lim || k.z >= lim) return AR_PG_KEY_EMPTY;
    const unsigned long long m = (1ull << AR_PG_KEY_BITS) - 1ull;
    return ((unsigned long long)k.f << (3 * AR_PG_KEY_BITS)) |
           ((unsigned long long)(unsigned)(k.z + lim) & m) << (2 * AR_PG_KEY_BITS) |
           ((unsigned long long)(unsigned)(k.y + lim) & m) << AR_PG_KEY_BITS |
           ((unsigned long long)(unsigned)(k.x + lim) & m);
}

AR_HD unsigned guide_hash(unsigned long long key)
{
    key ^= key >> 33;
    key *= 0xff51afd7ed558ccdull;
    key ^= key >> 33;
    key *= 0xc4ceb9fe1a85ec53ull;
    key ^= key >> 33;
    return (unsigned)key;
}

// probe index for a packed key, -1 when it has none
AR_HD int guide_lookup(const DevGuide& g, unsigned long long key)
{
    if (key == AR_PG_KEY_EMPTY || g.keys == nullptr) return -1;
    unsigned s = guide_hash(key) & g.mask;
    for (int i = 0; i < AR_PG_HASH_PROBES; ++i)
    {
        const unsigned long long k = AR_LDG(&g.keys[s]);
        if (k == key) return AR_LDG(&g.vals[s]);
        if (k == AR_PG_KEY_EMPTY) return -1;
        s = (s + 1u) & g.mask;
    }
    return -1;
}

// Radiance records emitted at path end (core/guiding/guiding.cuh:22-32)
struct GuideSamples
{
    float4* radiance;         // xyz
    float4* dir;              // xyz
    unsigned long long* key;  // packed voxel key, EMPTY = out of range
    int* count;
    int capacity;
    float4* pos;              // MLP guide only: vertex position
    float4* wr;               // MLP guide only: reflected view direction
};
// Device-side scene as the kernels see it (passed by value).
struct DevScene
{
    TravScene trav;
    TravScene sdf_trav;        // the SDF objects' own BVH (node_count 0: none)
    const Material* materials;
    const int* prim_material;  // per primitive id
    const int* prim_light;     // per primitive id, -1 when not a light
    const int* prim_slot;      // per primitive id: its slot in the BVH leaf array (SDF objects: in sdf_trav)
    const Light* lights;
    int light_count;
    const float* lut_rgb;      // RES^3 x 4
    const float* lut_lambda;   // 840 x 4
    const float* cie_cmf;      // 421 x 3
    const float* d65;          // 421
    int camera_inside;         // camera origin overlaps an object
    // profiling counters (null unless profiling): extend visits, extend tests,
    // shadow visits, shadow tests, extend rays, shadow rays
    unsigned long long* stats;
    DevGuide guide;
    // albedo textures: RGB float32 texels, per texture {texel offset, width,
    // height, 0}, per primitive id 6 uv floats (null when no texture is set)
    const float* texels;
    const int4* tex_info;
    const float* prim_uv;
    int tex_count;
    BoxMedium medium;  // participating medium (on = 0: none)
};

// stage ids for the per-stage profile
enum Stage
{
    ST_RAYGEN = 0,
    ST_EXTEND = 1,
    ST_SHADE = 2,
    ST_SHADOW = 3,
    ST_FINAL = 4,
    ST_COUNT = 5
};

struct StageEvent
{
    int stage;
    cudaEvent_t a, b;
};

// Per-path state of the wavefront integrator (structure of arrays).
// ints in a render wave's counter array (layout: AR_CNT_* in render.cu)
#define AR_CNT_COUNT 10

struct PathState
{
    uint64_t* rng;
    uint32_t* pixel;
    uint32_t* frame;
    float4* ray_o;      // xyz origin, w = lambda
    float4* ray_d;      // xyz direction, w = lambda pdf
    float* radiance;
    float* mask;
    uint32_t* depths;   // depth | nonDeltaDepth << 16
    uint32_t* flags;    // bit0 inside media, bit1 previous NEE valid
    float4* media_v;    // xyz media vertex, w = bits(media object index)
    int* media_depth;
    float4* prev;       // xyz last vertex, w = last BSDF pdf
    float* hit_t;
    int* hit_slot;
    int* q_slot;        // hit_slot again, indexed by the path's entry in the extended queue:
                        // k_shade reads it beside the queue entry instead of after it
    float4* hit_nrm;    // normal of SDF hits (computed by k_extend), xyz
    float* out_xyz;     // 3 per path
    int capacity;
    // guided rendering only: RGB probe query and the per-vertex radiance
    // collection (AR_PG_COLLECT_DEPTH slots of capacity entries each)
    float4* maskq;      // xyz query
    float4* pg_dir;     // xyz sampled direction, w = collected radiance
    float4* pg_loc;     // xyz vertex position, w = radiance mask
    float4* pg_vdir;    // xyz reflected direction (voxel face key)
    // replay adjoint only: the path's total radiance (first pass) and
    // d(loss)/d(radiance)
    float* adj_total;
    float* adj_delta;
    // MLP guide only: network inputs of the path's current hit and the 64
    // quantised cell weights inferred for it
    float4* q_pos;      // xyz hit position, w = 1 when the query is valid
    float4* q_wr;       // xyz reflected view direction
    uint8_t* q_dist;    // 64 per path
};

struct ShadowQueue
{
    int* path;
    float4* o;      // xyz origin, w = tmax
    float4* d;      // xyz direction, w = contribution if unoccluded
    float* v_occ;   // contribution if occluded
    uint8_t* valid_unocc;
    float* sdf_eps; // SDF objects' march tolerance at the shading vertex's depth
};

struct RenderLaunch
{
    int width, height, spp, max_depth;
    float cam_o[3], cam_d[3];
    float fov_deg;
    int use_nee;
    uint64_t seed;
    int first_frame;
    int profile;
    int guide;    // 0 none, 1 voxel probes, 2 MLP (voxel probes until the network has trained)
    int adjoint;  // 1: replay pass of ar_adjoint (gradient scatter, no output)
    float* grad;  // replay pass: float32 texel gradients
    int mlp_ready;  // guide 2: sample from the network instead of the voxel probes
    double* grad_medium;  // replay pass of ar_adjoint_medium: d loss / d (albedo, emission)
    int denoise;  // record the denoiser's G-buffer and sample moments
    int sample_block = 1;  // path order: samples per block (PathOrder)
    const ulonglong2* jumps = nullptr;  // per sample s: ar_pcg_jump((first_frame + s) << 32), or null
};

inline PathOrder path_order(const RenderLaunch& rl)
{
    return PathOrder{(uint32_t)((long long)rl.width * rl.height), (uint32_t)rl.spp, (uint32_t)rl.sample_block};
}

struct Ctx
{
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t order_event = nullptr;  // orders a caller's stream after the context's (ar_render_noalloc)
    // per depth of a wave: the next queue's length, copied to pinned host memory,
    // and the event after the copy (a ring of AR_BOUNCE_LOOKAHEAD + 1)
    cudaEvent_t bounce_ev[AR_BOUNCE_LOOKAHEAD + 1] = {};
    int* h_bounce_cnt = nullptr;
    float exposure = 1.0f;               // display exposure of ar_render_frame (ar_set_exposure)
    double* d_frame_xyz = nullptr;       // ar_render_frame: the frame's sample per pixel
    double* d_frame_dn = nullptr;        // ar_render_frame: denoiser input and output
    long long frame_cap = 0;             // pixels of the two buffers above
    std::string last_error;
    // host scene description
    std::vector<Material> materials;
    std::vector<Object> objects;         // one per scene object (any type)
    std::vector<int> object_material;
    std::vector<int> object_type;
    std::vector<float> object_tri;       // 9 per object (triangles)
    std::vector<float4> object_sdf;      // SDF objects: field parameters (one per object)
    // SDF volume cache (persists across scene builds, like the reference's SDFCacheManager)
    std::vector<std::vector<float>> vol_host;   // host copies (overlap tests, reads)
    std::vector<int> vol_dims;                  // 3 per volume
    std::vector<float*> vol_dev;                // device grids
    SdfVolume* d_vols = nullptr;                // device table
    float4* d_sdf_params = nullptr;
    int sdf_object_count = 0;                   // SDF objects in the scene
    int build_mode = 0;                         // AR_BUILD_HOST / AR_BUILD_GPU
    // refit: wide nodes grouped by depth, mesh indices, per-primitive bounds of the rest
    std::vector<int> refit_level_off;           // depth d: nodes [off[d], off[d+1]) of d_refit_nodes
    int* d_refit_nodes = nullptr;
    uint32_t* d_mesh_idx = nullptr;
    float* d_prim_box = nullptr;                // 6 per primitive id (objects; triangles recomputed)
    float* d_node_box = nullptr;                // 6 per wide node (refit scratch)
    float* d_refit_verts = nullptr;             // the latest refit's vertices (3 per mesh vertex)
    bool mesh_v_stale = false;                  // mesh_v lags d_refit_verts until a build needs it
    double last_build_ms = 0.0;                 // wall time of the last BVH build
    int* d_pend_list = nullptr;                 // shadow rays left for the SDF pass
    // the SDF objects' BVH
    arbvh::WideBVH sdf_bvh;
    void* d_sdf_nodes = nullptr;
    void* d_sdf_bvh_slots = nullptr;
    std::vector<float> mesh_v;           // 9 per mesh triangle
    std::vector<uint32_t> mesh_idx;      // 3 vertex indices per mesh triangle (for refits)
    int mesh_nv = 0;                     // vertices of the mesh
    std::vector<int> mesh_material;
    // built scene
    arbvh::WideBVH bvh;
    std::vector<Light> lights;
    bool built = false;
    int camera_inside = 0;
    // device buffers
    void* d_nodes = nullptr;
    void* d_slots = nullptr;
    Object* d_objects = nullptr;
    Material* d_materials = nullptr;
    int* d_prim_material = nullptr;
    int* d_prim_light = nullptr;
    int* d_prim_slot = nullptr;
    Light* d_lights = nullptr;
    float* d_lut_rgb = nullptr;
    float* d_lut_lambda = nullptr;
    float* d_cie = nullptr;
    float* d_d65 = nullptr;
    unsigned int* d_err = nullptr;
    int* d_counters = nullptr;
    // albedo textures
    std::vector<float> tex_texels;
    std::vector<int> tex_sizes;          // width, height per texture
    std::vector<float> mesh_uv;          // 6 per mesh triangle
    float* d_texels = nullptr;
    int4* d_tex_info = nullptr;
    float* d_prim_uv = nullptr;
    long long texel_floats = 0;          // of the built scene
    int tex_count = 0;
    // replay adjoint
    float* d_grad32 = nullptr;
    long long grad32_n = 0;
    float* d_adj = nullptr;              // 2 floats per wave path
    int adj_capacity = 0;
    double* d_grad_medium = nullptr;     // d loss / d (medium albedo, medium emission)
    // smooth-union SDF object and the participating medium
    std::vector<float> sdf_prims;        // 8 floats per primitive
    float sdf_k = 0.0f;
    int sdf_material = -1;
    float4* d_sdf = nullptr;
    SdfUnion sdf{};
    int sdf_id = -1;                     // primitive id of the SDF object
    BoxMedium medium{};
    // wavefront buffers
    PathState ps{};
    ShadowQueue sq{};
    int* d_queue[2] = {nullptr, nullptr};
    int2* d_pq = nullptr;  // the extended queue ordered for shading (k_partition)
    double* d_accum = nullptr;
    size_t accum_pixels = 0;
    int wave_capacity = 0;
    // timing of the last render (device ms) and launch count
    float last_render_ms = 0.0f;
    long long last_launches = 0;
    // profiling
    int profile = 0;  // bit0: stage events, bit1: traversal counters
    unsigned long long* d_stats = nullptr;  // 8 counters
    std::vector<StageEvent> stage_events;
    float stage_ms[ST_COUNT] = {0, 0, 0, 0, 0};
    long long stage_launches[ST_COUNT] = {0, 0, 0, 0, 0};
    unsigned long long stats[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    // voxel guide
    DevGuide guide{};
    unsigned long long* d_pg_keys = nullptr;  // hash slots: packed voxel key
    int* d_pg_vals = nullptr;                 // hash slots: probe index
    Probe* d_pg_probes = nullptr;
    Probe* d_pg_temp = nullptr;
    int* d_pg_meta = nullptr;     // [0] probe count, [1] sample count
    int pg_capacity = 0;
    int pg_hash_slots = 0;
    float pg_unit = 0.0f;
    GuideSamples gs{};
    int gs_capacity = 0;
    int pg_path_cap = 0;  // wavefront capacity the collection slots were sized for
    // MLP guide
    float* d_mlp_w32 = nullptr;   // master parameters
    uint16_t* d_mlp_wbf = nullptr;
    float* d_mlp_grad = nullptr;
    float* d_mlp_gpart = nullptr;
    ulonglong2* d_jumps = nullptr;  // per-sample stream jumps of the current render
    int jump_cap = 0;  // per-CTA gradient slices of a training step (SMs x AR_MLP_PARAMS)
    float* d_mlp_m = nullptr;
    float* d_mlp_v = nullptr;
    float* d_mlp_loss = nullptr;  // loss sum of the last training step
    int mlp_step = 0;
    int mlp_steps_per_frame = 8;
    int mlp_path_cap = 0;
    int* d_mlp_list = nullptr;    // compacted queue of the paths the network is queried for
    MlpBox mlp_box{};
    // denoiser records (denoise.cu)
    DnGBuf* d_dn_gb = nullptr;    // per pixel
    DnStat* d_dn_st = nullptr;    // per pixel
    float4* d_dn_rec = nullptr;   // per path in flight: first-hit record (2 float4)
    int dn_w = 0, dn_h = 0;       // image the records belong to (0: none)
    int dn_rec_cap = 0;
    float* d_dn_img = nullptr;    // filter input / output staging (float XYZ)
    double* d_dn_io = nullptr;    // host-image staging (double XYZ)
    long long dn_img_cap = 0;
};

// MLP guide (mlp.cu)
struct MlpDev
{
    const uint16_t* wbf;
    const float* w32;
    MlpBox box;
};
cudaError_t mlp_prepare_kernels();
cudaError_t launch_mlp_infer(const MlpDev& net, const float4* q_pos, const float4* q_wr, const int* queue,
                             const int* count, int n_direct, uint8_t* out, float* logits, unsigned* err, int sms,
                             cudaStream_t s);
// grad += the step's gradient; part: scratch of min(sms, tiles) x AR_MLP_PARAMS floats (one slice per CTA)
cudaError_t launch_mlp_train(const MlpDev& net, const float4* r_pos, const float4* r_wr, const float4* r_dir,
                             const float4* r_rad, const int* count, int n_direct, int n_train, int offset, float* grad,
                             float* part, float* loss_sum, unsigned* err, int sms, cudaStream_t s);
cudaError_t launch_mlp_bias_start(float* w32, const float4* r_rad, const int* count, cudaStream_t s);
cudaError_t launch_mlp_adam(float* w32, uint16_t* wbf, float* grad, float* m, float* v, int step, float lr,
                            cudaStream_t s);
cudaError_t launch_mlp_to_bf16(const float* w32, uint16_t* wbf, cudaStream_t s);
// frames of training before the guide switches from the voxel probes to the network
constexpr int AR_MLP_WARMUP_STEPS = 16;        // Adam steps (2 frames)
constexpr int AR_MLP_STEPS_PER_FRAME = 8;       // Adam steps after every frame, each on its own record subset
constexpr int AR_MLP_TRAIN_RECORDS = 1 << 14;  // records per step (spread over the frame's records)
constexpr int AR_MLP_MAX_NDD = 3;               // the network guides the first non-delta vertices, the probes the rest
constexpr float AR_MLP_LR = 1.0e-3f;

// voxel guide (guide.cu)
cudaError_t launch_guide_update(Ctx& c, long long* launches);
int guide_probe_count(Ctx& c);

DevScene dev_scene(const Ctx& c);
// 1 when a camera at cam_o starts inside a box, sphere or SDF object (host test;
// SDF objects read the host copy of the volume cache)
int camera_inside_any(const Ctx& c, const float cam_o[3]);

// Wavefront working set supplied by the caller (allocation-free rendering).
struct WaveBuffers
{
    PathState ps;
    ShadowQueue sq;
    int* queue[2];
    int2* pq;
    int* counters;   // AR_CNT_COUNT ints
    double* accum;   // 3 doubles per pixel
    int* pend_list;  // shadow rays left for the SDF pass
    cudaStream_t stream;
};
cudaError_t launch_render_wave_buffers(const DevScene& sc, const WaveBuffers& wb, int device, const RenderLaunch& rl,
                                       int camera_inside, long long first_path, int n, unsigned int* err);

// kernel launchers (render.cu / trace.cu)
cudaError_t launch_build_rgb_lut(float* lut, const float* weights_dev, cudaStream_t s);
cudaError_t launch_prepare_materials(Material* mats, int n, const float* lut, cudaStream_t s);
cudaError_t launch_trace(const DevScene& sc, const float* rays, int n, int any, int* prim_id, float* t,
                         unsigned int* err, cudaStream_t s, long long* launches);
cudaError_t launch_render_wave(Ctx& c, const RenderLaunch& rl, long long first_path, int n_paths,
                               float* per_sample_out, long long* launches);
cudaError_t launch_accumulate(Ctx& c, const RenderLaunch& rl, long long first_path, int n_paths, double* accum,
                              long long* launches);
// replay adjoint (adjoint.cu): per-path seed between the two passes, and the
// float32 -> float64 gradient fold after each wave
cudaError_t launch_adjoint_seed(Ctx& c, const RenderLaunch& rl, int n_paths, const float* dl_dxyz,
                                long long* launches);
cudaError_t launch_grad_fold(Ctx& c, double* grad64, long long n, long long* launches);
// denoiser (denoise.cu): fold one wave's first-hit records and sample XYZ into
// the per-pixel records, in sample order
cudaError_t launch_denoise_record(Ctx& c, const RenderLaunch& rl, long long first_path, int n_paths, long long* launches);
cudaError_t ensure_denoise(Ctx& c, int width, int height, int first_frame);
// v[i] *= inv for n doubles on stream s
cudaError_t launch_scale_means(double* v, long long n, double inv, cudaStream_t s);
void free_denoise(Ctx& c);
// SDF volume cache (sdfvol.cu)
void free_volumes(Ctx& c);
// GPU BVH build (bvh_gpu.cu): same format as arbvh::build_wide_bvh; "" on success
std::string build_wide_bvh_gpu(const std::vector<arbvh::PrimInput>& prims, arbvh::WideBVH& out, cudaStream_t s);
// refit of the main BVH after mesh vertices moved (bvh_gpu.cu)
cudaError_t refit_wide_bvh(Ctx& c, const float* verts_dev, cudaStream_t s);
} // namespace ar
