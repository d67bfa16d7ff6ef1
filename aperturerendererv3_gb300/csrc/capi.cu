// C-ABI implementation: context lifetime, scene upload, BVH / light-table /
// spectral-LUT setup, the render loop over waves, and the raw ray queries.
//
// Host-side logic mirrors SceneRenderer (core/scene.cu): the light table of
// UpdateSceneToDeviceIfDirty (core/scene.cu:677-706), the material factories
// (core/render/object.cuh:119-206), SceneObject's frame and bounds
// (core/render/object.cuh:249-315), and the headless Render loop
// (core/scene.cu:210-238) with FP64 accumulation instead of an FP32 running mean.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <new>

#include "../../include/aperture/ar.h"
#include "ar_internal.h"
#include "ar_rng.h"
#include "spectral_tables.inc"

struct ar_ctx
{
    ar::Ctx c;
};

namespace ar
{
DevScene dev_scene(const Ctx& c)
{
    DevScene s;
    s.trav.nodes = reinterpret_cast<const uint4*>(c.d_nodes);
    s.trav.slots = reinterpret_cast<const float4*>(c.d_slots);
    s.trav.objects = c.d_objects;
    s.trav.sdf_params = c.d_sdf_params;
    s.trav.sdf_vols = c.d_vols;
    s.trav.sdf_vol_count = (int)c.vol_dev.size();

    s.trav.node_count = (int)c.bvh.nodes.size();
    s.materials = c.d_materials;
    s.prim_material = c.d_prim_material;
    s.prim_light = c.d_prim_light;
    s.prim_slot = c.d_prim_slot;
    s.lights = c.d_lights;
    s.light_count = (int)c.lights.size();
    s.lut_rgb = c.d_lut_rgb;
    s.lut_lambda = c.d_lut_lambda;
    s.cie_cmf = c.d_cie;
    s.d65 = c.d_d65;
    s.camera_inside = c.camera_inside;
    s.stats = (c.profile & 2) ? c.d_stats : nullptr;
    s.guide = c.guide;
    s.trav.sdf = c.sdf;
    s.trav.sdf_id = c.sdf_id;
    s.sdf_trav = s.trav;
    s.sdf_trav.nodes = reinterpret_cast<const uint4*>(c.d_sdf_nodes);
    s.sdf_trav.slots = reinterpret_cast<const float4*>(c.d_sdf_bvh_slots);
    s.sdf_trav.node_count = c.d_sdf_nodes ? (int)c.sdf_bvh.nodes.size() : 0;
    s.medium = c.medium;
    s.texels = c.d_texels;
    s.tex_info = c.d_tex_info;
    s.prim_uv = c.d_prim_uv;
    s.tex_count = c.tex_count;
    return s;
}
// intersection::Overlap for one object (core/render/intersection.cuh:312-327);
// SDF objects evaluate their field on the host copy of the volume cache
// (OverlapSDFObject, core/object/sdf/sdf_base.cuh:165-176)
bool overlap_any(const Ctx& c, V3 p, int i)
{
    const Object& ob = c.objects[i];
    if (ob.type != AR_OBJECT_SDF) return overlap_object(p, ob);
    SdfObjField f;
    f.kind = ob.pad[0];
    f.prm = c.object_sdf[i];
    f.vol = nullptr;
    SdfVolume hv{};
    const int vi = ob.pad[1];
    if (f.kind == AR_SDF_OBJ_VOLUME && vi >= 0 && vi < (int)c.vol_host.size())
    {
        hv.data = c.vol_host[vi].data();
        hv.dx = c.vol_dims[3 * vi];
        hv.dy = c.vol_dims[3 * vi + 1];
        hv.dz = c.vol_dims[3 * vi + 2];
        hv.voxel_size_max = sdf_volume_voxel_size_max(hv.dx, hv.dy, hv.dz);
        f.vol = &hv;
    }
    const V3 lp = mul(ob.w2o, p - ob.center);
    return sdf_obj_eval(f, sdf_to_unit(lp, ob.extent)) <= 0.0f;
}

// 1 when the camera starts inside a non-triangle object (the first
// intersection::Overlap of CalculateRadiance, core/render/render.cuh:536-538)
int camera_inside_any(const Ctx& c, const float cam_o[3])
{
    const V3 co = v3(cam_o[0], cam_o[1], cam_o[2]);
    for (size_t i = 0; i < c.objects.size(); ++i)
        if (c.object_type[i] != AR_OBJECT_TRIANGLE && overlap_any(c, co, (int)i)) return 1;
    return 0;
}
} // namespace ar

namespace
{
using namespace ar;

ar_status fail(ar_ctx* ctx, ar_status code, const std::string& msg)
{
    if (ctx) ctx->c.last_error = msg;
    return code;
}

ar_status cuda_fail(ar_ctx* ctx, cudaError_t e, const char* where)
{
    return fail(ctx, AR_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

#define AR_CUDA(ctx, call)                                              \
    do                                                                  \
    {                                                                   \
        cudaError_t e_ = (call);                                        \
        if (e_ != cudaSuccess) return cuda_fail((ctx), e_, #call);      \
    } while (0)

template <typename T>
void free_dev(T*& p)
{
    if (p) cudaFree((void*)p);
    p = nullptr;
}

void free_scene(Ctx& c)
{
    free_dev(c.d_nodes);
    free_dev(c.d_slots);
    free_dev(c.d_objects);
    free_dev(c.d_materials);
    free_dev(c.d_prim_material);
    free_dev(c.d_prim_light);
    free_dev(c.d_prim_slot);
    free_dev(c.d_lights);
    free_dev(c.d_texels);
    free_dev(c.d_tex_info);
    free_dev(c.d_prim_uv);
    free_dev(c.d_sdf);
    free_dev(c.d_sdf_params);
    free_dev(c.d_sdf_nodes);
    free_dev(c.d_sdf_bvh_slots);
    free_dev(c.d_refit_nodes);
    free_dev(c.d_mesh_idx);
    free_dev(c.d_prim_box);
    free_dev(c.d_node_box);
    free_dev(c.d_refit_verts);
    c.refit_level_off.clear();
    c.sdf_object_count = 0;
    c.sdf = SdfUnion{};
    c.tex_count = 0;
    c.texel_floats = 0;
    c.built = false;
}

void free_waves(Ctx& c)
{
    PathState& p = c.ps;
    free_dev(p.rng); free_dev(p.pixel); free_dev(p.frame); free_dev(p.ray_o); free_dev(p.ray_d);
    free_dev(p.radiance); free_dev(p.mask); free_dev(p.depths); free_dev(p.flags); free_dev(p.media_v);
    free_dev(p.media_depth); free_dev(p.prev); free_dev(p.hit_t); free_dev(p.hit_slot); free_dev(p.q_slot); free_dev(p.hit_nrm); free_dev(c.d_pend_list); free_dev(p.out_xyz);
    free_dev(c.sq.path); free_dev(c.sq.o); free_dev(c.sq.d); free_dev(c.sq.v_occ); free_dev(c.sq.valid_unocc); free_dev(c.sq.sdf_eps);
    free_dev(c.d_queue[0]);
    free_dev(c.d_queue[1]);
    free_dev(c.d_pq);
    c.wave_capacity = 0;
    p.capacity = 0;
}

template <typename T>
cudaError_t alloc_dev(T*& p, size_t count)
{
    return cudaMalloc((void**)&p, std::max<size_t>(count, 1) * sizeof(T));
}

ar_status ensure_waves(ar_ctx* ctx, int cap)
{
    Ctx& c = ctx->c;
    if (c.wave_capacity >= cap) return AR_OK;
    free_waves(c);
    PathState& p = c.ps;
    const size_t n = (size_t)cap;
    AR_CUDA(ctx, alloc_dev(p.rng, n));
    AR_CUDA(ctx, alloc_dev(p.pixel, n));
    AR_CUDA(ctx, alloc_dev(p.frame, n));
    AR_CUDA(ctx, alloc_dev(p.ray_o, n));
    AR_CUDA(ctx, alloc_dev(p.ray_d, n));
    AR_CUDA(ctx, alloc_dev(p.radiance, n));
    AR_CUDA(ctx, alloc_dev(p.mask, n));
    AR_CUDA(ctx, alloc_dev(p.depths, n));
    AR_CUDA(ctx, alloc_dev(p.flags, n));
    AR_CUDA(ctx, alloc_dev(p.media_v, n));
    AR_CUDA(ctx, alloc_dev(p.media_depth, n));
    AR_CUDA(ctx, alloc_dev(p.prev, n));
    AR_CUDA(ctx, alloc_dev(p.hit_t, n));
    AR_CUDA(ctx, alloc_dev(p.hit_slot, n));
    AR_CUDA(ctx, alloc_dev(p.q_slot, n));
    AR_CUDA(ctx, alloc_dev(p.hit_nrm, n));
    AR_CUDA(ctx, alloc_dev(c.d_pend_list, n));
    AR_CUDA(ctx, alloc_dev(p.out_xyz, 3 * n));
    AR_CUDA(ctx, alloc_dev(c.sq.path, n));
    AR_CUDA(ctx, alloc_dev(c.sq.o, n));
    AR_CUDA(ctx, alloc_dev(c.sq.d, n));
    AR_CUDA(ctx, alloc_dev(c.sq.v_occ, n));
    AR_CUDA(ctx, alloc_dev(c.sq.valid_unocc, n));
    AR_CUDA(ctx, alloc_dev(c.sq.sdf_eps, n));
    AR_CUDA(ctx, alloc_dev(c.d_queue[0], n));
    AR_CUDA(ctx, alloc_dev(c.d_queue[1], n));
    AR_CUDA(ctx, alloc_dev(c.d_pq, n));
    p.capacity = cap;
    c.wave_capacity = cap;
    return AR_OK;
}

void free_guide(Ctx& c)
{
    free_dev(c.d_pg_keys);
    free_dev(c.d_pg_vals);
    free_dev(c.d_pg_probes);
    free_dev(c.d_pg_temp);
    free_dev(c.d_pg_meta);
    free_dev(c.gs.radiance);
    free_dev(c.gs.dir);
    free_dev(c.gs.key);
    free_dev(c.gs.count);
    free_dev(c.gs.pos);
    free_dev(c.gs.wr);
    free_dev(c.ps.maskq);
    free_dev(c.ps.pg_dir);
    free_dev(c.ps.pg_loc);
    free_dev(c.ps.pg_vdir);
    c.guide = DevGuide{};
    c.pg_capacity = 0;
    c.pg_hash_slots = 0;
    c.pg_unit = 0.0f;
    c.gs = GuideSamples{};
    c.gs_capacity = 0;
    c.pg_path_cap = 0;
}

// The voxel guide's probe pool and key hash (voxel = floor(p / unit), as the
// reference keys its sparse volume), kept while the unit stays the same.
ar_status ensure_guide_pool(ar_ctx* ctx, float unit)
{
    Ctx& c = ctx->c;
    if (!(c.d_pg_keys && c.pg_unit == unit))
    {
        free_guide(c);
        // probe pool of 131072 probes (182 MB) and a hash at load factor <= 1/4
        const int capacity = 131072;
        const int slots = 4 * capacity;
        AR_CUDA(ctx, cudaMalloc((void**)&c.d_pg_keys, (size_t)slots * sizeof(unsigned long long)));
        AR_CUDA(ctx, cudaMemset(c.d_pg_keys, 0xff, (size_t)slots * sizeof(unsigned long long)));
        AR_CUDA(ctx, cudaMalloc((void**)&c.d_pg_vals, (size_t)slots * sizeof(int)));
        AR_CUDA(ctx, cudaMemset(c.d_pg_vals, 0xff, (size_t)slots * sizeof(int)));
        AR_CUDA(ctx, cudaMalloc((void**)&c.d_pg_probes, (size_t)capacity * sizeof(Probe)));
        AR_CUDA(ctx, cudaMemset(c.d_pg_probes, 0, (size_t)capacity * sizeof(Probe)));
        AR_CUDA(ctx, cudaMalloc((void**)&c.d_pg_temp, (size_t)capacity * sizeof(Probe)));
        AR_CUDA(ctx, cudaMemset(c.d_pg_temp, 0, (size_t)capacity * sizeof(Probe)));
        AR_CUDA(ctx, cudaMalloc((void**)&c.d_pg_meta, 4 * sizeof(int)));
        AR_CUDA(ctx, cudaMemset(c.d_pg_meta, 0, 4 * sizeof(int)));
        c.pg_capacity = capacity;
        c.pg_hash_slots = slots;
        c.pg_unit = unit;
        c.guide.keys = c.d_pg_keys;
        c.guide.vals = c.d_pg_vals;
        c.guide.probes = c.d_pg_probes;
        c.guide.probe_count = 0;
        c.guide.mask = (unsigned)(slots - 1);
        c.guide.inv_unit = 1.0f / unit;
    }
    return AR_OK;
}

// Voxel-guide storage: dense index table over the scene's voxel box (voxel =
// floor(p / unit), as the reference keys its sparse volume) and a probe pool.
ar_status ensure_guide(ar_ctx* ctx, float unit, long long npix)
{
    Ctx& c = ctx->c;
    if (!(unit > 0.0f)) unit = 0.05f;
    if (c.d_pg_keys && c.pg_unit == unit && c.ps.maskq && c.pg_path_cap == c.ps.capacity &&
        (long long)c.gs_capacity >= AR_PG_COLLECT_DEPTH * npix)
        return AR_OK;
    ar_status st = ensure_guide_pool(ctx, unit);
    if (st != AR_OK) return st;
    // per-path collection slots use the wavefront buffers' stride; the record
    // buffer holds a whole update window (up to AR_PG_COLLECT_DEPTH records per
    // path of its frames; `npix` is the window's path count)
    const int wave_cap = c.ps.capacity;
    const size_t ns = (size_t)AR_PG_COLLECT_DEPTH * wave_cap;
    const size_t nrec = (size_t)AR_PG_COLLECT_DEPTH * (size_t)npix;
    if (c.gs_capacity < (long long)nrec)
    {
        free_dev(c.gs.radiance);
        free_dev(c.gs.dir);
        free_dev(c.gs.key);
        free_dev(c.gs.count);
        free_dev(c.gs.pos);  // reallocated at the new size by ensure_mlp when the network is on
        free_dev(c.gs.wr);
        AR_CUDA(ctx, alloc_dev(c.gs.radiance, nrec));
        AR_CUDA(ctx, alloc_dev(c.gs.dir, nrec));
        AR_CUDA(ctx, alloc_dev(c.gs.key, nrec));
        AR_CUDA(ctx, alloc_dev(c.gs.count, 1));
        AR_CUDA(ctx, cudaMemset(c.gs.count, 0, sizeof(int)));
        c.gs.capacity = (int)nrec;
        c.gs_capacity = (int)nrec;
    }
    free_dev(c.ps.maskq);
    free_dev(c.ps.pg_dir);
    free_dev(c.ps.pg_loc);
    free_dev(c.ps.pg_vdir);
    AR_CUDA(ctx, alloc_dev(c.ps.maskq, (size_t)wave_cap));
    AR_CUDA(ctx, alloc_dev(c.ps.pg_dir, ns));
    AR_CUDA(ctx, alloc_dev(c.ps.pg_loc, ns));
    AR_CUDA(ctx, alloc_dev(c.ps.pg_vdir, ns));
    c.pg_path_cap = wave_cap;
    return AR_OK;
}

void object_bounds(const Object& o, float lo[3], float hi[3]);

void free_mlp(Ctx& c)
{
    free_dev(c.d_mlp_w32);
    free_dev(c.d_mlp_wbf);
    free_dev(c.d_mlp_grad);
    free_dev(c.d_mlp_gpart);
    free_dev(c.d_mlp_m);
    free_dev(c.d_mlp_v);
    free_dev(c.d_mlp_loss);
    free_dev(c.ps.q_pos);
    free_dev(c.ps.q_wr);
    free_dev(c.ps.q_dist);
    free_dev(c.d_mlp_list);
    c.mlp_step = 0;
    c.mlp_path_cap = 0;
}

// Network state of the MLP guide: He-initialised weights (fixed seed; the
// output layer scaled by 0.1 so the first distributions are near uniform),
// Adam moments, per-path query buffers and the records' extra fields.  The
// position box spans the non-emissive geometry (a distant sun would squeeze
// everything else into a corner of the encoding).
// brings the host copy of the mesh up to the last refit's vertices
cudaError_t sync_mesh_host(Ctx& c)
{
    if (!c.mesh_v_stale) return cudaSuccess;
    std::vector<float> host((size_t)c.mesh_nv * 3);
    cudaError_t e = cudaStreamSynchronize(c.stream);
    if (e == cudaSuccess)
        e = cudaMemcpy(host.data(), c.d_refit_verts, host.size() * sizeof(float), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return e;
    const size_t nt = c.mesh_idx.size() / 3;
    for (size_t t = 0; t < nt; ++t)
        for (int j = 0; j < 3; ++j)
            for (int k = 0; k < 3; ++k) c.mesh_v[9 * t + 3 * j + k] = host[3 * (size_t)c.mesh_idx[3 * t + j] + k];
    c.mesh_v_stale = false;
    return cudaSuccess;
}

ar_status ensure_mlp(ar_ctx* ctx)
{
    Ctx& c = ctx->c;
    if (!c.d_mlp_w32)
    {
        std::vector<float> w(AR_MLP_PARAMS, 0.0f);
        uint64_t st = 0x853c49e6748fea9bull;
        auto gauss = [&st]() {
            // Box-Muller on a 64-bit LCG (Knuth MMIX constants)
            st = st * 6364136223846793005ull + 1442695040888963407ull;
            const double u1 = ((st >> 11) + 1.0) * (1.0 / 9007199254740993.0);
            st = st * 6364136223846793005ull + 1442695040888963407ull;
            const double u2 = (st >> 11) * (1.0 / 9007199254740992.0);
            return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
        };
        for (int l = 0; l < AR_MLP_LAYERS; ++l)
        {
            const int in = mlp_in_dim(l);
            const double sd = std::sqrt(2.0 / in) * (l == AR_MLP_LAYERS - 1 ? 0.1 : 1.0);
            for (int k = 0; k < 64 * in; ++k) w[mlp_w_offset(l) + k] = (float)(gauss() * sd);
        }
        AR_CUDA(ctx, alloc_dev(c.d_mlp_w32, (size_t)AR_MLP_PARAMS));
        AR_CUDA(ctx, alloc_dev(c.d_mlp_wbf, (size_t)AR_MLP_PARAMS));
        AR_CUDA(ctx, alloc_dev(c.d_mlp_grad, (size_t)AR_MLP_PARAMS));
        int sms = 0;
        AR_CUDA(ctx, cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c.device));
        AR_CUDA(ctx, alloc_dev(c.d_mlp_gpart, (size_t)std::max(1, sms) * AR_MLP_PARAMS));
        AR_CUDA(ctx, alloc_dev(c.d_mlp_m, (size_t)AR_MLP_PARAMS));
        AR_CUDA(ctx, alloc_dev(c.d_mlp_v, (size_t)AR_MLP_PARAMS));
        AR_CUDA(ctx, alloc_dev(c.d_mlp_loss, 1));
        AR_CUDA(ctx, cudaMemcpy(c.d_mlp_w32, w.data(), w.size() * sizeof(float), cudaMemcpyHostToDevice));
        AR_CUDA(ctx, cudaMemset(c.d_mlp_grad, 0, AR_MLP_PARAMS * sizeof(float)));
        AR_CUDA(ctx, cudaMemset(c.d_mlp_m, 0, AR_MLP_PARAMS * sizeof(float)));
        AR_CUDA(ctx, cudaMemset(c.d_mlp_v, 0, AR_MLP_PARAMS * sizeof(float)));
        AR_CUDA(ctx, cudaMemset(c.d_mlp_loss, 0, sizeof(float)));
        AR_CUDA(ctx, launch_mlp_to_bf16(c.d_mlp_w32, c.d_mlp_wbf, c.stream));
        AR_CUDA(ctx, mlp_prepare_kernels());
        c.mlp_step = 0;
        AR_CUDA(ctx, sync_mesh_host(c));
        // box of the non-emissive geometry
        float lo[3] = {3e38f, 3e38f, 3e38f}, hi[3] = {-3e38f, -3e38f, -3e38f};
        auto grow = [&](const float* a, const float* b) {
            for (int k = 0; k < 3; ++k)
            {
                lo[k] = std::min(lo[k], a[k]);
                hi[k] = std::max(hi[k], b[k]);
            }
        };
        for (size_t i = 0; i < c.objects.size(); ++i)
        {
            if (c.materials[c.object_material[i]].shading == AR_MAT_LIGHT) continue;
            float a[3], b[3];
            if (c.object_type[i] == AR_OBJECT_TRIANGLE)
            {
                const float* t = &c.object_tri[9 * i];
                for (int k = 0; k < 3; ++k)
                {
                    a[k] = std::min(t[k], std::min(t[3 + k], t[6 + k]));
                    b[k] = std::max(t[k], std::max(t[3 + k], t[6 + k]));
                }
            }
            else object_bounds(c.objects[i], a, b);
            grow(a, b);
        }
        for (size_t t = 0; t < c.mesh_material.size(); ++t)
        {
            if (c.materials[c.mesh_material[t]].shading == AR_MAT_LIGHT) continue;
            const float* v = &c.mesh_v[9 * t];
            for (int j = 0; j < 3; ++j) grow(v + 3 * j, v + 3 * j);
        }
        if (!(lo[0] <= hi[0]))
            for (int k = 0; k < 3; ++k)
            {
                lo[k] = c.bvh.root_lo[k];
                hi[k] = c.bvh.root_hi[k];
            }
        for (int k = 0; k < 3; ++k)
        {
            const float ext = std::max(hi[k] - lo[k], 1e-6f);
            c.mlp_box.lo[k] = lo[k] - 0.01f * ext;
            c.mlp_box.inv[k] = 1.0f / (1.02f * ext);
        }
    }
    if (c.mlp_path_cap != c.ps.capacity)
    {
        free_dev(c.ps.q_pos);
        free_dev(c.ps.q_wr);
        free_dev(c.ps.q_dist);
        free_dev(c.d_mlp_list);
        AR_CUDA(ctx, alloc_dev(c.d_mlp_list, (size_t)c.ps.capacity));
        AR_CUDA(ctx, alloc_dev(c.ps.q_pos, (size_t)c.ps.capacity));
        AR_CUDA(ctx, alloc_dev(c.ps.q_wr, (size_t)c.ps.capacity));
        AR_CUDA(ctx, alloc_dev(c.ps.q_dist, 64 * (size_t)c.ps.capacity));
        c.mlp_path_cap = c.ps.capacity;
    }
    if (!c.gs.pos)
    {
        AR_CUDA(ctx, alloc_dev(c.gs.pos, (size_t)c.gs.capacity));
        AR_CUDA(ctx, alloc_dev(c.gs.wr, (size_t)c.gs.capacity));
    }
    return AR_OK;
}

// one Adam step of the network on the frame's radiance records
// Adam steps after an update window of `frames` frames: mlp_steps_per_frame per frame
cudaError_t mlp_train_frame(Ctx& c, int frames, long long* launches)
{
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c.device);
    MlpDev net;
    net.wbf = c.d_mlp_wbf;
    net.w32 = c.d_mlp_w32;
    net.box = c.mlp_box;
    cudaError_t e = cudaSuccess;
    if (c.mlp_step == 0)
    {
        e = launch_mlp_bias_start(c.d_mlp_w32, c.gs.radiance, c.gs.count, c.stream);
        if (launches) *launches += 1;
    }
    const int steps = c.mlp_steps_per_frame * std::max(1, frames);
    for (int k = 0; k < steps && e == cudaSuccess; ++k)
    {
        // each step trains on its own subset of the frame's records; the loss of the last one is kept
        e = cudaMemsetAsync(c.d_mlp_loss, 0, sizeof(float), c.stream);
        if (e == cudaSuccess)
            e = launch_mlp_train(net, c.gs.pos, c.gs.wr, c.gs.dir, c.gs.radiance, c.gs.count, 0,
                                 AR_MLP_TRAIN_RECORDS, 1013 * k, c.d_mlp_grad, c.d_mlp_gpart, c.d_mlp_loss, c.d_err,
                                 sms, c.stream);
        if (e == cudaSuccess)
            e = launch_mlp_adam(c.d_mlp_w32, c.d_mlp_wbf, c.d_mlp_grad, c.d_mlp_m, c.d_mlp_v, c.mlp_step + 1,
                                AR_MLP_LR, c.stream);
        if (e == cudaSuccess) ++c.mlp_step;
        if (launches) *launches += 3;
    }
    return e;
}

// Material::Create* semantics: which fields each shading model keeps, clamps.
Material make_material(const ar_material& m)
{
    Material r;
    std::memset(&r, 0, sizeof(r));
    r.shading = m.shading;
    r.albedo = v3(1.0f, 1.0f, 1.0f);
    r.emissive = v3(0.0f, 0.0f, 0.0f);
    r.specular = 0.0f;
    r.metallic = 0.0f;
    r.roughness = 0.0f;
    r.ior = 1.5f;
    r.sigma_a = 100.0f;
    r.abbe = 20.0f;
    r.tilt = 0.0f;
    const V3 alb = v3(m.albedo[0], m.albedo[1], m.albedo[2]);
    const V3 emi = v3(m.emissive[0], m.emissive[1], m.emissive[2]);
    switch (m.shading)
    {
        case AR_SHADING_LIGHT:
            r.albedo = v3(0.0f, 0.0f, 0.0f);
            r.emissive = emi;
            break;
        case AR_SHADING_GLASS:
            r.albedo = alb;
            r.ior = m.ior;
            r.sigma_a = m.sigma_a;
            r.abbe = m.abbe;
            r.tilt = m.tilt;
            break;
        case AR_SHADING_GGX:
            r.albedo = alb;
            r.roughness = clampf(m.roughness, 0.01f, 1.0f);
            r.metallic = clampf(m.metallic, 0.0f, 1.0f);
            r.specular = clampf(m.specular, 0.0f, 1.0f);
            r.emissive = emi;
            break;
        default:
            r.shading = AR_SHADING_DIFFUSE;
            r.albedo = alb;
            r.emissive = emi;
            break;
    }
    r.albedo_tex = (m.albedo_texture > 0 && m.shading != AR_SHADING_LIGHT) ? m.albedo_texture - 1 : -1;
    return r;
}

float luminance(V3 c) { return dot(c, v3(0.2126f, 0.7152f, 0.0722f)); }

// SceneObject::GetArea (core/render/object.cuh:240-255)
float object_area(const Object& o)
{
    if (o.type == AR_OBJ_CUBE || o.type == AR_OBJECT_SDF)  // SceneObject::GetArea (core/render/object.cuh:249-263)
    {
        const float ex = fabsf(o.extent.x), ey = fabsf(o.extent.y), ez = fabsf(o.extent.z);
        return 8.0f * (ex * ey + ex * ez + ey * ez);
    }
    if (o.type == AR_OBJ_SPHERE)
    {
        const float r = fabsf(o.extent.x);
        return 4.0f * AR_PI_F * r * r;
    }
    return 0.0f;
}

// SceneObject::UpdateProxy bounds (core/render/object.cuh:262-293), widened by a
// relative 1e-6 so the BVH boxes enclose the intersection routine's rounding.
void object_bounds(const Object& o, float lo[3], float hi[3])
{
    V3 half;
    if (o.type == AR_OBJ_CUBE || o.type == AR_OBJECT_SDF)  // SceneObject::UpdateProxy (core/render/object.cuh:272-289)
    {
        const V3 ax = mul(o.o2w, v3(1, 0, 0)), ay = mul(o.o2w, v3(0, 1, 0)), az = mul(o.o2w, v3(0, 0, 1));
        half.x = fabsf(ax.x) * o.extent.x + fabsf(ay.x) * o.extent.y + fabsf(az.x) * o.extent.z;
        half.y = fabsf(ax.y) * o.extent.x + fabsf(ay.y) * o.extent.y + fabsf(az.y) * o.extent.z;
        half.z = fabsf(ax.z) * o.extent.x + fabsf(ay.z) * o.extent.y + fabsf(az.z) * o.extent.z;
    }
    else
    {
        const float r = max3(o.extent);
        half = v3(r, r, r);
    }
    const float c[3] = {o.center.x, o.center.y, o.center.z};
    const float h[3] = {half.x, half.y, half.z};
    for (int k = 0; k < 3; ++k)
    {
        const float pad = 1e-6f * (fabsf(c[k]) + h[k]) + 1e-30f;
        lo[k] = c[k] - h[k] - pad;
        hi[k] = c[k] + h[k] + pad;
    }
}

bool cuda_device_ok(int device, std::string* why)
{
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n <= device || device < 0)
    {
        *why = std::string("no CUDA device ") + std::to_string(device) + (e != cudaSuccess ? std::string(": ") + cudaGetErrorString(e) : std::string());
        return false;
    }
    return true;
}
// Validates the render parameters and fills the launch description; resets
// the per-render profile state and decides whether the camera starts inside
// an object (camera_inside_any).
ar_status prepare_launch(ar_ctx* ctx, const ar_render_params* prm, RenderLaunch& rl)
{
    Ctx& c = ctx->c;
    if (!c.built) return fail(ctx, AR_ERR_STATE, "render before ar_scene_build");
    if (prm->width <= 0 || prm->height <= 0 || prm->spp <= 0 || prm->max_depth <= 0 || prm->max_depth > 0xffff)
        return fail(ctx, AR_ERR_INVALID, "render: bad resolution, spp or depth");
    if ((long long)prm->width * prm->height > 0x7fffffffll)
        return fail(ctx, AR_ERR_INVALID, "render: more than 2^31 - 1 pixels");  // pixel indices are 32-bit
    AR_CUDA(ctx, cudaSetDevice(c.device));
    rl = RenderLaunch{};
    rl.width = prm->width;
    rl.height = prm->height;
    rl.spp = prm->spp;
    rl.max_depth = prm->max_depth;
    for (int k = 0; k < 3; ++k)
    {
        rl.cam_o[k] = prm->cam_origin[k];
        rl.cam_d[k] = prm->cam_dir[k];
    }
    rl.fov_deg = prm->fov_deg;
    rl.use_nee = prm->use_nee;
    rl.seed = prm->seed;
    rl.first_frame = prm->first_frame;
    // samples per block of the path order (PathOrder): a warp holds 32 samples
    // of one pixel; guided renders use a block that divides their update
    // window, so that a window stays one run of paths
    rl.sample_block = std::min(AR_SAMPLE_BLOCK, std::max(1, rl.spp));
    // the stream jump of every sample of the render, once (k_raygen reads it)
    if (c.jump_cap < rl.spp)
    {
        free_dev(c.d_jumps);
        c.jump_cap = 0;
        AR_CUDA(ctx, cudaMalloc((void**)&c.d_jumps, (size_t)rl.spp * sizeof(ulonglong2)));
        c.jump_cap = rl.spp;
    }
    {
        std::vector<ulonglong2> jumps((size_t)rl.spp);
        for (int s = 0; s < rl.spp; ++s)
        {
            uint64_t m, a;
            ar_pcg_jump((uint64_t)((uint32_t)s + (uint32_t)rl.first_frame) << 32, &m, &a);
            jumps[(size_t)s] = make_ulonglong2(m, a);
        }
        AR_CUDA(ctx, cudaMemcpyAsync(c.d_jumps, jumps.data(), jumps.size() * sizeof(ulonglong2), cudaMemcpyHostToDevice,
                                     c.stream));
    }
    rl.jumps = c.d_jumps;
    rl.profile = prm->profile;
    c.profile = prm->profile & 3;
    c.stage_events.clear();
    for (int k = 0; k < ST_COUNT; ++k)
    {
        c.stage_ms[k] = 0.0f;
        c.stage_launches[k] = 0;
    }
    if (c.profile)
    {
        if (!c.d_stats) AR_CUDA(ctx, cudaMalloc((void**)&c.d_stats, 8 * sizeof(unsigned long long)));
        AR_CUDA(ctx, cudaMemsetAsync(c.d_stats, 0, 8 * sizeof(unsigned long long), c.stream));
    }
    // camera inside a medium (intersection::Overlap, core/render/intersection.cuh:312-327)
    c.camera_inside = camera_inside_any(c, rl.cam_o);
    return AR_OK;
}

} // namespace

extern "C" {

int ar_abi_version(void) { return 4; }

ar_status ar_create(ar_ctx** out, int device)
{
    if (!out) return AR_ERR_INVALID;
    *out = nullptr;
    std::string why;
    if (!cuda_device_ok(device, &why)) return AR_ERR_CUDA;
    ar_ctx* ctx = new (std::nothrow) ar_ctx();
    if (!ctx) return AR_ERR_NOMEM;
    Ctx& c = ctx->c;
    c.device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c.order_event, cudaEventDisableTiming);
    for (int k = 0; k <= AR_BOUNCE_LOOKAHEAD && e == cudaSuccess; ++k)
        e = cudaEventCreateWithFlags(&c.bounce_ev[k], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaHostAlloc((void**)&c.h_bounce_cnt, (AR_BOUNCE_LOOKAHEAD + 1) * sizeof(int), cudaHostAllocDefault);
    if (e == cudaSuccess) e = cudaMalloc((void**)&c.d_err, sizeof(unsigned int));
    if (e == cudaSuccess) e = cudaMemset(c.d_err, 0, sizeof(unsigned int));
    if (e == cudaSuccess) e = cudaMalloc((void**)&c.d_counters, AR_CNT_COUNT * sizeof(int));
    // spectral tables: CIE CMFs, D65, lambda LUT (built on the host: 840 encoder runs)
    if (e == cudaSuccess) e = cudaMalloc((void**)&c.d_cie, sizeof(AR_TAB_CMF));
    if (e == cudaSuccess) e = cudaMemcpy(c.d_cie, AR_TAB_CMF, sizeof(AR_TAB_CMF), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMalloc((void**)&c.d_d65, sizeof(AR_TAB_D65));
    if (e == cudaSuccess) e = cudaMemcpy(c.d_d65, AR_TAB_D65, sizeof(AR_TAB_D65), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
    {
        std::vector<float> lam(AR_LAMBDA_LUT_RES * 4);
        const float step = (780.0f - 360.0f) / static_cast<float>(AR_LAMBDA_LUT_RES);
        for (int i = 0; i < AR_LAMBDA_LUT_RES; ++i) lambda_encode(360.0f + (i + 0.5f) * step, &lam[4 * i], AR_TAB_LAM_MLP);
        e = cudaMalloc((void**)&c.d_lut_lambda, lam.size() * sizeof(float));
        if (e == cudaSuccess) e = cudaMemcpy(c.d_lut_lambda, lam.data(), lam.size() * sizeof(float), cudaMemcpyHostToDevice);
    }
    if (e != cudaSuccess)
    {
        ar_destroy(ctx);
        return AR_ERR_CUDA;
    }
    *out = ctx;
    return AR_OK;
}

ar_status ar_destroy(ar_ctx* ctx)
{
    if (!ctx) return AR_ERR_INVALID;
    Ctx& c = ctx->c;
    cudaSetDevice(c.device);
    if (c.stream) cudaStreamSynchronize(c.stream);
    free_scene(c);
    free_guide(c);
    free_mlp(c);
    free_denoise(c);
    free_volumes(c);
    free_waves(c);
    free_dev(c.d_lut_rgb);
    free_dev(c.d_lut_lambda);
    free_dev(c.d_cie);
    free_dev(c.d_d65);
    free_dev(c.d_err);
    free_dev(c.d_counters);
    free_dev(c.d_accum);
    free_dev(c.d_stats);
    free_dev(c.d_grad32);
    free_dev(c.d_adj);
    free_dev(c.d_grad_medium);
    free_dev(c.d_frame_xyz);
    free_dev(c.d_frame_dn);
    free_dev(c.d_jumps);
    if (c.order_event) cudaEventDestroy(c.order_event);
    for (cudaEvent_t& ev : c.bounce_ev)
        if (ev) cudaEventDestroy(ev);
    if (c.h_bounce_cnt) cudaFreeHost(c.h_bounce_cnt);
    if (c.stream) cudaStreamDestroy(c.stream);
    delete ctx;
    return AR_OK;
}

const char* ar_last_error(ar_ctx* ctx) { return ctx ? ctx->c.last_error.c_str() : "null context"; }

ar_status ar_scene_set_materials(ar_ctx* ctx, const ar_material* m, int n)
{
    if (!ctx) return AR_ERR_INVALID;
    if (n < 0 || (n > 0 && !m)) return fail(ctx, AR_ERR_INVALID, "materials: bad pointer or count");
    Ctx& c = ctx->c;
    c.materials.resize(n);
    for (int i = 0; i < n; ++i) c.materials[i] = make_material(m[i]);
    c.built = false;
    return AR_OK;
}

ar_status ar_scene_set_objects(ar_ctx* ctx, const ar_object* o, int n)
{
    if (!ctx) return AR_ERR_INVALID;
    if (n < 0 || (n > 0 && !o)) return fail(ctx, AR_ERR_INVALID, "objects: bad pointer or count");
    Ctx& c = ctx->c;
    c.objects.assign(n, Object{});
    c.object_material.resize(n);
    c.object_type.resize(n);
    c.object_tri.assign((size_t)n * 9, 0.0f);
    c.object_sdf.assign((size_t)n, make_float4(0.0f, 0.0f, 0.0f, 0.0f));
    for (int i = 0; i < n; ++i)
    {
        const ar_object& s = o[i];
        if (s.type != AR_OBJECT_CUBE && s.type != AR_OBJECT_SPHERE && s.type != AR_OBJECT_TRIANGLE &&
            s.type != AR_OBJECT_SDF)
            return fail(ctx, AR_ERR_INVALID, "objects: unsupported type " + std::to_string(s.type));
        if (s.type == AR_OBJECT_SDF && s.sdf_type != AR_SDF_OBJECT_TORUS && s.sdf_type != AR_SDF_OBJECT_VOLUME)
            return fail(ctx, AR_ERR_INVALID, "objects: SDF objects are a torus or a cached volume");
        Object& ob = c.objects[i];
        std::memset(&ob, 0, sizeof(ob));
        ob.type = s.type;
        if (s.type == AR_OBJECT_SDF)
        {
            ob.pad[0] = s.sdf_type;
            ob.pad[1] = s.sdf_volume;
        }
        c.object_sdf[i] = make_float4(s.sdf_params[0], s.sdf_params[1], s.sdf_params[2], s.sdf_params[3]);
        ob.center = v3(s.center[0], s.center[1], s.center[2]);
        ob.extent = v3(fabsf(s.extent[0]), fabsf(s.extent[1]), fabsf(s.extent[2]));
        object_frame(v3(s.rotation_deg[0], s.rotation_deg[1], s.rotation_deg[2]), &ob.o2w, &ob.w2o);
        c.object_material[i] = s.material;
        c.object_type[i] = s.type;
        if (s.type == AR_OBJECT_TRIANGLE)
        {
            for (int k = 0; k < 3; ++k)
            {
                c.object_tri[9 * (size_t)i + k] = s.v0[k];
                c.object_tri[9 * (size_t)i + 3 + k] = s.v1[k];
                c.object_tri[9 * (size_t)i + 6 + k] = s.v2[k];
            }
        }
    }
    c.built = false;
    return AR_OK;
}

ar_status ar_scene_set_mesh(ar_ctx* ctx, const float* v, int nv, const uint32_t* idx, int nt, const int32_t* mat)
{
    if (!ctx) return AR_ERR_INVALID;
    if (nt < 0 || nv < 0 || (nt > 0 && (!v || !idx || !mat))) return fail(ctx, AR_ERR_INVALID, "mesh: bad pointer or count");
    Ctx& c = ctx->c;
    c.mesh_v_stale = false;
    c.mesh_v.resize((size_t)nt * 9);
    c.mesh_material.resize(nt);
    c.mesh_idx.assign(idx ? idx : nullptr, idx ? idx + 3 * (size_t)nt : nullptr);
    c.mesh_nv = nv;
    for (int t = 0; t < nt; ++t)
    {
        for (int j = 0; j < 3; ++j)
        {
            const uint32_t vi = idx[3 * (size_t)t + j];
            if (vi >= (uint32_t)nv) return fail(ctx, AR_ERR_INVALID, "mesh: vertex index out of range");
            for (int k = 0; k < 3; ++k) c.mesh_v[9 * (size_t)t + 3 * j + k] = v[3 * (size_t)vi + k];
        }
        c.mesh_material[t] = mat[t];
    }
    c.built = false;
    return AR_OK;
}

ar_status ar_scene_set_textures(ar_ctx* ctx, const float* texels, const int32_t* sizes, int n)
{
    if (!ctx) return AR_ERR_INVALID;
    if (n < 0 || (n > 0 && (!texels || !sizes))) return fail(ctx, AR_ERR_INVALID, "textures: bad pointer or count");
    Ctx& c = ctx->c;
    long long total = 0;
    for (int i = 0; i < n; ++i)
    {
        const int w = sizes[2 * i], h = sizes[2 * i + 1];
        if (w <= 0 || h <= 0 || (long long)w * h > (1ll << 28)) return fail(ctx, AR_ERR_INVALID, "textures: bad size");
        total += (long long)w * h;
    }
    if (total > (1ll << 30)) return fail(ctx, AR_ERR_INVALID, "textures: more than 2^30 texels");
    c.tex_sizes.assign(sizes, sizes + 2 * (size_t)n);
    c.tex_texels.assign(texels, texels + 3 * (size_t)total);
    c.built = false;
    return AR_OK;
}

ar_status ar_scene_set_mesh_uv(ar_ctx* ctx, const float* uv, int nt)
{
    if (!ctx) return AR_ERR_INVALID;
    if (nt < 0 || (nt > 0 && !uv)) return fail(ctx, AR_ERR_INVALID, "mesh uv: bad pointer or count");
    Ctx& c = ctx->c;
    c.mesh_uv.assign(uv, uv + 6 * (size_t)nt);
    c.built = false;
    return AR_OK;
}

ar_status ar_scene_set_sdf_union(ar_ctx* ctx, const float* prims, int n, float smooth_k, int32_t material)
{
    if (!ctx) return AR_ERR_INVALID;
    if (n < 0 || n > AR_SDF_MAX_PRIMS || (n > 0 && !prims)) return fail(ctx, AR_ERR_INVALID, "sdf union: bad pointer or count");
    if (n > 0 && !(smooth_k > 0.0f)) return fail(ctx, AR_ERR_INVALID, "sdf union: smooth width must be positive");
    Ctx& c = ctx->c;
    for (int i = 0; i < n; ++i)
    {
        const int kind = (int)prims[8 * i];
        if (kind != AR_SDF_SPHERE && kind != AR_SDF_BOX && kind != AR_SDF_TORUS)
            return fail(ctx, AR_ERR_INVALID, "sdf union: unknown primitive kind");
    }
    c.sdf_prims.assign(prims, prims + 8 * (size_t)n);
    c.sdf_k = smooth_k;
    c.sdf_material = material;
    c.built = false;
    return AR_OK;
}

ar_status ar_scene_set_medium(ar_ctx* ctx, const ar_medium* m)
{
    if (!ctx) return AR_ERR_INVALID;
    Ctx& c = ctx->c;
    if (!m)
    {
        c.medium = BoxMedium{};
        return AR_OK;
    }
    if (!(m->sigma_t > 0.0f) || !(m->albedo >= 0.0f && m->albedo <= 1.0f) || !(m->g > -1.0f && m->g < 1.0f) ||
        !(m->emission >= 0.0f))
        return fail(ctx, AR_ERR_INVALID, "medium: sigma_t > 0, albedo in [0, 1], |g| < 1, emission >= 0");
    for (int k = 0; k < 3; ++k)
        if (!(m->box_lo[k] < m->box_hi[k])) return fail(ctx, AR_ERR_INVALID, "medium: empty box");
    c.medium.on = 1;
    c.medium.lo = v3(m->box_lo[0], m->box_lo[1], m->box_lo[2]);
    c.medium.hi = v3(m->box_hi[0], m->box_hi[1], m->box_hi[2]);
    c.medium.sigma_t = m->sigma_t;
    c.medium.albedo = m->albedo;
    c.medium.g = m->g;
    c.medium.emission = m->emission;
    return AR_OK;
}

ar_status ar_scene_texel_count(ar_ctx* ctx, int64_t* n_floats)
{
    if (!ctx || !n_floats) return AR_ERR_INVALID;
    if (!ctx->c.built) return fail(ctx, AR_ERR_STATE, "texel count before ar_scene_build");
    *n_floats = ctx->c.texel_floats;
    return AR_OK;
}

ar_status ar_scene_update_texels(ar_ctx* ctx, const float* texels, int64_t n_floats, int is_device, void* stream)
{
    if (!ctx || (n_floats > 0 && !texels)) return AR_ERR_INVALID;
    Ctx& c = ctx->c;
    if (!c.built) return fail(ctx, AR_ERR_STATE, "texel update before ar_scene_build");
    if (n_floats != c.texel_floats) return fail(ctx, AR_ERR_INVALID, "texel update: count differs from the scene's");
    if (n_floats == 0) return AR_OK;
    AR_CUDA(ctx, cudaSetDevice(c.device));
    cudaStream_t s = stream ? (cudaStream_t)stream : c.stream;
    AR_CUDA(ctx, cudaMemcpyAsync(c.d_texels, texels, (size_t)n_floats * sizeof(float),
                                 is_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s));
    // later work on the context's stream sees the new texels
    if (s != c.stream) AR_CUDA(ctx, cudaStreamSynchronize(s));
    return AR_OK;
}

ar_status ar_scene_build(ar_ctx* ctx)
{
    if (!ctx) return AR_ERR_INVALID;
    Ctx& c = ctx->c;
    AR_CUDA(ctx, cudaSetDevice(c.device));
    AR_CUDA(ctx, sync_mesh_host(c));
    const int nobj = (int)c.objects.size();
    const int nmesh = (int)c.mesh_material.size();
    const int nsdf = c.sdf_prims.empty() ? 0 : 1;  // the smooth-union SDF is one primitive, after the mesh
    const long long nprim = (long long)nobj + nmesh + nsdf;
    const int nmat = (int)c.materials.size();
    if (nprim == 0) return fail(ctx, AR_ERR_INVALID, "scene is empty");
    if ((long long)nobj + nmesh == 0) return fail(ctx, AR_ERR_INVALID, "scene has no object or triangle besides the SDF");
    for (int i = 0; i < nobj; ++i)
        if (c.object_material[i] < 0 || c.object_material[i] >= nmat) return fail(ctx, AR_ERR_INVALID, "object material index out of range");
    for (int i = 0; i < nmesh; ++i)
        if (c.mesh_material[i] < 0 || c.mesh_material[i] >= nmat) return fail(ctx, AR_ERR_INVALID, "mesh material index out of range");
    const int ntex = (int)(c.tex_sizes.size() / 2);
    for (int i = 0; i < nmat; ++i)
        if (c.materials[i].albedo_tex >= ntex) return fail(ctx, AR_ERR_INVALID, "material texture index out of range");
    if (!c.mesh_uv.empty() && c.mesh_uv.size() != 6 * (size_t)nmesh)
        return fail(ctx, AR_ERR_INVALID, "mesh uv count differs from the mesh's triangle count");
    if (nsdf && (c.sdf_material < 0 || c.sdf_material >= nmat || c.materials[c.sdf_material].shading == AR_MAT_LIGHT))
        return fail(ctx, AR_ERR_INVALID, "sdf union: material index out of range or a light");
    float sdf_lo[3] = {3e38f, 3e38f, 3e38f}, sdf_hi[3] = {-3e38f, -3e38f, -3e38f};
    for (size_t i = 0; i < c.sdf_prims.size() / 8; ++i)
    {
        const float* q = &c.sdf_prims[8 * i];
        const int kind = (int)q[0];
        float h[3];
        if (kind == AR_SDF_SPHERE) h[0] = h[1] = h[2] = q[4];
        else if (kind == AR_SDF_BOX)
        {
            h[0] = q[4];
            h[1] = q[5];
            h[2] = q[6];
        }
        else
        {
            h[0] = h[2] = q[4] + q[5];
            h[1] = q[5];
        }
        for (int k = 0; k < 3; ++k)
        {
            // the smooth union reaches at most k / 4 beyond its primitives
            const float pad = 0.25f * c.sdf_k + 1e-4f * (fabsf(q[1 + k]) + h[k]) + 1e-6f;
            sdf_lo[k] = std::min(sdf_lo[k], q[1 + k] - fabsf(h[k]) - pad);
            sdf_hi[k] = std::max(sdf_hi[k], q[1 + k] + fabsf(h[k]) + pad);
        }
    }

    // primitives for the BVH (the SDF object, if any, is marched after the BVH traversal)
    const long long nbvh = (long long)nobj + nmesh;
    std::vector<arbvh::PrimInput> prims((size_t)nbvh);
    std::vector<int> prim_material((size_t)nprim), prim_light((size_t)nprim, -1);
    if (nsdf) prim_material[nbvh] = c.sdf_material;
    for (long long i = 0; i < nbvh; ++i)
    {
        arbvh::PrimInput& p = prims[i];
        p.id = (uint32_t)i;
        const float* tv = nullptr;
        if (i < nobj)
        {
            prim_material[i] = c.object_material[i];
            if (c.object_type[i] == AR_OBJECT_TRIANGLE) tv = &c.object_tri[9 * (size_t)i];
            else
            {
                p.kind = c.object_type[i] == AR_OBJECT_CUBE   ? AR_PRIM_KIND_BOX
                         : c.object_type[i] == AR_OBJECT_SDF ? AR_PRIM_KIND_SDF
                                                             : AR_PRIM_KIND_SPHERE;
                object_bounds(c.objects[i], p.lo, p.hi);
            }
        }
        else
        {
            prim_material[i] = c.mesh_material[i - nobj];
            tv = &c.mesh_v[9 * (size_t)(i - nobj)];
        }
        if (tv)
        {
            p.kind = AR_PRIM_KIND_TRI;
            std::memcpy(p.v, tv, 9 * sizeof(float));
            for (int k = 0; k < 3; ++k)
            {
                p.lo[k] = std::min(tv[k], std::min(tv[3 + k], tv[6 + k]));
                p.hi[k] = std::max(tv[k], std::max(tv[3 + k], tv[6 + k]));
            }
        }
    }
    // SDF objects get their own BVH, traversed in a separate pass, so the main
    // traversal carries no SDF code
    std::vector<arbvh::PrimInput> sdf_prims;
    {
        size_t w = 0;
        for (size_t i = 0; i < prims.size(); ++i)
        {
            if (prims[i].kind == AR_PRIM_KIND_SDF) sdf_prims.push_back(prims[i]);
            else prims[w++] = prims[i];
        }
        prims.resize(w);
    }
    const int n_sdf_objects = (int)sdf_prims.size();
    std::string err;
    const auto tb0 = std::chrono::steady_clock::now();
    if (c.build_mode == AR_BUILD_GPU)
    {
        err = build_wide_bvh_gpu(prims, c.bvh, c.stream);
        if (!err.empty()) return fail(ctx, AR_ERR_CUDA, err);
    }
    else if (!arbvh::build_wide_bvh(prims, c.bvh, &err))
        return fail(ctx, AR_ERR_INVALID, "BVH build: " + err);
    c.last_build_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - tb0).count();
    if (c.bvh.depth >= AR_TRAV_STACK) return fail(ctx, AR_ERR_INVALID, "BVH deeper than the traversal stack");
    c.sdf_bvh = arbvh::WideBVH{};
    if (!sdf_prims.empty() && !arbvh::build_wide_bvh(sdf_prims, c.sdf_bvh, &err))
        return fail(ctx, AR_ERR_INVALID, "SDF object BVH build: " + err);
    if (c.sdf_bvh.depth >= AR_TRAV_STACK) return fail(ctx, AR_ERR_INVALID, "SDF object BVH deeper than the traversal stack");
    std::vector<int> prim_slot((size_t)nprim, -1);
    for (const arbvh::WideBVH* b : {&c.bvh, &c.sdf_bvh})
        for (size_t s = 0; s < b->slots.size(); ++s)
        {
            uint32_t tag;
            std::memcpy(&tag, &b->slots[s].a[3], 4);
            prim_slot[tag & AR_PRIM_ID_MASK] = (int)s;  // SDF objects: a slot of the SDF objects' BVH
        }

    // light table (core/scene.cu:677-706): every primitive with a light material
    c.lights.clear();
    float total = 0.0f;
    std::vector<float> weights;
    for (long long i = 0; i < nprim; ++i)
    {
        const Material& m = c.materials[prim_material[i]];
        if (m.shading != AR_MAT_LIGHT) continue;
        Light L;
        L.obj = (int)i;
        L.type = (i < nobj) ? c.object_type[i] : AR_OBJ_TRIANGLE;
        L.material = prim_material[i];
        const float area = (i < nobj) ? object_area(c.objects[i]) : 0.0f;
        const float w = fmaxf(area * luminance(m.emissive), 1.0e-20f);
        total += w;
        weights.push_back(w);
        prim_light[i] = (int)c.lights.size();
        c.lights.push_back(L);
    }
    float acc = 0.0f;
    for (size_t k = 0; k < c.lights.size(); ++k)
    {
        c.lights[k].select_prob = weights[k] / total;
        acc += c.lights[k].select_prob;
        c.lights[k].cdf = acc;
    }

    // device upload (a rebuilt scene starts with an empty guide)
    free_scene(c);
    free_guide(c);
    free_mlp(c);
    c.sdf_object_count = n_sdf_objects;
    std::vector<Object> objs(c.objects);
    if (objs.empty()) objs.resize(1);
    AR_CUDA(ctx, alloc_dev(c.d_nodes, c.bvh.nodes.size() * sizeof(ar_wide_node)));
    AR_CUDA(ctx, cudaMemcpy(c.d_nodes, c.bvh.nodes.data(), c.bvh.nodes.size() * sizeof(ar_wide_node), cudaMemcpyHostToDevice));
    // triangle slots carry their primitive's material and light index in the
    // spare w lanes of their second and third float4 (read by the shading's hit
    // reconstruction; the traversal reads only the vertices and the tag)
    for (ar_prim_slot& sl : c.bvh.slots)
    {
        uint32_t tag;
        std::memcpy(&tag, &sl.a[3], 4);
        if ((tag >> AR_PRIM_KIND_SHIFT) != AR_PRIM_KIND_TRI) continue;
        const int32_t mi = prim_material[tag & AR_PRIM_ID_MASK], li = prim_light[tag & AR_PRIM_ID_MASK];
        std::memcpy(&sl.b[3], &mi, 4);
        std::memcpy(&sl.c[3], &li, 4);
    }
    AR_CUDA(ctx, alloc_dev(c.d_slots, c.bvh.slots.size() * sizeof(ar_prim_slot)));
    AR_CUDA(ctx, cudaMemcpy(c.d_slots, c.bvh.slots.data(), c.bvh.slots.size() * sizeof(ar_prim_slot), cudaMemcpyHostToDevice));
    if (nmesh > 0 && !c.bvh.nodes.empty())
    {
        // refit tables: wide nodes by depth (children always follow their parent), mesh
        // indices, the bounds of the non-triangle primitives
        std::vector<int> level_nodes, cur{0}, next;
        c.refit_level_off.assign(1, 0);
        while (!cur.empty())
        {
            next.clear();
            for (int ni : cur)
            {
                level_nodes.push_back(ni);
                const ar_wide_node& nd = c.bvh.nodes[ni];
                int rank = 0;
                for (int sl = 0; sl < 8; ++sl)
                    if (nd.meta[sl] & 0x80u) next.push_back((int)nd.child_base + rank++);
            }
            c.refit_level_off.push_back((int)level_nodes.size());
            cur.swap(next);
        }
        std::vector<float> pbox((size_t)std::max(nobj, 1) * 6, 0.0f);
        for (int i = 0; i < nobj; ++i)
            if (c.object_type[i] != AR_OBJECT_TRIANGLE && c.object_type[i] != AR_OBJECT_SDF)
                object_bounds(c.objects[i], &pbox[6 * (size_t)i], &pbox[6 * (size_t)i + 3]);
        AR_CUDA(ctx, alloc_dev(c.d_refit_nodes, level_nodes.size()));
        AR_CUDA(ctx, cudaMemcpy(c.d_refit_nodes, level_nodes.data(), level_nodes.size() * sizeof(int), cudaMemcpyHostToDevice));
        AR_CUDA(ctx, alloc_dev(c.d_mesh_idx, c.mesh_idx.size()));
        AR_CUDA(ctx, cudaMemcpy(c.d_mesh_idx, c.mesh_idx.data(), c.mesh_idx.size() * sizeof(uint32_t), cudaMemcpyHostToDevice));
        AR_CUDA(ctx, alloc_dev(c.d_prim_box, pbox.size()));
        AR_CUDA(ctx, cudaMemcpy(c.d_prim_box, pbox.data(), pbox.size() * sizeof(float), cudaMemcpyHostToDevice));
        AR_CUDA(ctx, alloc_dev(c.d_node_box, 6 * c.bvh.nodes.size()));
    }
    AR_CUDA(ctx, alloc_dev(c.d_objects, objs.size()));
    AR_CUDA(ctx, cudaMemcpy(c.d_objects, objs.data(), objs.size() * sizeof(Object), cudaMemcpyHostToDevice));
    {
        std::vector<float4> sp(c.object_sdf);
        if (sp.empty()) sp.resize(1);
        AR_CUDA(ctx, alloc_dev(c.d_sdf_params, sp.size()));
        AR_CUDA(ctx, cudaMemcpy(c.d_sdf_params, sp.data(), sp.size() * sizeof(float4), cudaMemcpyHostToDevice));
    }
    if (!c.sdf_bvh.nodes.empty())
    {
        AR_CUDA(ctx, alloc_dev(c.d_sdf_nodes, c.sdf_bvh.nodes.size() * sizeof(ar_wide_node)));
        AR_CUDA(ctx, cudaMemcpy(c.d_sdf_nodes, c.sdf_bvh.nodes.data(), c.sdf_bvh.nodes.size() * sizeof(ar_wide_node),
                                cudaMemcpyHostToDevice));
        AR_CUDA(ctx, alloc_dev(c.d_sdf_bvh_slots, c.sdf_bvh.slots.size() * sizeof(ar_prim_slot)));
        AR_CUDA(ctx, cudaMemcpy(c.d_sdf_bvh_slots, c.sdf_bvh.slots.data(), c.sdf_bvh.slots.size() * sizeof(ar_prim_slot),
                                cudaMemcpyHostToDevice));
    }
    AR_CUDA(ctx, alloc_dev(c.d_prim_material, (size_t)nprim));
    AR_CUDA(ctx, cudaMemcpy(c.d_prim_material, prim_material.data(), nprim * sizeof(int), cudaMemcpyHostToDevice));
    AR_CUDA(ctx, alloc_dev(c.d_prim_light, (size_t)nprim));
    AR_CUDA(ctx, cudaMemcpy(c.d_prim_light, prim_light.data(), nprim * sizeof(int), cudaMemcpyHostToDevice));
    AR_CUDA(ctx, alloc_dev(c.d_prim_slot, (size_t)nprim));
    AR_CUDA(ctx, cudaMemcpy(c.d_prim_slot, prim_slot.data(), nprim * sizeof(int), cudaMemcpyHostToDevice));
    AR_CUDA(ctx, alloc_dev(c.d_lights, c.lights.size()));
    if (!c.lights.empty())
        AR_CUDA(ctx, cudaMemcpy(c.d_lights, c.lights.data(), c.lights.size() * sizeof(Light), cudaMemcpyHostToDevice));

    // spectral RGB LUT (2 GiB, built once per context on the GPU)
    if (!c.d_lut_rgb)
    {
        const size_t bytes = (size_t)AR_LUT_RES * AR_LUT_RES * AR_LUT_RES * 4 * sizeof(float);
        AR_CUDA(ctx, cudaMalloc((void**)&c.d_lut_rgb, bytes));
        float* d_w = nullptr;
        AR_CUDA(ctx, cudaMalloc((void**)&d_w, sizeof(AR_TAB_RGB_MLP)));
        cudaError_t e = cudaMemcpy(d_w, AR_TAB_RGB_MLP, sizeof(AR_TAB_RGB_MLP), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = launch_build_rgb_lut(c.d_lut_rgb, d_w, c.stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
        cudaFree(d_w);
        if (e != cudaSuccess)
        {
            free_dev(c.d_lut_rgb);
            return cuda_fail(ctx, e, "spectral LUT build");
        }
    }
    // albedo textures: texels, per-texture {offset, width, height}, per-primitive uv
    if (ntex > 0)
    {
        std::vector<int4> info((size_t)ntex);
        long long off = 0;
        for (int i = 0; i < ntex; ++i)
        {
            info[i] = make_int4((int)off, c.tex_sizes[2 * i], c.tex_sizes[2 * i + 1], 0);
            off += (long long)c.tex_sizes[2 * i] * c.tex_sizes[2 * i + 1];
        }
        AR_CUDA(ctx, alloc_dev(c.d_texels, c.tex_texels.size()));
        AR_CUDA(ctx, cudaMemcpy(c.d_texels, c.tex_texels.data(), c.tex_texels.size() * sizeof(float), cudaMemcpyHostToDevice));
        AR_CUDA(ctx, alloc_dev(c.d_tex_info, info.size()));
        AR_CUDA(ctx, cudaMemcpy(c.d_tex_info, info.data(), info.size() * sizeof(int4), cudaMemcpyHostToDevice));
        std::vector<float> uv((size_t)nprim * 6, 0.0f);
        if (!c.mesh_uv.empty()) std::memcpy(&uv[(size_t)nobj * 6], c.mesh_uv.data(), c.mesh_uv.size() * sizeof(float));
        AR_CUDA(ctx, alloc_dev(c.d_prim_uv, uv.size()));
        AR_CUDA(ctx, cudaMemcpy(c.d_prim_uv, uv.data(), uv.size() * sizeof(float), cudaMemcpyHostToDevice));
        c.tex_count = ntex;
        c.texel_floats = (long long)c.tex_texels.size();
    }
    if (nsdf)
    {
        const int n = (int)(c.sdf_prims.size() / 8);
        std::vector<float> up(c.sdf_prims);
        for (int i = 0; i < n; ++i)
            up[8 * i + 7] = sdf_bounding_radius(up[8 * i], up[8 * i + 4], up[8 * i + 5], up[8 * i + 6]);
        AR_CUDA(ctx, alloc_dev(c.d_sdf, 2 * (size_t)n));
        AR_CUDA(ctx, cudaMemcpy(c.d_sdf, up.data(), up.size() * sizeof(float), cudaMemcpyHostToDevice));
        c.sdf.prims = c.d_sdf;
        c.sdf.count = n;
        c.sdf.k = c.sdf_k;
        c.sdf.lo = v3(sdf_lo[0], sdf_lo[1], sdf_lo[2]);
        c.sdf.hi = v3(sdf_hi[0], sdf_hi[1], sdf_hi[2]);
        c.sdf_id = (int)nbvh;
    }
    std::vector<Material> mats(c.materials);
    AR_CUDA(ctx, alloc_dev(c.d_materials, std::max<size_t>(mats.size(), 1)));
    if (!mats.empty())
    {
        AR_CUDA(ctx, cudaMemcpy(c.d_materials, mats.data(), mats.size() * sizeof(Material), cudaMemcpyHostToDevice));
        AR_CUDA(ctx, launch_prepare_materials(c.d_materials, (int)mats.size(), c.d_lut_rgb, c.stream));
        AR_CUDA(ctx, cudaStreamSynchronize(c.stream));
    }
    c.built = true;
    return AR_OK;
}

ar_status ar_scene_set_build_mode(ar_ctx* ctx, int32_t mode)
{
    if (!ctx) return AR_ERR_INVALID;
    if (mode != AR_BUILD_HOST && mode != AR_BUILD_GPU) return fail(ctx, AR_ERR_INVALID, "build mode: host or GPU");
    ctx->c.build_mode = mode;
    ctx->c.built = false;
    return AR_OK;
}

ar_status ar_scene_refit_mesh(ar_ctx* ctx, const float* vertices, int n_vertices, int is_device, void* stream)
{
    if (!ctx || !vertices) return AR_ERR_INVALID;
    Ctx& c = ctx->c;
    if (!c.built) return fail(ctx, AR_ERR_STATE, "refit before ar_scene_build");
    if (c.mesh_idx.empty() || !c.d_mesh_idx) return fail(ctx, AR_ERR_STATE, "refit: the scene has no mesh");
    if (n_vertices != c.mesh_nv) return fail(ctx, AR_ERR_INVALID, "refit: vertex count differs from the mesh's");
    AR_CUDA(ctx, cudaSetDevice(c.device));
    cudaStream_t s = stream ? (cudaStream_t)stream : c.stream;
    const size_t bytes = (size_t)n_vertices * 3 * sizeof(float);
    if (!c.d_refit_verts) AR_CUDA(ctx, alloc_dev(c.d_refit_verts, (size_t)n_vertices * 3));
    // the context keeps the vertices on the device; its host copy of the mesh
    // (rebuilds, the MLP guide's bounds) is brought up to date when next needed
    AR_CUDA(ctx, cudaMemcpyAsync(c.d_refit_verts, vertices, bytes,
                                 is_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s));
    AR_CUDA(ctx, refit_wide_bvh(c, c.d_refit_verts, s));
    AR_CUDA(ctx, cudaStreamSynchronize(s));
    c.mesh_v_stale = true;
    return AR_OK;
}

ar_status ar_scene_build_time(ar_ctx* ctx, double* ms)
{
    if (!ctx || !ms) return AR_ERR_INVALID;
    *ms = ctx->c.last_build_ms;
    return AR_OK;
}

ar_status ar_scene_stats(ar_ctx* ctx, int64_t* n_nodes, int64_t* n_slots, int32_t* depth, int64_t* device_bytes)
{
    if (!ctx) return AR_ERR_INVALID;
    const Ctx& c = ctx->c;
    if (n_nodes) *n_nodes = (int64_t)c.bvh.nodes.size();
    if (n_slots) *n_slots = (int64_t)c.bvh.slots.size();
    if (depth) *depth = c.bvh.depth;
    if (device_bytes)
        *device_bytes = (int64_t)(c.bvh.nodes.size() * sizeof(ar_wide_node) + c.bvh.slots.size() * sizeof(ar_prim_slot));
    return AR_OK;
}

ar_status ar_render(ar_ctx* ctx, const ar_render_params* prm, double* out_xyz, int out_is_device, float* per_sample_xyz,
                    void* stream)
{
    (void)stream;
    if (!ctx || !prm || !out_xyz) return AR_ERR_INVALID;
    Ctx& c = ctx->c;
    RenderLaunch rl;
    ar_status st = prepare_launch(ctx, prm, rl);
    if (st != AR_OK) return st;
    const long long npix = (long long)rl.width * rl.height;
    const long long total = npix * rl.spp;
    rl.guide = prm->guide;
    if (rl.guide < 0 || rl.guide > 2) return fail(ctx, AR_ERR_INVALID, "render: unknown guide mode");
    if (rl.guide)
    {
        // an update window of guide_frames frames stays one run of paths when
        // the sample block divides it
        const int gf = std::max(1, prm->guide_frames);
        while (gf % rl.sample_block != 0) rl.sample_block >>= 1;
    }
    // automatic: up to 2^25 paths in flight (about 8 GB of path and shadow-ray
    // state); each depth of a wave is three launches whose ramp-up and tail
    // cost the same whatever the wave's size, so few large waves keep the GPU
    // full (the 64-sample 1920 x 1080 terrain: 712 Msamples/s with 2^21-path
    // waves, 1083 with 2^25)
    int cap = prm->wave_paths > 0 ? prm->wave_paths : AR_WAVE_PATHS_AUTO;
    if ((long long)cap > total) cap = (int)total;
    // guided frames learn after every update window of guide_frames frames:
    // waves never straddle a window
    if (prm->guide_frames < 0) return fail(ctx, AR_ERR_INVALID, "render: negative guide_frames");
    const long long window = rl.guide ? npix * std::max(1, prm->guide_frames) : total;
    if (rl.guide && (long long)cap > window) cap = (int)window;
    st = ensure_waves(ctx, cap);
    if (st != AR_OK) return st;
    if (rl.guide)
    {
        st = ensure_guide(ctx, prm->guide_unit, std::min(window, total));
        if (st != AR_OK) return st;
    }
    if (rl.guide == 2)
    {
        st = ensure_mlp(ctx);
        if (st != AR_OK) return st;
    }
    if (prm->denoise_record != 0 && prm->denoise_record != 1)
        return fail(ctx, AR_ERR_INVALID, "render: denoise_record must be 0 or 1");
    rl.denoise = prm->denoise_record;
    if (rl.denoise) AR_CUDA(ctx, ensure_denoise(c, rl.width, rl.height, rl.first_frame));
    c.mlp_steps_per_frame = prm->guide_train_steps > 0 ? prm->guide_train_steps : AR_MLP_STEPS_PER_FRAME;
    rl.mlp_ready = (rl.guide == 2 && c.mlp_step >= AR_MLP_WARMUP_STEPS) ? 1 : 0;
    if (c.accum_pixels < (size_t)npix)
    {
        free_dev(c.d_accum);
        AR_CUDA(ctx, cudaMalloc((void**)&c.d_accum, (size_t)npix * 3 * sizeof(double)));
        c.accum_pixels = (size_t)npix;
    }
    AR_CUDA(ctx, cudaMemsetAsync(c.d_accum, 0, (size_t)npix * 3 * sizeof(double), c.stream));
    float* d_samples = nullptr;
    if (per_sample_xyz) AR_CUDA(ctx, cudaMalloc((void**)&d_samples, (size_t)cap * 3 * sizeof(float)));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, c.stream);
    long long launches = 0;
    cudaError_t e = cudaSuccess;
    for (long long first = 0; first < total && e == cudaSuccess;)
    {
        // a wave never crosses an update window in guided mode
        long long n_ll = std::min<long long>(cap, total - first);
        if (rl.guide) n_ll = std::min<long long>(n_ll, window - first % window);
        const int n = (int)n_ll;
        e = launch_render_wave(c, rl, first, n, d_samples, &launches);
        if (e == cudaSuccess) e = launch_accumulate(c, rl, first, n, c.d_accum, &launches);
        if (e == cudaSuccess && rl.denoise) e = launch_denoise_record(c, rl, first, n, &launches);
        if (e == cudaSuccess && per_sample_xyz)
            e = cudaMemcpyAsync(per_sample_xyz + 3 * first, d_samples, (size_t)n * 3 * sizeof(float), cudaMemcpyDeviceToHost, c.stream);
        first += n;
        if (rl.guide && e == cudaSuccess && (first % window == 0 || first == total))
        {
            // end of an update window (one frame by default): learn from its radiance
            // records (core/scene.cu:258-273); the network trains first (the probe
            // update clears the record count)
            if (rl.guide == 2)
            {
                const long long frames = (first - ((first - 1) / window) * window + npix - 1) / npix;
                e = mlp_train_frame(c, (int)frames, &launches);
                rl.mlp_ready = c.mlp_step >= AR_MLP_WARMUP_STEPS ? 1 : 0;
            }
            if (e == cudaSuccess) e = launch_guide_update(c, &launches);
            c.guide.probe_count = 1;
        }
    }
    cudaEventRecord(e1, c.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
    if (e == cudaSuccess) cudaEventElapsedTime(&c.last_render_ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (d_samples) cudaFree(d_samples);
    if (e == cudaSuccess && per_sample_xyz)
    {
        // samples arrive in path order; hand them back sample-major, pixel-minor
        const std::vector<float> by_path(per_sample_xyz, per_sample_xyz + 3 * (size_t)total);
        const PathOrder po = path_order(rl);
        for (long long g = 0; g < total; ++g)
        {
            uint32_t u, s;
            path_slot(po, (unsigned long long)g, &u, &s);
            const size_t px = slot_pixel(u, (uint32_t)rl.width, (uint32_t)rl.height);
            float* dst = per_sample_xyz + 3 * ((size_t)s * npix + px);
            for (int k = 0; k < 3; ++k) dst[k] = by_path[3 * (size_t)g + k];
        }
    }
    c.last_launches = launches;
    for (const StageEvent& se : c.stage_events)
    {
        float ms = 0.0f;
        if (e == cudaSuccess && cudaEventElapsedTime(&ms, se.a, se.b) == cudaSuccess) c.stage_ms[se.stage] += ms;
        cudaEventDestroy(se.a);
        cudaEventDestroy(se.b);
    }
    c.stage_events.clear();
    if ((c.profile & 2) && e == cudaSuccess)
        e = cudaMemcpy(c.stats, c.d_stats, 8 * sizeof(unsigned long long), cudaMemcpyDeviceToHost);
    c.profile = 0;
    if (e != cudaSuccess) return cuda_fail(ctx, e, "render");
    // mean over samples, scaled on the device and copied once
    const size_t out_bytes = (size_t)npix * 3 * sizeof(double);
    AR_CUDA(ctx, launch_scale_means(c.d_accum, npix * 3, 1.0 / (double)rl.spp, c.stream));
    c.last_launches += 1;
    AR_CUDA(ctx, cudaMemcpyAsync(out_xyz, c.d_accum, out_bytes,
                                 out_is_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, c.stream));
    AR_CUDA(ctx, cudaStreamSynchronize(c.stream));
    unsigned int word = 0;
    AR_CUDA(ctx, cudaMemcpy(&word, c.d_err, sizeof(word), cudaMemcpyDeviceToHost));
    if (word) return fail(ctx, AR_ERR_DEVICE, "device error word set: " + std::to_string(word));
    return AR_OK;
}

} // extern "C"

namespace
{
// Replay adjoint driver: per wave a radiance pass, the per-path seed and the
// replay pass that scatters gradients (texels into float32, folded into
// grad_texels in float64 after each wave; medium parameters into grad_medium).
ar_status run_adjoint(ar_ctx* ctx, const ar_render_params* prm, const float* dl_dxyz, double* grad_texels,
                      double* grad_medium, void* stream)
{
    Ctx& c = ctx->c;
    if (prm->guide != AR_GUIDE_NONE) return fail(ctx, AR_ERR_INVALID, "adjoint: guided rendering is not differentiated");
    if (prm->profile) return fail(ctx, AR_ERR_INVALID, "adjoint: profiling is not supported");
    RenderLaunch rl;
    ar_status st = prepare_launch(ctx, prm, rl);
    if (st != AR_OK) return st;
    if (stream) AR_CUDA(ctx, cudaStreamSynchronize((cudaStream_t)stream));
    const long long npix = (long long)rl.width * rl.height;
    const long long total = npix * rl.spp;
    // smaller automatic waves than rendering: gradients gather in float32 per wave
    int cap = prm->wave_paths > 0 ? prm->wave_paths : AR_WAVE_PATHS_ADJOINT;
    if ((long long)cap > total) cap = (int)total;
    st = ensure_waves(ctx, cap);
    if (st != AR_OK) return st;
    if (c.adj_capacity < c.ps.capacity)
    {
        free_dev(c.d_adj);
        AR_CUDA(ctx, alloc_dev(c.d_adj, 2 * (size_t)c.ps.capacity));
        c.adj_capacity = c.ps.capacity;
    }
    c.ps.adj_total = c.d_adj;
    c.ps.adj_delta = c.d_adj + c.ps.capacity;
    if (grad_texels)
    {
        if (c.grad32_n < c.texel_floats)
        {
            free_dev(c.d_grad32);
            AR_CUDA(ctx, alloc_dev(c.d_grad32, (size_t)c.texel_floats));
            AR_CUDA(ctx, cudaMemset(c.d_grad32, 0, (size_t)c.texel_floats * sizeof(float)));
            c.grad32_n = c.texel_floats;
        }
        AR_CUDA(ctx, cudaMemsetAsync(grad_texels, 0, (size_t)c.texel_floats * sizeof(double), c.stream));
    }
    if (grad_medium) AR_CUDA(ctx, cudaMemsetAsync(grad_medium, 0, 2 * sizeof(double), c.stream));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, c.stream);
    long long launches = 0;
    cudaError_t e = cudaSuccess;
    RenderLaunch replay = rl;
    replay.adjoint = 1;
    replay.grad = grad_texels ? c.d_grad32 : nullptr;
    replay.grad_medium = grad_medium;
    for (long long first = 0; first < total && e == cudaSuccess;)
    {
        const int n = (int)std::min<long long>(cap, total - first);
        e = launch_render_wave(c, rl, first, n, nullptr, &launches);                           // radiance of each path
        if (e == cudaSuccess) e = launch_adjoint_seed(c, rl, n, dl_dxyz, &launches);           // its adjoint
        if (e == cudaSuccess) e = launch_render_wave(c, replay, first, n, nullptr, &launches);  // replay + scatter
        if (e == cudaSuccess && grad_texels) e = launch_grad_fold(c, grad_texels, c.texel_floats, &launches);
        first += n;
    }
    cudaEventRecord(e1, c.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
    if (e == cudaSuccess) cudaEventElapsedTime(&c.last_render_ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    c.last_launches = launches;
    c.ps.adj_total = nullptr;
    c.ps.adj_delta = nullptr;
    c.profile = 0;
    if (e != cudaSuccess) return cuda_fail(ctx, e, "adjoint");
    unsigned int word = 0;
    AR_CUDA(ctx, cudaMemcpy(&word, c.d_err, sizeof(word), cudaMemcpyDeviceToHost));
    if (word) return fail(ctx, AR_ERR_DEVICE, "device error word set: " + std::to_string(word));
    return AR_OK;
}
} // namespace

extern "C" {

ar_status ar_adjoint(ar_ctx* ctx, const ar_render_params* prm, const float* dl_dxyz, double* grad_texels, void* stream)
{
    if (!ctx || !prm || !dl_dxyz || !grad_texels) return AR_ERR_INVALID;
    if (!ctx->c.built) return fail(ctx, AR_ERR_STATE, "adjoint before ar_scene_build");
    if (ctx->c.texel_floats == 0) return fail(ctx, AR_ERR_STATE, "adjoint: the scene has no textures");
    return run_adjoint(ctx, prm, dl_dxyz, grad_texels, nullptr, stream);
}

ar_status ar_adjoint_medium(ar_ctx* ctx, const ar_render_params* prm, const float* dl_dxyz, double* grad2, void* stream)
{
    if (!ctx || !prm || !dl_dxyz || !grad2) return AR_ERR_INVALID;
    Ctx& c = ctx->c;
    if (!c.built) return fail(ctx, AR_ERR_STATE, "adjoint before ar_scene_build");
    if (!c.medium.on) return fail(ctx, AR_ERR_STATE, "adjoint: the scene has no medium");
    AR_CUDA(ctx, cudaSetDevice(c.device));
    if (!c.d_grad_medium) AR_CUDA(ctx, alloc_dev(c.d_grad_medium, 2));
    const ar_status st = run_adjoint(ctx, prm, dl_dxyz, nullptr, c.d_grad_medium, stream);
    if (st != AR_OK) return st;
    AR_CUDA(ctx, cudaMemcpy(grad2, c.d_grad_medium, 2 * sizeof(double), cudaMemcpyDeviceToHost));
    return AR_OK;
}

ar_status ar_trace_closest(ar_ctx* ctx, const float* rays, int n, int32_t* prim_id, float* t, void* stream)
{
    if (!ctx || n < 0 || (n > 0 && (!rays || !prim_id))) return AR_ERR_INVALID;
    Ctx& c = ctx->c;
    if (!c.built) return fail(ctx, AR_ERR_STATE, "trace before ar_scene_build");
    cudaStream_t s = stream ? (cudaStream_t)stream : c.stream;
    long long L = 0;
    const cudaError_t e = launch_trace(dev_scene(c), rays, n, 0, prim_id, t, c.d_err, s, &L);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "trace_closest");
    c.last_launches = L;
    return AR_OK;
}

ar_status ar_trace_any(ar_ctx* ctx, const float* rays, int n, int32_t* hit, void* stream)
{
    if (!ctx || n < 0 || (n > 0 && (!rays || !hit))) return AR_ERR_INVALID;
    Ctx& c = ctx->c;
    if (!c.built) return fail(ctx, AR_ERR_STATE, "trace before ar_scene_build");
    cudaStream_t s = stream ? (cudaStream_t)stream : c.stream;
    long long L = 0;
    const cudaError_t e = launch_trace(dev_scene(c), rays, n, 1, hit, nullptr, c.d_err, s, &L);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "trace_any");
    c.last_launches = L;
    return AR_OK;
}

ar_status ar_last_render_stats(ar_ctx* ctx, float* ms, int64_t* launches)
{
    if (!ctx) return AR_ERR_INVALID;
    if (ms) *ms = ctx->c.last_render_ms;
    if (launches) *launches = ctx->c.last_launches;
    return AR_OK;
}

ar_status ar_guide_stats(ar_ctx* ctx, int32_t* n_probes, int32_t* capacity)
{
    if (!ctx) return AR_ERR_INVALID;
    Ctx& c = ctx->c;
    AR_CUDA(ctx, cudaSetDevice(c.device));
    AR_CUDA(ctx, cudaStreamSynchronize(c.stream));
    if (n_probes) *n_probes = guide_probe_count(c);
    if (capacity) *capacity = c.pg_capacity;
    return AR_OK;
}

ar_status ar_guide_reset(ar_ctx* ctx, int32_t* n_probes)
{
    if (!ctx) return AR_ERR_INVALID;
    Ctx& c = ctx->c;
    AR_CUDA(ctx, cudaSetDevice(c.device));
    AR_CUDA(ctx, cudaStreamSynchronize(c.stream));
    if (n_probes) *n_probes = guide_probe_count(c);
    free_guide(c);
    free_mlp(c);
    return AR_OK;
}

// Probe set of the voxel guide, ordered by probe index: keys as pg::GetVoxelGrid
// returns them (x, y, z, face), the Texture<4> texels and counts.
ar_status ar_guide_read(ar_ctx* ctx, int32_t* n, int32_t capacity, int32_t* keys, float* texels, uint64_t* counts)
{
    if (!ctx || !n) return AR_ERR_INVALID;
    Ctx& c = ctx->c;
    AR_CUDA(ctx, cudaSetDevice(c.device));
    AR_CUDA(ctx, cudaStreamSynchronize(c.stream));
    const int np = c.d_pg_keys ? guide_probe_count(c) : 0;
    *n = np;
    if (!keys && !texels && !counts) return AR_OK;
    if (capacity < np) return fail(ctx, AR_ERR_INVALID, "guide_read: capacity below the probe count");
    if (keys)
    {
        std::vector<unsigned long long> hk((size_t)c.pg_hash_slots);
        std::vector<int> hv((size_t)c.pg_hash_slots);
        AR_CUDA(ctx, cudaMemcpy(hk.data(), c.d_pg_keys, hk.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
        AR_CUDA(ctx, cudaMemcpy(hv.data(), c.d_pg_vals, hv.size() * sizeof(int), cudaMemcpyDeviceToHost));
        const int lim = 1 << (AR_PG_KEY_BITS - 1);
        const unsigned long long m = (1ull << AR_PG_KEY_BITS) - 1ull;
        for (int i = 0; i < 4 * np; ++i) keys[i] = INT32_MIN;
        for (size_t sl = 0; sl < hk.size(); ++sl)
        {
            const unsigned long long k = hk[sl];
            const int v = hv[sl];
            if (k == AR_PG_KEY_EMPTY || v < 0 || v >= np) continue;
            keys[4 * v + 0] = (int)(k & m) - lim;
            keys[4 * v + 1] = (int)((k >> AR_PG_KEY_BITS) & m) - lim;
            keys[4 * v + 2] = (int)((k >> (2 * AR_PG_KEY_BITS)) & m) - lim;
            keys[4 * v + 3] = (int)(k >> (3 * AR_PG_KEY_BITS));
        }
    }
    if (texels || counts)
    {
        std::vector<Probe> pr((size_t)np);
        if (np) AR_CUDA(ctx, cudaMemcpy(pr.data(), c.d_pg_probes, pr.size() * sizeof(Probe), cudaMemcpyDeviceToHost));
        for (int i = 0; i < np; ++i)
        {
            if (texels) std::memcpy(texels + (size_t)i * AR_GUIDE_PROBE_FLOATS, pr[i].data, AR_GUIDE_PROBE_FLOATS * sizeof(float));
            if (counts) counts[i] = pr[i].count;
        }
    }
    return AR_OK;
}

// Replaces the probe set (keys, texels and counts as ar_guide_read gives them)
// and sets the voxel unit; the next guided ar_render with the same guide_unit
// samples from these probes and keeps learning into them.
ar_status ar_guide_write(ar_ctx* ctx, int32_t n, const int32_t* keys, const float* texels, const uint64_t* counts,
                         float unit)
{
    if (!ctx || n < 0 || (n > 0 && (!keys || !texels || !counts))) return AR_ERR_INVALID;
    Ctx& c = ctx->c;
    if (!(unit > 0.0f)) unit = 0.05f;
    AR_CUDA(ctx, cudaSetDevice(c.device));
    AR_CUDA(ctx, cudaStreamSynchronize(c.stream));
    ar_status st = ensure_guide_pool(ctx, unit);
    if (st != AR_OK) return st;
    if (n > c.pg_capacity) return fail(ctx, AR_ERR_INVALID, "guide_write: more probes than the pool holds");
    std::vector<unsigned long long> hk((size_t)c.pg_hash_slots, AR_PG_KEY_EMPTY);
    std::vector<int> hv((size_t)c.pg_hash_slots, -1);
    for (int i = 0; i < n; ++i)
    {
        const unsigned long long k = guide_pack(VoxelKey{keys[4 * i], keys[4 * i + 1], keys[4 * i + 2], keys[4 * i + 3]});
        if (k == AR_PG_KEY_EMPTY) return fail(ctx, AR_ERR_INVALID, "guide_write: key out of range");
        unsigned sl = guide_hash(k) & c.guide.mask;
        int probe = 0;
        for (; probe < AR_PG_HASH_PROBES; ++probe)
        {
            if (hk[sl] == k) return fail(ctx, AR_ERR_INVALID, "guide_write: duplicate key");
            if (hk[sl] == AR_PG_KEY_EMPTY) break;
            sl = (sl + 1u) & c.guide.mask;
        }
        if (probe == AR_PG_HASH_PROBES) return fail(ctx, AR_ERR_INVALID, "guide_write: hash chain too long");
        hk[sl] = k;
        hv[sl] = i;
    }
    std::vector<Probe> pr((size_t)n);
    for (int i = 0; i < n; ++i)
    {
        pr[i] = Probe{};
        std::memcpy(pr[i].data, texels + (size_t)i * AR_GUIDE_PROBE_FLOATS, AR_GUIDE_PROBE_FLOATS * sizeof(float));
        pr[i].count = counts[i];
    }
    AR_CUDA(ctx, cudaMemcpy(c.d_pg_keys, hk.data(), hk.size() * sizeof(unsigned long long), cudaMemcpyHostToDevice));
    AR_CUDA(ctx, cudaMemcpy(c.d_pg_vals, hv.data(), hv.size() * sizeof(int), cudaMemcpyHostToDevice));
    AR_CUDA(ctx, cudaMemset(c.d_pg_probes, 0, (size_t)c.pg_capacity * sizeof(Probe)));
    AR_CUDA(ctx, cudaMemset(c.d_pg_temp, 0, (size_t)c.pg_capacity * sizeof(Probe)));
    if (n) AR_CUDA(ctx, cudaMemcpy(c.d_pg_probes, pr.data(), pr.size() * sizeof(Probe), cudaMemcpyHostToDevice));
    const int meta[4] = {n, 0, 0, 0};
    AR_CUDA(ctx, cudaMemcpy(c.d_pg_meta, meta, sizeof(meta), cudaMemcpyHostToDevice));
    c.guide.probe_count = n > 0 ? 1 : 0;
    return AR_OK;
}

// Radiance records of the last guided frame, in the order the kernels wrote
// them: key (x, y, z, face), direction, XYZ radiance.
ar_status ar_guide_read_records(ar_ctx* ctx, int32_t* n, int32_t capacity, int32_t* keys, float* dirs,
                                float* radiance)
{
    if (!ctx || !n) return AR_ERR_INVALID;
    Ctx& c = ctx->c;
    AR_CUDA(ctx, cudaSetDevice(c.device));
    AR_CUDA(ctx, cudaStreamSynchronize(c.stream));
    int meta[4] = {0, 0, 0, 0};
    if (c.d_pg_meta) AR_CUDA(ctx, cudaMemcpy(meta, c.d_pg_meta, sizeof(meta), cudaMemcpyDeviceToHost));
    const int nr = std::min(meta[1], c.gs.capacity);
    *n = nr;
    if (!keys && !dirs && !radiance) return AR_OK;
    if (capacity < nr) return fail(ctx, AR_ERR_INVALID, "guide_read_records: capacity below the record count");
    std::vector<unsigned long long> k((size_t)nr);
    std::vector<float4> d((size_t)nr), r((size_t)nr);
    if (nr)
    {
        AR_CUDA(ctx, cudaMemcpy(k.data(), c.gs.key, k.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
        AR_CUDA(ctx, cudaMemcpy(d.data(), c.gs.dir, d.size() * sizeof(float4), cudaMemcpyDeviceToHost));
        AR_CUDA(ctx, cudaMemcpy(r.data(), c.gs.radiance, r.size() * sizeof(float4), cudaMemcpyDeviceToHost));
    }
    const int lim = 1 << (AR_PG_KEY_BITS - 1);
    const unsigned long long m = (1ull << AR_PG_KEY_BITS) - 1ull;
    for (int i = 0; i < nr; ++i)
    {
        if (keys)
        {
            if (k[i] == AR_PG_KEY_EMPTY)
            {
                keys[4 * i] = keys[4 * i + 1] = keys[4 * i + 2] = keys[4 * i + 3] = INT32_MIN;
            }
            else
            {
                keys[4 * i + 0] = (int)(k[i] & m) - lim;
                keys[4 * i + 1] = (int)((k[i] >> AR_PG_KEY_BITS) & m) - lim;
                keys[4 * i + 2] = (int)((k[i] >> (2 * AR_PG_KEY_BITS)) & m) - lim;
                keys[4 * i + 3] = (int)(k[i] >> (3 * AR_PG_KEY_BITS));
            }
        }
        if (dirs)
        {
            dirs[3 * i] = d[i].x;
            dirs[3 * i + 1] = d[i].y;
            dirs[3 * i + 2] = d[i].z;
        }
        if (radiance)
        {
            radiance[3 * i] = r[i].x;
            radiance[3 * i + 1] = r[i].y;
            radiance[3 * i + 2] = r[i].z;
        }
    }
    return AR_OK;
}

ar_status ar_guide_mlp_stats(ar_ctx* ctx, int32_t* steps, float* last_loss)
{
    if (!ctx) return AR_ERR_INVALID;
    Ctx& c = ctx->c;
    AR_CUDA(ctx, cudaSetDevice(c.device));
    AR_CUDA(ctx, cudaStreamSynchronize(c.stream));
    if (steps) *steps = c.mlp_step;
    if (last_loss)
    {
        *last_loss = 0.0f;
        if (c.d_mlp_loss) AR_CUDA(ctx, cudaMemcpy(last_loss, c.d_mlp_loss, sizeof(float), cudaMemcpyDeviceToHost));
    }
    return AR_OK;
}

ar_status ar_last_render_profile(ar_ctx* ctx, ar_render_profile* out)
{
    if (!ctx || !out) return AR_ERR_INVALID;
    const Ctx& c = ctx->c;
    out->raygen_ms = c.stage_ms[ST_RAYGEN];
    out->extend_ms = c.stage_ms[ST_EXTEND];
    out->shade_ms = c.stage_ms[ST_SHADE];
    out->shadow_ms = c.stage_ms[ST_SHADOW];
    out->finalize_ms = c.stage_ms[ST_FINAL];
    out->extend_node_visits = (int64_t)c.stats[0];
    out->extend_prim_tests = (int64_t)c.stats[1];
    out->shadow_node_visits = (int64_t)c.stats[2];
    out->shadow_prim_tests = (int64_t)c.stats[3];
    out->extend_rays = (int64_t)c.stats[4];
    out->shadow_rays = (int64_t)c.stats[5];
    out->extend_launches = c.stage_launches[ST_EXTEND];
    out->shade_launches = c.stage_launches[ST_SHADE];
    out->shadow_launches = c.stage_launches[ST_SHADOW];
    return AR_OK;
}

ar_status ar_get_error_word(ar_ctx* ctx, uint32_t* word)
{
    if (!ctx || !word) return AR_ERR_INVALID;
    unsigned int w = 0;
    AR_CUDA(ctx, cudaMemcpy(&w, ctx->c.d_err, sizeof(w), cudaMemcpyDeviceToHost));
    *word = w;
    return AR_OK;
}

ar_status ar_clear_error_word(ar_ctx* ctx)
{
    if (!ctx) return AR_ERR_INVALID;
    AR_CUDA(ctx, cudaMemset(ctx->c.d_err, 0, sizeof(unsigned int)));
    return AR_OK;
}

ar_status ar_host_trace_closest(const float* tris, int ntri, const float* rays, int nray, int32_t* ids, float* t,
                                int64_t* node_visits)
{
    if (ntri < 0 || nray < 0 || (ntri > 0 && !tris) || (nray > 0 && (!rays || !ids))) return AR_ERR_INVALID;
    std::vector<arbvh::PrimInput> prims((size_t)ntri);
    for (int i = 0; i < ntri; ++i)
    {
        arbvh::PrimInput& p = prims[i];
        const float* v = tris + 9 * (size_t)i;
        std::memcpy(p.v, v, 9 * sizeof(float));
        p.id = (uint32_t)i;
        p.kind = AR_PRIM_KIND_TRI;
        for (int k = 0; k < 3; ++k)
        {
            p.lo[k] = std::min(v[k], std::min(v[3 + k], v[6 + k]));
            p.hi[k] = std::max(v[k], std::max(v[3 + k], v[6 + k]));
        }
    }
    arbvh::WideBVH bvh;
    std::string err;
    if (!arbvh::build_wide_bvh(prims, bvh, &err)) return AR_ERR_INVALID;
    TravScene sc;
    sc.nodes = reinterpret_cast<const uint4*>(bvh.nodes.data());
    sc.slots = reinterpret_cast<const float4*>(bvh.slots.data());
    sc.objects = nullptr;
    sc.sdf_params = nullptr;
    sc.sdf_vols = nullptr;
    sc.sdf_vol_count = 0;
    sc.node_count = (int)bvh.nodes.size();
    sc.sdf = SdfUnion{};
    sc.sdf_id = -1;
    unsigned int errw = 0;
    unsigned long long stats[2] = {0, 0};
    for (int r = 0; r < nray; ++r)
    {
        const float* q = rays + 8 * (size_t)r;
        const TravResult res = traverse<false>(sc, v3(q[0], q[1], q[2]), v3(q[4], q[5], q[6]), q[3], q[7], &errw, stats);
        ids[r] = res.id;
        if (t) t[r] = res.slot >= 0 ? res.t : -1.0f;
    }
    if (node_visits) *node_visits = (int64_t)stats[0];
    return errw ? AR_ERR_DEVICE : AR_OK;
}

ar_status ar_host_guide_eval(const float* in, int n, float* out)
{
    // same record layout as the oracle's guide mode: leaf (AR_PG_RES2 x float4), then
    // n x {dir 3, normal 3, query 3, pos 3, uv 2, seed as 2 floats}
    if (n < 0 || !in || !out) return AR_ERR_INVALID;
    Probe* pr = new (std::nothrow) Probe();
    if (!pr) return AR_ERR_NOMEM;
    std::memset(pr, 0, sizeof(Probe));
    for (int i = 0; i < AR_PG_RES2; ++i) pr->data[i] = make_float4(in[4 * i], in[4 * i + 1], in[4 * i + 2], in[4 * i + 3]);
    generate_mipmaps(*pr);
    for (int i = 0; i < AR_PG_TEXELS_PAD; ++i)
    {
        out[4 * i] = pr->data[i].x;
        out[4 * i + 1] = pr->data[i].y;
        out[4 * i + 2] = pr->data[i].z;
        out[4 * i + 3] = pr->data[i].w;
    }
    const float* rec = in + AR_PG_RES2 * 4;
    for (int i = 0; i < n; ++i)
    {
        const float* r = rec + (size_t)i * 16;
        const V3 dir = v3(r[0], r[1], r[2]), nrm = v3(r[3], r[4], r[5]), q = v3(r[6], r[7], r[8]);
        const V3 pos = v3(r[9], r[10], r[11]);
        uint64_t seed;
        std::memcpy(&seed, r + 14, 8);
        float* o = out + AR_PG_TEXELS_PAD * 4 + (size_t)i * 14;
        const VoxelKey k = voxel_key(pos, dir, 1.0f / 0.05);
        o[0] = (float)k.f;
        o[1] = (float)k.x;
        o[2] = (float)k.y;
        o[3] = (float)k.z;
        sphere_to_uv(dir, &o[4], &o[5]);
        const V3 s = uv_to_sphere(r[12], r[13]);
        o[6] = s.x;
        o[7] = s.y;
        o[8] = s.z;
        o[9] = octahedron_hemisphere_pdf(*pr, dir, nrm, q);
        struct HostRand
        {
            ar_pcg g;
            float operator()() { return ar_rand1(&g); }
        } R;
        R.g = ar_pcg_init(seed, (uint64_t)i, 0);
        const GuideSample gsmp = sample_octahedron_hemisphere(*pr, R, nrm, q);
        o[10] = gsmp.dir.x;
        o[11] = gsmp.dir.y;
        o[12] = gsmp.dir.z;
        o[13] = gsmp.pdf;
    }
    delete pr;
    return AR_OK;
}

ar_status ar_host_rgb_encode(const float* rgb, int n, float* out)
{
    if (n < 0 || (n > 0 && (!rgb || !out))) return AR_ERR_INVALID;
    for (int i = 0; i < n; ++i) rgb_encode(rgb + 3 * (size_t)i, out + 4 * (size_t)i, AR_TAB_RGB_MLP);
    return AR_OK;
}

ar_status ar_host_lambda_encode(const float* lam, int n, float* out)
{
    if (n < 0 || (n > 0 && (!lam || !out))) return AR_ERR_INVALID;
    for (int i = 0; i < n; ++i) lambda_encode(lam[i], out + 4 * (size_t)i, AR_TAB_LAM_MLP);
    return AR_OK;
}

ar_status ar_host_sample_lambda(const float* u3, int n, float* lam, float* pdf)
{
    if (n < 0 || (n > 0 && (!u3 || !lam || !pdf))) return AR_ERR_INVALID;
    for (int i = 0; i < n; ++i)
    {
        const LambdaSample s = sample_cie1931(u3[3 * i], u3[3 * i + 1], u3[3 * i + 2]);
        lam[i] = s.lambda;
        pdf[i] = s.pdf;
    }
    return AR_OK;
}

} // extern "C"
