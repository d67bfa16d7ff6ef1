// Wavefront spectral path tracer (sm_103a) and the spectral LUT builder.
//
// The reference runs one megakernel thread per pixel sample through the whole
// path (CalculateRadiance, core/render/render.cuh:460-999).  Here each bounce is
// split into kernels over compacted queues of live paths:
//   raygen  -> camera ray + hero wavelength           (core/scene.cu:146-164, render.cuh:466-473)
//   extend  -> closest-hit traversal                  (render.cuh:77-108)
//   shade   -> material sample/eval, hit offset, emitter MIS, NEE light sample,
//              Russian roulette, next ray             (render.cuh:109-163, 541-907)
//   shadow  -> any-hit traversal of the NEE segments  (render.cuh:254-263)
//   finalize/accumulate -> XYZ per sample, FP64 per-pixel sums in sample order.
// Per path, random numbers are drawn in exactly the reference's order, so the
// GPU replays the reference's paths (see ar_rng.h for the stream layout).
// Queues are compacted with warp ballots and one atomic per warp.
#include <cuda_runtime.h>

#include <algorithm>

#include "ar_internal.h"
#include "ar_rng.h"

namespace ar
{
#define AR_BLOCK 256

__device__ __forceinline__ int lane_id() { return threadIdx.x & 31; }

// warp-aggregated append: one atomic per warp, order within the warp by lane
__device__ __forceinline__ int warp_append_slot(int* counter, bool pred)
{
    const unsigned m = __ballot_sync(0xffffffffu, pred);
    int base = 0;
    if (lane_id() == 0 && m) base = atomicAdd(counter, __popc(m));
    base = __shfl_sync(0xffffffffu, base, 0);
    return base + __popc(m & ((1u << lane_id()) - 1u));
}

struct DevRand
{
    ar_pcg g;
    __device__ float operator()() { return ar_rand1(&g); }
};

// ---------------------------------------------------------------- LUT build
// RGB -> basis LUT, one lattice point per thread; MLP weights staged in shared
// memory (34 KB, read as broadcast), the same arithmetic as rgb_encode.
__global__ void __launch_bounds__(AR_BLOCK) k_build_rgb_lut(float4* __restrict__ lut, const float* __restrict__ w)
{
    __shared__ float sw[AR_RGB_MLP_FLOATS];
    for (int i = threadIdx.x; i < AR_RGB_MLP_FLOATS; i += blockDim.x) sw[i] = w[i];
    __syncthreads();
    const long long total = (long long)AR_LUT_RES * AR_LUT_RES * AR_LUT_RES;
    const float invRes = 1.0f / static_cast<float>(AR_LUT_RES);
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < total; v += (long long)gridDim.x * blockDim.x)
    {
        const int x = (int)(v % AR_LUT_RES);
        const int y = (int)((v / AR_LUT_RES) % AR_LUT_RES);
        const int z = (int)(v / ((long long)AR_LUT_RES * AR_LUT_RES));
        const float in3[3] = {(x + 0.5f) * invRes, (y + 0.5f) * invRes, (z + 0.5f) * invRes};
        float o[4];
        rgb_encode(in3, o, sw);
        lut[v] = make_float4(o[0], o[1], o[2], o[3]);
    }
}

cudaError_t launch_build_rgb_lut(float* lut, const float* weights_dev, cudaStream_t s)
{
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    k_build_rgb_lut<<<sms * 4, AR_BLOCK, 0, s>>>(reinterpret_cast<float4*>(lut), weights_dev);
    return cudaGetLastError();
}

// Per-material spectral colours (albedo and emission bases), computed with
// the same trilinear LUT query the reference performs per interaction.
__global__ void k_prepare_materials(Material* mats, int n, const float* __restrict__ lut)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const PlainFetch f{lut};
    mats[i].albedo_c = prepare_color(mats[i].albedo, f);
    mats[i].emissive_c = prepare_color(mats[i].emissive, f);
}

cudaError_t launch_prepare_materials(Material* mats, int n, const float* lut, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    k_prepare_materials<<<(n + 127) / 128, 128, 0, s>>>(mats, n, lut);
    return cudaGetLastError();
}

// ---------------------------------------------------------------- hit reconstruction
// Full hit record for primitive slot `slot` at distance t (the traversal's t);
// SDF hits (the union and SDF objects) take the normal k_extend stored in *sdf_nrm.
__device__ __forceinline__ void hit_context(const DevScene& sc, int slot, V3 o, V3 d, float t, Hit* h,
                                            const float4* sdf_nrm)
{
    if (slot == AR_SLOT_SDF)
    {
        const int id = sc.trav.sdf_id;
        h->hit = true;
        h->obj = id;
        h->light = sc.prim_light[id];
        h->material = sc.prim_material[id];
        h->dist = t;
        h->pos = o + d * t;
        const float4 n = *sdf_nrm;
        h->nrm = v3(n.x, n.y, n.z);
        h->local_pos = h->pos;
        return;
    }
    const bool sdf_obj = slot <= AR_SLOT_SDFOBJ_BASE;
    const float4 a = sdf_obj ? __ldg(&sc.sdf_trav.slots[3 * (size_t)(AR_SLOT_SDFOBJ_BASE - slot)])
                             : __ldg(&sc.trav.slots[3 * (size_t)slot + 0]);
    const uint32_t tag = __float_as_uint(a.w);
    const uint32_t kind = tag >> AR_PRIM_KIND_SHIFT;
    const int id = (int)(tag & AR_PRIM_ID_MASK);
    h->hit = true;
    h->obj = id;
    h->dist = t;
    if (kind == AR_PRIM_KIND_TRI)
    {
        // triangle slots carry their primitive's material and light index in the
        // spare w lanes (filled at upload): no dependent per-primitive table reads
        const float4 b = __ldg(&sc.trav.slots[3 * (size_t)slot + 1]);
        const float4 c = __ldg(&sc.trav.slots[3 * (size_t)slot + 2]);
        h->material = __float_as_int(b.w);
        h->light = __float_as_int(c.w);
        tri_frame(o, d, t, v3(a.x, a.y, a.z), v3(b.x, b.y, b.z), v3(c.x, c.y, c.z), &h->pos, &h->nrm);
        h->local_pos = v3(0.0f, 0.0f, 0.0f);
    }
    else if (kind == AR_PRIM_KIND_SDF)
    {
        h->material = sc.prim_material[id];
        h->light = sc.prim_light[id];
        // IntersectSDFObject's hit frame (core/object/sdf/sdf_base.cuh:140-151); slot is in sdf_trav
        const Object ob = sc.trav.objects[id];
        const V3 lo = mul(ob.w2o, o - ob.center);
        const V3 ld = normalize(mul(ob.w2o, d));
        const V3 lp = lo + ld * t;
        h->pos = mul(ob.o2w, lp) + ob.center;
        const float4 n = *sdf_nrm;
        h->nrm = v3(n.x, n.y, n.z);
        h->local_pos = lp;
    }
    else
    {
        h->material = sc.prim_material[id];
        h->light = sc.prim_light[id];
        const Object ob = sc.trav.objects[id];
        if (kind == AR_PRIM_KIND_BOX) intersect_box(o, d, ob, h, true);
        else intersect_sphere(o, d, ob, h, true);
    }
}

// Albedo texel at a triangle hit: the mesh uv interpolated with the
// barycentric weights of pos, nearest texel, clamped to the edge.  Returns the
// texel index (in RGB units) or -1 when the primitive is not a triangle.
__device__ __forceinline__ int albedo_texel(const DevScene& sc, int tex, int slot, int prim, V3 pos)
{
    if (slot < 0) return -1;
    const float4 a = __ldg(&sc.trav.slots[3 * (size_t)slot + 0]);
    if ((__float_as_uint(a.w) >> AR_PRIM_KIND_SHIFT) != AR_PRIM_KIND_TRI) return -1;
    const float4 b = __ldg(&sc.trav.slots[3 * (size_t)slot + 1]);
    const float4 c = __ldg(&sc.trav.slots[3 * (size_t)slot + 2]);
    const V3 v0 = v3(a.x, a.y, a.z);
    const V3 e1 = v3(b.x, b.y, b.z) - v0, e2 = v3(c.x, c.y, c.z) - v0, d = pos - v0;
    const float d00 = dot(e1, e1), d01 = dot(e1, e2), d11 = dot(e2, e2);
    const float d20 = dot(d, e1), d21 = dot(d, e2);
    const float den = d00 * d11 - d01 * d01;
    float b1 = 0.0f, b2 = 0.0f;
    if (den > 0.0f)
    {
        b1 = (d11 * d20 - d01 * d21) / den;
        b2 = (d00 * d21 - d01 * d20) / den;
    }
    const float b0 = 1.0f - b1 - b2;
    const float* uv = sc.prim_uv + 6 * (size_t)prim;
    float u = b0 * __ldg(uv + 0) + b1 * __ldg(uv + 2) + b2 * __ldg(uv + 4);
    float v = b0 * __ldg(uv + 1) + b1 * __ldg(uv + 3) + b2 * __ldg(uv + 5);
    if (!(u == u)) u = 0.0f;
    if (!(v == v)) v = 0.0f;
    const int4 ti = __ldg(&sc.tex_info[tex]);
    const int x = min(max((int)floorf(fminf(fmaxf(u, 0.0f), 1.0f) * (float)ti.y), 0), ti.y - 1);
    const int y = min(max((int)floorf(fminf(fmaxf(v, 0.0f), 1.0f) * (float)ti.z), 0), ti.z - 1);
    return ti.x + y * ti.y + x;
}

// counters of a render wave (c.d_counters / the allocation-free scratch)
#define AR_CNT_Q0 0          // queue 0 length
#define AR_CNT_Q1 1          // queue 1 length
#define AR_CNT_SHADOW 2
#define AR_CNT_MLP 3
#define AR_CNT_FETCH 4       // k_extend, k_shadow fetch counters
#define AR_CNT_PEND 6        // pending SDF work of k_extend, k_shadow
#define AR_CNT_PART 8        // k_partition: hits placed from the front, misses from the back

// ---------------------------------------------------------------- raygen
struct CamParams
{
    V3 o, d, right, up;
    float tan_x, tan_y;
};

__global__ void __launch_bounds__(AR_BLOCK) k_raygen(PathState ps, int* queue, int* counter, long long first_path, int n,
                                                   int width, int height, uint64_t seed, int first_frame, CamParams cam,
                                                   int camera_inside, int* fetch_reset, bool media_record,
                                                   bool frame_record, PathOrder po,
                                                   const ulonglong2* __restrict__ jumps)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k == 0)
    {
        *counter = n;
        *fetch_reset = 0;  // the first k_extend's fetch counter
    }
    // stream jumps per sample: the render's table, or (allocation-free renders)
    // those of the samples this block's paths can belong to (its first path's
    // block of samples and the next: 2 x po.block frames), computed once
    __shared__ uint64_t s_jump[2 * AR_SAMPLE_BLOCK][2];
    uint32_t s_base = 0u, n_jump = 0u;
    if (!jumps)  // the same for every thread of the launch
    {
        const long long g_first = first_path + (long long)blockIdx.x * blockDim.x;
        s_base = (uint32_t)(g_first / ((long long)po.npix * po.block)) * po.block;
        n_jump = 2 * po.block;
        if (threadIdx.x < n_jump)
        {
            uint64_t m, c;
            ar_pcg_jump((uint64_t)(s_base + threadIdx.x + (uint32_t)first_frame) << 32, &m, &c);
            s_jump[threadIdx.x][0] = m;
            s_jump[threadIdx.x][1] = c;
        }
        __syncthreads();
    }
    if (k >= n) return;
    const long long g = first_path + k;
    uint32_t slot, smp;
    path_slot(po, (unsigned long long)g, &slot, &smp);
    const uint32_t pixel = slot_pixel(slot, (uint32_t)width, (uint32_t)height);
    const uint32_t frame = smp + (uint32_t)first_frame;
    const int i = (int)(pixel % (uint32_t)width), j = (int)(pixel / (uint32_t)width);
    DevRand R;
    const uint32_t jf = smp - s_base;
    if (jumps)
    {
        const ulonglong2 jm = jumps[smp];
        R.g = ar_pcg_init_jumped(seed, pixel, frame, jm.x, jm.y);
    }
    else if (smp >= s_base && jf < n_jump)
        R.g = ar_pcg_init_jumped(seed, pixel, frame, s_jump[jf][0], s_jump[jf][1]);
    else
        R.g = ar_pcg_init(seed, pixel, frame);  // blocks spanning more samples (images under 256 pixels)
    const float u = (i + R()) / static_cast<float>(width);
    const float v = (j + R()) / static_cast<float>(height);
    const float nx = u * 2.f - 1.f;
    const float ny = (float)((1.0 - (double)v) * 2.f - 1.f);
    const float sx = nx * cam.tan_x;
    const float sy = ny * cam.tan_y;
    V3 dir = normalize(cam.d + cam.right * sx + cam.up * sy);
    dir = normalize(dir);  // CalculateRadiance normalizes its input again
    const float r0 = R(), r1 = R(), r2 = R();
    const LambdaSample ls = sample_cie1931(r0, r1, r2);
    ps.rng[k] = R.g.state;
    ps.pixel[k] = pixel;
    if (frame_record) ps.frame[k] = frame;  // read by the guided shading only
    ps.ray_o[k] = make_float4(cam.o.x, cam.o.y, cam.o.z, ls.lambda);
    ps.ray_d[k] = make_float4(dir.x, dir.y, dir.z, ls.pdf);
    ps.radiance[k] = 0.0f;
    ps.mask[k] = 1.0f;
    ps.depths[k] = 0u;
    ps.flags[k] = camera_inside ? 1u : 0u;
    // the media record is read only by shading instantiations that track media
    // (and by k_extend for rays inside an object); prev (last vertex, pdf) is
    // read only after a vertex has written it (flag bit 1)
    if (media_record)
    {
        ps.media_v[k] = make_float4(cam.o.x, cam.o.y, cam.o.z, __int_as_float(-1));
        ps.media_depth[k] = 0;
    }
    queue[k] = k;
}

// ---------------------------------------------------------------- extend
// The traversal kernels are persistent over the queue: a warp's lanes take
// rays from a global fetch counter, step their traversals, and whenever at
// least a threshold of lanes have finished, the warp fetches that many new rays
// (one atomic per warp), so lanes do not idle behind the warp's longest ray.
#ifndef AR_EXT_REFILL_MIN
#define AR_EXT_REFILL_MIN 4      // closest hit: idle lanes that trigger a refill
#endif
#ifndef AR_EXT_STEPS
#define AR_EXT_STEPS 8           // closest hit: node visits between refill checks
#endif
#ifndef AR_SHD_REFILL_MIN
#define AR_SHD_REFILL_MIN 8      // shadow rays
#endif
#ifndef AR_SHD_STEPS
#define AR_SHD_STEPS 16
#endif
#ifndef AR_EXT_REFILL_MIN0
#define AR_EXT_REFILL_MIN0 32    // camera rays: a warp refills only when all its lanes are idle
#endif
#ifndef AR_SHD_REFILL_MIN0
#define AR_SHD_REFILL_MIN0 32    // shadow rays of the first vertices
#endif
#ifndef AR_SHADE_MLP_MIN_BLOCKS
#define AR_SHADE_MLP_MIN_BLOCKS 2    // k_shade<2> (MLP guide): blocks per SM it is compiled for (at 1,
                                     // 201 registers and 11 % of warps active: 3.5 % slower)
#endif
#ifndef AR_SHADE_PATHS_PER_THREAD
#define AR_SHADE_PATHS_PER_THREAD 16  // k_shade's grid: one thread per this many paths of the wave (a
                                      // grid-stride loop that prefetches each next pass's path state;
                                      // 64-spp terrain step: 2, 4, 8, 16 paths per thread gave 85.1,
                                      // 83.8, 83.0, 82.8 ms)
#endif
#ifndef AR_TRAV_MIN_BLOCKS
#define AR_TRAV_MIN_BLOCKS 4     // blocks per SM the traversal kernels are compiled for (64 registers)
#endif

// Warp-wide fetch of rays for the idle lanes: true and *q = the lane's queue
// index when it got one; *exhausted (warp-uniform) once the queue is used up.
__device__ __forceinline__ bool warp_refill(int* fetch, int n, bool active, bool* exhausted, int* q, int min_idle)
{
    const unsigned idle = __ballot_sync(0xffffffffu, !active);
    if (*exhausted || __popc(idle) < min_idle) return false;
    const int need = __popc(idle);
    const int leader = __ffs(idle) - 1;
    int base = 0;
    if (lane_id() == leader) base = atomicAdd(fetch, need);
    base = __shfl_sync(0xffffffffu, base, leader);
    if (base + need >= n) *exhausted = true;
    if (active) return false;
    *q = base + __popc(idle & ((1u << lane_id()) - 1u));
    return *q < n;
}

// Counters a kernel zeroes for later kernels of the wave (block 0, thread 0,
// before any other work): each is one that the kernel itself does not use and
// that no kernel still running could use, so the per-depth counter resets need
// no memset launches.
struct CounterReset
{
    int* a;
    int* b;
    int* c;
    int* d;
    int* e = nullptr;
    int* f = nullptr;
};

__device__ __forceinline__ void reset_counters(const CounterReset& r)
{
    if (blockIdx.x == 0 && threadIdx.x == 0)
    {
        if (r.a) *r.a = 0;
        if (r.b) *r.b = 0;
        if (r.c) *r.c = 0;
        if (r.d) *r.d = 0;
        if (r.e) *r.e = 0;
        if (r.f) *r.f = 0;
    }
}

// Shadow rays the traversal left unoccluded, for k_sdf_shadow (list ==
// nullptr when the scene has no SDF geometry).
struct SdfPending
{
    int* list;
    int* count;
};

// closest hit of a finished traversal of the main BVH
__device__ __forceinline__ void extend_finish(const DevScene& sc, const PathState& ps, int p, int q,
                                              const TravState<false>& st)
{
    const TravResult r = st.result();
    if (sc.stats)
    {
        atomicAdd(&sc.stats[0], (unsigned long long)st.n_visits);
        atomicAdd(&sc.stats[1], (unsigned long long)st.n_tests);
        atomicAdd(&sc.stats[4], 1ull);
    }
    ps.hit_t[p] = r.t;
    ps.hit_slot[p] = r.slot;
    ps.q_slot[q] = r.slot;
}

// The SDF pass of the closest hits (scenes with SDF geometry only): the SDF
// objects' BVH from the main BVH's hit, then the smooth union (marched up to
// the hit so far; it has the largest primitive id, so a hit at equal t wins),
// and the normal of an SDF hit (central differences of the field), which
// k_shade reads from hit_nrm.  Rays inside an SDF object test only it.
__global__ void __launch_bounds__(AR_BLOCK) k_sdf_extend(DevScene sc, PathState ps, const int* __restrict__ queue,
                                                       const int* __restrict__ counter)
{
    const int n = *counter;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x)
    {
        const int p = queue[q];
        const float4 ro = ps.ray_o[p], rd = ps.ray_d[p];
        const V3 o = v3(ro.x, ro.y, ro.z), d = v3(rd.x, rd.y, rd.z);
        const float tmin = intersect_eps((int)(ps.depths[p] >> 16));
        const float seps = 0.5f * fmaxf(tmin, 1.0e-3f);
        int slot = ps.hit_slot[p];
        float t = ps.hit_t[p];
        int sdf_obj_slot = -1;  // slot in the SDF objects' BVH of an SDF object hit
        if (slot == AR_SLOT_SOLO)
        {
            const int s = sc.prim_slot[__float_as_int(ps.media_v[p].w)];
            int id;
            const float th = prim_hit<true>(sc.sdf_trav, s, make_shear(d), o, d, &id, tmin, seps);
            slot = -1;
            t = 0.0f;
            if (th >= tmin)
            {
                sdf_obj_slot = s;
                t = th;
            }
        }
        else
        {
            TravResult r;
            r.slot = slot;
            r.t = slot >= 0 ? t : __int_as_float(0x7f800000);
            r.id = slot >= 0 ? (int)(__float_as_uint(sc.trav.slots[3 * (size_t)slot].w) & AR_PRIM_ID_MASK) : -1;
            const TravResult r2 = sdf_bvh_trace<false>(sc.sdf_trav, o, d, tmin, __int_as_float(0x7f800000), seps, r);
            if (r2.id != r.id)
            {
                sdf_obj_slot = r2.slot;
                slot = -1;
                t = r2.t;
            }
            const bool any = slot >= 0 || sdf_obj_slot >= 0;
            if (sc.trav.sdf.count > 0)
            {
                const float ts = sdf_march(sc.trav.sdf, o, d, sdf_eps(tmin), any ? t : 3.0e38f);
                if (ts >= tmin && (!any || ts < t))
                {
                    t = ts;
                    slot = AR_SLOT_SDF;
                    sdf_obj_slot = -1;
                }
            }
        }
        if (slot == AR_SLOT_SDF)
        {
            const V3 nn = sdf_normal(sc.trav.sdf, o + d * t, 1.0e-4f);
            ps.hit_nrm[p] = make_float4(nn.x, nn.y, nn.z, 0.0f);
        }
        else if (sdf_obj_slot >= 0)
        {
            const int id = (int)(__float_as_uint(sc.sdf_trav.slots[3 * (size_t)sdf_obj_slot].w) & AR_PRIM_ID_MASK);
            const Object ob = sc.trav.objects[id];
            const V3 lo = mul(ob.w2o, o - ob.center);
            const V3 ld = normalize(mul(ob.w2o, d));
            const V3 nn = sdf_obj_normal(sdf_obj_field(sc.trav, ob, id), ob.extent, ob.o2w, lo + ld * t, seps);
            ps.hit_nrm[p] = make_float4(nn.x, nn.y, nn.z, 0.0f);
            slot = AR_SLOT_SDFOBJ_BASE - sdf_obj_slot;
        }
        ps.hit_t[p] = t;
        ps.hit_slot[p] = slot;
        ps.q_slot[q] = slot;
    }
}

__global__ void __launch_bounds__(AR_BLOCK, AR_TRAV_MIN_BLOCKS) k_extend(DevScene sc, PathState ps, const int* __restrict__ queue,
                                                   const int* __restrict__ counter, int* fetch, unsigned int* err,
                                                   int min_idle, CounterReset rs)
{
    reset_counters(rs);
    const int n = *counter;
    TravState<false> st;
    uint2 stk[AR_TRAV_STACK];
    int p = 0, q = 0;
    bool active = false, exhausted = false;
    while (true)
    {
        if (warp_refill(fetch, n, active, &exhausted, &q, min_idle))
        {
            p = queue[q];
            const float4 ro = ps.ray_o[p], rd = ps.ray_d[p];
            const V3 o = v3(ro.x, ro.y, ro.z), d = v3(rd.x, rd.y, rd.z);
            const float tmin = intersect_eps((int)(ps.depths[p] >> 16));
            // the media record is read only for rays inside an object (rare)
            const int mobj = (ps.flags[p] & 1u) ? __float_as_int(ps.media_v[p].w) : -1;
            if (mobj >= 0)
            {
                // inside a medium: intersect only the enclosing object (render.cuh:89-92);
                // an SDF object is left to the SDF pass
                if (sc.trav.objects[mobj].type == AR_OBJ_SDF)
                {
                    ps.hit_t[p] = 0.0f;
                    ps.hit_slot[p] = AR_SLOT_SOLO;
                    ps.q_slot[q] = AR_SLOT_SOLO;
                }
                else
                {
                    const int s = sc.prim_slot[mobj];
                    int id;
                    const float th = prim_hit<false>(sc.trav, s, make_shear(d), o, d, &id, tmin);
                    ps.hit_t[p] = th >= tmin ? th : 0.0f;
                    ps.hit_slot[p] = th >= tmin ? s : -1;
                    ps.q_slot[q] = th >= tmin ? s : -1;
                }
                if (sc.stats) atomicAdd(&sc.stats[4], 1ull);
            }
            else
            {
                st.init(sc.trav, o, d, tmin, __int_as_float(0x7f800000), stk);
                active = true;
            }
        }
        if (__ballot_sync(0xffffffffu, active) == 0)
        {
            if (exhausted) break;
            continue;
        }
        if (active)
        {
            for (int it = 0; it < AR_EXT_STEPS; ++it)
            {
                if (!st.step(sc.trav, err))
                {
                    extend_finish(sc, ps, p, q, st);
                    active = false;
                    break;
                }
            }
        }
    }
}

// Camera rays (depth 0) as warp packets.  A warp takes 32 consecutive queue
// entries; in the path order they are samples of one pixel (or of a few
// neighbouring pixels), so the rays share the camera's origin and nearly
// share a direction.  The warp walks the BVH once for all of them: lanes 0-7
// test the 8 children of the current node against the whole packet with
// interval arithmetic over the lanes' inverse directions (a conservative test:
// a child that any lane's ray meets is never rejected), and every lane then
// runs its own exact primitive tests over the union of the leaves the packet
// meets, keeping its own closest hit with the smaller-id rule for equal t.  A
// lane therefore sees every primitive its own traversal would: the hits are
// the per-ray traversal's, bit for bit.  Warps whose rays do not share an
// origin and a direction octant (or with fewer than 32 rays) run the per-ray
// traversal instead.
#define AR_PACKET_MAX_VISITS (1 << 22)  // node visits of one packet before it gives up (error word)

__device__ __forceinline__ float warp_min(float v)
{
    for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

__device__ __forceinline__ float warp_max(float v)
{
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

__global__ void __launch_bounds__(AR_BLOCK) k_extend_camera(DevScene sc, PathState ps, const int* __restrict__ queue,
                                                           const int* __restrict__ counter, unsigned int* err,
                                                           CounterReset rs)
{
    reset_counters(rs);
    const int n = *counter;
    __shared__ uint2 s_stack[AR_BLOCK / 32][AR_TRAV_STACK];
    const int lane = lane_id(), wib = threadIdx.x >> 5;
    uint2* stack = s_stack[wib];
    const int warps = gridDim.x * (blockDim.x >> 5);
    for (int w = blockIdx.x * (blockDim.x >> 5) + wib; (long long)w * 32 < n; w += warps)
    {
        const int q = w * 32 + lane;
        const bool active = q < n;
        const int p = active ? queue[q] : 0;
        V3 o = v3(0, 0, 0), d = v3(1, 1, 1);
        float tmin = 0.0f;
        if (active)
        {
            const float4 ro = ps.ray_o[p], rd = ps.ray_d[p];
            o = v3(ro.x, ro.y, ro.z);
            d = v3(rd.x, rd.y, rd.z);
            tmin = intersect_eps((int)(ps.depths[p] >> 16));
        }
        const uint32_t oct = (d.x < 0.0f ? 1u : 0u) | (d.y < 0.0f ? 2u : 0u) | (d.z < 0.0f ? 4u : 0u);
        const V3 o0 = v3(__shfl_sync(0xffffffffu, o.x, 0), __shfl_sync(0xffffffffu, o.y, 0),
                         __shfl_sync(0xffffffffu, o.z, 0));
        const uint32_t oct0 = __shfl_sync(0xffffffffu, oct, 0);
        const float tmin0 = __shfl_sync(0xffffffffu, tmin, 0);
        const bool same = active && o.x == o0.x && o.y == o0.y && o.z == o0.z && oct == oct0 && tmin == tmin0 &&
                          d.x != 0.0f && d.y != 0.0f && d.z != 0.0f;
        const bool packet = __all_sync(0xffffffffu, same) && sc.trav.node_count > 0;
        if (!packet)
        {
            // the per-ray traversal, each lane to the end of its ray
            if (active)
            {
                TravState<false> st;
                uint2 stk[AR_TRAV_STACK];
                st.init(sc.trav, o, d, tmin, __int_as_float(0x7f800000), stk);
                while (st.step(sc.trav, err)) {}
                extend_finish(sc, ps, p, q, st);
            }
            continue;
        }
        // ---- packet: interval inverse directions (all of one sign per axis)
        const V3 inv = v3(inv_safe(d.x), inv_safe(d.y), inv_safe(d.z));
        const V3 inv_lo = v3(warp_min(inv.x), warp_min(inv.y), warp_min(inv.z));
        const V3 inv_hi = v3(warp_max(inv.x), warp_max(inv.y), warp_max(inv.z));
        const V3 inv_abs = v3(fmaxf(fabsf(inv_lo.x), fabsf(inv_hi.x)), fmaxf(fabsf(inv_lo.y), fabsf(inv_hi.y)),
                              fmaxf(fabsf(inv_lo.z), fabsf(inv_hi.z)));
        const RayShear sh = make_shear(d);
        float res_t = __int_as_float(0x7f800000);
        int res_slot = -1, res_id = -1;
        uint32_t n_visits = 0, n_tests = 0;
        int node = 0, sp = 0;
        bool failed = false;
        while (true)
        {
            if (node >= 0)
            {
                if (++n_visits > AR_PACKET_MAX_VISITS)
                {
                    failed = true;
                    break;
                }
                const uint4* np = sc.trav.nodes + 5 * (size_t)node;
                const uint4 w0 = __ldg(np + 0), w1 = __ldg(np + 1), w2 = __ldg(np + 2), w3 = __ldg(np + 3),
                            w4 = __ldg(np + 4);
                const uint32_t imask = w0.w >> 24;
                const uint32_t child_base = w1.x, prim_base = w1.y;
                // lanes 0-7 test the 8 children against the whole packet; the packet's far limit: the farthest closest-hit so far (t >= 0: bit order is value order)
                const float tlim = __uint_as_float(__reduce_max_sync(0xffffffffu, __float_as_uint(res_t)));
                const bool hit = lane < 8 && packet_child_meets(w0, w1, w2, w3, w4, lane, o0, oct0, inv_lo, inv_hi,
                                                                inv_abs, tmin0, tlim);
                const uint32_t hb = __ballot_sync(0xffffffffu, hit) & 0xffu;
                uint32_t hit_int = 0u, hit_leaf = 0u;
                for (uint32_t m = hb; m; m &= m - 1u)
                {
                    const uint32_t sl = (uint32_t)(__ffs(m) - 1);
                    const uint32_t bit = 1u << (sl ^ oct0);
                    if ((imask >> sl) & 1u) hit_int |= bit;
                    else hit_leaf |= bit;
                }
                // every lane tests the primitives of the packet's leaves (near first) with its own ray
                while (hit_leaf)
                {
                    const uint32_t i = (uint32_t)(__ffs(hit_leaf) - 1);
                    hit_leaf &= hit_leaf - 1u;
                    const int sl = (int)(i ^ oct0);
                    const uint32_t meta = byte_of(w1.z, w1.w, sl);
                    const int cnt = (int)(meta >> 5);
                    const int first = (int)(prim_base + (meta & 31u));
                    for (int k = 0; k < cnt; ++k)
                    {
                        int id;
                        ++n_tests;
                        const float t = prim_hit<false>(sc.trav, first + k, sh, o, d, &id, tmin);
                        if (!(t >= tmin)) continue;
                        if (t < res_t || (t == res_t && res_id >= 0 && id < res_id))
                        {
                            res_t = t;
                            res_slot = first + k;
                            res_id = id;
                        }
                    }
                }
                node = -1;
                if (hit_int)
                {
                    const uint32_t i = (uint32_t)(__ffs(hit_int) - 1);
                    hit_int &= hit_int - 1u;
                    const uint32_t sl = i ^ oct0;
                    node = (int)(child_base + __popc(imask & ((1u << sl) - 1u)));
                    if (hit_int)
                    {
                        if (sp < AR_TRAV_STACK)
                        {
                            if (lane == 0) stack[sp] = make_uint2(child_base, hit_int | (imask << 8));
                            ++sp;
                        }
                        else
                        {
                            failed = true;
                            break;
                        }
                    }
                    __syncwarp();
                    continue;
                }
            }
            if (sp == 0) break;
            // the top group gives its nearest child; the group stays while children remain
            __syncwarp();
            const uint2 e = stack[sp - 1];
            uint32_t m = e.y & 0xffu;
            const uint32_t im = e.y >> 8;
            const uint32_t i = (uint32_t)(__ffs(m) - 1);
            m &= m - 1u;
            const uint32_t sl = i ^ oct0;
            node = (int)(e.x + __popc(im & ((1u << sl) - 1u)));
            __syncwarp();
            if (m)
            {
                if (lane == 0) stack[sp - 1].y = m | (im << 8);
            }
            else
                --sp;
            __syncwarp();
        }
        if (failed && lane == 0) atomicOr(err, AR_DEVERR_STACK);
        if (sc.stats)
        {
            atomicAdd(&sc.stats[0], (unsigned long long)n_visits);
            atomicAdd(&sc.stats[1], (unsigned long long)n_tests);
            atomicAdd(&sc.stats[4], 1ull);
        }
        ps.hit_t[p] = res_slot >= 0 ? res_t : __int_as_float(0x7f800000);
        ps.hit_slot[p] = res_slot;
        ps.q_slot[q] = res_slot;
    }
}

// MLP guide: the network inputs (position and reflected view direction) of
// the queued paths that hit a surface at one of their first AR_MLP_MAX_NDD
// non-delta vertices, outside media; those paths are appended to `list` (the
// inference queue) and flagged in q_pos.w, the others flagged off.
__global__ void __launch_bounds__(AR_BLOCK) k_mlp_query(DevScene sc, PathState ps, const int* __restrict__ queue,
                                                      const int* __restrict__ counter, int* list, int* list_counter)
{
    const int n = *counter;
    const int stride = gridDim.x * blockDim.x;
    for (int base = (blockIdx.x * blockDim.x + threadIdx.x) & ~31; base < n; base += stride)
    {
        const int q = base + lane_id();
        bool want = false;
        int p = 0;
        if (q < n)
        {
            p = queue[q];
            const int slot = ps.hit_slot[p];
            const int ndd = (int)(ps.depths[p] >> 16);
            want = slot != -1 && ndd < AR_MLP_MAX_NDD && (ps.flags[p] & 1u) == 0u;
            if (want)
            {
                const float4 ro = ps.ray_o[p], rd = ps.ray_d[p];
                Hit h;
                hit_context(sc, slot, v3(ro.x, ro.y, ro.z), v3(rd.x, rd.y, rd.z), ps.hit_t[p], &h, &ps.hit_nrm[p]);
                const V3 wr = reflect(v3(rd.x, rd.y, rd.z), h.nrm);
                ps.q_pos[p] = make_float4(h.pos.x, h.pos.y, h.pos.z, 1.0f);
                ps.q_wr[p] = make_float4(wr.x, wr.y, wr.z, 0.0f);
            }
            else
            {
                ps.q_pos[p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            }
        }
        const int slot_out = warp_append_slot(list_counter, want);
        if (want) list[slot_out] = p;
    }
}

// ---------------------------------------------------------------- shade
#ifndef AR_SHADE_LEAN_MIN_BLOCKS
#define AR_SHADE_LEAN_MIN_BLOCKS 2  // the same for the opaque-surface instantiation (AR_FEAT_SURFACE)
#endif
#ifndef AR_SHADE_MIN_BLOCKS
#define AR_SHADE_MIN_BLOCKS 2    // blocks per SM the unguided / voxel-guided shade kernels are compiled for
#endif
struct ShadeParams
{
    int use_nee;
    int max_depth;
    float* grad;  // replay adjoint: float32 texel gradients (3 per texel), or null
    int mlp_ready;  // MLP guide: the network has trained long enough to replace the voxel probes
    double* grad_medium;  // replay adjoint: d loss / d (medium albedo, medium emission), or null
    float4* gbuf;         // denoiser: first-hit record per path (2 float4), or null
};

// CollectRadiance (core/render/render.cuh:353-432) on the path's collection
// slots; valid bits live in flags bits 8..12.
__device__ __forceinline__ void collect_radiance(const PathState& ps, int p, uint32_t& fl, float endpointLe, V3 nextDir,
                                                 float segContrib, float rrProb, int ndd, bool allowStart, bool advance,
                                                 V3 rayDir, V3 hitLoc, V3 hitNrm)
{
    const int cap = ps.capacity;
    if (endpointLe != 0.0f)
    {
        const int hi = min(ndd, AR_PG_COLLECT_DEPTH);
        for (int i = 0; i < hi; ++i)
        {
            const float m = ps.pg_loc[i * cap + p].w;
            if (m != 0.0f)
            {
                float4 d = ps.pg_dir[i * cap + p];
                d.w = d.w + m * endpointLe;
                ps.pg_dir[i * cap + p] = d;
                fl |= 1u << (8 + i);
            }
        }
    }
    if (allowStart && ndd < AR_PG_COLLECT_DEPTH)
    {
        const float4 l = ps.pg_loc[ndd * cap + p];
        if (l.w == 0.0f)
        {
            const float w = ps.pg_dir[ndd * cap + p].w;
            ps.pg_dir[ndd * cap + p] = make_float4(nextDir.x, nextDir.y, nextDir.z, w);
            ps.pg_loc[ndd * cap + p] = make_float4(hitLoc.x, hitLoc.y, hitLoc.z, 1.0f);
            const V3 vd = reflect(rayDir, hitNrm);
            ps.pg_vdir[ndd * cap + p] = make_float4(vd.x, vd.y, vd.z, mlp_pack_normal(hitNrm));
        }
    }
    if (advance)
    {
        const float invQ = (float)(1.0 / (double)rrProb);
        const int hi = min(ndd + (allowStart ? 1 : 0), AR_PG_COLLECT_DEPTH);
        for (int i = 0; i < hi; ++i)
        {
            float4 l = ps.pg_loc[i * cap + p];
            if (l.w != 0.0f)
            {
                l.w = l.w * (segContrib * invQ);
                ps.pg_loc[i * cap + p] = l;
            }
        }
    }
}

// Prefetch into L2 of the path state k_shade reads first (and of the hit's
// primitive slot), for a path this thread shades in its next pass.
__device__ __forceinline__ void prefetch_l2(const void* a) { asm volatile("prefetch.global.L2 [%0];" ::"l"(a)); }

__device__ __forceinline__ void prefetch_shade_inputs(const DevScene& sc, const PathState& ps, int2 e)
{
    const int p = e.x;
    prefetch_l2(&ps.ray_o[p]);
    prefetch_l2(&ps.ray_d[p]);
    prefetch_l2(&ps.rng[p]);
    prefetch_l2(&ps.pixel[p]);
    prefetch_l2(&ps.depths[p]);
    prefetch_l2(&ps.flags[p]);
    prefetch_l2(&ps.radiance[p]);
    prefetch_l2(&ps.mask[p]);
    prefetch_l2(&ps.hit_t[p]);
    if (e.y >= 0)
    {
        const float4* sl = sc.trav.slots + 3 * (size_t)e.y;
        prefetch_l2(sl);
        prefetch_l2(sl + 2);
    }
}

// The extended queue ordered for shading: hits with their slot from the front,
// misses from the back.  k_shade then gives whole warps and blocks to one kind
// of work (a hit runs the BSDF, NEE and roulette; a miss adds the sky and
// ends) without reordering inside the kernel.  One atomic per block and end.
// Which thread shades which path does not change any path's result.
__global__ void __launch_bounds__(AR_BLOCK) k_partition(const int* __restrict__ queue, const int* __restrict__ q_slot,
                                                        const int* __restrict__ counter, int2* __restrict__ out,
                                                        int* front, int* back)
{
    const int n = *counter;
    __shared__ int s_hits[AR_BLOCK / 32], s_miss[AR_BLOCK / 32], s_base[2];
    const int w = threadIdx.x >> 5;
    for (int bbase = blockIdx.x * blockDim.x; bbase < n; bbase += gridDim.x * blockDim.x)
    {
        const int q = bbase + (int)threadIdx.x;
        const bool valid = q < n;
        const int p = valid ? queue[q] : -1;
        const int slot = valid ? q_slot[q] : -1;
        const bool hit = valid && slot != -1;
        const unsigned hb = __ballot_sync(0xffffffffu, hit), mb = __ballot_sync(0xffffffffu, valid && !hit);
        if (lane_id() == 0)
        {
            s_hits[w] = __popc(hb);
            s_miss[w] = __popc(mb);
        }
        __syncthreads();
        int hbase = 0, mbase = 0, th = 0, tm = 0;
        for (int k = 0; k < AR_BLOCK / 32; ++k)
        {
            if (k < w)
            {
                hbase += s_hits[k];
                mbase += s_miss[k];
            }
            th += s_hits[k];
            tm += s_miss[k];
        }
        if (threadIdx.x == 0)
        {
            s_base[0] = th ? atomicAdd(front, th) : 0;
            s_base[1] = tm ? atomicAdd(back, tm) : 0;
        }
        __syncthreads();
        const unsigned below = (1u << lane_id()) - 1u;
        if (hit) out[s_base[0] + hbase + __popc(hb & below)] = make_int2(p, slot);
        else if (valid) out[n - 1 - (s_base[1] + mbase + __popc(mb & below))] = make_int2(p, -1);
        __syncthreads();  // the shared counts are rewritten by the next pass
    }
}

// Scene features a k_shade instantiation handles, fixed at compile time: the
// BSDF models (AR_MATS_* bits), the participating medium and albedo textures.
// Scenes of opaque surfaces only (no glass, medium or textures, the camera
// outside every object) run an instantiation without that code: the same
// arithmetic for everything it keeps, less code and fewer registers.
#define AR_FEAT_MEDIUM (1 << 4)
#define AR_FEAT_TEX (1 << 5)
#define AR_FEAT_ALL (AR_MATS_ALL | AR_FEAT_MEDIUM | AR_FEAT_TEX)
#define AR_FEAT_SURFACE (AR_MATS_DIFFUSE | AR_MATS_LIGHT | AR_MATS_GGX)

template <int GUIDE, bool ADJ, int FEAT = AR_FEAT_ALL>
__global__ void __launch_bounds__(AR_BLOCK, GUIDE == 2 ? AR_SHADE_MLP_MIN_BLOCKS
                                            : (FEAT == AR_FEAT_SURFACE ? AR_SHADE_LEAN_MIN_BLOCKS : AR_SHADE_MIN_BLOCKS))
    k_shade(DevScene sc, PathState ps, ShadowQueue sq, const int2* __restrict__ queue,
                                                  const int* __restrict__ counter, int* next_queue, int* next_counter,
                                                  int* shadow_counter, ShadeParams prm)
{
    const int n = *counter;
    // blocks past the queue have nothing to do (the same for every thread of the
    // block): deep bounces often have few or no paths left
    if ((long long)blockIdx.x * blockDim.x >= n) return;
    __shared__ float s_lam[AR_LAMBDA_LUT_RES * 4];
    for (int i = threadIdx.x; i < AR_LAMBDA_LUT_RES * 4; i += blockDim.x) s_lam[i] = sc.lut_lambda[i];
    __syncthreads();
    const int stride = gridDim.x * blockDim.x;
    float g_med_albedo = 0.0f, g_med_emission = 0.0f;  // replay adjoint of the medium parameters
    // The queue comes from k_partition: {path, hit slot}, hits first.
    // Without glass the path never enters an object: its media record stays
    // the default and is neither read nor written.  Unguided forward renders
    // read nothing of an ended path but its radiance.
    constexpr bool TRACK_MEDIA = (FEAT & AR_MATS_GLASS) != 0;
    constexpr bool STORE_ENDED = GUIDE != 0 || ADJ;
    for (int bbase = blockIdx.x * blockDim.x; bbase < n; bbase += stride)
    {
        const int qq = bbase + (int)threadIdx.x;
        const bool active = qq < n;
        // the entry this thread shades in its next pass, read now; its state is
        // prefetched once this pass's own loads have arrived
        const int qn = qq + stride;
        const int2 next = qn < n ? queue[qn] : make_int2(-1, -1);
        bool keep = false;
        bool shadow = false;
        int p = 0;
        V3 sh_o = v3(0, 0, 0), sh_d = v3(0, 0, 0);
        float sh_tmax = 0.0f, sh_vun = 0.0f, sh_vocc = 0.0f, sh_sdf_eps = 0.0f;
        bool sh_valid = false;
        if (active)
        {
            const int2 entry = queue[qq];
            p = entry.x;
            const float4 ro = ps.ray_o[p], rd = ps.ray_d[p];
            const V3 rayO = v3(ro.x, ro.y, ro.z), rayD = v3(rd.x, rd.y, rd.z);
            const float lambda = ro.w;
            const Basis lb = query_lambda(lambda, s_lam);
            const float d65 = d65_norm(lambda, sc.d65);
            const uint32_t dep = ps.depths[p];
            int depth = (int)(dep & 0xffffu);
            int ndd = (int)(dep >> 16);
            uint32_t fl = ps.flags[p];
            Media media = media_default();
            if constexpr (TRACK_MEDIA)
            {
                const float4 mv = ps.media_v[p];
                media.inside = (fl & 1u) != 0u;
                media.vertex = v3(mv.x, mv.y, mv.z);
                media.obj = __float_as_int(mv.w);
                media.depth = ps.media_depth[p];
            }
            float radiance = ps.radiance[p];
            float mask = ps.mask[p];
            const bool prev_did_nee = (fl & 2u) != 0u;
            DevRand R;
            R.g.state = ps.rng[p];
            R.g.inc = ar_pcg_increment(ps.pixel[p]);

            const float eps = intersect_eps(ndd);
            const int slot = entry.y;
            Hit h;
            h.hit = false;
            h.obj = -1;
            h.light = -1;
            h.dist = 0.0f;
            h.pos = v3(0, 0, 0);
            h.nrm = v3(0, 0, 0);
            h.local_pos = v3(0, 0, 0);
            if (slot != -1) hit_context(sc, slot, rayO, rayD, ps.hit_t[p], &h, &ps.hit_nrm[p]);
            if (next.x >= 0) prefetch_shade_inputs(sc, ps, next);

            // ---- participating medium: a free flight sampled in the medium box
            // ends the segment early with probability 1 - transmittance
            bool scatter = false;
            if ((FEAT & AR_FEAT_MEDIUM) && sc.medium.on)
            {
                float m0, m1;
                if (medium_segment(sc.medium, rayO, rayD, 0.0f, h.hit ? h.dist : 3.0e38f, &m0, &m1))
                {
                    const float ts = m0 - arm_logf(R()) / sc.medium.sigma_t;
                    if (ts < m1)
                    {
                        scatter = true;
                        h.hit = false;
                        h.obj = -1;
                        h.light = -1;
                        h.dist = ts;
                        h.pos = rayO + rayD * ts;
                        h.nrm = v3(0.0f, 0.0f, 0.0f);
                    }
                }
            }

            // ---- Trace (render.cuh:109-155)
            BsdfSample S = bsdf_sample_default();
            Material mat;
            mat.shading = AR_MAT_DIFFUSE;
            if (!h.hit && !scatter && media.inside)
            {
                S.miss_thin = true;
                S.brdf = 1.0f;
                S.next_dir = rayD;
                S.pdf = 1.0f;
                h.local_pos = rayO;
                h.obj = media.obj;
                S.delta = true;
                S.emissive = v3(0, 0, 0);
                S.media.inside = false;
                S.media.vertex = h.local_pos;
            }
            int texel = -1;
            if (h.hit)
            {
                mat = sc.materials[h.material];
                if ((FEAT & AR_FEAT_TEX) && mat.albedo_tex >= 0 && sc.tex_count > 0)
                {
                    texel = albedo_texel(sc, mat.albedo_tex, slot, h.obj, h.pos);
                    if (texel >= 0)
                    {
                        const float* tx = sc.texels + 3 * (size_t)texel;
                        mat.albedo = v3(__ldg(tx), __ldg(tx + 1), __ldg(tx + 2));
                        mat.albedo_c = prepare_color(mat.albedo, PlainFetch{sc.lut_rgb});
                    }
                }
                S = evaluate_material<FEAT & AR_MATS_ALL>(lambda, lb, R, mat, rayD, h, media);
            }
            else if (scatter)
            {
                // Henyey-Greenstein phase sampling; throughput x albedo
                const float e0 = R();
                const float e1 = R();
                const DirSample ph = hg_sample(e0, e1, rayD, sc.medium.g);
                S.next_dir = ph.dir;
                S.pdf = ph.pdf;
                S.brdf = sc.medium.albedo * ph.pdf;
                S.delta = false;
                S.emissive = v3(0.0f, 0.0f, 0.0f);
                S.media = media;
            }
            else
            {
                S.brdf = 1.0f;
                S.delta = false;
                S.next_dir = rayD;
                S.pdf = 1.0f;
                S.emissive = sky_lighting(rayD);
                S.media.inside = false;
            }
            // denoiser G-buffer of the camera ray's hit (RecordScreenGBuffer at
            // depth 0, core/render/render.cuh:640-643): albedo (texel when
            // textured), material index (-1: no surface), normal, distance
            if constexpr (!ADJ)
            {
                if (prm.gbuf && depth == 0)
                {
                    const int mid = h.hit ? h.material : -1;
                    const V3 alb = h.hit ? mat.albedo : v3(0.0f, 0.0f, 0.0f);
                    prm.gbuf[2 * (size_t)p] = make_float4(alb.x, alb.y, alb.z, __int_as_float(mid));
                    prm.gbuf[2 * (size_t)p + 1] = make_float4(h.nrm.x, h.nrm.y, h.nrm.z, h.dist);
                }
            }
            {
                const float offsetEPS = eps * fmaxf(1.0f, length(h.pos));
                h.pos = h.pos + signf(dot(h.nrm, S.next_dir)) * h.nrm * offsetEPS * (R() + 0.5f);
            }
            media = S.media;

            // ---- guided mixture sampling (render.cuh:553-638)
            const Probe* probe = nullptr;
            V3 maskq = v3(1.0f, 1.0f, 1.0f);
            float pgProb = 0.0f;
            bool mlp_on = false;           // GUIDE == 2: this vertex mixes in the network's distribution
            const uint8_t* qcells = nullptr;  // its 64 quantised cell weights (the path's inference record)
            float q_total = 1.0f;
            if constexpr (GUIDE)
            {
                const float4 mq = ps.maskq[p];
                maskq = v3(mq.x, mq.y, mq.z);
                pgProb = guide_probability((int)ps.frame[p]);  // the path's own frame (waves may hold several)
                const bool eligible = h.hit && !S.delta && !S.pure_light && !media.inside;
                if constexpr (GUIDE == 2)
                {
                    if (eligible && prm.mlp_ready && ps.q_pos[p].w > 0.0f)
                    {
                        const uint8_t* q = ps.q_dist + 64 * (size_t)p;
                        qcells = q;
                        q_total = mlp_total(q);
                        mlp_on = true;
                        const float pB = S.pdf;
                        const float pP = mlp_hemisphere_pdf(q, 1.0f / q_total, S.next_dir, h.nrm);
                        if (pB > 1.0e-12f && pP > 1.0e-12f)
                        {
                            if (R() < pgProb)
                            {
                                const GuideSample g = mlp_sample_hemisphere(q, q_total, R, h.nrm);
                                if (dot(g.dir, h.nrm) > 1.0e-12f)
                                {
                                    const float pBs = bsdf_pdf<FEAT & AR_MATS_ALL>(lb, mat, h.nrm, rayD, g.dir);
                                    S.next_dir = g.dir;
                                    S.brdf = eval_bsdf_cos<FEAT & AR_MATS_ALL>(lambda, lb, mat, rayD, g.dir, h, media);
                                    S.pdf = (1.0f - pgProb) * fmaxf(pBs, 1.0e-12f) + pgProb * g.pdf;
                                }
                                else
                                {
                                    mlp_on = false;
                                }
                            }
                            else
                            {
                                S.pdf = (1.0f - pgProb) * pB + pgProb * pP;
                            }
                        }
                        else
                        {
                            mlp_on = false;
                        }
                    }
                }
                if (!mlp_on && eligible && sc.guide.probe_count > 0)
                {
                    const VoxelKey key = voxel_key(h.pos, reflect(rayD, h.nrm), sc.guide.inv_unit);
                    const int idx = guide_lookup(sc.guide, guide_pack(key));
                    if (idx >= 0)
                    {
                        probe = &sc.guide.probes[idx];
                        const float pB = S.pdf;
                        const float pP = octahedron_hemisphere_pdf(*probe, S.next_dir, h.nrm, maskq);
                        if (pB > 1.0e-12f && pP > 1.0e-12f)
                        {
                            if (R() < pgProb)
                            {
                                const GuideSample g = sample_octahedron_hemisphere(*probe, R, h.nrm, maskq);
                                if (dot(g.dir, h.nrm) > 1.0e-12f)
                                {
                                    const float pBs = bsdf_pdf<FEAT & AR_MATS_ALL>(lb, mat, h.nrm, rayD, g.dir);
                                    S.next_dir = g.dir;
                                    S.brdf = eval_bsdf_cos<FEAT & AR_MATS_ALL>(lambda, lb, mat, rayD, g.dir, h, media);
                                    S.pdf = (1.0f - pgProb) * fmaxf(pBs, 1.0e-12f) + pgProb * g.pdf;
                                }
                                else
                                {
                                    probe = nullptr;
                                }
                            }
                            else
                            {
                                S.pdf = (1.0f - pgProb) * pB + pgProb * pP;
                            }
                        }
                        else
                        {
                            probe = nullptr;
                        }
                    }
                }
            }

            // ---- emission (render.cuh:647-723)
            V3 endpointLe = v3(0.0f, 0.0f, 0.0f);
            float medium_unit = 0.0f;  // emission released at this scattering point per unit emission
            if (scatter)
            {
                medium_unit = mask * (1.0f - sc.medium.albedo) * d65;
                radiance = radiance + medium_unit * sc.medium.emission;
            }
            else if (!h.hit)
            {
                if (!S.miss_thin)
                {
                    endpointLe = S.emissive;
                    const PlainFetch f{sc.lut_rgb};
                    radiance = radiance + mask * interact_rgb(lb, S.emissive, f) * d65;
                }
            }
            else if (h.light >= 0)
            {
                float misW = 1.0f;
                if (prm.use_nee && depth > 0 && prev_did_nee)
                {
                    const float4 pv = ps.prev[p];
                    const float pB = fmaxf(pv.w, 0.0f);
                    const Light L = sc.lights[h.light];
                    float pL = 0.0f;
                    const V3 lastPos = v3(pv.x, pv.y, pv.z);
                    if (L.type == AR_OBJ_CUBE) pL = box_light_pdf_omega(sc.trav.objects[L.obj], L.select_prob, lastPos, h.pos, h.nrm);
                    else if (L.type == AR_OBJ_SPHERE) pL = sphere_light_pdf_omega(sc.trav.objects[L.obj], L.select_prob, lastPos, h.pos, h.nrm);
                    if (pL >= 0.0f && pB > 0.0f) misW = power_heuristic(pB, pL);
                }
                endpointLe = S.emissive * misW;
                radiance = radiance + mask * interact(mat.emissive_c, lb) * d65 * misW;
            }
            else if (!all_zero(S.emissive))
            {
                endpointLe = S.emissive;
            }
            if constexpr (ADJ)
            {
                // replay adjoint: every contribution still to come on this path
                // (NEE here, emission and NEE further on) carries this vertex's
                // albedo once; radiance holds the contributions that do not
                if (scatter && prm.grad_medium)
                {
                    // later contributions carry this albedo once; the emission here carries (1 - albedo)
                    const float dlt = ps.adj_delta[p];
                    const float a = sc.medium.albedo;
                    const float rest = ps.adj_total[p] - radiance;
                    if (a > 1.0e-8f) g_med_albedo += dlt * rest / a;
                    // d/d albedo of (1 - albedo) x emission x mask, and d/d emission
                    g_med_albedo -= dlt * mask * sc.medium.emission * d65;
                    g_med_emission += dlt * medium_unit;
                }
                if (prm.grad && texel >= 0 && mat.shading == AR_MAT_DIFFUSE)
                {
                    const float rest = ps.adj_total[p] - radiance;
                    const float dlt = ps.adj_delta[p];
                    const float alb = interact(mat.albedo_c, lb);
                    if (rest != 0.0f && dlt != 0.0f && alb > 1.0e-8f)
                    {
                        const V3 g = interact_rgb_grad(lb, mat.albedo, PlainFetch{sc.lut_rgb}) * (dlt * rest / alb);
                        float* gp = prm.grad + 3 * (size_t)texel;
                        if (g.x != 0.0f) atomicAdd(gp + 0, g.x);
                        if (g.y != 0.0f) atomicAdd(gp + 1, g.y);
                        if (g.z != 0.0f) atomicAdd(gp + 2, g.z);
                    }
                }
            }
            if constexpr (GUIDE)
            {
                const PlainFetch f{sc.lut_rgb};
                collect_radiance(ps, p, fl, interact_rgb(lb, endpointLe, f) * d65, S.next_dir, 0.0f, 1.0f, ndd, false,
                                 false, rayD, h.pos, h.nrm);
            }

            const bool ended = (!h.hit && !S.miss_thin && !scatter) || S.terminate;
            if (!ended)
            {
                // ---- NEE (render.cuh:766-827, 206-343)
                if (!S.miss_thin)
                {
                    const float useNEERate = sqrtf(saturate(mask));
                    bool neeValid = false;
                    if (prm.use_nee && ndd < AR_NEE_MAX_NON_DELTA_DEPTH && !S.delta && !media.inside && R() < useNEERate)
                    {
                        LightSample ls;
                        ls.valid = false;
                        if (sc.light_count > 0)
                        {
                            const float r = R();
                            int pick = sc.light_count - 1;
                            float pickProb = 0.0f;
                            // first light whose running CDF exceeds r (same as the sequential scan)
                            int lo = 0, hi = sc.light_count;
                            while (lo < hi)
                            {
                                const int mid = (lo + hi) >> 1;
                                if (r < sc.lights[mid].cdf) hi = mid;
                                else lo = mid + 1;
                            }
                            if (lo < sc.light_count)
                            {
                                pick = lo;
                                pickProb = sc.lights[lo].select_prob;
                            }
                            const Light L = sc.lights[pick];
                            if (L.type == AR_OBJ_CUBE) ls = sample_box_light(R, sc.trav.objects[L.obj], h.pos);
                            else if (L.type == AR_OBJ_SPHERE) ls = sample_sphere_light(R, sc.trav.objects[L.obj], h.pos);
                            if (ls.valid)
                            {
                                ls.obj = L.obj;
                                ls.material = L.material;
                                ls.p_facet = ls.p_facet * pickProb;
                            }
                        }
                        const float vZero = mask * 0.0f * d65;
                        if (!ls.valid)
                        {
                            radiance = radiance + vZero;
                        }
                        else
                        {
                            const float pATotal = fmaxf(1e-20f, ls.p_a * ls.p_facet);
                            const V3 lun = ls.point - h.pos;
                            const float dist2 = fmaxf(dot(lun, lun), (float)1.0e-12);
                            const V3 L = lun * arm_rsqrtf(dist2);
                            const float cosX = scatter ? 1.0f : fmaxf(0.0f, dot(h.nrm, L));
                            const float cosY = fmaxf(0.0f, dot(ls.normal, -L));
                            float vUn = vZero;
                            bool validUn = false;
                            if (!(cosX <= 0.0f || cosY <= 0.0f))
                            {
                                const float brdfCos =
                                    scatter ? sc.medium.albedo * hg_pdf(dot(rayD, L), sc.medium.g)
                                            : eval_bsdf_cos<FEAT & AR_MATS_ALL>(lambda, lb, mat, rayD, L, h, media_default());
                                const float G = (cosY / dist2);
                                const float le = interact(sc.materials[ls.material].emissive_c, lb);
                                const float contribution = brdfCos * le * (G / pATotal);
                                const float pLight = area_to_solid_angle_pdf(h.pos, ls.point, ls.normal, ls.p_facet * ls.p_a);
                                float pBsdf = scatter ? hg_pdf(dot(rayD, L), sc.medium.g)
                                                      : fmaxf(bsdf_pdf<FEAT & AR_MATS_ALL>(lb, mat, h.nrm, rayD, L), 0.0f);
                                if constexpr (GUIDE)
                                {
                                    if (probe)
                                        pBsdf = (1.0f - pgProb) * pBsdf +
                                                pgProb * octahedron_hemisphere_pdf(*probe, L, h.nrm, maskq);
                                    if (mlp_on)
                                        pBsdf = (1.0f - pgProb) * pBsdf +
                                                pgProb * mlp_hemisphere_pdf(qcells, 1.0f / q_total, L, h.nrm);
                                }
                                const float misW = power_heuristic(pLight, pBsdf);
                                vUn = mask * (contribution * misW) * d65;
                                if ((FEAT & AR_FEAT_MEDIUM) && sc.medium.on)
                                    vUn *= medium_transmittance(sc.medium, h.pos, L, sqrtf(dist2));
                                validUn = true;
                            }
                            // shadow segment (intersection.cuh:285-310)
                            V3 dirS = ls.point - h.pos;
                            const float distance = length(dirS);
                            bool traced = false;
                            if (distance > 0.0f)
                            {
                                dirS = dirS / distance;
                                const float seps = intersect_eps(depth) * fmaxf(1.0f, fmaxf(length(h.pos), length(ls.point)));
                                const float tmax = fmaxf(0.0f, distance - seps);
                                if (tmax > 0.0f)
                                {
                                    traced = true;
                                    shadow = true;
                                    sh_o = h.pos;
                                    sh_d = dirS;
                                    sh_tmax = tmax;
                                    sh_sdf_eps = 0.5f * intersect_eps(depth);  // SDF_EPS of the NEE depth
                                    sh_vun = vUn;
                                    sh_vocc = vZero;
                                    sh_valid = validUn;
                                }
                            }
                            if (!traced)
                            {
                                radiance = radiance + vUn;
                                neeValid = validUn;
                            }
                        }
                    }
                    fl = (fl & ~2u) | (neeValid ? 2u : 0u);
                    ps.prev[p] = make_float4(h.pos.x, h.pos.y, h.pos.z, S.pdf);
                }
                // ---- Russian roulette (render.cuh:829-859)
                const float contrib = S.brdf / fmaxf(S.pdf, 1e-12f);
                float pSurvive = 1.0f;
                bool survived = true;
                if (ndd >= AR_MIN_TRACING_DEPTH)
                {
                    const float basic = clampf(mask * 0.5f + mask * 0.5f, 0.05f, 0.95f);
                    pSurvive = lerpf(basic, 1.0f, media.inside ? AR_DELTA_RR_TERMINATE_REDUCE : 0.0f);
                    if (R() > pSurvive) survived = false;
                }
                if (survived)
                {
                    if constexpr (GUIDE)
                    {
                        const bool allowStart = h.hit && !S.delta && !S.pure_light && !media.inside;
                        collect_radiance(ps, p, fl, 0.0f, S.next_dir, contrib, pSurvive, ndd, allowStart, true, rayD, h.pos,
                                         h.nrm);
                    }
                    mask = mask * contrib;
                    mask = mask / pSurvive;
                    if constexpr (GUIDE)
                    {
                        const V3 xyz = lambda_to_xyz(lambda, sc.cie_cmf);
                        V3 q = vmax(mask * xyz, (float)AR_PG_QUERY_EPS);
                        const float div = (float)((double)sum3(q) + AR_PG_QUERY_EPS);
                        q = q / div;
                        ps.maskq[p] = make_float4(q.x, q.y, q.z, 0.0f);
                    }
                    if (!S.delta) ++ndd;
                    ++depth;
                    if (depth < prm.max_depth)
                    {
                        keep = true;
                        ps.ray_o[p] = make_float4(h.pos.x, h.pos.y, h.pos.z, lambda);
                        ps.ray_d[p] = make_float4(S.next_dir.x, S.next_dir.y, S.next_dir.z, rd.w);
                        ps.mask[p] = mask;
                        ps.depths[p] = (uint32_t)depth | ((uint32_t)ndd << 16);
                        fl = (fl & ~1u) | (media.inside ? 1u : 0u);
                        if constexpr (TRACK_MEDIA)
                        {
                            ps.media_v[p] = make_float4(media.vertex.x, media.vertex.y, media.vertex.z,
                                                        __int_as_float(media.obj));
                            ps.media_depth[p] = media.depth;
                        }
                    }
                }
            }
            ps.radiance[p] = radiance;
            if (STORE_ENDED || keep)
            {
                ps.flags[p] = fl;
                ps.rng[p] = R.g.state;
            }
        }
        const int nq = warp_append_slot(next_counter, keep);
        if (keep) next_queue[nq] = p;
        const int sqi = warp_append_slot(shadow_counter, shadow);
        if (shadow)
        {
            sq.path[sqi] = p;
            sq.o[sqi] = make_float4(sh_o.x, sh_o.y, sh_o.z, sh_tmax);
            sq.d[sqi] = make_float4(sh_d.x, sh_d.y, sh_d.z, sh_vun);
            sq.v_occ[sqi] = sh_vocc;
            sq.valid_unocc[sqi] = sh_valid ? 1 : 0;
            sq.sdf_eps[sqi] = sh_sdf_eps;
        }
    }
    if constexpr (ADJ)
    {
        if (prm.grad_medium)
        {
            for (int o = 16; o > 0; o >>= 1)
            {
                g_med_albedo += __shfl_xor_sync(0xffffffffu, g_med_albedo, o);
                g_med_emission += __shfl_xor_sync(0xffffffffu, g_med_emission, o);
            }
            if (lane_id() == 0 && (g_med_albedo != 0.0f || g_med_emission != 0.0f))
            {
                atomicAdd(prm.grad_medium, (double)g_med_albedo);
                atomicAdd(prm.grad_medium + 1, (double)g_med_emission);
            }
        }
    }
}

// ---------------------------------------------------------------- shadow
__device__ __forceinline__ void shadow_apply(const PathState& ps, const ShadowQueue& sq, int i, int p, bool occluded)
{
    ps.radiance[p] = ps.radiance[p] + (occluded ? sq.v_occ[i] : sq.d[i].w);
    const bool valid = occluded ? true : (sq.valid_unocc[i] != 0);
    ps.flags[p] = (ps.flags[p] & ~2u) | (valid ? 2u : 0u);
}

__device__ __forceinline__ void shadow_finish(const DevScene& sc, const PathState& ps, const ShadowQueue& sq, int i,
                                              int p, const TravState<true>& st, const SdfPending& pend)
{
    const bool occluded = st.result().slot >= 0;
    if (sc.stats)
    {
        atomicAdd(&sc.stats[2], (unsigned long long)st.n_visits);
        atomicAdd(&sc.stats[3], (unsigned long long)st.n_tests);
        atomicAdd(&sc.stats[5], 1ull);
    }
    if (!occluded && pend.list) pend.list[atomicAdd(pend.count, 1)] = i;
    else shadow_apply(ps, sq, i, p, occluded);
}

// the SDF pass of the shadow rays the main BVH left unoccluded
__global__ void __launch_bounds__(AR_BLOCK) k_sdf_shadow(DevScene sc, PathState ps, ShadowQueue sq, SdfPending pend)
{
    const int n = *pend.count;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
    {
        const int i = pend.list[k];
        const int p = sq.path[i];
        const float4 o4 = sq.o[i], d4 = sq.d[i];
        const V3 o = v3(o4.x, o4.y, o4.z), d = v3(d4.x, d4.y, d4.z);
        const float tmax = o4.w;
        TravResult r;
        r.t = tmax;
        r.slot = -1;
        r.id = -1;
        bool occluded = sdf_bvh_trace<true>(sc.sdf_trav, o, d, 0.0f, tmax, sq.sdf_eps[i], r).slot >= 0;
        if (!occluded && sc.trav.sdf.count > 0)
        {
            const float ts = sdf_march(sc.trav.sdf, o, d, sdf_eps(0.0f), tmax);
            occluded = ts >= 0.0f && ts < tmax;
        }
        shadow_apply(ps, sq, i, p, occluded);
    }
}

__global__ void __launch_bounds__(AR_BLOCK, AR_TRAV_MIN_BLOCKS) k_shadow(DevScene sc, PathState ps, ShadowQueue sq, const int* __restrict__ counter,
                                                   int* fetch, SdfPending pend, unsigned int* err, int min_idle,
                                                   CounterReset rs)
{
    reset_counters(rs);
    const int n = *counter;
    TravState<true> st;
    uint2 stk[AR_TRAV_STACK];
    int i = 0, p = 0;
    bool active = false, exhausted = false;
    while (true)
    {
        int q;
        if (warp_refill(fetch, n, active, &exhausted, &q, min_idle))
        {
            i = q;
            p = sq.path[i];
            const float4 o = sq.o[i], d = sq.d[i];
            st.init(sc.trav, v3(o.x, o.y, o.z), v3(d.x, d.y, d.z), 0.0f, o.w, stk);
            active = true;
        }
        if (__ballot_sync(0xffffffffu, active) == 0)
        {
            if (exhausted) break;
            continue;
        }
        if (active)
        {
            for (int it = 0; it < AR_SHD_STEPS; ++it)
            {
                if (!st.step(sc.trav, err))
                {
                    shadow_finish(sc, ps, sq, i, p, st, pend);
                    active = false;
                    break;
                }
            }
        }
    }
}

// ---------------------------------------------------------------- finalize / accumulate
__device__ __forceinline__ float nan_inf_to_zero(float x)
{
    if (x != x) return 0.0f;
    if (fabsf(x) == __int_as_float(0x7f800000)) return x > 0.0f ? 0.0f : -0.0f;
    return x;
}

__global__ void k_finalize(DevScene sc, PathState ps, int n, float* __restrict__ extra_out)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const float lambda = ps.ray_o[k].w;
    const float pdf = ps.ray_d[k].w;
    const V3 xyz = lambda_to_xyz(lambda, sc.cie_cmf);
    const float r = nan_inf_to_zero(ps.radiance[k]);
    const float x = fmaxf(0.0f, clampf(xyz.x * r / pdf, 0.0f, AR_RADIANCE_CLAMP));
    const float y = fmaxf(0.0f, clampf(xyz.y * r / pdf, 0.0f, AR_RADIANCE_CLAMP));
    const float z = fmaxf(0.0f, clampf(xyz.z * r / pdf, 0.0f, AR_RADIANCE_CLAMP));
    ps.out_xyz[3 * k + 0] = x;
    ps.out_xyz[3 * k + 1] = y;
    ps.out_xyz[3 * k + 2] = z;
    if (extra_out)
    {
        extra_out[3 * k + 0] = x;
        extra_out[3 * k + 1] = y;
        extra_out[3 * k + 2] = z;
    }
}

// guided rendering: clear the collection slots and set the probe query
__global__ void k_guide_init(PathState ps, int n)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    ps.maskq[k] = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
    for (int i = 0; i < AR_PG_COLLECT_DEPTH; ++i)
    {
        ps.pg_dir[i * ps.capacity + k] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        ps.pg_loc[i * ps.capacity + k] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        ps.pg_vdir[i * ps.capacity + k] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
}

// radiance records of finished paths (core/render/render.cuh:909-963)
__global__ void k_guide_emit(DevScene sc, PathState ps, int n, GuideSamples gs)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const uint32_t fl = ps.flags[k];
    if (((fl >> 8) & 31u) == 0u) return;
    const float lambda = ps.ray_o[k].w;
    const float pdf = ps.ray_d[k].w;
    const V3 lxyz = lambda_to_xyz(lambda, sc.cie_cmf);
    for (int i = 0; i < AR_PG_COLLECT_DEPTH; ++i)
    {
        if (!((fl >> (8 + i)) & 1u)) continue;
        const float4 d = ps.pg_dir[i * ps.capacity + k];
        const V3 xyz = lxyz * d.w / pdf;
        const float strength = fminf(max3(xyz), AR_PG_COLLECT_MAX);
        if (strength < AR_PG_COLLECT_MIN) continue;
        const float4 l = ps.pg_loc[i * ps.capacity + k];
        const float4 vd = ps.pg_vdir[i * ps.capacity + k];
        const VoxelKey key = voxel_key(v3(l.x, l.y, l.z), v3(vd.x, vd.y, vd.z), sc.guide.inv_unit);
        const unsigned long long packed = guide_pack(key);
        const int slot = atomicAdd(gs.count, 1);
        if (slot >= gs.capacity) continue;
        const V3 rad = vmax(xyz, 0.0f);
        gs.radiance[slot] = make_float4(rad.x, rad.y, rad.z, 0.0f);
        gs.dir[slot] = make_float4(d.x, d.y, d.z, 0.0f);
        gs.key[slot] = packed;
        if (gs.pos)
        {
            gs.pos[slot] = make_float4(l.x, l.y, l.z, 1.0f);
            gs.wr[slot] = make_float4(vd.x, vd.y, vd.z, vd.w);  // w: the packed surface normal
        }
    }
}

// per pixel, adds the wave's samples in increasing sample order (deterministic)
// one thread per pixel slot u of a frame (slot_pixel(u) is its pixel): the
// wave's samples of that pixel are added in frame order
__global__ void k_accumulate(const float* __restrict__ out_xyz, long long first_path, int n, int width, int height,
                             PathOrder po, double* __restrict__ accum)
{
    const long long npix = (long long)width * height;
    const long long u = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (u >= npix) return;
    // this wave's samples of slot u, in sample order
    uint32_t smp = path_first_sample(po, (uint32_t)u, (unsigned long long)first_path);
    if (smp >= po.spp || (long long)path_index(po, (uint32_t)u, smp) >= first_path + n) return;
    const long long p = slot_pixel((uint32_t)u, (uint32_t)width, (uint32_t)height);
    double sx = accum[3 * p], sy = accum[3 * p + 1], sz = accum[3 * p + 2];
    bool any = false;
    for (long long g; smp < po.spp && (g = (long long)path_index(po, (uint32_t)u, smp)) < first_path + n; ++smp)
    {
        const long long k = g - first_path;
        sx += (double)out_xyz[3 * k];
        sy += (double)out_xyz[3 * k + 1];
        sz += (double)out_xyz[3 * k + 2];
        any = true;
    }
    if (any)
    {
        accum[3 * p] = sx;
        accum[3 * p + 1] = sy;
        accum[3 * p + 2] = sz;
    }
}

static CamParams make_camera(const RenderLaunch& rl)
{
    CamParams c;
    c.o = v3(rl.cam_o[0], rl.cam_o[1], rl.cam_o[2]);
    c.d = v3(rl.cam_d[0], rl.cam_d[1], rl.cam_d[2]);
    const float FOV = rl.fov_deg * 3.1415926f / 180.0f;
    const float aspect = static_cast<float>(rl.width) / fmaxf(1.0f, static_cast<float>(rl.height));
    c.tan_y = arm_tanf(0.5f * FOV);
    c.tan_x = c.tan_y * aspect;
    c.right = normalize(cross(c.d, v3(0.0f, 1.0f, 0.0f)));
    c.up = normalize(cross(c.d, c.right));
    return c;
}

// records a stage interval when profiling
struct StageScope
{
    Ctx& c;
    int stage;
    cudaEvent_t a = nullptr;
    StageScope(Ctx& cc, int st) : c(cc), stage(st)
    {
        if (c.profile & 1)
        {
            cudaEventCreate(&a);
            cudaEventRecord(a, c.stream);
        }
    }
    ~StageScope()
    {
        if (c.profile & 1)
        {
            cudaEvent_t b;
            cudaEventCreate(&b);
            cudaEventRecord(b, c.stream);
            c.stage_events.push_back(StageEvent{stage, a, b});
            c.stage_launches[stage] += 1;
        }
    }
};

cudaError_t launch_render_wave(Ctx& c, const RenderLaunch& rl, long long first_path, int n, float* per_sample_out,
                               long long* launches)
{
    const DevScene sc = dev_scene(c);
    cudaStream_t s = c.stream;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c.device);
    const int grid_n = (n + AR_BLOCK - 1) / AR_BLOCK;
    // the persistent traversal kernels launch as many blocks as stay
    // resident: they fetch rays from a counter, so extra blocks would only add
    // launch cost (most deep bounces have few or no paths left)
    const int grid_t = sms * AR_TRAV_MIN_BLOCKS;
    int* cnt = c.d_counters;  // AR_CNT_* layout
    const CamParams cam = make_camera(rl);
    // opaque surfaces only: the shading instantiation without glass, medium and texture code
    bool lean = !c.medium.on && c.tex_count == 0 && !c.camera_inside && !rl.guide && !rl.adjoint;
    for (const Material& m : c.materials) lean = lean && m.shading != AR_MAT_GLASS;
    {
        StageScope st(c, ST_RAYGEN);
        k_raygen<<<grid_n, AR_BLOCK, 0, s>>>(c.ps, c.d_queue[0], &cnt[AR_CNT_Q0], first_path, n, rl.width, rl.height,
                                             rl.seed, rl.first_frame, cam, c.camera_inside, &cnt[AR_CNT_FETCH], !lean,
                                             rl.guide != 0, path_order(rl), rl.jumps);
        if (rl.guide) k_guide_init<<<grid_n, AR_BLOCK, 0, s>>>(c.ps, n);
    }
    long long L = rl.guide ? 2 : 1;
    ShadeParams prm;
    prm.use_nee = rl.use_nee;
    prm.max_depth = rl.max_depth;
    prm.grad = rl.grad;
    prm.grad_medium = rl.grad_medium;
    prm.mlp_ready = rl.mlp_ready;
    prm.gbuf = rl.denoise ? c.d_dn_rec : nullptr;
    MlpDev net;
    net.wbf = c.d_mlp_wbf;
    net.w32 = c.d_mlp_w32;
    net.box = c.mlp_box;
    // SDF geometry: its work leaves the traversal kernels for k_sdf_extend / k_sdf_shadow
    const bool has_sdf = c.sdf_object_count > 0 || c.sdf.count > 0;
    const SdfPending pend_shd{has_sdf ? c.d_pend_list : nullptr, &cnt[AR_CNT_PEND]};
    // Each depth's next-queue length is copied to pinned host memory behind
    // the depth's launches.  The host stays AR_BOUNCE_LOOKAHEAD depths ahead of
    // the GPU: before it queues depth b it reads the length left by depth
    // b - AR_BOUNCE_LOOKAHEAD, which bounds every later queue.  A zero ends the
    // wave's depth loop (every later depth would find an empty queue), and the
    // bound sizes the grids of the queue-sized kernels, so deep bounces with
    // few paths left (or none, at depth limits like 1000) cost launches of a
    // few blocks instead of a wave-sized grid.
    constexpr int K = AR_BOUNCE_LOOKAHEAD;
    long long bound = n;  // upper bound of the current depth's queue length
    for (int b = 0; b < rl.max_depth; ++b)
    {
        if (b >= K)
        {
            const int slot = (b - K) % (K + 1);
            const cudaError_t we = cudaEventSynchronize(c.bounce_ev[slot]);
            if (we != cudaSuccess) return we;
            const int known = c.h_bounce_cnt[slot];  // queue length of depth b - K + 1
            if (known <= 0) break;
            bound = std::min<long long>(bound, known);
        }
        const int grid_s = std::max(2 * sms, (int)((bound + AR_BLOCK * AR_SHADE_PATHS_PER_THREAD - 1) /
                                                   (AR_BLOCK * AR_SHADE_PATHS_PER_THREAD)));
        const int cur = b & 1, nxt = cur ^ 1;
        int* qn = &cnt[AR_CNT_Q0 + cur];
        // k_extend zeroes the next queue, shadow queue, shadow fetch and pending
        // counters; k_shadow zeroes the next k_extend's fetch counter
        const CounterReset ext_rs{&cnt[AR_CNT_Q0 + nxt], &cnt[AR_CNT_SHADOW], &cnt[AR_CNT_FETCH + 1],
                                  &cnt[AR_CNT_PEND], &cnt[AR_CNT_PART], &cnt[AR_CNT_PART + 1]};
        const CounterReset shd_rs{&cnt[AR_CNT_FETCH], nullptr, nullptr, nullptr};
        {
            StageScope st(c, ST_EXTEND);
            if (b == 0 && !c.camera_inside && rl.sample_block >= 32)
            {
                // camera rays: one packet per warp when a warp holds 32 samples of one
                // pixel; wider warps traverse per ray (2-pixel warps of 16-sample blocks:
                // guided terrain 971 -> 931 Msamples/s as packets; one-sample frames hold
                // an 8x4 tile, whose union of nodes is larger still)
                const int grid_c = std::max(1, (n + AR_BLOCK - 1) / AR_BLOCK);
                k_extend_camera<<<grid_c, AR_BLOCK, 0, s>>>(sc, c.ps, c.d_queue[cur], qn, c.d_err, ext_rs);
            }
            else
                k_extend<<<grid_t, AR_BLOCK, 0, s>>>(sc, c.ps, c.d_queue[cur], qn, &cnt[AR_CNT_FETCH], c.d_err,
                                                     b == 0 ? AR_EXT_REFILL_MIN0 : AR_EXT_REFILL_MIN, ext_rs);
            if (has_sdf)
            {
                k_sdf_extend<<<grid_s, AR_BLOCK, 0, s>>>(sc, c.ps, c.d_queue[cur], qn);
                ++L;
            }
        }
        {
            StageScope st(c, ST_SHADE);
            k_partition<<<grid_s, AR_BLOCK, 0, s>>>(c.d_queue[cur], c.ps.q_slot, qn, c.d_pq, &cnt[AR_CNT_PART],
                                                    &cnt[AR_CNT_PART + 1]);
            ++L;
            if (rl.guide == 2 && rl.mlp_ready)
            {
                // network inference for every queued hit (tensor cores), before shading
                cudaMemsetAsync(&cnt[AR_CNT_MLP], 0, sizeof(int), s);
                k_mlp_query<<<grid_s, AR_BLOCK, 0, s>>>(sc, c.ps, c.d_queue[cur], qn, c.d_mlp_list, &cnt[AR_CNT_MLP]);
                launch_mlp_infer(net, c.ps.q_pos, c.ps.q_wr, c.d_mlp_list, &cnt[AR_CNT_MLP], 0, c.ps.q_dist, nullptr, c.d_err,
                                 sms, s);
                L += 2;
            }
            int* shc = &cnt[AR_CNT_SHADOW];
            int* nq = c.d_queue[nxt];
            int* nn = &cnt[AR_CNT_Q0 + nxt];
            const int2* pq = c.d_pq;
            if (rl.guide == 2)
                k_shade<2, false><<<grid_s, AR_BLOCK, 0, s>>>(sc, c.ps, c.sq, pq, qn, nq, nn, shc, prm);
            else if (rl.guide)
                k_shade<1, false><<<grid_s, AR_BLOCK, 0, s>>>(sc, c.ps, c.sq, pq, qn, nq, nn, shc, prm);
            else if (rl.adjoint)
                k_shade<0, true><<<grid_s, AR_BLOCK, 0, s>>>(sc, c.ps, c.sq, pq, qn, nq, nn, shc, prm);
            else if (lean)
                k_shade<0, false, AR_FEAT_SURFACE><<<grid_s, AR_BLOCK, 0, s>>>(sc, c.ps, c.sq, pq, qn, nq, nn, shc, prm);
            else
                k_shade<0, false><<<grid_s, AR_BLOCK, 0, s>>>(sc, c.ps, c.sq, pq, qn, nq, nn, shc, prm);
        }
        {
            StageScope st(c, ST_SHADOW);
            k_shadow<<<grid_t, AR_BLOCK, 0, s>>>(sc, c.ps, c.sq, &cnt[AR_CNT_SHADOW], &cnt[AR_CNT_FETCH + 1], pend_shd,
                                                 c.d_err, b == 0 ? AR_SHD_REFILL_MIN0 : AR_SHD_REFILL_MIN, shd_rs);
            if (has_sdf)
            {
                k_sdf_shadow<<<grid_s, AR_BLOCK, 0, s>>>(sc, c.ps, c.sq, pend_shd);
                ++L;
            }
        }
        L += 3;
        {
            const int slot = b % (K + 1);
            cudaMemcpyAsync(&c.h_bounce_cnt[slot], &cnt[AR_CNT_Q0 + nxt], sizeof(int), cudaMemcpyDeviceToHost, s);
            cudaEventRecord(c.bounce_ev[slot], s);
        }
    }
    if (rl.adjoint)
    {
        if (launches) *launches += L;
        return cudaGetLastError();
    }
    {
        StageScope st(c, ST_FINAL);
        k_finalize<<<grid_n, AR_BLOCK, 0, s>>>(sc, c.ps, n, per_sample_out);
        if (rl.guide)
        {
            k_guide_emit<<<grid_n, AR_BLOCK, 0, s>>>(sc, c.ps, n, c.gs);
            ++L;
        }
    }
    ++L;
    if (launches) *launches += L;
    return cudaGetLastError();
}

// Wave launch over caller-provided buffers (used by the allocation-free entry
// point); same kernel sequence as launch_render_wave.
cudaError_t launch_render_wave_buffers(const DevScene& sc, const WaveBuffers& wb, int device, const RenderLaunch& rl,
                                       int camera_inside, long long first_path, int n, unsigned int* err)
{
    cudaStream_t s = wb.stream;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const int grid_n = (n + AR_BLOCK - 1) / AR_BLOCK;
    const int grid_t = sms * AR_TRAV_MIN_BLOCKS;
    const int grid_s = std::max(2 * sms, (n + AR_BLOCK * AR_SHADE_PATHS_PER_THREAD - 1) / (AR_BLOCK * AR_SHADE_PATHS_PER_THREAD));
    int* cnt = wb.counters;  // AR_CNT_* layout
    const CamParams cam = make_camera(rl);
    k_raygen<<<grid_n, AR_BLOCK, 0, s>>>(wb.ps, wb.queue[0], &cnt[AR_CNT_Q0], first_path, n, rl.width, rl.height, rl.seed,
                                         rl.first_frame, cam, camera_inside, &cnt[AR_CNT_FETCH], true, false,
                                         path_order(rl), nullptr);
    ShadeParams prm;
    prm.use_nee = rl.use_nee;
    prm.max_depth = rl.max_depth;
    prm.grad = nullptr;
    prm.grad_medium = nullptr;
    prm.mlp_ready = 0;
    prm.gbuf = nullptr;
    const bool has_sdf = sc.sdf_trav.node_count > 0 || sc.trav.sdf.count > 0;
    const SdfPending pend_shd{has_sdf ? wb.pend_list : nullptr, &cnt[AR_CNT_PEND]};
    for (int b = 0; b < rl.max_depth; ++b)
    {
        const int cur = b & 1, nxt = cur ^ 1;
        const CounterReset ext_rs{&cnt[AR_CNT_Q0 + nxt], &cnt[AR_CNT_SHADOW], &cnt[AR_CNT_FETCH + 1],
                                  &cnt[AR_CNT_PEND], &cnt[AR_CNT_PART], &cnt[AR_CNT_PART + 1]};
        const CounterReset shd_rs{&cnt[AR_CNT_FETCH], nullptr, nullptr, nullptr};
        k_extend<<<grid_t, AR_BLOCK, 0, s>>>(sc, wb.ps, wb.queue[cur], &cnt[AR_CNT_Q0 + cur], &cnt[AR_CNT_FETCH], err,
                                             b == 0 ? AR_EXT_REFILL_MIN0 : AR_EXT_REFILL_MIN, ext_rs);
        if (has_sdf) k_sdf_extend<<<grid_s, AR_BLOCK, 0, s>>>(sc, wb.ps, wb.queue[cur], &cnt[AR_CNT_Q0 + cur]);
        k_partition<<<grid_s, AR_BLOCK, 0, s>>>(wb.queue[cur], wb.ps.q_slot, &cnt[AR_CNT_Q0 + cur], wb.pq,
                                                &cnt[AR_CNT_PART], &cnt[AR_CNT_PART + 1]);
        k_shade<0, false><<<grid_s, AR_BLOCK, 0, s>>>(sc, wb.ps, wb.sq, wb.pq, &cnt[AR_CNT_Q0 + cur],
                                                   wb.queue[nxt], &cnt[AR_CNT_Q0 + nxt], &cnt[AR_CNT_SHADOW], prm);
        k_shadow<<<grid_t, AR_BLOCK, 0, s>>>(sc, wb.ps, wb.sq, &cnt[AR_CNT_SHADOW], &cnt[AR_CNT_FETCH + 1], pend_shd, err,
                                             b == 0 ? AR_SHD_REFILL_MIN0 : AR_SHD_REFILL_MIN, shd_rs);
        if (has_sdf) k_sdf_shadow<<<grid_s, AR_BLOCK, 0, s>>>(sc, wb.ps, wb.sq, pend_shd);
    }
    k_finalize<<<grid_n, AR_BLOCK, 0, s>>>(sc, wb.ps, n, nullptr);
    const long long npix = (long long)rl.width * rl.height;
    k_accumulate<<<(int)((npix + AR_BLOCK - 1) / AR_BLOCK), AR_BLOCK, 0, s>>>(wb.ps.out_xyz, first_path, n, rl.width,
                                                                             rl.height, path_order(rl), wb.accum);
    return cudaGetLastError();
}

// per-pixel sums -> means (one double multiply each, as the host would do it)
__global__ void k_scale_means(double* v, long long n, double inv)
{
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < n) v[i] *= inv;
}

cudaError_t launch_scale_means(double* v, long long n, double inv, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    k_scale_means<<<(int)((n + 255) / 256), 256, 0, s>>>(v, n, inv);
    return cudaGetLastError();
}

cudaError_t launch_accumulate(Ctx& c, const RenderLaunch& rl, long long first_path, int n, double* accum, long long* launches)
{
    const long long npix = (long long)rl.width * rl.height;
    const int grid = (int)((npix + AR_BLOCK - 1) / AR_BLOCK);
    k_accumulate<<<grid, AR_BLOCK, 0, c.stream>>>(c.ps.out_xyz, first_path, n, rl.width, rl.height, path_order(rl),
                                                  accum);
    if (launches) *launches += 1;
    return cudaGetLastError();
}
} // namespace ar
