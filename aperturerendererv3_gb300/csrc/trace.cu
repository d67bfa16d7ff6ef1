// Raw ray queries against the scene BVH (closest hit / any hit), the kernels
// behind ar_trace_closest / ar_trace_any.  One ray per thread, rays read as two
// float4 (origin + tmin, direction + tmax).
#include <cuda_runtime.h>

#include "ar_internal.h"

namespace ar
{
template <bool AnyHit>
__global__ void __launch_bounds__(256) k_trace(TravScene sc, TravScene sdf_objects, const float4* __restrict__ rays, int n,
                                             int* __restrict__ out, float* __restrict__ tout, unsigned int* err)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        const float4 a = __ldg(&rays[2 * (size_t)i]);
        const float4 b = __ldg(&rays[2 * (size_t)i + 1]);
        const V3 o = v3(a.x, a.y, a.z), d = v3(b.x, b.y, b.z);
        TravResult r = traverse<AnyHit>(sc, o, d, a.w, b.w, err);
        if (sdf_objects.node_count > 0 && (!AnyHit || r.slot < 0))
        {
            // SDF objects (their own BVH), marched with half of max(tmin, 1e-3)
            const TravResult r2 = sdf_bvh_trace<AnyHit>(sdf_objects, o, d, a.w, b.w, 0.5f * fmaxf(a.w, 1.0e-3f), r);
            if (r2.id != r.id)
            {
                r = r2;
                r.slot = AR_SLOT_SDFOBJ_BASE - r2.slot;
            }
        }
        const bool hit = r.id >= 0;
        if (sc.sdf.count > 0 && (!AnyHit || !hit))
        {
            // the smooth-union SDF object (largest primitive id: a BVH hit at equal t wins)
            const float ts = sdf_march(sc.sdf, o, d, sdf_eps(a.w), hit ? r.t : b.w);
            if (ts >= a.w && ts < b.w && (!hit || ts < r.t))
            {
                r.t = ts;
                r.slot = AR_SLOT_SDF;
                r.id = sc.sdf_id;
            }
        }
        if (AnyHit)
        {
            out[i] = r.slot != -1 ? 1 : 0;
        }
        else
        {
            out[i] = r.id;
            if (tout) tout[i] = r.slot != -1 ? r.t : -1.0f;
        }
    }
}

cudaError_t launch_trace(const DevScene& sc, const float* rays, int n, int any, int* prim_id, float* t, unsigned int* err,
                         cudaStream_t s, long long* launches)
{
    if (n <= 0) return cudaSuccess;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int blocks = (int)std::min<long long>((n + 255) / 256, (long long)sms * 16);
    const float4* r4 = reinterpret_cast<const float4*>(rays);
    if (any) k_trace<true><<<blocks, 256, 0, s>>>(sc.trav, sc.sdf_trav, r4, n, prim_id, nullptr, err);
    else k_trace<false><<<blocks, 256, 0, s>>>(sc.trav, sc.sdf_trav, r4, n, prim_id, t, err);
    if (launches) *launches += 1;
    return cudaGetLastError();
}
} // namespace ar
