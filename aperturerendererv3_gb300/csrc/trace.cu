// Raw ray queries against the scene BVH (closest hit / any hit), the kernels
// behind ar_trace_closest / ar_trace_any.  One ray per thread, rays read as two
// float4 (origin + tmin, direction + tmax).
#include <cuda_runtime.h>

#include "ar_internal.h"

namespace ar
{
template <bool AnyHit>
__global__ void __launch_bounds__(256) k_trace(TravScene sc, const float4* __restrict__ rays, int n, int* __restrict__ out,
                                             float* __restrict__ tout, unsigned int* err)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        const float4 a = __ldg(&rays[2 * (size_t)i]);
        const float4 b = __ldg(&rays[2 * (size_t)i + 1]);
        const V3 o = v3(a.x, a.y, a.z), d = v3(b.x, b.y, b.z);
        TravResult r = traverse<AnyHit>(sc, o, d, a.w, b.w, err);
        if (sc.sdf.count > 0 && (!AnyHit || r.slot < 0))
        {
            // the SDF object (largest primitive id: a BVH hit at equal t wins)
            const float ts = sdf_march(sc.sdf, o, d, sdf_eps(a.w), r.slot < 0 ? b.w : r.t);
            if (ts >= a.w && ts < b.w && (r.slot < 0 || ts < r.t))
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
    if (any) k_trace<true><<<blocks, 256, 0, s>>>(sc.trav, r4, n, prim_id, nullptr, err);
    else k_trace<false><<<blocks, 256, 0, s>>>(sc.trav, r4, n, prim_id, t, err);
    if (launches) *launches += 1;
    return cudaGetLastError();
}
} // namespace ar
