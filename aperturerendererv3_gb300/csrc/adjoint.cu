// Replay adjoint of the albedo textures (no counterpart in the reference).
//
// ar_adjoint runs every wave twice over the same random streams: the first
// pass is the ordinary render and leaves each path's total radiance L; the
// seed kernel below turns d(loss)/d(image) into the path's scalar adjoint
// delta = sum_c dl/dXYZ_c * dXYZ_c/dL / spp; the second pass (k_shade<*, true>)
// scatters delta * (L - radiance so far) * d(albedo)/d(rgb) / albedo into a
// float32 gradient buffer at every textured diffuse vertex.  After each wave
// the float32 buffer is folded into the caller's float64 gradient and
// cleared, so float32 sums only ever span one wave.
#include <cuda_runtime.h>

#include "ar_internal.h"

namespace ar
{
__global__ void k_adjoint_seed(DevScene sc, PathState ps, int n, const float* __restrict__ dl_dxyz, float inv_spp)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const float lambda = ps.ray_o[k].w;
    const float pdf = ps.ray_d[k].w;
    float r = ps.radiance[k];
    if (!(r == r) || fabsf(r) == __int_as_float(0x7f800000)) r = 0.0f;
    const V3 xyz = lambda_to_xyz(lambda, sc.cie_cmf);
    const uint32_t pix = ps.pixel[k];
    const float* g = dl_dxyz + 3 * (size_t)pix;
    // the image is clamp(xyz * L / pdf, 0, AR_RADIANCE_CLAMP) per channel
    const float cx = xyz.x * r / pdf, cy = xyz.y * r / pdf, cz = xyz.z * r / pdf;
    float d = 0.0f;
    if (cx > 0.0f && cx < AR_RADIANCE_CLAMP) d += g[0] * (xyz.x / pdf);
    if (cy > 0.0f && cy < AR_RADIANCE_CLAMP) d += g[1] * (xyz.y / pdf);
    if (cz > 0.0f && cz < AR_RADIANCE_CLAMP) d += g[2] * (xyz.z / pdf);
    ps.adj_total[k] = r;
    ps.adj_delta[k] = d * inv_spp;
}

__global__ void k_grad_fold(float* __restrict__ g32, double* __restrict__ g64, long long n)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += stride)
    {
        const float v = g32[i];
        if (v != 0.0f)
        {
            g64[i] += (double)v;
            g32[i] = 0.0f;
        }
    }
}

cudaError_t launch_adjoint_seed(Ctx& c, const RenderLaunch& rl, int n, const float* dl_dxyz, long long* launches)
{
    const DevScene sc = dev_scene(c);
    k_adjoint_seed<<<(n + 255) / 256, 256, 0, c.stream>>>(sc, c.ps, n, dl_dxyz, 1.0f / (float)rl.spp);
    if (launches) *launches += 1;
    return cudaGetLastError();
}

cudaError_t launch_grad_fold(Ctx& c, double* grad64, long long n, long long* launches)
{
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c.device);
    const long long want = (n + 255) / 256;
    const int grid = (int)std::min<long long>(want, (long long)sms * 16);
    if (grid > 0) k_grad_fold<<<grid, 256, 0, c.stream>>>(c.d_grad32, grad64, n);
    if (launches) *launches += 1;
    return cudaGetLastError();
}
} // namespace ar
