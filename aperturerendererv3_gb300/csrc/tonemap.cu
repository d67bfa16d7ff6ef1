// Display transform of a rendered image on the GPU (the reference applies it
// per pixel on the host in Camera::RenderToFile, core/camera.cu:64-89, and on
// the device for its window, core/scene.cu:22-133).
#include <cuda_runtime.h>

#include "../../include/aperture/ar.h"
#include "ar_internal.h"
#include "ar_tonemap.h"

namespace ar
{
__global__ void k_tonemap(const double* __restrict__ xyz, long long n, float exposure, int tone, uchar4* __restrict__ out)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    {
        const V3 c = v3((float)xyz[3 * i], (float)xyz[3 * i + 1], (float)xyz[3 * i + 2]);
        const V3 rgb = tonemap_pixel(c, exposure, tone);
        out[i] = make_uchar4((unsigned char)(rgb.x * 255.0f), (unsigned char)(rgb.y * 255.0f),
                             (unsigned char)(rgb.z * 255.0f), 255);
    }
}
} // namespace ar

struct ar_ctx
{
    ar::Ctx c;
};

extern "C" ar_status ar_tonemap(ar_ctx* ctx, const double* xyz, int xyz_is_device, int width, int height, float exposure,
                                int tone, uint8_t* rgba)
{
    using namespace ar;
    if (!ctx || !xyz || !rgba || width <= 0 || height <= 0) return AR_ERR_INVALID;
    if (tone != AR_TONE_ACES && tone != AR_TONE_GAMMA && tone != AR_TONE_LINEAR) return AR_ERR_INVALID;
    Ctx& c = ctx->c;
    if (cudaSetDevice(c.device) != cudaSuccess) return AR_ERR_CUDA;
    const long long n = (long long)width * height;
    double* dx = nullptr;
    uchar4* dout = nullptr;
    cudaError_t e = cudaSuccess;
    const double* src = xyz;
    if (!xyz_is_device)
    {
        e = cudaMalloc(&dx, (size_t)n * 3 * sizeof(double));
        if (e == cudaSuccess) e = cudaMemcpyAsync(dx, xyz, (size_t)n * 3 * sizeof(double), cudaMemcpyHostToDevice, c.stream);
        src = dx;
    }
    if (e == cudaSuccess) e = cudaMalloc(&dout, (size_t)n * sizeof(uchar4));
    if (e == cudaSuccess)
    {
        const int grid = (int)std::min<long long>((n + 255) / 256, 4096);
        k_tonemap<<<grid, 256, 0, c.stream>>>(src, n, exposure, tone, dout);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(rgba, dout, (size_t)n * sizeof(uchar4), cudaMemcpyDeviceToHost, c.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
    if (dx) cudaFree(dx);
    if (dout) cudaFree(dout);
    return e == cudaSuccess ? AR_OK : AR_ERR_CUDA;
}
