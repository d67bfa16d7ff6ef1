// Progressive one-frame-per-call rendering for interactive callers: the
// reference's SceneRenderer::Render(hdr, ldr, size, origin, dir, frameIndex,
// toneType, odd, even, ...) (core/scene.hpp:109-114, core/scene.cu:240-366)
// and SetExposure (core/scene.hpp:97, core/scene.cu:752-755).
//
// One call renders one sample per pixel with the frame's random streams (the
// same paths as sample `frame_index` of ar_render), then
//   k_frame_blend  folds it into the caller's float32 running mean
//                  (RenderCamera, core/scene.cu:178-192: lerp with rate
//                  1 / (1 + frame), odd frames into `odd`, even into `even` at
//                  rate 1 / (1 + frame / 2));
//   k_frame_ldr    writes the display image (the Tonemap kernel's plain
//                  branch, core/scene.cu:113-131: XYZ -> linear sRGB, times the
//                  exposure, tone 0 linear / 1 gamma / 2 ACES, 0xAARRGGBB).
// With params->denoise_record the running mean is filtered by the bilateral
// denoiser first and the display image is made from the filtered one, as the
// reference does with SceneSetting::bDenoise_ (core/scene.cu:324-348).
#include <cuda_runtime.h>

#include <algorithm>

#include "../../include/aperture/ar.h"
#include "ar_internal.h"
#include "ar_tonemap.h"

namespace ar
{
// lerp(a, b, v) = a (1 - v) + b v in float (core/vector.cuh:241), no contraction
__device__ __forceinline__ float frame_lerp(float a, float b, float v)
{
    return __fadd_rn(__fmul_rn(a, __fsub_rn(1.0f, v)), __fmul_rn(b, v));
}

__global__ void k_frame_blend(const double* __restrict__ sample, long long n, int frame, float* __restrict__ hdr,
                              float* __restrict__ odd, float* __restrict__ even)
{
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    // one sample per pixel: the FP64 sum of one float32 sample holds it exactly
    float r[3];
    for (int k = 0; k < 3; ++k) r[k] = fmaxf(0.0f, (float)sample[3 * i + k]);
    const float rate = __fdiv_rn(1.0f, (float)(1 + frame));
    for (int k = 0; k < 3; ++k) hdr[3 * i + k] = frame_lerp(hdr[3 * i + k], r[k], rate);
    if (odd && even)
    {
        const float half = __fdiv_rn(1.0f, (float)(1 + (frame >> 1)));
        float* t = (frame % 2 == 1) ? odd : even;
        for (int k = 0; k < 3; ++k) t[3 * i + k] = frame_lerp(t[3 * i + k], r[k], half);
    }
}

template <typename T>
__global__ void k_frame_ldr(const T* __restrict__ xyz, long long n, int tone, float exposure, uint32_t* __restrict__ ldr)
{
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const V3 lin = xyz_to_srgb_linear(v3((float)xyz[3 * i], (float)xyz[3 * i + 1], (float)xyz[3 * i + 2]));
    V3 v = lin * exposure;
    if (tone == 1) v = gamma22(v);
    else if (tone == 2) v = aces(v);
    const uint32_t r = (uint32_t)(255.0f * saturate(v.x));
    const uint32_t g = (uint32_t)(255.0f * saturate(v.y));
    const uint32_t b = (uint32_t)(255.0f * saturate(v.z));
    ldr[i] = 0xff000000u | (r << 16) | (g << 8) | b;
}

__global__ void k_float_to_double(const float* __restrict__ a, long long n, double* __restrict__ b)
{
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < n) b[i] = (double)a[i];
}
} // namespace ar

struct ar_ctx
{
    ar::Ctx c;
};

extern "C" ar_status ar_set_exposure(ar_ctx* ctx, float exposure)
{
    if (!ctx || !(exposure == exposure)) return AR_ERR_INVALID;
    ctx->c.exposure = exposure;
    return AR_OK;
}

extern "C" ar_status ar_render_frame(ar_ctx* ctx, const ar_render_params* params, int32_t frame_index, int32_t tone_type,
                                     float* hdr, uint32_t* ldr, float* odd, float* even, void* stream)
{
    using namespace ar;
    if (!ctx || !params || !hdr) return AR_ERR_INVALID;
    Ctx& c = ctx->c;
    if (frame_index < 0 || tone_type < 0 || tone_type > 2 || (odd == nullptr) != (even == nullptr))
    {
        c.last_error = "render_frame: bad frame index, tone type, or only one of odd / even";
        return AR_ERR_INVALID;
    }
    if (params->width <= 0 || params->height <= 0)
    {
        c.last_error = "render_frame: bad resolution";
        return AR_ERR_INVALID;
    }
    const long long n = (long long)params->width * params->height;
    if (cudaSetDevice(c.device) != cudaSuccess) return AR_ERR_CUDA;
    if (c.frame_cap < n)
    {
        if (c.d_frame_xyz) cudaFree(c.d_frame_xyz);
        if (c.d_frame_dn) cudaFree(c.d_frame_dn);
        c.d_frame_xyz = nullptr;
        c.d_frame_dn = nullptr;
        c.frame_cap = 0;
        if (cudaMalloc((void**)&c.d_frame_xyz, (size_t)n * 3 * sizeof(double)) != cudaSuccess ||
            cudaMalloc((void**)&c.d_frame_dn, (size_t)n * 6 * sizeof(double)) != cudaSuccess)
        {
            c.last_error = "render_frame: device allocation failed";
            return AR_ERR_NOMEM;
        }
        c.frame_cap = n;
    }
    // the caller's stream (if any) is done with its buffers before the frame starts
    if (stream && cudaStreamSynchronize((cudaStream_t)stream) != cudaSuccess) return AR_ERR_CUDA;
    ar_render_params p = *params;
    p.spp = 1;
    p.first_frame = frame_index;
    p.profile = 0;
    ar_status st = ar_render(ctx, &p, c.d_frame_xyz, 1, nullptr, nullptr);
    if (st != AR_OK) return st;
    const int block = 256;
    const int grid = (int)((n + block - 1) / block);
    k_frame_blend<<<grid, block, 0, c.stream>>>(c.d_frame_xyz, n, frame_index, hdr, odd, even);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess && ldr)
    {
        if (params->denoise_record)
        {
            // filter the running mean, then display the filtered image
            double* din = c.d_frame_dn;
            double* dout = c.d_frame_dn + 3 * n;
            k_float_to_double<<<(int)((3 * n + block - 1) / block), block, 0, c.stream>>>(hdr, 3 * n, din);
            e = cudaGetLastError();
            if (e == cudaSuccess)
            {
                st = ar_denoise(ctx, din, 1, dout, 1, c.stream);
                if (st != AR_OK) return st;
                k_frame_ldr<double><<<grid, block, 0, c.stream>>>(dout, n, tone_type, c.exposure, ldr);
            }
        }
        else
        {
            k_frame_ldr<float><<<grid, block, 0, c.stream>>>(hdr, n, tone_type, c.exposure, ldr);
        }
        if (e == cudaSuccess) e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
    if (e != cudaSuccess)
    {
        c.last_error = std::string("render_frame: ") + cudaGetErrorString(e);
        return AR_ERR_CUDA;
    }
    return AR_OK;
}
