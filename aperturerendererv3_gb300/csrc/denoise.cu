// Denoiser of the accumulated image (SceneRenderer::Render with bDenoise_,
// core/scene.cu:324-348, and core/denoise/*).
//
// Recording: k_shade writes the camera ray's first-hit record per path; after
// each wave, k_denoise_record walks every pixel's samples of that wave in
// sample order and folds them into the pixel's G-buffer means and sample
// moments (the reference updates them inside its megakernel, one sample per
// thread per frame).
//
// Filtering: k_bilateral is the reference's Bilateral16x16<7>
// (core/denoise/denoise.cuh:360-443) restructured for the SM: one 1024-thread
// block per 32 x 32 output tile stages the 46 x 46 pixels it reads as
// per-pixel keys (dn_make_key, 96 B each, 203 KB per block) in shared memory,
// planar, so a warp reads 32 consecutive words per field; the t-test of a pair
// is evaluated first and the G-buffer weight only for pairs that pass (a
// failing pair contributes weight 0 in the reference as well).
#include <cuda_runtime.h>

#include <algorithm>

#include "../../include/aperture/ar.h"
#include "ar_denoise.h"
#include "ar_internal.h"
#include "ar_t_quantile.h"

namespace ar
{
namespace
{
constexpr int TX = 32, TY = 32;                      // output tile
constexpr int SX = TX + 2 * AR_DN_RADIUS;            // 46
constexpr int SY = TY + 2 * AR_DN_RADIUS;            // 46
constexpr int SPAN = SX * SY;                        // staged pixels per tile
constexpr int TAPS = (2 * AR_DN_RADIUS + 1) * (2 * AR_DN_RADIUS + 1);
// planes of the staged keys (one float or one 32-bit word per pixel each)
enum
{
    P_COL = 0,
    P_NRM = 3,
    P_DEP = 6,
    P_H = 7,      // 5 words of half pairs: (albedo x, y), (albedo z, metallic), (roughness, model 0),
                  // (model 1, model 2), (model 3, model 4)
    P_TH = 12,
    P_VTH = 15,
    P_UP = 18,
    P_LO = 21,
    P_COUNT = 24
};
constexpr size_t SMEM_BYTES = ((size_t)P_COUNT * SPAN + AR_DN_TQ_SIZE + TAPS) * sizeof(float);
} // namespace

__global__ void k_denoise_record(const float4* __restrict__ rec, const float* __restrict__ out_xyz,
                                 const Material* __restrict__ mats, long long first_path, int n, int width, int height,
                                 PathOrder po, DnGBuf* __restrict__ gb, DnStat* __restrict__ st)
{
    // one thread per pixel slot (slot_pixel maps it to its pixel): this wave's
    // samples of the slot, in sample order
    const long long npix = (long long)width * height;
    const long long u = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (u >= npix) return;
    uint32_t smp = path_first_sample(po, (uint32_t)u, (unsigned long long)first_path);
    if (smp >= po.spp || (long long)path_index(po, (uint32_t)u, smp) >= first_path + n) return;
    const long long p = slot_pixel((uint32_t)u, (uint32_t)width, (uint32_t)height);
    DnGBuf b = gb[p];
    DnStat s = st[p];
    for (long long g; smp < po.spp && (g = (long long)path_index(po, (uint32_t)u, smp)) < first_path + n; ++smp)
    {
        const long long k = g - first_path;
        const float4 r0 = rec[2 * k], r1 = rec[2 * k + 1];
        const int mid = __float_as_int(r0.w);
        if (mid >= 0)
        {
            const Material& m = mats[mid];
            dn_record_gbuffer(b, true, v3(r0.x, r0.y, r0.z), v3(r1.x, r1.y, r1.z), m.metallic, m.roughness, r1.w,
                              m.shading);
        }
        else
        {
            dn_record_gbuffer(b, false, v3(0, 0, 0), v3(0, 0, 0), 0.0f, 0.0f, 0.0f, AR_DN_NO_HIT);
        }
        const float xyz[3] = {out_xyz[3 * k], out_xyz[3 * k + 1], out_xyz[3 * k + 2]};
        dn_record_stat(s, xyz);
    }
    gb[p] = b;
    st[p] = s;
}

__device__ __forceinline__ uint32_t half2_bits(__half a, __half b)
{
    return (uint32_t)__half_as_ushort(a) | ((uint32_t)__half_as_ushort(b) << 16);
}
__device__ __forceinline__ __half half_lo(uint32_t w) { return __ushort_as_half((unsigned short)(w & 0xffffu)); }
__device__ __forceinline__ __half half_hi(uint32_t w) { return __ushort_as_half((unsigned short)(w >> 16)); }

// |a - b| of two halves as the reference's device code computes it: a half
// subtraction (rounded to half), then widened
__device__ __forceinline__ float hdiff(__half a, __half b) { return __half2float(__hsub(a, b)); }

__global__ void __launch_bounds__(TX * TY, 1) k_bilateral(const double* __restrict__ in_xyz, double* __restrict__ out_xyz,
                                                         const DnGBuf* __restrict__ gb, const DnStat* __restrict__ st,
                                                         const float* __restrict__ tq_global, int W, int H)
{
    extern __shared__ float sm[];
    uint32_t* smu = reinterpret_cast<uint32_t*>(sm);
    float* s_tq = sm + (size_t)P_COUNT * SPAN;
    float* s_sp = s_tq + AR_DN_TQ_SIZE;
    const int tid = threadIdx.y * TX + threadIdx.x;
    for (int i = tid; i < AR_DN_TQ_SIZE; i += TX * TY) s_tq[i] = tq_global[i];
    for (int i = tid; i < TAPS; i += TX * TY)
    {
        const int dj = i / (2 * AR_DN_RADIUS + 1) - AR_DN_RADIUS, di = i % (2 * AR_DN_RADIUS + 1) - AR_DN_RADIUS;
        s_sp[i] = arm_expf((float)(-(di * di + dj * dj)) * DnSigma::kSpatial);
    }
    // stage the tile's keys (clamped to the image, as the reference's tile load)
    const int gx0 = blockIdx.x * TX - AR_DN_RADIUS, gy0 = blockIdx.y * TY - AR_DN_RADIUS;
    for (int e = tid; e < SPAN; e += TX * TY)
    {
        const int sy = e / SX, sx = e % SX;
        const int gy = min(max(gy0 + sy, 0), H - 1), gx = min(max(gx0 + sx, 0), W - 1);
        const long long q = (long long)gy * W + gx;
        const V3 c = v3((float)in_xyz[3 * q], (float)in_xyz[3 * q + 1], (float)in_xyz[3 * q + 2]);
        const DnKey k = dn_make_key(gb[q], st[q], c);
        for (int ch = 0; ch < 3; ++ch)
        {
            sm[(P_COL + ch) * SPAN + e] = k.col[ch];
            sm[(P_NRM + ch) * SPAN + e] = k.nrm[ch];
            sm[(P_TH + ch) * SPAN + e] = k.theta[ch];
            sm[(P_VTH + ch) * SPAN + e] = k.vth[ch];
            sm[(P_UP + ch) * SPAN + e] = k.up[ch];
            sm[(P_LO + ch) * SPAN + e] = k.lo[ch];
        }
        sm[P_DEP * SPAN + e] = k.depth;
        smu[P_H * SPAN + e] = half2_bits(__float2half_rn(k.alb[0]), __float2half_rn(k.alb[1]));
        smu[(P_H + 1) * SPAN + e] = half2_bits(__float2half_rn(k.alb[2]), k.mr[0]);
        smu[(P_H + 2) * SPAN + e] = half2_bits(k.mr[1], k.model[0]);
        smu[(P_H + 3) * SPAN + e] = half2_bits(k.model[1], k.model[2]);
        smu[(P_H + 4) * SPAN + e] = half2_bits(k.model[3], k.model[4]);
    }
    __syncthreads();
    const int ox = blockIdx.x * TX + threadIdx.x, oy = blockIdx.y * TY + threadIdx.y;
    if (ox >= W || oy >= H) return;

    // centre key
    const int ce = (threadIdx.y + AR_DN_RADIUS) * SX + threadIdx.x + AR_DN_RADIUS;
    float cCol[3], cNrm[3], cTh[3], cVth[3], cUp[3], cLo[3];
    for (int ch = 0; ch < 3; ++ch)
    {
        cCol[ch] = sm[(P_COL + ch) * SPAN + ce];
        cNrm[ch] = sm[(P_NRM + ch) * SPAN + ce];
        cTh[ch] = sm[(P_TH + ch) * SPAN + ce];
        cVth[ch] = sm[(P_VTH + ch) * SPAN + ce];
        cUp[ch] = sm[(P_UP + ch) * SPAN + ce];
        cLo[ch] = sm[(P_LO + ch) * SPAN + ce];
    }
    const float cDep = sm[P_DEP * SPAN + ce];
    const uint32_t cH0 = smu[P_H * SPAN + ce], cH1 = smu[(P_H + 1) * SPAN + ce], cH2 = smu[(P_H + 2) * SPAN + ce],
                   cH3 = smu[(P_H + 3) * SPAN + ce], cH4 = smu[(P_H + 4) * SPAN + ce];
    const float cAlb0 = __half2float(half_lo(cH0)), cAlb1 = __half2float(half_hi(cH0)),
                cAlb2 = __half2float(half_lo(cH1));

    constexpr float CENTER_EPS = 1.0e-6f;
    float acc0 = cCol[0] * CENTER_EPS, acc1 = cCol[1] * CENTER_EPS, acc2 = cCol[2] * CENTER_EPS;
    float accW = CENTER_EPS;
    for (int jj = 0; jj <= 2 * AR_DN_RADIUS; ++jj)
    {
        const int row = (threadIdx.y + jj) * SX + threadIdx.x;
#pragma unroll 3
        for (int ii = 0; ii <= 2 * AR_DN_RADIUS; ++ii)
        {
            const int e = row + ii;
            // ComputeTStatisticFinal (core/denoise/denoise.cuh:309-321): all three
            // channels below their Welch-t threshold
            // (a channel that fails decides the pair; the rest need not be evaluated)
            bool pass = true;
#pragma unroll
            for (int ch = 0; ch < 3; ++ch)
            {
                if (!pass) break;
                const float t = cTh[ch] - sm[(P_TH + ch) * SPAN + e];
                const float t2 = t * t;
                const float vB = sm[(P_VTH + ch) * SPAN + e];
                const float wAsym = (t2 + vB) / fmaxf(t2 + cVth[ch] + vB, 1.0e-6f);
                const float T = sqrtf(0.5f / (1.0f - wAsym) - 1.0f);
                const float u = cUp[ch] + sm[(P_UP + ch) * SPAN + e];
                const float nu = u * u / (cLo[ch] + sm[(P_LO + ch) * SPAN + e]);
                pass = T < dn_t_quantile(s_tq, nu);
            }
            float weight = 0.0f;
            if (pass)
            {
                // ComputeSVGFWeight (core/denoise/denoise.cuh:178-242)
                float wTerm = 0.0f;
                const uint32_t b0 = smu[P_H * SPAN + e], b1 = smu[(P_H + 1) * SPAN + e];
                {
                    const float d0 = cAlb0 - __half2float(half_lo(b0));
                    const float d1 = cAlb1 - __half2float(half_hi(b0));
                    const float d2 = cAlb2 - __half2float(half_lo(b1));
                    wTerm += (d0 * d0 + d1 * d1 + d2 * d2) * DnSigma::kAlbedo;
                }
                {
                    const float dv = cNrm[0] * sm[P_NRM * SPAN + e] + cNrm[1] * sm[(P_NRM + 1) * SPAN + e] +
                                     cNrm[2] * sm[(P_NRM + 2) * SPAN + e];
                    const float d = 1.0f - dv;
                    wTerm += d * d * DnSigma::kNormal;
                }
                {
                    const float b = sm[P_DEP * SPAN + e];
                    const float denom = fmaxf(fmaxf(cDep, b), 1.0e-6f);
                    const float d = (cDep - b) / denom;
                    wTerm += d * d * DnSigma::kDepth;
                }
                const uint32_t b2 = smu[(P_H + 2) * SPAN + e];
                {
                    const float dm = hdiff(half_hi(cH1), half_hi(b1));
                    wTerm += dm * dm * DnSigma::kMetallic;
                }
                {
                    const float dr = hdiff(half_lo(cH2), half_lo(b2));
                    wTerm += dr * dr * DnSigma::kRough;
                }
                {
                    const uint32_t b3 = smu[(P_H + 3) * SPAN + e], b4 = smu[(P_H + 4) * SPAN + e];
                    float l1 = 0.0f;
                    l1 += fabsf(hdiff(half_hi(cH2), half_hi(b2)));
                    l1 += fabsf(hdiff(half_lo(cH3), half_lo(b3)));
                    l1 += fabsf(hdiff(half_hi(cH3), half_hi(b3)));
                    l1 += fabsf(hdiff(half_lo(cH4), half_lo(b4)));
                    l1 += fabsf(hdiff(half_hi(cH4), half_hi(b4)));
                    const float tv = 0.5f * l1;
                    wTerm += tv * tv * DnSigma::kModel;
                }
                weight = arm_expf(-wTerm) * s_sp[jj * (2 * AR_DN_RADIUS + 1) + ii];
            }
            acc0 = acc0 + sm[P_COL * SPAN + e] * weight;
            acc1 = acc1 + sm[(P_COL + 1) * SPAN + e] * weight;
            acc2 = acc2 + sm[(P_COL + 2) * SPAN + e] * weight;
            accW = accW + weight;
        }
    }
    // CompositeSample (core/denoise/denoise.cuh:211-220)
    const long long o = (long long)oy * W + ox;
    out_xyz[3 * o + 0] = (double)fmaxf(arm_expf(acc0 / accW) - 1.0f, 0.0f);
    out_xyz[3 * o + 1] = (double)fmaxf(arm_expf(acc1 / accW) - 1.0f, 0.0f);
    out_xyz[3 * o + 2] = (double)fmaxf(arm_expf(acc2 / accW) - 1.0f, 0.0f);
}

cudaError_t launch_denoise_record(Ctx& c, const RenderLaunch& rl, long long first_path, int n, long long* launches)
{
    const long long npix = (long long)rl.width * rl.height;
    const int grid = (int)((npix + 255) / 256);
    k_denoise_record<<<grid, 256, 0, c.stream>>>(c.d_dn_rec, c.ps.out_xyz, c.d_materials, first_path, n, rl.width,
                                                 rl.height, path_order(rl), c.d_dn_gb, c.d_dn_st);
    if (launches) *launches += 1;
    return cudaGetLastError();
}
} // namespace ar

struct ar_ctx
{
    ar::Ctx c;
};

namespace
{
float* g_tq_dev[64] = {};  // t-quantile table per device

cudaError_t tq_table(int device, const float** out)
{
    if (device < 0 || device >= 64) return cudaErrorInvalidDevice;
    if (!g_tq_dev[device])
    {
        float* p = nullptr;
        cudaError_t e = cudaMalloc((void**)&p, sizeof(ar_t_quantile_0025));
        if (e == cudaSuccess) e = cudaMemcpy(p, ar_t_quantile_0025, sizeof(ar_t_quantile_0025), cudaMemcpyHostToDevice);
        if (e != cudaSuccess)
        {
            if (p) cudaFree(p);
            return e;
        }
        e = cudaFuncSetAttribute(ar::k_bilateral, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ar::SMEM_BYTES);
        if (e != cudaSuccess)
        {
            cudaFree(p);
            return e;
        }
        g_tq_dev[device] = p;
    }
    *out = g_tq_dev[device];
    return cudaSuccess;
}
} // namespace

namespace ar
{
// Allocates the per-pixel records for a width x height image (zeroed when the
// image changes or a render starts at frame 0) and the per-path first-hit
// records for the wave capacity.
cudaError_t ensure_denoise(Ctx& c, int width, int height, int first_frame)
{
    cudaError_t e = cudaSuccess;
    const long long npix = (long long)width * height;
    if (c.dn_rec_cap < c.ps.capacity)
    {
        if (c.d_dn_rec) cudaFree(c.d_dn_rec);
        c.d_dn_rec = nullptr;
        c.dn_rec_cap = 0;
        e = cudaMalloc((void**)&c.d_dn_rec, 2 * (size_t)c.ps.capacity * sizeof(float4));
        if (e != cudaSuccess) return e;
        c.dn_rec_cap = c.ps.capacity;
    }
    const bool resize = c.dn_w != width || c.dn_h != height;
    if (resize)
    {
        if (c.d_dn_gb) cudaFree(c.d_dn_gb);
        if (c.d_dn_st) cudaFree(c.d_dn_st);
        c.d_dn_gb = nullptr;
        c.d_dn_st = nullptr;
        c.dn_w = c.dn_h = 0;
        e = cudaMalloc((void**)&c.d_dn_gb, (size_t)npix * sizeof(DnGBuf));
        if (e == cudaSuccess) e = cudaMalloc((void**)&c.d_dn_st, (size_t)npix * sizeof(DnStat));
        if (e != cudaSuccess) return e;
        c.dn_w = width;
        c.dn_h = height;
    }
    if (resize || first_frame == 0)
    {
        e = cudaMemsetAsync(c.d_dn_gb, 0, (size_t)npix * sizeof(DnGBuf), c.stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(c.d_dn_st, 0, (size_t)npix * sizeof(DnStat), c.stream);
    }
    return e;
}

void free_denoise(Ctx& c)
{
    if (c.d_dn_gb) cudaFree(c.d_dn_gb);
    if (c.d_dn_st) cudaFree(c.d_dn_st);
    if (c.d_dn_rec) cudaFree(c.d_dn_rec);
    if (c.d_dn_io) cudaFree(c.d_dn_io);
    c.d_dn_gb = nullptr;
    c.d_dn_st = nullptr;
    c.d_dn_rec = nullptr;
    c.d_dn_io = nullptr;
    c.dn_w = c.dn_h = 0;
    c.dn_rec_cap = 0;
    c.dn_img_cap = 0;
}
} // namespace ar

extern "C" {

ar_status ar_denoise(ar_ctx* ctx, const double* xyz_in, int in_is_device, double* xyz_out, int out_is_device,
                     void* stream)
{
    using namespace ar;
    if (!ctx || !xyz_in || !xyz_out) return AR_ERR_INVALID;
    Ctx& c = ctx->c;
    if (c.dn_w <= 0 || c.dn_h <= 0) return AR_ERR_STATE;
    if (cudaSetDevice(c.device) != cudaSuccess) return AR_ERR_CUDA;
    cudaStream_t s = stream ? (cudaStream_t)stream : c.stream;
    const long long npix = (long long)c.dn_w * c.dn_h;
    const size_t bytes = (size_t)npix * 3 * sizeof(double);
    const float* tq = nullptr;
    cudaError_t e = tq_table(c.device, &tq);
    // device staging for host images: input and output halves of one buffer
    if (e == cudaSuccess && (!in_is_device || !out_is_device) && c.dn_img_cap < npix)
    {
        if (c.d_dn_io) cudaFree(c.d_dn_io);
        c.d_dn_io = nullptr;
        c.dn_img_cap = 0;
        e = cudaMalloc((void**)&c.d_dn_io, 2 * bytes);
        if (e == cudaSuccess) c.dn_img_cap = npix;
    }
    const double* src = xyz_in;
    double* dst = xyz_out;
    if (e == cudaSuccess && !in_is_device)
    {
        e = cudaMemcpyAsync(c.d_dn_io, xyz_in, bytes, cudaMemcpyHostToDevice, s);
        src = c.d_dn_io;
    }
    if (!out_is_device) dst = c.d_dn_io + 3 * npix;
    if (e == cudaSuccess)
    {
        const dim3 block(TX, TY), grid((c.dn_w + TX - 1) / TX, (c.dn_h + TY - 1) / TY);
        k_bilateral<<<grid, block, SMEM_BYTES, s>>>(src, dst, c.d_dn_gb, c.d_dn_st, tq, c.dn_w, c.dn_h);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess && !out_is_device) e = cudaMemcpyAsync(xyz_out, dst, bytes, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    return e == cudaSuccess ? AR_OK : AR_ERR_CUDA;
}

ar_status ar_denoise_read(ar_ctx* ctx, int32_t* width, int32_t* height, void* gbuffer, void* moments)
{
    using namespace ar;
    if (!ctx) return AR_ERR_INVALID;
    Ctx& c = ctx->c;
    if (width) *width = c.dn_w;
    if (height) *height = c.dn_h;
    if (!gbuffer && !moments) return AR_OK;
    if (c.dn_w <= 0) return AR_ERR_STATE;
    if (cudaSetDevice(c.device) != cudaSuccess) return AR_ERR_CUDA;
    const size_t npix = (size_t)c.dn_w * c.dn_h;
    cudaError_t e = cudaStreamSynchronize(c.stream);
    if (e == cudaSuccess && gbuffer) e = cudaMemcpy(gbuffer, c.d_dn_gb, npix * sizeof(DnGBuf), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && moments) e = cudaMemcpy(moments, c.d_dn_st, npix * sizeof(DnStat), cudaMemcpyDeviceToHost);
    return e == cudaSuccess ? AR_OK : AR_ERR_CUDA;
}

ar_status ar_denoise_write(ar_ctx* ctx, int32_t width, int32_t height, const void* gbuffer, const void* moments)
{
    using namespace ar;
    if (!ctx || width <= 0 || height <= 0 || !gbuffer || !moments) return AR_ERR_INVALID;
    Ctx& c = ctx->c;
    if (cudaSetDevice(c.device) != cudaSuccess) return AR_ERR_CUDA;
    const size_t npix = (size_t)width * height;
    if (c.dn_w != width || c.dn_h != height)
    {
        if (c.d_dn_gb) cudaFree(c.d_dn_gb);
        if (c.d_dn_st) cudaFree(c.d_dn_st);
        c.d_dn_gb = nullptr;
        c.d_dn_st = nullptr;
        c.dn_w = c.dn_h = 0;
        if (cudaMalloc((void**)&c.d_dn_gb, npix * sizeof(DnGBuf)) != cudaSuccess) return AR_ERR_NOMEM;
        if (cudaMalloc((void**)&c.d_dn_st, npix * sizeof(DnStat)) != cudaSuccess) return AR_ERR_NOMEM;
        c.dn_w = width;
        c.dn_h = height;
    }
    cudaError_t e = cudaStreamSynchronize(c.stream);
    if (e == cudaSuccess) e = cudaMemcpy(c.d_dn_gb, gbuffer, npix * sizeof(DnGBuf), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(c.d_dn_st, moments, npix * sizeof(DnStat), cudaMemcpyHostToDevice);
    return e == cudaSuccess ? AR_OK : AR_ERR_CUDA;
}

} // extern "C"
