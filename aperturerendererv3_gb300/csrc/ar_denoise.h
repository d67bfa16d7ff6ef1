// Screen-space denoiser of the accumulated image: the reference's bilateral
// filter with G-buffer edge stops and a per-pixel-pair Welch t-test on the
// moments of the Box-Cox transformed samples (core/denoise/denoise.cuh:85-444,
// core/denoise/denoise_statistic.cuh:10-70).
//
// Two per-pixel records, both updated once per sample in sample order:
//   DnGBuf  running means of the first hit's albedo, normal, metallic,
//           roughness (stored as halves after every update, as the reference
//           stores them), hit distance (float), and the histogram of the first
//           hit's shading model (5 bins, the last one "no hit");
//   DnStat  sample count, mean and M2/n, M3/n of BoxCox(XYZ) per channel
//           (Welford updates with the M2/M3 sums carried in double).
// The filter stages per-pixel keys (everything a pixel contributes to a pair
// weight) in shared memory; every floating-point operation follows the
// reference's device code in the same order, so results match it bit for bit
// on the same records.  Device only.
#pragma once
#include <cstdint>
#include <cuda_fp16.h>

#include "ar_vec.h"

#define AR_DN_RADIUS 7                   // Bilateral16x16<7> (core/scene.cu:341)
#define AR_DN_MODELS 5                   // diffuse, light, glass, GGX, no hit (EShadingModel::MAT_MAX)
#define AR_DN_NO_HIT 4
#define AR_DN_TQ_SIZE 1024               // T_QUANTILE_LUT_SIZE (core/denoise/t_quantile.cuh:6)

namespace ar
{
// 40 B per pixel.  h: albedo xyz, normal xyz, metallic, roughness, model histogram[5], pad
struct DnGBuf
{
    __half h[14];
    float depth;
    uint32_t valid;   // samples whose camera ray hit a surface
    uint32_t frames;  // all samples
};

// 40 B per pixel
struct DnStat
{
    uint32_t num;
    float mean[3], m2n[3], m3n[3];
};

// Filter constants (FilterParams, core/denoise/denoise.cuh:12-31), evaluated
// in float like the reference's constexpr expressions.
struct DnSigma
{
    static constexpr float kAlbedo = 1.0f / (2.0f * 1.0f * 1.0f);
    static constexpr float kNormal = 1.0f / (2.0f * 0.5f * 0.5f);
    static constexpr float kDepth = 1.0f / (2.0f * 0.25f * 0.25f);
    static constexpr float kMetallic = 1.0f / (2.0f * 0.5f * 0.5f);
    static constexpr float kRough = 1.0f / (2.0f * 0.5f * 0.5f);
    static constexpr float kModel = 1.0f / (2.0f * 0.1f * 0.1f);
    static constexpr float kSpatial = 1.0f / (2.0f * 2.0f * 2.0f);
};

// ---------------------------------------------------------------- recording

// RecordShadingModel (core/denoise/denoise.cuh:85-104)
__device__ __forceinline__ void dn_record_model(DnGBuf& g, int model)
{
    if (g.frames == 0u)
        for (int i = 0; i < AR_DN_MODELS; ++i) g.h[8 + i] = __float2half_rn(0.0f);
    const uint64_t f = g.frames;
    const float affix = 1.0f / (float)(f + 1ull);
    const float pre = (float)f / (float)(f + 1ull);
#pragma unroll
    for (int i = 0; i < AR_DN_MODELS; ++i)
    {
        const __half scaled = __float2half_rn(__half2float(g.h[8 + i]) * pre);
        // the bin of this sample's model gains affix (a select, not an indexed
        // store, so the record stays in registers)
        g.h[8 + i] = (i == model) ? __float2half_rn(__half2float(scaled) + affix) : scaled;
    }
}

// RecordScreenGBuffer (core/denoise/denoise.cuh:106-158) for one sample.
// hit = false records "no hit" in the model histogram only.
__device__ __forceinline__ void dn_record_gbuffer(DnGBuf& g, bool hit, V3 albedo, V3 nrm, float metallic,
                                                  float roughness, float dist, int model)
{
    if (hit)
    {
        if (g.valid == 0u)
        {
            for (int i = 0; i < 8; ++i) g.h[i] = __float2half_rn(0.0f);
            g.depth = 0.0f;
        }
        const uint64_t v = g.valid;
        const float affix = 1.0f / (float)(v + 1ull);
        const float pre = (float)v / (float)(v + 1ull);
        for (int i = 0; i < 8; ++i) g.h[i] = __float2half_rn(__half2float(g.h[i]) * pre);
        g.depth = g.depth * pre;
        const float x[8] = {albedo.x, albedo.y, albedo.z, nrm.x, nrm.y, nrm.z, metallic, roughness};
        for (int i = 0; i < 8; ++i) g.h[i] = __float2half_rn(__half2float(g.h[i]) + affix * x[i]);
        g.depth = g.depth + affix * dist;
        g.valid += 1u;
        dn_record_model(g, model);
    }
    else
    {
        dn_record_model(g, AR_DN_NO_HIT);
    }
    g.frames += 1u;
}

// RecordScreenStatisticBuffer (core/denoise/denoise_statistic.cuh:36-69) for
// one sample's clamped XYZ.
__device__ __forceinline__ void dn_record_stat(DnStat& s, const float xyz[3])
{
    const uint32_t n0 = s.num;
    const uint32_t n1 = n0 + 1u;
    s.num = n1;
    const float invN1 = 1.0f / (float)n1;
    for (int c = 0; c < 3; ++c)
    {
        const float bc = (arm_powf(fmaxf(xyz[c], 0.0f), 0.5f) - 1.0f) * 2.0f;  // BoxCox05
        const float delta = bc - s.mean[c];
        const float dn = delta * invN1;
        const float mean1 = s.mean[c] + dn;
        const double m2_0 = (double)s.m2n[c] * (double)n0;
        const double m2_1 = m2_0 + (double)(delta * (delta - dn));
        const double m3_0 = (double)s.m3n[c] * (double)n0;
        const float d2 = delta * delta;
        const float dn2 = dn * dn;
        const double m3_1 = m3_0 - 3.0 * ((double)dn * m2_1) + (double)(delta * (d2 - dn2));
        s.mean[c] = mean1;
        s.m2n[c] = (float)(m2_1 / (double)n1);
        s.m3n[c] = (float)(m3_1 / (double)n1);
    }
}

// ---------------------------------------------------------------- filter keys

// What one pixel contributes to a pair weight, derived once per pixel from its
// records: the pure per-pixel parts of ComputeSVGFWeight (normalised normal),
// ComputeTStatistic (core/denoise/denoise.cuh:241-264) and ComputeWelchNu
// (:293-306), and SeparateSample (:200-209).
struct DnKey
{
    float col[3];          // log(c + 1)
    float alb[3];
    float nrm[3];          // normalize(normal mean)
    float depth;
    __half mr[2];          // metallic, roughness
    __half model[AR_DN_MODELS + 1];
    float theta[3];        // mean + M3/n / 6 / s^2
    float vth[3];          // s^2 / n
    float up[3];           // s^2 / n (Welch numerator term, float division)
    float lo[3];           // up^2 / max(n - 1, 1)
};

__device__ __forceinline__ DnKey dn_make_key(const DnGBuf& g, const DnStat& s, V3 color)
{
    DnKey k;
    k.col[0] = arm_logf(color.x + 1.0f);
    k.col[1] = arm_logf(color.y + 1.0f);
    k.col[2] = arm_logf(color.z + 1.0f);
    k.alb[0] = __half2float(g.h[0]);
    k.alb[1] = __half2float(g.h[1]);
    k.alb[2] = __half2float(g.h[2]);
    const V3 n = normalize(v3(__half2float(g.h[3]), __half2float(g.h[4]), __half2float(g.h[5])));
    k.nrm[0] = n.x;
    k.nrm[1] = n.y;
    k.nrm[2] = n.z;
    k.depth = g.depth;
    k.mr[0] = g.h[6];
    k.mr[1] = g.h[7];
    for (int i = 0; i < AR_DN_MODELS; ++i) k.model[i] = g.h[8 + i];
    k.model[AR_DN_MODELS] = __float2half_rn(0.0f);
    const double num = (double)s.num;
    const uint32_t nm1 = s.num - 1u;
    const double invNumMinus1 = 1.0 / (double)(nm1 > 1u ? nm1 : 1u);
    const uint32_t wm1 = s.num - 1u;
    const float wden = (float)(wm1 > 1u ? wm1 : 1u);
    for (int c = 0; c < 3; ++c)
    {
        const double m2 = (double)s.m2n[c] * num;
        const float var = (float)(m2 * invNumMinus1);
        k.vth[c] = (float)((double)var / num);
        k.theta[c] = s.mean[c] + s.m3n[c] / 6.0f / var;
        const float up = var / (float)s.num;
        k.up[c] = up;
        k.lo[c] = up * up / wden;
    }
    return k;
}

// LookupTQuantile005 (core/denoise/t_quantile.cuh:17-26); the float -> int
// conversion saturates and maps NaN to 0, as the GPU's conversion does.
__device__ __forceinline__ float dn_t_quantile(const float* tq, float nu)
{
    const float f = floorf(nu);
    int i;
    if (f != f) i = 0;
    else if (f >= 2147483648.0f) i = 2147483647;
    else if (f <= -2147483648.0f) i = (-2147483647 - 1);
    else i = (int)f;
    uint32_t idx = (i <= 0) ? 0u : (uint32_t)(i - 1);
    if (idx > AR_DN_TQ_SIZE - 1) idx = AR_DN_TQ_SIZE - 1;
    return tq[idx];
}
} // namespace ar
