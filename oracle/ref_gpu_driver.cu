// Headless driver that times the reference's own GPU renderer (the
// RenderCamera megakernel, core/scene.cu:135-208, through the progressive
// SceneRenderer::Render, core/scene.cu:240-366) on its own Cornell box
// (SceneHelper::CreateCornellBox, core/helper/scene_helper.h:10-91).
//
// TEST / MEASUREMENT INFRASTRUCTURE ONLY (see oracle/prepare_ref.py,
// prepare_gpu): compiled against a copy of the reference's core/ tree with
// only the Linux build fixes and one launch bound, with the reference's own
// flags (-use_fast_math -maxrregcount=168, CMakeLists.txt:119-121) for sm_103a.
//
// usage: ref_gpu <out.bin> <width> <height> <frames> <guide 0|1>
// Renders `frames` frames into a zeroed HDR buffer after a warm-up, writes the
// HDR running mean (float XYZ, 3 per pixel) and prints one JSON line.
#include <cstdio>
#include <cstdlib>
#include <chrono>
#include <vector>

#include "scene.hpp"
#include "helper/scene_helper.h"

int main(int argc, char** argv)
{
    if (argc != 6)
    {
        fprintf(stderr, "usage: ref_gpu <out.bin> <width> <height> <frames> <guide 0|1>\n");
        return 2;
    }
    const int W = atoi(argv[2]), H = atoi(argv[3]), frames = atoi(argv[4]), guide = atoi(argv[5]);
    if (W <= 0 || H <= 0 || frames <= 0) return 2;
    const std::vector<SceneObject> scene = SceneHelper::CreateCornellBox();
    SceneRenderer r(scene);
    r.sceneSetting_.bUsePathGuiding_ = guide != 0;
    const int2 size{W, H};
    const size_t n = (size_t)W * H;
    float3* hdr = nullptr;
    unsigned int* ldr = nullptr;
    pg::PathGuidingSample* samples = nullptr;
    if (cudaMalloc(&hdr, n * sizeof(float3)) != cudaSuccess || cudaMalloc(&ldr, n * sizeof(unsigned int)) != cudaSuccess)
        return 3;
    if (guide)
    {
        // the radiance-record buffer the reference's GUI registers (core/GUI.hpp:262-272)
        r.maxRadianceSampleCount_ = n * PATH_GUIDING_COLLECT_DEPTH;
        if (cudaMalloc(&samples, r.maxRadianceSampleCount_ * sizeof(pg::PathGuidingSample)) != cudaSuccess) return 3;
        cudaMemset(samples, 0, r.maxRadianceSampleCount_ * sizeof(pg::PathGuidingSample));
        r.sharedCollectedRadianceSampleDevice_ = samples;
    }
    const float3 origin{0.0f, 0.0f, 1.1f}, dir{0.0f, 0.0f, -1.0f};
    cudaMemset(hdr, 0, n * sizeof(float3));
    // warm-up: spectral LUT build, scene upload, first frames
    for (int f = 0; f < 4; ++f) r.Render(hdr, ldr, size, origin, dir, f, 2, nullptr, nullptr, samples, nullptr, nullptr);
    cudaDeviceSynchronize();
    if (guide) r.MarkNeedResetGuiding();
    cudaMemset(hdr, 0, n * sizeof(float3));
    cudaDeviceSynchronize();
    const auto t0 = std::chrono::steady_clock::now();
    for (int f = 0; f < frames; ++f) r.Render(hdr, ldr, size, origin, dir, f, 2, nullptr, nullptr, samples, nullptr, nullptr);
    cudaDeviceSynchronize();
    const auto t1 = std::chrono::steady_clock::now();
    const cudaError_t err = cudaGetLastError();
    std::vector<float3> host(n);
    cudaMemcpy(host.data(), hdr, n * sizeof(float3), cudaMemcpyDeviceToHost);
    FILE* fo = fopen(argv[1], "wb");
    if (!fo) return 4;
    fwrite(host.data(), sizeof(float3), n, fo);
    fclose(fo);
    const double s = std::chrono::duration<double>(t1 - t0).count();
    printf("\n{\"frames\": %d, \"width\": %d, \"height\": %d, \"s\": %.6f, \"ms_per_frame\": %.6f, "
           "\"msamples_per_s\": %.6f, \"guide\": %d, \"cuda_error\": \"%s\"}\n",
           frames, W, H, s, 1e3 * s / frames, (double)n * frames / s / 1e6, guide, cudaGetErrorString(err));
    fflush(stdout);
    cudaFree(hdr);
    cudaFree(ldr);
    if (samples) cudaFree(samples);
    return err == cudaSuccess ? 0 : 5;
}
