// SDF volume cache (SDFCacheManager, core/object/sdf/sdf_cache_manager.cuh and
// .cu): grids of signed distances that SDF objects of the volume kind sample.
// A volume is filled on the GPU from one of the reference's functors (torus,
// diamond) as FillSDFVolume does, or taken from caller data; the context keeps
// a host copy for overlap tests and reads.  Volumes persist across scene
// builds until ar_sdf_volume_clear, as the reference's cache does.
#include <cuda_runtime.h>

#include <cstring>
#include <string>

#include "../../include/aperture/ar.h"
#include "ar_internal.h"

namespace ar
{
__global__ void k_fill_sdf_volume(float* __restrict__ out, int fn, float4 prm, int dx, int dy, int dz)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int z = blockIdx.z * blockDim.z + threadIdx.z;
    if (x >= dx || y >= dy || z >= dz) return;
    out[sdf_index3(x, y, z, dx, dy)] = sdf_fill_voxel(fn, prm, x, y, z, dx, dy, dz);
}

void free_volumes(Ctx& c)
{
    for (float* p : c.vol_dev)
        if (p) cudaFree(p);
    c.vol_dev.clear();
    c.vol_host.clear();
    c.vol_dims.clear();
    if (c.d_vols) cudaFree(c.d_vols);
    c.d_vols = nullptr;
}
} // namespace ar

struct ar_ctx
{
    ar::Ctx c;
};

namespace
{
using namespace ar;

ar_status vol_fail(ar_ctx* ctx, ar_status code, const std::string& msg)
{
    ctx->c.last_error = msg;
    return code;
}

// republishes the device table after a change
cudaError_t publish(Ctx& c)
{
    if (c.d_vols) cudaFree(c.d_vols);
    c.d_vols = nullptr;
    if (c.vol_dev.empty()) return cudaSuccess;
    std::vector<SdfVolume> t(c.vol_dev.size());
    for (size_t i = 0; i < t.size(); ++i)
    {
        t[i].data = c.vol_dev[i];
        t[i].dx = c.vol_dims[3 * i];
        t[i].dy = c.vol_dims[3 * i + 1];
        t[i].dz = c.vol_dims[3 * i + 2];
        t[i].voxel_size_max = sdf_volume_voxel_size_max(t[i].dx, t[i].dy, t[i].dz);
    }
    cudaError_t e = cudaMalloc((void**)&c.d_vols, t.size() * sizeof(SdfVolume));
    if (e == cudaSuccess) e = cudaMemcpy(c.d_vols, t.data(), t.size() * sizeof(SdfVolume), cudaMemcpyHostToDevice);
    return e;
}

bool dims_ok(const int32_t* dims)
{
    return dims && dims[0] > 0 && dims[1] > 0 && dims[2] > 0 &&
           (long long)dims[0] * dims[1] * dims[2] <= (1ll << 31) / 4;
}

// appends a volume whose device grid is already filled
ar_status append(ar_ctx* ctx, float* dev, std::vector<float>&& host, const int32_t* dims, int32_t* index)
{
    Ctx& c = ctx->c;
    c.vol_dev.push_back(dev);
    c.vol_host.push_back(std::move(host));
    c.vol_dims.insert(c.vol_dims.end(), {dims[0], dims[1], dims[2]});
    const cudaError_t e = publish(c);
    if (e != cudaSuccess) return vol_fail(ctx, AR_ERR_CUDA, std::string("sdf volume: ") + cudaGetErrorString(e));
    if (index) *index = (int32_t)c.vol_dev.size() - 1;
    return AR_OK;
}
} // namespace

extern "C" {

ar_status ar_sdf_volume_add(ar_ctx* ctx, int32_t fn, const float* params, const int32_t* dims, int32_t* index)
{
    if (!ctx || !params) return AR_ERR_INVALID;
    if (fn != AR_SDF_FN_TORUS && fn != AR_SDF_FN_DIAMOND) return vol_fail(ctx, AR_ERR_INVALID, "sdf volume: unknown functor");
    if (!dims_ok(dims)) return vol_fail(ctx, AR_ERR_INVALID, "sdf volume: bad dimensions");
    Ctx& c = ctx->c;
    if (cudaSetDevice(c.device) != cudaSuccess) return AR_ERR_CUDA;
    const size_t n = (size_t)dims[0] * dims[1] * dims[2];
    float* dev = nullptr;
    cudaError_t e = cudaMalloc((void**)&dev, n * sizeof(float));
    if (e == cudaSuccess)
    {
        const dim3 block(8, 8, 8);
        const dim3 grid((dims[0] + 7) / 8, (dims[1] + 7) / 8, (dims[2] + 7) / 8);
        k_fill_sdf_volume<<<grid, block, 0, c.stream>>>(dev, fn, make_float4(params[0], params[1], params[2], params[3]),
                                                        dims[0], dims[1], dims[2]);
        e = cudaGetLastError();
    }
    std::vector<float> host(n);
    if (e == cudaSuccess) e = cudaMemcpyAsync(host.data(), dev, n * sizeof(float), cudaMemcpyDeviceToHost, c.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
    if (e != cudaSuccess)
    {
        if (dev) cudaFree(dev);
        return vol_fail(ctx, AR_ERR_CUDA, std::string("sdf volume fill: ") + cudaGetErrorString(e));
    }
    return append(ctx, dev, std::move(host), dims, index);
}

ar_status ar_sdf_volume_add_data(ar_ctx* ctx, const float* voxels, const int32_t* dims, int32_t* index)
{
    if (!ctx || !voxels) return AR_ERR_INVALID;
    if (!dims_ok(dims)) return vol_fail(ctx, AR_ERR_INVALID, "sdf volume: bad dimensions");
    Ctx& c = ctx->c;
    if (cudaSetDevice(c.device) != cudaSuccess) return AR_ERR_CUDA;
    const size_t n = (size_t)dims[0] * dims[1] * dims[2];
    float* dev = nullptr;
    cudaError_t e = cudaMalloc((void**)&dev, n * sizeof(float));
    if (e == cudaSuccess) e = cudaMemcpy(dev, voxels, n * sizeof(float), cudaMemcpyHostToDevice);
    if (e != cudaSuccess)
    {
        if (dev) cudaFree(dev);
        return vol_fail(ctx, AR_ERR_CUDA, std::string("sdf volume upload: ") + cudaGetErrorString(e));
    }
    return append(ctx, dev, std::vector<float>(voxels, voxels + n), dims, index);
}

ar_status ar_sdf_volume_read(ar_ctx* ctx, int32_t index, float* voxels, int32_t* dims)
{
    if (!ctx) return AR_ERR_INVALID;
    Ctx& c = ctx->c;
    if (index < 0 || index >= (int32_t)c.vol_host.size()) return vol_fail(ctx, AR_ERR_INVALID, "sdf volume: bad index");
    if (dims)
        for (int k = 0; k < 3; ++k) dims[k] = c.vol_dims[3 * index + k];
    if (voxels) std::memcpy(voxels, c.vol_host[index].data(), c.vol_host[index].size() * sizeof(float));
    return AR_OK;
}

ar_status ar_sdf_volume_clear(ar_ctx* ctx)
{
    if (!ctx) return AR_ERR_INVALID;
    Ctx& c = ctx->c;
    if (cudaSetDevice(c.device) != cudaSuccess) return AR_ERR_CUDA;
    cudaStreamSynchronize(c.stream);
    free_volumes(c);
    return AR_OK;
}

} // extern "C"
