// Voxel-guide learning on the GPU: the per-frame update that the reference runs
// on its second stream (SceneRenderer::UpdatePathGuidingSample,
// core/scene.cu:409-570; kernels in core/guiding/guiding.cuh:293-517).
//
// The reference filters, sorts and uniques the frame's radiance records with
// thrust, grows a sparse index volume by copying, assigns probe ids on the
// host side and rebuilds each probe's mips in a single lane.  Here the sparse
// index is an open-addressing hash of packed voxel keys, so the whole update
// is three kernels with no host round trip:
//   k_pg_claim       every record finds or inserts its key (atomicCAS on the
//                    slot's key) and a new key takes the next probe index
//   k_pg_accumulate  radiance x Jacobian added into the probe's leaf texel;
//                    warp-aggregated when lanes share a texel
//   k_pg_merge       one warp per probe: FP64 running-mean blend of the leaf,
//                    count update (capped), then the mip pyramid level by level
//                    with all lanes busy; the temporary probe is cleared.
#include <cuda_runtime.h>

#include "ar_internal.h"

namespace ar
{
__global__ void k_pg_claim(GuideSamples gs, unsigned long long* keys, int* vals, unsigned mask, int* meta,
                           int capacity)
{
    const int n = min(*gs.count, gs.capacity);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        const unsigned long long key = gs.key[i];
        if (key == AR_PG_KEY_EMPTY) continue;
        unsigned s = guide_hash(key) & mask;
        for (int probe = 0; probe < AR_PG_HASH_PROBES; ++probe)
        {
            const unsigned long long prev = atomicCAS(&keys[s], AR_PG_KEY_EMPTY, key);
            if (prev == AR_PG_KEY_EMPTY)
            {
                const int idx = atomicAdd(&meta[0], 1);
                vals[s] = idx < capacity ? idx : -3;  // -3: pool full, the key stays unguided
                break;
            }
            if (prev == key) break;
            s = (s + 1u) & mask;
        }
    }
}

__global__ void k_pg_accumulate(GuideSamples gs, DevGuide g, Probe* temp)
{
    const int n = min(*gs.count, gs.capacity);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        const int idx = guide_lookup(g, gs.key[i]);
        if (idx < 0) continue;
        const float4 dd = gs.dir[i];
        const V3 dir = normalize(v3(dd.x, dd.y, dd.z));
        int px, py;
        direction_to_leaf(dir, &px, &py);
        const float J = clarberg_jacobian();
        const float4 r = gs.radiance[i];
        float4* leaf = &temp[idx].data[py * AR_PG_RES + px];
        atomicAdd(&leaf->x, r.x * J);
        atomicAdd(&leaf->y, r.y * J);
        atomicAdd(&leaf->z, r.z * J);
        atomicAdd(&temp[idx].count, 1ull);
    }
}

__global__ void __launch_bounds__(256) k_pg_merge(Probe* probes, Probe* temp, const int* meta, int capacity)
{
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const int nprobe = min(meta[0], capacity);
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int p = warp; p < nprobe; p += nwarps)
    {
        Probe& tp = temp[p];
        const unsigned long long countNew = tp.count;
        if (countNew == 0ull) continue;
        Probe& op = probes[p];
        const unsigned long long countOld = op.count;
        const double invDen = 1.0 / static_cast<double>(countOld + countNew);
        const double alpha = static_cast<double>(countOld) * invDen;
        for (int k = lane; k < AR_PG_RES2; k += 32)
        {
            float4 o = op.data[k];
            const float4 nv = tp.data[k];
            o.x = static_cast<float>(static_cast<double>(o.x) * alpha + static_cast<double>(nv.x) * invDen);
            o.y = static_cast<float>(static_cast<double>(o.y) * alpha + static_cast<double>(nv.y) * invDen);
            o.z = static_cast<float>(static_cast<double>(o.z) * alpha + static_cast<double>(nv.z) * invDen);
            o.x = fmaxf(o.x, AR_PG_PROBE_MIN);
            o.y = fmaxf(o.y, AR_PG_PROBE_MIN);
            o.z = fmaxf(o.z, AR_PG_PROBE_MIN);
            o.w = fmaxf(o.w, AR_PG_PROBE_MIN);
            op.data[k] = o;
            tp.data[k] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        }
        __syncwarp();
        // mip levels: each output texel = mean of its 4 children, all lanes busy
        int srcRes = AR_PG_RES, srcOff = 0, dstOff = AR_PG_RES2;
        for (int level = 0; level < AR_PG_LEVELS - 1; ++level)
        {
            const int dr = srcRes >> 1;
            for (int t = lane; t < dr * dr; t += 32)
            {
                const int x = t % dr, y = t / dr;
                const float4 a = op.data[srcOff + (2 * y) * srcRes + 2 * x];
                const float4 b = op.data[srcOff + (2 * y) * srcRes + 2 * x + 1];
                const float4 c = op.data[srcOff + (2 * y + 1) * srcRes + 2 * x];
                const float4 d = op.data[srcOff + (2 * y + 1) * srcRes + 2 * x + 1];
                float4 o;
                o.x = (a.x + b.x + c.x + d.x) * 0.25f;
                o.y = (a.y + b.y + c.y + d.y) * 0.25f;
                o.z = (a.z + b.z + c.z + d.z) * 0.25f;
                o.w = (a.w + b.w + c.w + d.w) * 0.25f;
                op.data[dstOff + y * dr + x] = o;
            }
            __syncwarp();
            srcOff = dstOff;
            srcRes = dr;
            dstOff = srcOff + srcRes * srcRes;
        }
        if (lane == 0)
        {
            op.data[AR_PG_TEXELS] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            const unsigned long long s = countOld + countNew;
            op.count = s < AR_PG_MAX_COUNT ? s : AR_PG_MAX_COUNT;
            tp.count = 0ull;
        }
        __syncwarp();
    }
}

cudaError_t launch_guide_update(Ctx& c, long long* launches)
{
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c.device);
    cudaStream_t s = c.stream;
    k_pg_claim<<<sms * 4, 256, 0, s>>>(c.gs, c.d_pg_keys, c.d_pg_vals, c.guide.mask, c.d_pg_meta, c.pg_capacity);
    k_pg_accumulate<<<sms * 4, 256, 0, s>>>(c.gs, c.guide, c.d_pg_temp);
    k_pg_merge<<<sms * 8, 256, 0, s>>>(c.d_pg_probes, c.d_pg_temp, c.d_pg_meta, c.pg_capacity);
    // the frame's record count stays readable (ar_guide_read_records) after the reset
    cudaMemcpyAsync(&c.d_pg_meta[1], c.gs.count, sizeof(int), cudaMemcpyDeviceToDevice, s);
    cudaMemsetAsync(c.gs.count, 0, sizeof(int), s);
    if (launches) *launches += 3;
    return cudaGetLastError();
}

int guide_probe_count(Ctx& c)
{
    int n = 0;
    if (c.d_pg_meta) cudaMemcpy(&n, c.d_pg_meta, sizeof(int), cudaMemcpyDeviceToHost);
    return n < c.pg_capacity ? n : c.pg_capacity;
}
} // namespace ar
