// Tensor-core (tcgen05) kernels of the MLP path guide, and the self-test that
// checks the operand descriptors against a host GEMM.
#include <cuda_runtime.h>

#include <vector>

#include <cuda_bf16.h>

#include "ar_internal.h"
#include "ar_umma.cuh"
#include "../../include/aperture/ar.h"

namespace ar
{
// ------------------------------------------------------------------ MLP guide
// Network parameters as the kernels see them: MlpDev (ar_internal.h), bf16
// weights at mlp_w_offset (bias slots unused) and the float32 master block
// the biases are read from.

namespace mlpk
{
constexpr int W_BYTES = 64 * 144 * 2 + 4 * 64 * 64 * 2;  // weight tiles, all layers
constexpr int X_BYTES = 128 * 144 * 2;                   // encoded inputs of one tile
constexpr int H_BYTES = 128 * 64 * 2;                    // one hidden layer of one tile
constexpr int DY_BYTES = 128 * 128 * 2;                  // layer gradient, M padded to 128
constexpr int INF_WG = 4;                                // warpgroups (tiles in flight) per CTA
// per warpgroup one buffer: the encoded inputs, then (layer 0 done) the hidden layer
constexpr int INF_SMEM = W_BYTES + INF_WG * X_BYTES + 5 * 64 * 4;
constexpr int TR_SMEM = W_BYTES + X_BYTES + 4 * H_BYTES + 2 * DY_BYTES + 2 * 5 * 64 * 4;
constexpr uint32_t TR_TMEM_COLS = 512;
// TMEM columns of the weight-gradient accumulators (working accumulator at 0)
__host__ __device__ constexpr int dw_col(int l) { return l == 0 ? 64 : 208 + 64 * (l - 1); }

__device__ __forceinline__ int w_tile_offset(int l) { return l == 0 ? 0 : 64 * 144 * 2 + (l - 1) * 64 * 64 * 2; }

__device__ __forceinline__ uint32_t pack_bf16(float a, float b)
{
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const uint32_t*>(&h);
}

// one row of eight bf16 values (a 16-byte core-matrix row)
__device__ __forceinline__ void store8(uint8_t* tile, int C, int row, int col8, const float* v)
{
    uint4 u;
    u.x = pack_bf16(v[0], v[1]);
    u.y = pack_bf16(v[2], v[3]);
    u.z = pack_bf16(v[4], v[5]);
    u.w = pack_bf16(v[6], v[7]);
    *reinterpret_cast<uint4*>(tile + umma::tile_offset(row, col8, C)) = u;
}

__device__ __forceinline__ void load8(const uint8_t* tile, int C, int row, int col8, float* v)
{
    const uint4 u = *reinterpret_cast<const uint4*>(tile + umma::tile_offset(row, col8, C));
    const uint32_t w[4] = {u.x, u.y, u.z, u.w};
    for (int k = 0; k < 4; ++k)
    {
        const __nv_bfloat162 h = *reinterpret_cast<const __nv_bfloat162*>(&w[k]);
        const float2 f = __bfloat1622float2(h);
        v[2 * k] = f.x;
        v[2 * k + 1] = f.y;
    }
}

// 12-band sin/cos encoding of the six inputs into row `row` of the X tile.
// Bands 0, 4 and 8 come from sincospif; the three bands after each by angle
// doubling (sin 2a = 2 sin a cos a, cos 2a = (cos a - sin a)(cos a + sin a)),
// whose rounding (a few 1e-7 after three doublings) is far below the bf16
// rounding of the features.  A quarter of the transcendental calls.
__device__ __forceinline__ void encode_row(uint8_t* X, int row, const float in6[6])
{
    for (int d = 0; d < 6; ++d)
        for (int k = 0; k < 3; ++k)
        {
            float v[8];
            float sn, cs;
            sincospif(in6[d] * (float)(1 << (4 * k)), &sn, &cs);
            for (int b = 0; b < 4; ++b)
            {
                v[2 * b] = sn;
                v[2 * b + 1] = cs;
                const float s2 = 2.0f * sn * cs;
                cs = (cs - sn) * (cs + sn);
                sn = s2;
            }
            store8(X, AR_MLP_IN, row, mlp_feature(d, 4 * k, 0), v);
        }
}

// weight tiles (rows = outputs, columns = inputs) from the bf16 parameter block
__device__ void load_weights(uint8_t* W, const uint16_t* __restrict__ wbf, float* sbias, const float* __restrict__ w32)
{
    for (int l = 0; l < AR_MLP_LAYERS; ++l)
    {
        const int in = mlp_in_dim(l);
        const uint16_t* src = wbf + mlp_w_offset(l);
        uint8_t* dst = W + w_tile_offset(l);
        for (int c = threadIdx.x; c < 64 * (in / 8); c += blockDim.x)
        {
            const int o = c / (in / 8), i8 = (c % (in / 8)) * 8;
            *reinterpret_cast<uint4*>(dst + umma::tile_offset(o, i8, in)) =
                *reinterpret_cast<const uint4*>(src + o * in + i8);
        }
    }
    for (int k = threadIdx.x; k < 5 * 64; k += blockDim.x) sbias[k] = w32[mlp_b_offset(k / 64) + (k % 64)];
}

__device__ __forceinline__ void wg_sync(int wg)
{
    asm volatile("bar.sync %0, 128;" ::"r"(1 + wg) : "memory");
}

// all smem writes of the warpgroup visible to its next tensor-core operation
__device__ __forceinline__ void wg_publish(int wg)
{
    umma::fence_async_smem();
    umma::fence_before_sync();
    wg_sync(wg);
    umma::fence_after_sync();
}

// 64 FP32 accumulator columns of this thread's row (TMEM lane = row)
__device__ __forceinline__ void load_row64(uint32_t tmem, int warp_in_wg, int col0, float* v)
{
    const uint32_t base = tmem + ((uint32_t)(warp_in_wg * 32) << 16) + (uint32_t)col0;
    for (int j = 0; j < 4; ++j) umma::tmem_ld16(base + 16 * j, v + 16 * j);
}
} // namespace mlpk

// Inference: 128 shading points per tile, INF_WG tiles in flight per CTA (one
// per warpgroup), weights staged once per CTA.  Inputs: per path (queue mode:
// path p = queue[q], q < *count) or per index (direct mode).  Output: 64
// quantised cell weights per point (and, in direct mode, optionally the raw
// output layer).
__global__ void __launch_bounds__(128 * mlpk::INF_WG, 1)
    k_mlp_infer(MlpDev net, const float4* __restrict__ q_pos, const float4* __restrict__ q_wr,
                const int* __restrict__ queue, const int* __restrict__ count, int n_direct, uint8_t* __restrict__ out,
                float* __restrict__ logits_out, unsigned* err)
{
    using namespace mlpk;
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t* W = smem;
    const int wg = threadIdx.x >> 7, row = threadIdx.x & 127, warp_in_wg = (threadIdx.x >> 5) & 3;
    uint8_t* X = smem + W_BYTES + wg * X_BYTES;
    uint8_t* H = X;  // the layer-0 product has completed before the first hidden row is written
    float* sbias = reinterpret_cast<float*>(smem + W_BYTES + INF_WG * X_BYTES);
    __shared__ uint64_t mbar[INF_WG];
    __shared__ uint32_t tmem_slot;
    __shared__ int abort_flag[INF_WG];
    load_weights(W, net.wbf, sbias, net.w32);
    if (threadIdx.x < 32) umma::tmem_alloc(&tmem_slot, 64 * INF_WG);
    if (threadIdx.x < INF_WG)
    {
        umma::mbar_init(&mbar[threadIdx.x], 1);
        abort_flag[threadIdx.x] = 0;
    }
    umma::fence_async_smem();
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tmem = tmem_slot + (uint32_t)(wg * 64);
    const int n = queue ? *count : n_direct;
    const int tiles = (n + 127) / 128;
    uint32_t phase = 0;
    for (int tile = blockIdx.x * INF_WG + wg; tile < tiles; tile += gridDim.x * INF_WG)
    {
        const int qi = tile * 128 + row;
        const bool valid = qi < n;
        const int p = valid ? (queue ? queue[qi] : qi) : 0;
        float in6[6] = {0, 0, 0, 0, 0, 0};
        if (valid)
        {
            const float4 a = q_pos[p], b = q_wr[p];
            mlp_inputs(net.box, v3(a.x, a.y, a.z), v3(b.x, b.y, b.z), in6);
        }
        encode_row(X, row, in6);
        wg_publish(wg);
        float v[64];
        for (int l = 0; l < AR_MLP_LAYERS; ++l)
        {
            const int in = mlp_in_dim(l);
            if (row == 0)
            {
                const uint32_t a0 = umma::smem_addr(l == 0 ? X : H), b0 = umma::smem_addr(W + w_tile_offset(l));
                const uint32_t idesc = umma::make_idesc(128, 64, false, false);
                for (int k = 0; k < in / 16; ++k)
                    umma::mma(tmem, umma::tile_desc(a0, in, 0, 16 * k, false), umma::tile_desc(b0, in, 0, 16 * k, false),
                              idesc, k > 0);
                umma::commit(&mbar[wg]);
            }
            if (!umma::mbar_wait(&mbar[wg], phase))
            {
                atomicOr(err, AR_DEVERR_MLP);
                abort_flag[wg] = 1;
                umma::mbar_wait(&mbar[wg], phase);
            }
            phase ^= 1u;
            umma::fence_after_sync();
            load_row64(tmem, warp_in_wg, 0, v);
            const float* b = sbias + 64 * l;
            if (l < AR_MLP_LAYERS - 1)
            {
                for (int c = 0; c < 8; ++c)
                {
                    float h[8];
                    for (int i = 0; i < 8; ++i) h[i] = fmaxf(v[8 * c + i] + b[8 * c + i], 0.0f);
                    mlpk::store8(H, 64, row, 8 * c, h);
                }
                wg_publish(wg);
            }
            else
            {
                float mx = -3.0e38f;
                for (int i = 0; i < 64; ++i)
                {
                    v[i] += b[i];
                    mx = fmaxf(mx, v[i]);
                }
                if (valid)
                {
                    if (logits_out)
                        for (int i = 0; i < 64; ++i) logits_out[(size_t)qi * 64 + i] = v[i];
                    if (out)
                    {
                        uint32_t w[16];
                        for (int k = 0; k < 16; ++k)
                        {
                            uint32_t word = 0;
                            for (int j = 0; j < 4; ++j)
                            {
                                const float e = __expf(v[4 * k + j] - mx);
                                word |= (uint32_t)__float2int_rn(fminf(255.0f, 255.0f * e)) << (8 * j);
                            }
                            w[k] = word;
                        }
                        uint4* dst = reinterpret_cast<uint4*>(out + (size_t)p * 64);
                        for (int k = 0; k < 4; ++k) dst[k] = make_uint4(w[4 * k], w[4 * k + 1], w[4 * k + 2], w[4 * k + 3]);
                    }
                }
                umma::fence_before_sync();
                wg_sync(wg);
                umma::fence_after_sync();
            }
        }
        if (abort_flag[wg]) break;
    }
    umma::fence_before_sync();
    __syncthreads();
    if (threadIdx.x < 32) umma::tmem_free(tmem_slot, 64 * INF_WG);
}

// Training: forward, loss gradient and backward over tiles of 128 radiance
// records; weight gradients accumulate in TMEM for all of a CTA's tiles and are
// added to the float32 gradient block at the end.  Loss per record: the
// radiance-weighted cross-entropy of the record direction's cell under the
// softmax p of the 64 outputs, Y (logsumexp(y) - y_cell), averaged over the
// records used.  Each CTA stores its whole gradient (weights and biases, zeros
// included) into its own slice of `part` (gridDim.x x AR_MLP_PARAMS floats);
// k_mlp_grad_sum adds the slices in CTA order.  Its minimiser is
// p(cell | position, view) proportional to
// E[Y 1(direction in cell)], the radiance the records carried into each cell:
// what a voxel probe's leaf accumulates (radiance x Jacobian per texel over
// the records of its voxel and face, core/guiding/guiding.cuh:373-418), so the
// network learns the probes' distribution, including the density of the
// directions the records were sampled with.
__global__ void __launch_bounds__(128, 1)
    k_mlp_train(MlpDev net, const float4* __restrict__ r_pos, const float4* __restrict__ r_wr,
                const float4* __restrict__ r_dir, const float4* __restrict__ r_rad, const int* __restrict__ count_ptr,
                int n_direct, int n_train, int offset, float* __restrict__ part, float* __restrict__ loss_sum,
                unsigned* err)
{
    using namespace mlpk;
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t* W = smem;
    uint8_t* X = W + W_BYTES;
    uint8_t* Hs = X + X_BYTES;  // 4 hidden tiles
    uint8_t* DY = Hs + 4 * H_BYTES;  // 2 gradient tiles, 128 columns
    float* sbias = reinterpret_cast<float*>(DY + 2 * DY_BYTES);
    float* sdb = sbias + 5 * 64;
    __shared__ uint64_t mbar;
    __shared__ uint32_t tmem_slot;
    __shared__ int abort_flag;
    __shared__ float sloss;
    const int row = threadIdx.x, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    load_weights(W, net.wbf, sbias, net.w32);
    for (int i = threadIdx.x; i < 2 * DY_BYTES / 16; i += blockDim.x) reinterpret_cast<uint4*>(DY)[i] = make_uint4(0, 0, 0, 0);
    for (int i = threadIdx.x; i < 5 * 64; i += blockDim.x) sdb[i] = 0.0f;
    if (warp == 0) umma::tmem_alloc(&tmem_slot, TR_TMEM_COLS);
    if (threadIdx.x == 0)
    {
        umma::mbar_init(&mbar, 1);
        abort_flag = 0;
        sloss = 0.0f;
    }
    umma::fence_async_smem();
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tmem = tmem_slot;
    const int count = count_ptr ? *count_ptr : n_direct;
    const int n_use = min(count, n_train);
    const int stride = n_use > 0 ? max(1, count / n_use) : 1;
    const float inv_n = n_use > 0 ? 1.0f / (float)n_use : 0.0f;
    const int tiles = (n_use + 127) / 128;
    uint32_t phase = 0;
    bool first = true;
    float my_loss = 0.0f;
    for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x)
    {
        const int s = tile * 128 + row;
        const bool valid = s < n_use;
        const int rec = valid ? (int)(((long long)s * stride + offset) % count) : 0;
        float in6[6] = {0, 0, 0, 0, 0, 0};
        int cell = 0;
        float target = 0.0f;
        if (valid)
        {
            const float4 a = r_pos[rec], w = r_wr[rec], d = r_dir[rec], L = r_rad[rec];
            mlp_inputs(net.box, v3(a.x, a.y, a.z), v3(w.x, w.y, w.z), in6);
            cell = mlp_cell(normalize(v3(d.x, d.y, d.z)));
            target = fmaxf(L.y, 0.0f);
        }
        encode_row(X, row, in6);
        wg_publish(0);
        // ---- forward
        float v[64];
        for (int l = 0; l < AR_MLP_LAYERS; ++l)
        {
            const int in = mlp_in_dim(l);
            if (row == 0)
            {
                const uint32_t a0 = umma::smem_addr(l == 0 ? X : Hs + (l - 1) * H_BYTES);
                const uint32_t b0 = umma::smem_addr(W + w_tile_offset(l));
                const uint32_t idesc = umma::make_idesc(128, 64, false, false);
                for (int k = 0; k < in / 16; ++k)
                    umma::mma(tmem, umma::tile_desc(a0, in, 0, 16 * k, false), umma::tile_desc(b0, in, 0, 16 * k, false),
                              idesc, k > 0);
                umma::commit(&mbar);
            }
            if (!umma::mbar_wait(&mbar, phase))
            {
                atomicOr(err, AR_DEVERR_MLP);
                abort_flag = 1;
                umma::mbar_wait(&mbar, phase);
            }
            phase ^= 1u;
            umma::fence_after_sync();
            load_row64(tmem, warp, 0, v);
            const float* b = sbias + 64 * l;
            if (l < AR_MLP_LAYERS - 1)
            {
                uint8_t* Ho = Hs + l * H_BYTES;
                for (int c = 0; c < 8; ++c)
                {
                    float h[8];
                    for (int i = 0; i < 8; ++i) h[i] = fmaxf(v[8 * c + i] + b[8 * c + i], 0.0f);
                    store8(Ho, 64, row, 8 * c, h);
                }
            }
            else
            {
                // radiance-weighted cross-entropy of the record's cell under the
                // softmax of the outputs: weight Y, d loss / d y_j = Y (p_j - [j == cell])
                float mx = -3.0e38f;
                for (int i = 0; i < 64; ++i)
                {
                    v[i] += b[i];
                    mx = fmaxf(mx, v[i]);
                }
                float se = 0.0f;
                for (int i = 0; i < 64; ++i) se += __expf(v[i] - mx);
                const float inv_se = 1.0f / se;
                const float wgt = valid ? target * inv_n : 0.0f;
                if (valid && target > 0.0f) my_loss += target * (mx + __logf(se) - v[cell]);
                for (int c = 0; c < 8; ++c)
                {
                    float g[8];
                    for (int i = 0; i < 8; ++i)
                    {
                        const int j = 8 * c + i;
                        g[i] = wgt * (__expf(v[j] - mx) * inv_se - (j == cell ? 1.0f : 0.0f));
                    }
                    store8(DY, 128, row, 8 * c, g);
                    for (int i = 0; i < 8; ++i)
                    {
                        float t = g[i];
                        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
                        if (lane == 0 && t != 0.0f) atomicAdd(&sdb[4 * 64 + 8 * c + i], t);
                    }
                }
            }
            wg_publish(0);
        }
        // ---- backward
        int cur = 0;
        for (int l = AR_MLP_LAYERS - 1; l >= 0; --l)
        {
            const int in = mlp_in_dim(l);
            uint8_t* dyc = DY + cur * DY_BYTES;
            const uint8_t* inbuf = l == 0 ? X : Hs + (l - 1) * H_BYTES;
            if (row == 0)
            {
                // dW_l += dY_l^T . input_l   (M = outputs padded to 128, N = inputs, K = 128 records)
                const uint32_t a0 = umma::smem_addr(dyc), b0 = umma::smem_addr(inbuf);
                const uint32_t idw = umma::make_idesc(128, in, true, true);
                for (int k = 0; k < 8; ++k)
                    umma::mma(tmem + dw_col(l), umma::tile_desc(a0, 128, 16 * k, 0, true),
                              umma::tile_desc(b0, in, 16 * k, 0, true), idw, !(first && k == 0));
                if (l > 0)
                {
                    // dH = dY_l . W_l   (K = 64 outputs)
                    const uint32_t w0 = umma::smem_addr(W + w_tile_offset(l));
                    const uint32_t idx = umma::make_idesc(128, 64, false, true);
                    for (int k = 0; k < 4; ++k)
                        umma::mma(tmem, umma::tile_desc(a0, 128, 0, 16 * k, false), umma::tile_desc(w0, 64, 16 * k, 0, true),
                                  idx, k > 0);
                }
                umma::commit(&mbar);
            }
            if (!umma::mbar_wait(&mbar, phase))
            {
                atomicOr(err, AR_DEVERR_MLP);
                abort_flag = 1;
                umma::mbar_wait(&mbar, phase);
            }
            phase ^= 1u;
            umma::fence_after_sync();
            if (l > 0)
            {
                load_row64(tmem, warp, 0, v);
                const uint8_t* hin = Hs + (l - 1) * H_BYTES;
                uint8_t* dyn = DY + (cur ^ 1) * DY_BYTES;
                for (int c = 0; c < 8; ++c)
                {
                    float h[8], g[8];
                    load8(hin, 64, row, 8 * c, h);
                    for (int i = 0; i < 8; ++i) g[i] = h[i] > 0.0f ? v[8 * c + i] : 0.0f;
                    store8(dyn, 128, row, 8 * c, g);
                    for (int i = 0; i < 8; ++i)
                    {
                        float t = g[i];
                        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
                        if (lane == 0 && t != 0.0f) atomicAdd(&sdb[(l - 1) * 64 + 8 * c + i], t);
                    }
                }
            }
            wg_publish(0);
            cur ^= 1;
        }
        first = false;
        if (abort_flag) break;
    }
    // ---- flush: this CTA's weight gradients (TMEM lanes 0-63 = outputs) and
    // bias gradients into its slice of `part`, the loss into loss_sum
    for (int o = 16; o > 0; o >>= 1) my_loss += __shfl_xor_sync(0xffffffffu, my_loss, o);
    if (lane == 0 && my_loss != 0.0f) atomicAdd(&sloss, my_loss);
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    float* slice = part + (size_t)blockIdx.x * AR_MLP_PARAMS;
    if (warp < 2)
    {
        const int o = warp * 32 + lane;
        for (int l = 0; l < AR_MLP_LAYERS; ++l)
        {
            const int in = mlp_in_dim(l);
            for (int j = 0; j < in / 16; ++j)
            {
                float g[16];
                if (!first) umma::tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(dw_col(l) + 16 * j), g);
                else
                    for (int i = 0; i < 16; ++i) g[i] = 0.0f;  // no tile: the accumulators were never written
                float4* dst = reinterpret_cast<float4*>(slice + mlp_w_offset(l) + o * in + 16 * j);
                for (int i = 0; i < 4; ++i) dst[i] = make_float4(g[4 * i], g[4 * i + 1], g[4 * i + 2], g[4 * i + 3]);
            }
        }
    }
    for (int k = threadIdx.x; k < 5 * 64; k += blockDim.x) slice[mlp_b_offset(k / 64) + (k % 64)] = sdb[k];
    if (threadIdx.x == 0 && loss_sum && sloss != 0.0f) atomicAdd(loss_sum, sloss);
    umma::fence_before_sync();
    __syncthreads();
    if (warp == 0) umma::tmem_free(tmem, TR_TMEM_COLS);
}

// grad += the sum of the training CTAs' gradient slices, in CTA order
__global__ void k_mlp_grad_sum(const float* __restrict__ part, int slices, float* __restrict__ grad)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= AR_MLP_PARAMS) return;
    float acc = 0.0f;
    for (int b = 0; b < slices; ++b) acc += part[(size_t)b * AR_MLP_PARAMS + i];
    grad[i] += acc;
}

// Adam on the float32 master parameters; refreshes the bf16 copy and clears
// the gradient block.
__global__ void k_mlp_adam(float* __restrict__ w32, uint16_t* __restrict__ wbf, float* __restrict__ grad,
                           float* __restrict__ m, float* __restrict__ v, int n, float lr, float b1, float b2, float eps,
                           float bc1, float bc2)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float g = grad[i];
    grad[i] = 0.0f;
    const float mi = b1 * m[i] + (1.0f - b1) * g;
    const float vi = b2 * v[i] + (1.0f - b2) * g * g;
    m[i] = mi;
    v[i] = vi;
    const float w = w32[i] - lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
    w32[i] = w;
    const __nv_bfloat16 h = __float2bfloat16_rn(w);
    wbf[i] = *reinterpret_cast<const uint16_t*>(&h);
}

__global__ void k_mlp_to_bf16(const float* __restrict__ w32, uint16_t* __restrict__ wbf, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const __nv_bfloat16 h = __float2bfloat16_rn(w32[i]);
    wbf[i] = *reinterpret_cast<const uint16_t*>(&h);
}

cudaError_t mlp_prepare_kernels()
{
    cudaError_t e = cudaFuncSetAttribute(k_mlp_infer, cudaFuncAttributeMaxDynamicSharedMemorySize, mlpk::INF_SMEM);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize, mlpk::TR_SMEM);
    return e;
}

cudaError_t launch_mlp_infer(const MlpDev& net, const float4* q_pos, const float4* q_wr, const int* queue,
                             const int* count, int n_direct, uint8_t* out, float* logits, unsigned* err, int sms,
                             cudaStream_t s)
{
    k_mlp_infer<<<sms, 128 * mlpk::INF_WG, mlpk::INF_SMEM, s>>>(net, q_pos, q_wr, queue, count, n_direct, out, logits, err);
    return cudaGetLastError();
}

cudaError_t launch_mlp_train(const MlpDev& net, const float4* r_pos, const float4* r_wr, const float4* r_dir,
                             const float4* r_rad, const int* count, int n_direct, int n_train, int offset, float* grad,
                             float* part, float* loss_sum, unsigned* err, int sms, cudaStream_t s)
{
    const int tiles = (n_train + 127) / 128;
    const int grid = std::max(1, std::min(sms, tiles));
    k_mlp_train<<<grid, 128, mlpk::TR_SMEM, s>>>(net, r_pos, r_wr, r_dir, r_rad, count, n_direct, n_train, offset,
                                                  part, loss_sum, err);
    k_mlp_grad_sum<<<(AR_MLP_PARAMS + 255) / 256, 256, 0, s>>>(part, grid, grad);
    return cudaGetLastError();
}

// Output biases start at the log of the first frame's mean record radiance (a
// data-dependent start: the outputs predict log mean radiance, far from zero,
// and the sampled distribution only depends on differences between outputs).
__global__ void k_mlp_bias_start(float* __restrict__ w32, const float4* __restrict__ r_rad, const int* __restrict__ count)
{
    __shared__ float ssum[256];
    __shared__ int scnt[256];
    const int n = *count;
    const int use = min(n, 65536);
    const int stride = use > 0 ? max(1, n / use) : 1;
    float sum = 0.0f;
    int cnt = 0;
    for (int i = threadIdx.x; i < use; i += blockDim.x)
    {
        sum += fmaxf(r_rad[(long long)i * stride % n].y, 0.0f);
        ++cnt;
    }
    ssum[threadIdx.x] = sum;
    scnt[threadIdx.x] = cnt;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1)
    {
        if (threadIdx.x < o)
        {
            ssum[threadIdx.x] += ssum[threadIdx.x + o];
            scnt[threadIdx.x] += scnt[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x < 64 && scnt[0] > 0)
        w32[mlp_b_offset(AR_MLP_LAYERS - 1) + threadIdx.x] = __logf(ssum[0] / (float)scnt[0] + 1.0e-6f);
}

cudaError_t launch_mlp_bias_start(float* w32, const float4* r_rad, const int* count, cudaStream_t s)
{
    k_mlp_bias_start<<<1, 256, 0, s>>>(w32, r_rad, count);
    return cudaGetLastError();
}

cudaError_t launch_mlp_adam(float* w32, uint16_t* wbf, float* grad, float* m, float* v, int step, float lr,
                            cudaStream_t s)
{
    const float b1 = 0.9f, b2 = 0.999f;
    const float bc1 = 1.0f - powf(b1, (float)step), bc2 = 1.0f - powf(b2, (float)step);
    k_mlp_adam<<<(AR_MLP_PARAMS + 255) / 256, 256, 0, s>>>(w32, wbf, grad, m, v, AR_MLP_PARAMS, lr, b1, b2, 1.0e-8f,
                                                           bc1, bc2);
    return cudaGetLastError();
}

cudaError_t launch_mlp_to_bf16(const float* w32, uint16_t* wbf, cudaStream_t s)
{
    k_mlp_to_bf16<<<(AR_MLP_PARAMS + 255) / 256, 256, 0, s>>>(w32, wbf, AR_MLP_PARAMS);
    return cudaGetLastError();
}

namespace
{
constexpr int ST_MAX_A = 128 * 144;  // elements
constexpr int ST_MAX_B = 144 * 144;

// D[128 x N] = A * B^T.  A is M x K (K-major) or K x M (MN-major), B is N x K
// (K-major) or K x N (MN-major), given row-major in global memory; both are
// staged into the core-matrix layout.  swap != 0 exchanges the two descriptor
// strides (the test runs both and keeps the one that matches the host GEMM).
// The staging buffers are twice the operand size, so either stride reading
// stays inside them.
__global__ void __launch_bounds__(128) k_umma_selftest(const uint16_t* __restrict__ A, const uint16_t* __restrict__ B,
                                                       int a_mn, int b_mn, int N, int K, int swap,
                                                       float* __restrict__ D, int* status)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t* sa = smem;
    uint8_t* sb = smem + 2 * ST_MAX_A * 2;
    __shared__ uint64_t mbar;
    __shared__ uint32_t tmem_slot;
    const int M = 128;
    const int a_rows = a_mn ? K : M, a_cols = a_mn ? M : K;
    const int b_rows = b_mn ? K : N, b_cols = b_mn ? N : K;
    for (int i = threadIdx.x; i < 2 * ST_MAX_A; i += blockDim.x) reinterpret_cast<uint16_t*>(sa)[i] = 0;
    for (int i = threadIdx.x; i < 2 * ST_MAX_B; i += blockDim.x) reinterpret_cast<uint16_t*>(sb)[i] = 0;
    __syncthreads();
    for (int i = threadIdx.x; i < a_rows * a_cols; i += blockDim.x)
    {
        const int r = i / a_cols, c = i % a_cols;
        *reinterpret_cast<uint16_t*>(sa + umma::tile_offset(r, c, a_cols)) = A[i];
    }
    for (int i = threadIdx.x; i < b_rows * b_cols; i += blockDim.x)
    {
        const int r = i / b_cols, c = i % b_cols;
        *reinterpret_cast<uint16_t*>(sb + umma::tile_offset(r, c, b_cols)) = B[i];
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (warp == 0) umma::tmem_alloc(&tmem_slot, 256);
    if (threadIdx.x == 0) umma::mbar_init(&mbar, 1);
    umma::fence_async_smem();
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tmem = tmem_slot;
    if (threadIdx.x == 0)
    {
        const uint32_t a0 = umma::smem_addr(sa), b0 = umma::smem_addr(sb);
        const uint32_t idesc = umma::make_idesc(M, N, a_mn != 0, b_mn != 0);
        for (int k = 0; k < K / 16; ++k)
        {
            // K advances by 16: two column chunks (K-major) or two row groups (MN-major)
            uint64_t ad = a_mn ? umma::tile_desc(a0, a_cols, 16 * k, 0, true) : umma::tile_desc(a0, a_cols, 0, 16 * k, false);
            uint64_t bd = b_mn ? umma::tile_desc(b0, b_cols, 16 * k, 0, true) : umma::tile_desc(b0, b_cols, 0, 16 * k, false);
            if (swap)
            {
                // exchange the two stride fields (bits 16-29 and 32-45)
                const uint64_t m1 = 0x3FFFull << 16, m2 = 0x3FFFull << 32;
                ad = (ad & ~(m1 | m2)) | ((ad & m1) << 16) | ((ad & m2) >> 16);
                bd = (bd & ~(m1 | m2)) | ((bd & m1) << 16) | ((bd & m2) >> 16);
            }
            umma::mma(tmem, ad, bd, idesc, k > 0);
        }
        umma::commit(&mbar);
    }
    bool ok = umma::mbar_wait(&mbar, 0);
    if (!ok)
    {
        if (lane == 0) atomicOr(status, 1);
        ok = umma::mbar_wait(&mbar, 0);  // let the MMAs drain before the TMEM goes back
    }
    umma::fence_after_sync();
    if (ok)
    {
        const int row = warp * 32 + lane;
        for (int j = 0; j < N / 16; ++j)
        {
            float v[16];
            umma::tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(16 * j), v);
            for (int i = 0; i < 16; ++i) D[row * N + 16 * j + i] = v[i];
        }
    }
    umma::fence_before_sync();
    __syncthreads();
    if (warp == 0) umma::tmem_free(tmem, 256);
}
} // namespace
} // namespace ar

extern "C" ar_status ar_diag_umma_gemm(int device, const uint16_t* a, const uint16_t* b, int a_mn, int b_mn, int n, int k,
                                       int swap, float* d)
{
    using namespace ar;
    if (!a || !b || !d || (n != 64 && n != 128 && n != 144) || (k != 64 && k != 128 && k != 144)) return AR_ERR_INVALID;
    const int a_elems = 128 * k, b_elems = n * k;
    if (a_elems > ST_MAX_A || b_elems > ST_MAX_B) return AR_ERR_INVALID;
    if (cudaSetDevice(device) != cudaSuccess) return AR_ERR_CUDA;
    uint16_t *da = nullptr, *db = nullptr;
    float* dd = nullptr;
    int* dst = nullptr;
    cudaError_t e = cudaMalloc(&da, a_elems * 2);
    if (e == cudaSuccess) e = cudaMalloc(&db, b_elems * 2);
    if (e == cudaSuccess) e = cudaMalloc(&dd, 128 * n * 4);
    if (e == cudaSuccess) e = cudaMalloc(&dst, 4);
    if (e == cudaSuccess) e = cudaMemcpy(da, a, a_elems * 2, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(db, b, b_elems * 2, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(dst, 0, 4);
    const int smem = 2 * ST_MAX_A * 2 + 2 * ST_MAX_B * 2;
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_umma_selftest, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e == cudaSuccess)
    {
        k_umma_selftest<<<1, 128, smem>>>(da, db, a_mn, b_mn, n, k, swap, dd, dst);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    int st = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&st, dst, 4, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(d, dd, 128 * n * 4, cudaMemcpyDeviceToHost);
    cudaFree(da);
    cudaFree(db);
    cudaFree(dd);
    cudaFree(dst);
    if (e != cudaSuccess) return AR_ERR_CUDA;
    return st ? AR_ERR_DEVICE : AR_OK;
}

extern "C" ar_status ar_diag_mlp(int device, const float* params, const float* in6, const float* dirs, const float* nrm,
                                 const float* lum, int n, float* logits, float* grad, float* loss)
{
    using namespace ar;
    static_assert(AR_MLP_PARAMS == 25920, "parameter block size");
    if (!params || !in6 || !dirs || !lum || !logits || !grad || !loss || n <= 0 || n > (1 << 20)) return AR_ERR_INVALID;
    if (cudaSetDevice(device) != cudaSuccess) return AR_ERR_CUDA;
    std::vector<float4> pos(n), wr(n), dir(n), rad(n);
    for (int i = 0; i < n; ++i)
    {
        const float* x = in6 + 6 * (size_t)i;
        pos[i] = make_float4(x[0], x[1], x[2], 1.0f);
        // the packed normal rides along in the record (the cross-entropy loss does not read it)
        const V3 dn = nrm ? v3(nrm[3 * (size_t)i], nrm[3 * (size_t)i + 1], nrm[3 * (size_t)i + 2])
                          : -v3(dirs[3 * (size_t)i], dirs[3 * (size_t)i + 1], dirs[3 * (size_t)i + 2]);
        wr[i] = make_float4(2.0f * x[3] - 1.0f, 2.0f * x[4] - 1.0f, 2.0f * x[5] - 1.0f, mlp_pack_normal(normalize(dn)));
        dir[i] = make_float4(dirs[3 * (size_t)i], dirs[3 * (size_t)i + 1], dirs[3 * (size_t)i + 2], 0.0f);
        rad[i] = make_float4(0.0f, lum[i], 0.0f, 0.0f);
    }
    float *w32 = nullptr, *dgrad = nullptr, *dpart = nullptr, *dlog = nullptr, *dloss = nullptr;
    uint16_t* wbf = nullptr;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    float4* dbuf = nullptr;
    unsigned* derr = nullptr;
    cudaError_t e = cudaMalloc(&w32, AR_MLP_PARAMS * 4);
    if (e == cudaSuccess) e = cudaMalloc(&wbf, AR_MLP_PARAMS * 2);
    if (e == cudaSuccess) e = cudaMalloc(&dgrad, AR_MLP_PARAMS * 4);
    if (e == cudaSuccess) e = cudaMalloc(&dpart, (size_t)std::max(1, sms) * AR_MLP_PARAMS * 4);
    if (e == cudaSuccess) e = cudaMalloc(&dlog, (size_t)n * 64 * 4);
    if (e == cudaSuccess) e = cudaMalloc(&dloss, 4);
    if (e == cudaSuccess) e = cudaMalloc(&dbuf, (size_t)n * 4 * sizeof(float4));
    if (e == cudaSuccess) e = cudaMalloc(&derr, 4);
    if (e == cudaSuccess) e = cudaMemcpy(w32, params, AR_MLP_PARAMS * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(dgrad, 0, AR_MLP_PARAMS * 4);
    if (e == cudaSuccess) e = cudaMemset(dloss, 0, 4);
    if (e == cudaSuccess) e = cudaMemset(derr, 0, 4);
    float4* dp = dbuf;
    float4* dw = dbuf + n;
    float4* dd = dbuf + 2 * (size_t)n;
    float4* dr = dbuf + 3 * (size_t)n;
    if (e == cudaSuccess) e = cudaMemcpy(dp, pos.data(), n * sizeof(float4), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dw, wr.data(), n * sizeof(float4), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dd, dir.data(), n * sizeof(float4), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dr, rad.data(), n * sizeof(float4), cudaMemcpyHostToDevice);
    MlpDev net;
    net.wbf = wbf;
    net.w32 = w32;
    for (int k = 0; k < 3; ++k)
    {
        net.box.lo[k] = 0.0f;
        net.box.inv[k] = 1.0f;
    }
    if (e == cudaSuccess) e = mlp_prepare_kernels();
    if (e == cudaSuccess) e = launch_mlp_to_bf16(w32, wbf, 0);
    if (e == cudaSuccess) e = launch_mlp_infer(net, dp, dw, nullptr, nullptr, n, nullptr, dlog, derr, sms, 0);
    if (e == cudaSuccess) e = launch_mlp_train(net, dp, dw, dd, dr, nullptr, n, n, 0, dgrad, dpart, dloss, derr, sms, 0);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    unsigned herr = 0;
    if (e == cudaSuccess) e = cudaMemcpy(logits, dlog, (size_t)n * 64 * 4, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(grad, dgrad, AR_MLP_PARAMS * 4, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(loss, dloss, 4, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(&herr, derr, 4, cudaMemcpyDeviceToHost);
    cudaFree(w32);
    cudaFree(wbf);
    cudaFree(dgrad);
    cudaFree(dpart);
    cudaFree(dlog);
    cudaFree(dloss);
    cudaFree(dbuf);
    cudaFree(derr);
    if (e != cudaSuccess) return AR_ERR_CUDA;
    return herr ? AR_ERR_DEVICE : AR_OK;
}
