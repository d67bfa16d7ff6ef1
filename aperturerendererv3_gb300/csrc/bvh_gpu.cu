// GPU build of the 8-wide compressed BVH (the same node and slot format as the
// host builder, ar_bvh.h), and its refit after mesh vertices move (the tree is
// kept; slots take the new vertices, boxes are recomputed from the leaves up).  The reference
// builds its BVH on the host (BuildBVH, core/bvh/bvh.cuh:142-422); for meshes of
// millions of triangles the build dominates scene setup, so this path runs it
// on the GPU:
//   1. Morton codes of primitive centroids (63 bits) in the centroid bounds,
//      scaled by the largest extent on every axis (cells stay cubes);
//   2. a stable LSD radix sort of (code, primitive) pairs, 8-bit digits;
//   3. the binary radix tree over the sorted codes (Karras, "Maximizing
//      parallelism in the construction of BVHs, octrees, and k-d trees", HPG
//      2012), equal codes ordered by position;
//   4. node boxes bottom-up (the second child to arrive at a node merges);
//   5. collapse to width 8, one level of wide nodes per launch: a wide node
//      opens its largest-area child until it has 8 children; a binary node
//      covering at most 3 primitives is a leaf; children take octant slots by
//      the greedy alignment rule of the host builder; boxes are quantized
//      conservatively against the node's box, as on the host.
// Hit results do not depend on the tree (closest hits are the smallest t, equal
// t the smallest id), so a GPU-built BVH answers exactly as the host-built one.
#include <cuda_runtime.h>

#include <cfloat>
#include <cmath>
#include <string>
#include <vector>

#include "../../include/aperture/ar.h"
#include "ar_bvh_build.h"
#include "ar_internal.h"

namespace ar
{
namespace lbvh
{
constexpr int kMaxLeaf = 3;
constexpr int kSortBlock = 256;
constexpr int kSortTiles = 16;  // tiles of kSortBlock keys per block per pass

__device__ __forceinline__ unsigned int fmin_bits(float f)  // order-preserving float -> uint
{
    const unsigned int u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float bits_fmin(unsigned int u)
{
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

// centroid bounds: bounds[0..2] min, [3..5] max, as ordered uints
__global__ void k_centroid_bounds(const arbvh::PrimInput* __restrict__ prims, int n, unsigned int* bounds)
{
    float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        for (int k = 0; k < 3; ++k)
        {
            const float c = 0.5f * (prims[i].lo[k] + prims[i].hi[k]);
            lo[k] = fminf(lo[k], c);
            hi[k] = fmaxf(hi[k], c);
        }
    for (int k = 0; k < 3; ++k)
    {
        for (int o = 16; o > 0; o >>= 1)
        {
            lo[k] = fminf(lo[k], __shfl_xor_sync(0xffffffffu, lo[k], o));
            hi[k] = fmaxf(hi[k], __shfl_xor_sync(0xffffffffu, hi[k], o));
        }
        if ((threadIdx.x & 31) == 0)
        {
            atomicMin(&bounds[k], fmin_bits(lo[k]));
            atomicMax(&bounds[3 + k], fmin_bits(hi[k]));
        }
    }
}

// spreads the low 21 bits of v to every third bit
__device__ __forceinline__ unsigned long long expand_bits21(unsigned long long v)
{
    v &= 0x1fffffull;
    v = (v | (v << 32)) & 0x1f00000000ffffull;
    v = (v | (v << 16)) & 0x1f0000ff0000ffull;
    v = (v | (v << 8)) & 0x100f00f00f00f00full;
    v = (v | (v << 4)) & 0x10c30c30c30c30c3ull;
    v = (v | (v << 2)) & 0x1249249249249249ull;
    return v;
}

__global__ void k_morton(const arbvh::PrimInput* __restrict__ prims, int n, const unsigned int* bounds,
                         unsigned long long* keys, unsigned int* vals)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float lo[3], ext = 0.0f;
    for (int k = 0; k < 3; ++k)
    {
        lo[k] = bits_fmin(bounds[k]);
        ext = fmaxf(ext, bits_fmin(bounds[3 + k]) - lo[k]);
    }
    unsigned long long code = 0;
    for (int k = 0; k < 3; ++k)
    {
        const float c = 0.5f * (prims[i].lo[k] + prims[i].hi[k]);
        float u = ext > 0.0f ? (c - lo[k]) / ext : 0.0f;
        u = fminf(fmaxf(u, 0.0f), 1.0f);
        const unsigned long long q = min((unsigned long long)(u * 2097152.0f), 2097151ull);
        code |= expand_bits21(q) << (2 - k);
    }
    keys[i] = code;
    vals[i] = (unsigned int)i;
}

// ---- stable LSD radix sort, 8-bit digits.  A block owns kSortTiles
// consecutive tiles of kSortBlock keys; pass: histogram per block, exclusive
// scan over (digit, block), stable scatter (rank within a tile from warp
// matches and per-warp digit counts, tiles in order).
__global__ void k_sort_hist(const unsigned long long* __restrict__ keys, int n, int shift, unsigned int* hist, int nblocks)
{
    __shared__ unsigned int h[256];
    for (int i = threadIdx.x; i < 256; i += blockDim.x) h[i] = 0;
    __syncthreads();
    const long long base = (long long)blockIdx.x * kSortBlock * kSortTiles;
    for (int t = 0; t < kSortTiles; ++t)
    {
        const long long i = base + (long long)t * kSortBlock + threadIdx.x;
        if (i < n) atomicAdd(&h[(unsigned int)(keys[i] >> shift) & 0xffu], 1u);
    }
    __syncthreads();
    for (int d = threadIdx.x; d < 256; d += blockDim.x) hist[(size_t)d * nblocks + blockIdx.x] = h[d];
}

// exclusive scan of hist (256 x nblocks, digit-major) in place; one block
__global__ void k_sort_scan(unsigned int* hist, int total)
{
    __shared__ unsigned int carry;
    __shared__ unsigned int part[1024];
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < total; base += 1024)
    {
        const int i = base + threadIdx.x;
        const unsigned int v = i < total ? hist[i] : 0u;
        part[threadIdx.x] = v;
        __syncthreads();
        for (int o = 1; o < 1024; o <<= 1)
        {
            const unsigned int a = threadIdx.x >= o ? part[threadIdx.x - o] : 0u;
            __syncthreads();
            part[threadIdx.x] += a;
            __syncthreads();
        }
        if (i < total) hist[i] = carry + part[threadIdx.x] - v;
        __syncthreads();
        if (threadIdx.x == 1023) carry += part[1023];
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kSortBlock) k_sort_scatter(const unsigned long long* __restrict__ keys,
                                                           const unsigned int* __restrict__ vals, int n, int shift,
                                                           const unsigned int* __restrict__ hist, int nblocks,
                                                           unsigned long long* __restrict__ okeys,
                                                           unsigned int* __restrict__ ovals)
{
    constexpr int W = kSortBlock / 32;
    __shared__ unsigned int run[256];         // next output position per digit
    __shared__ unsigned int wcnt[W][256];     // per-warp digit counts of the tile
    for (int d = threadIdx.x; d < 256; d += blockDim.x) run[d] = hist[(size_t)d * nblocks + blockIdx.x];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long base = (long long)blockIdx.x * kSortBlock * kSortTiles;
    for (int t = 0; t < kSortTiles; ++t)
    {
        for (int k = threadIdx.x; k < W * 256; k += blockDim.x) (&wcnt[0][0])[k] = 0;
        __syncthreads();
        const long long i = base + (long long)t * kSortBlock + threadIdx.x;
        const bool valid = i < n;
        const unsigned long long key = valid ? keys[i] : 0ull;
        const unsigned int dig = valid ? ((unsigned int)(key >> shift) & 0xffu) : 256u;
        const unsigned int peers = __match_any_sync(0xffffffffu, dig);
        const unsigned int rank_in_warp = __popc(peers & ((1u << lane) - 1u));
        if (valid && rank_in_warp == 0) wcnt[warp][dig] = __popc(peers);
        __syncthreads();
        unsigned int pos = 0;
        if (valid)
        {
            unsigned int before = 0;
            for (int w = 0; w < warp; ++w) before += wcnt[w][dig];
            pos = run[dig] + before + rank_in_warp;
            okeys[pos] = key;
            ovals[pos] = vals[i];
        }
        __syncthreads();
        // advance the running offsets by this tile's digit counts
        for (int d = threadIdx.x; d < 256; d += blockDim.x)
        {
            unsigned int c = 0;
            for (int w = 0; w < W; ++w) c += wcnt[w][d];
            run[d] += c;
        }
        __syncthreads();
    }
}

// ---- radix tree (Karras 2012).  Internal nodes 0..n-2, leaves n-1+k for sorted
// position k.  first/last: the sorted range a node covers.
__device__ __forceinline__ int delta(const unsigned long long* keys, int n, int i, int j)
{
    if (j < 0 || j >= n) return -1;
    const unsigned long long a = keys[i], b = keys[j];
    if (a != b) return __clzll(a ^ b);
    return 64 + __clz((unsigned int)i ^ (unsigned int)j);
}

__global__ void k_radix_tree(const unsigned long long* __restrict__ keys, int n, int2* child, int* parent, int2* range)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    const int d = (delta(keys, n, i, i + 1) - delta(keys, n, i, i - 1)) >= 0 ? 1 : -1;
    const int dmin = delta(keys, n, i, i - d);
    int lmax = 2;
    while (delta(keys, n, i, i + lmax * d) > dmin) lmax <<= 1;
    int l = 0;
    for (int t = lmax >> 1; t >= 1; t >>= 1)
        if (delta(keys, n, i, i + (l + t) * d) > dmin) l += t;
    const int j = i + l * d;
    const int dnode = delta(keys, n, i, j);
    int s = 0;
    int t = l;
    do
    {
        t = (t + 1) >> 1;
        if (delta(keys, n, i, i + (s + t) * d) > dnode) s += t;
    } while (t > 1);
    const int split = i + s * d + min(d, 0);
    const int first = min(i, j), last = max(i, j);
    const int left = (first == split) ? (n - 1 + split) : split;
    const int right = (last == split + 1) ? (n - 1 + split + 1) : split + 1;
    child[i] = make_int2(left, right);
    parent[left] = i;
    parent[right] = i;
    range[i] = make_int2(first, last);
}

struct Box6
{
    float lo[3], hi[3];
};

__global__ void k_boxes(const arbvh::PrimInput* __restrict__ prims, const unsigned int* __restrict__ order, int n,
                        const int2* __restrict__ child, const int* __restrict__ parent, Box6* box, int* flag)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    int node = n - 1 + k;
    const arbvh::PrimInput& p = prims[order[k]];
    for (int a = 0; a < 3; ++a)
    {
        box[node].lo[a] = p.lo[a];
        box[node].hi[a] = p.hi[a];
    }
    if (n == 1) return;
    node = parent[node];
    while (true)
    {
        __threadfence();
        if (atomicAdd(&flag[node], 1) == 0) return;  // the other child is not done yet
        __threadfence();
        const int2 c = child[node];
        // the other child's box was written by another SM: read it from L2
        const float* bx = reinterpret_cast<const float*>(&box[c.x]);
        const float* by = reinterpret_cast<const float*>(&box[c.y]);
        Box6 b;
        for (int a = 0; a < 3; ++a)
        {
            b.lo[a] = fminf(__ldcg(bx + a), __ldcg(by + a));
            b.hi[a] = fmaxf(__ldcg(bx + 3 + a), __ldcg(by + 3 + a));
        }
        box[node] = b;
        if (node == 0) return;
        node = parent[node];
        if (node < 0 || node >= n - 1) return;  // malformed tree: the build reports a count mismatch
    }
}

__device__ __forceinline__ double box_area(const Box6& b)
{
    const double dx = fmax(0.0, (double)b.hi[0] - b.lo[0]);
    const double dy = fmax(0.0, (double)b.hi[1] - b.lo[1]);
    const double dz = fmax(0.0, (double)b.hi[2] - b.lo[2]);
    return 2.0 * (dx * dy + dy * dz + dz * dx);
}

// number of sorted primitives under binary node b
__device__ __forceinline__ int node_count(int b, int n, const int2* range)
{
    if (b >= n - 1) return 1;
    const int2 r = range[b];
    return r.y - r.x + 1;
}
__device__ __forceinline__ int node_first(int b, int n, const int2* range)
{
    return b >= n - 1 ? b - (n - 1) : range[b].x;
}

struct CollapseArgs
{
    const arbvh::PrimInput* prims;
    const unsigned int* order;
    int n;
    const int2* child;
    const int2* range;
    const Box6* box;
    ar_wide_node* nodes;
    ar_prim_slot* slots;
    int* node_counter;
    int* slot_counter;
    int node_cap;
};

// one wide node per queue entry (wide index, binary index); internal children
// are appended to the next level's queue
__global__ void k_collapse(CollapseArgs a, const int2* __restrict__ queue, int nq, int2* next, int* next_count,
                           unsigned int* err)
{
    const int qi = blockIdx.x * blockDim.x + threadIdx.x;
    if (qi >= nq) return;
    const int wi = queue[qi].x, b = queue[qi].y;
    const int n = a.n;
    int ch[8];
    int nch = 0;
    if (node_count(b, n, a.range) <= kMaxLeaf) ch[nch++] = b;
    else
    {
        ch[nch++] = a.child[b].x;
        ch[nch++] = a.child[b].y;
    }
    while (nch < 8)
    {
        int pick = -1;
        double best = -1.0;
        for (int i = 0; i < nch; ++i)
        {
            if (node_count(ch[i], n, a.range) <= kMaxLeaf) continue;
            const double ar = box_area(a.box[ch[i]]);
            if (ar > best)
            {
                best = ar;
                pick = i;
            }
        }
        if (pick < 0) break;
        const int c = ch[pick];
        ch[pick] = a.child[c].x;
        ch[nch++] = a.child[c].y;
    }
    Box6 nb;
    for (int k = 0; k < 3; ++k)
    {
        nb.lo[k] = FLT_MAX;
        nb.hi[k] = -FLT_MAX;
    }
    for (int i = 0; i < nch; ++i)
        for (int k = 0; k < 3; ++k)
        {
            nb.lo[k] = fminf(nb.lo[k], a.box[ch[i]].lo[k]);
            nb.hi[k] = fmaxf(nb.hi[k], a.box[ch[i]].hi[k]);
        }
    double nc[3];
    for (int k = 0; k < 3; ++k) nc[k] = 0.5 * ((double)nb.lo[k] + nb.hi[k]);
    // octant slots: greedy over (child, slot) by decreasing alignment, ties to
    // the earlier candidate (the host builder's stable sort)
    double cost[8][8];
    for (int i = 0; i < nch; ++i)
    {
        double off[3];
        for (int k = 0; k < 3; ++k) off[k] = 0.5 * ((double)a.box[ch[i]].lo[k] + a.box[ch[i]].hi[k]) - nc[k];
        for (int s = 0; s < 8; ++s)
        {
            double c = 0.0;
            for (int k = 0; k < 3; ++k) c += ((s >> k) & 1) ? off[k] : -off[k];
            cost[i][s] = c;
        }
    }
    int slot_of[8], child_in_slot[8];
    for (int i = 0; i < 8; ++i)
    {
        slot_of[i] = -1;
        child_in_slot[i] = -1;
    }
    for (int round = 0; round < nch; ++round)
    {
        int bi = -1, bs = -1;
        double bc = 0.0;
        for (int i = 0; i < nch; ++i)
        {
            if (slot_of[i] >= 0) continue;
            for (int s = 0; s < 8; ++s)
            {
                if (child_in_slot[s] >= 0) continue;
                if (bi < 0 || cost[i][s] > bc)
                {
                    bc = cost[i][s];
                    bi = i;
                    bs = s;
                }
            }
        }
        slot_of[bi] = bs;
        child_in_slot[bs] = bi;
    }
    ar_wide_node node;
    memset(&node, 0, sizeof(node));
    memset(node.qlo, 0xff, sizeof(node.qlo));  // empty slots: an inverted box that no ray meets
    node.px = nb.lo[0];
    node.py = nb.lo[1];
    node.pz = nb.lo[2];
    double scale[3];
    for (int k = 0; k < 3; ++k)
    {
        const double ext = (double)nb.hi[k] - nb.lo[k];
        int e = -126;
        if (ext > 0.0)
        {
            e = (int)ceil(log2(ext / 255.0));
            while (ldexp(255.0, e) < ext) ++e;
            e = max(-126, min(127, e));
        }
        node.e[k] = (uint8_t)(e + 127);
        scale[k] = ldexp(1.0, e);
    }
    int n_int = 0, n_prims = 0;
    for (int i = 0; i < nch; ++i)
    {
        const int c = node_count(ch[i], n, a.range);
        if (c <= kMaxLeaf) n_prims += c;
        else ++n_int;
    }
    const int child_base = n_int ? atomicAdd(a.node_counter, n_int) : 0;
    const int prim_base = n_prims ? atomicAdd(a.slot_counter, n_prims) : 0;
    if (child_base + n_int > a.node_cap || prim_base + n_prims > n)
    {
        atomicOr(err, AR_DEVERR_QUEUE);
        return;
    }
    node.child_base = (uint32_t)child_base;
    node.prim_base = (uint32_t)prim_base;
    const double p[3] = {nb.lo[0], nb.lo[1], nb.lo[2]};
    int rank = 0, off = 0;
    for (int s = 0; s < 8; ++s)
    {
        const int ci = child_in_slot[s];
        if (ci < 0) continue;
        const int c = ch[ci];
        const Box6& cb = a.box[c];
        for (int k = 0; k < 3; ++k)
        {
            double ql = floor(((double)cb.lo[k] - p[k]) / scale[k]);
            double qh = ceil(((double)cb.hi[k] - p[k]) / scale[k]);
            ql = fmin(fmax(ql, 0.0), 255.0);
            qh = fmin(fmax(qh, 0.0), 255.0);
            node.qlo[k][s] = (uint8_t)ql;
            node.qhi[k][s] = (uint8_t)qh;
        }
        const int cnt = node_count(c, n, a.range);
        if (cnt > kMaxLeaf)
        {
            node.imask |= (uint8_t)(1u << s);
            node.meta[s] = (uint8_t)(0x80u | (uint32_t)rank);
            const int qn = atomicAdd(next_count, 1);
            if (qn < a.node_cap) next[qn] = make_int2(child_base + rank, c);
            else atomicOr(err, AR_DEVERR_QUEUE);
            ++rank;
        }
        else
        {
            node.meta[s] = (uint8_t)(((uint32_t)cnt << 5) | (uint32_t)off);
            const int first = node_first(c, n, a.range);
            for (int j = 0; j < cnt; ++j)
            {
                const arbvh::PrimInput& pi = a.prims[a.order[first + j]];
                ar_prim_slot sl;
                memset(&sl, 0, sizeof(sl));
                const uint32_t tag = pi.id | (pi.kind << AR_PRIM_KIND_SHIFT);
                if (pi.kind == AR_PRIM_KIND_TRI)
                    for (int k = 0; k < 3; ++k)
                    {
                        sl.a[k] = pi.v[k];
                        sl.b[k] = pi.v[3 + k];
                        sl.c[k] = pi.v[6 + k];
                    }
                sl.a[3] = __uint_as_float(tag);
                a.slots[prim_base + off + j] = sl;
            }
            off += cnt;
        }
    }
    a.nodes[wi] = node;
}
} // namespace lbvh

// ---- refit
// triangle slots take the moved vertices (slot tag -> triangle id - n_objects)
__global__ void k_refit_slots(float4* slots, int nslots, const float* __restrict__ verts, const uint32_t* __restrict__ idx,
                              int nobj)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nslots) return;
    const uint32_t tag = __float_as_uint(slots[3 * (size_t)s].w);
    if ((tag >> AR_PRIM_KIND_SHIFT) != AR_PRIM_KIND_TRI) return;
    const int id = (int)(tag & AR_PRIM_ID_MASK);
    if (id < nobj) return;  // a triangle object: not part of the mesh
    const size_t t = (size_t)(id - nobj);
    for (int j = 0; j < 3; ++j)
    {
        const float* v = verts + 3 * (size_t)idx[3 * t + j];
        float4 w = slots[3 * (size_t)s + j];
        w.x = v[0];
        w.y = v[1];
        w.z = v[2];
        slots[3 * (size_t)s + j] = w;
    }
}

// one depth of wide nodes: child boxes from the leaves' primitives or the
// deeper level's node boxes, then the node re-quantized as the builders do
__global__ void k_refit_level(ar_wide_node* nodes, const int* __restrict__ list, int nlist,
                              const float4* __restrict__ slots, const float* __restrict__ prim_box, float* node_box)
{
    const int li = blockIdx.x * blockDim.x + threadIdx.x;
    if (li >= nlist) return;
    const int ni = list[li];
    ar_wide_node node = nodes[ni];
    float cb[8][6];
    float nb[6] = {FLT_MAX, FLT_MAX, FLT_MAX, -FLT_MAX, -FLT_MAX, -FLT_MAX};
    int rank = 0;
    for (int s = 0; s < 8; ++s)
    {
        const uint32_t meta = node.meta[s];
        if (meta == 0u) continue;
        float b[6] = {FLT_MAX, FLT_MAX, FLT_MAX, -FLT_MAX, -FLT_MAX, -FLT_MAX};
        if (meta & 0x80u)
        {
            const float* src = node_box + 6 * (size_t)(node.child_base + rank);
            for (int k = 0; k < 6; ++k) b[k] = src[k];
            ++rank;
        }
        else
        {
            const int cnt = (int)(meta >> 5), first = (int)(node.prim_base + (meta & 31u));
            for (int j = 0; j < cnt; ++j)
            {
                const float4 a = slots[3 * (size_t)(first + j)];
                const uint32_t tag = __float_as_uint(a.w);
                if ((tag >> AR_PRIM_KIND_SHIFT) == AR_PRIM_KIND_TRI)
                {
                    const float4 bb = slots[3 * (size_t)(first + j) + 1], cc = slots[3 * (size_t)(first + j) + 2];
                    b[0] = fminf(b[0], fminf(a.x, fminf(bb.x, cc.x)));
                    b[1] = fminf(b[1], fminf(a.y, fminf(bb.y, cc.y)));
                    b[2] = fminf(b[2], fminf(a.z, fminf(bb.z, cc.z)));
                    b[3] = fmaxf(b[3], fmaxf(a.x, fmaxf(bb.x, cc.x)));
                    b[4] = fmaxf(b[4], fmaxf(a.y, fmaxf(bb.y, cc.y)));
                    b[5] = fmaxf(b[5], fmaxf(a.z, fmaxf(bb.z, cc.z)));
                }
                else
                {
                    const float* pb = prim_box + 6 * (size_t)(tag & AR_PRIM_ID_MASK);
                    for (int k = 0; k < 3; ++k)
                    {
                        b[k] = fminf(b[k], pb[k]);
                        b[3 + k] = fmaxf(b[3 + k], pb[3 + k]);
                    }
                }
            }
        }
        for (int k = 0; k < 6; ++k) cb[s][k] = b[k];
        for (int k = 0; k < 3; ++k)
        {
            nb[k] = fminf(nb[k], b[k]);
            nb[3 + k] = fmaxf(nb[3 + k], b[3 + k]);
        }
    }
    node.px = nb[0];
    node.py = nb[1];
    node.pz = nb[2];
    double scale[3];
    for (int k = 0; k < 3; ++k)
    {
        const double ext = (double)nb[3 + k] - nb[k];
        int e = -126;
        if (ext > 0.0)
        {
            e = (int)ceil(log2(ext / 255.0));
            while (ldexp(255.0, e) < ext) ++e;
            e = max(-126, min(127, e));
        }
        node.e[k] = (uint8_t)(e + 127);
        scale[k] = ldexp(1.0, e);
    }
    for (int s = 0; s < 8; ++s)
    {
        if (node.meta[s] == 0u) continue;
        for (int k = 0; k < 3; ++k)
        {
            double ql = floor(((double)cb[s][k] - nb[k]) / scale[k]);
            double qh = ceil(((double)cb[s][3 + k] - nb[k]) / scale[k]);
            node.qlo[k][s] = (uint8_t)fmin(fmax(ql, 0.0), 255.0);
            node.qhi[k][s] = (uint8_t)fmin(fmax(qh, 0.0), 255.0);
        }
    }
    nodes[ni] = node;
    for (int k = 0; k < 6; ++k) node_box[6 * (size_t)ni + k] = nb[k];
}

cudaError_t refit_wide_bvh(Ctx& c, const float* verts_dev, cudaStream_t s)
{
    const int nslots = (int)c.bvh.slots.size();
    if (nslots == 0) return cudaSuccess;
    k_refit_slots<<<(nslots + 255) / 256, 256, 0, s>>>(reinterpret_cast<float4*>(c.d_slots), nslots, verts_dev,
                                                        c.d_mesh_idx, (int)c.objects.size());
    cudaError_t e = cudaGetLastError();
    for (int d = (int)c.refit_level_off.size() - 2; d >= 0 && e == cudaSuccess; --d)
    {
        const int a = c.refit_level_off[d], b = c.refit_level_off[d + 1];
        if (b <= a) continue;
        k_refit_level<<<(b - a + 127) / 128, 128, 0, s>>>(reinterpret_cast<ar_wide_node*>(c.d_nodes), c.d_refit_nodes + a,
                                                         b - a, reinterpret_cast<const float4*>(c.d_slots), c.d_prim_box,
                                                         c.d_node_box);
        e = cudaGetLastError();
    }
    return e;
}

// Builds `prims` into out (host copies of nodes and slots, for the scene's
// bookkeeping) on the GPU; returns the error string or "".
std::string build_wide_bvh_gpu(const std::vector<arbvh::PrimInput>& prims, arbvh::WideBVH& out, cudaStream_t s)
{
    using namespace lbvh;
    out.nodes.clear();
    out.slots.clear();
    out.depth = 0;
    const int n = (int)prims.size();
    if (n == 0) return "";
    std::vector<void*> bufs;
    auto dalloc = [&](size_t bytes) -> void* {
        void* p = nullptr;
        if (cudaMalloc(&p, bytes) != cudaSuccess) return nullptr;
        bufs.push_back(p);
        return p;
    };
    auto cleanup = [&]() {
        for (void* p : bufs) cudaFree(p);
    };
    const int nblocks = (n + kSortBlock * kSortTiles - 1) / (kSortBlock * kSortTiles);
    const int node_cap = n;  // wide nodes never outnumber primitives
    auto* dprims = (arbvh::PrimInput*)dalloc(sizeof(arbvh::PrimInput) * n);
    auto* bounds = (unsigned int*)dalloc(6 * sizeof(unsigned int));
    auto* k0 = (unsigned long long*)dalloc(8ull * n);
    auto* v0 = (unsigned int*)dalloc(4ull * n);
    auto* k1 = (unsigned long long*)dalloc(8ull * n);
    auto* v1 = (unsigned int*)dalloc(4ull * n);
    auto* hist = (unsigned int*)dalloc(4ull * 256 * nblocks);
    auto* child = (int2*)dalloc(sizeof(int2) * (size_t)std::max(1, n - 1));
    auto* range = (int2*)dalloc(sizeof(int2) * (size_t)std::max(1, n - 1));
    auto* parent = (int*)dalloc(sizeof(int) * (size_t)(2 * n));
    auto* flag = (int*)dalloc(sizeof(int) * (size_t)std::max(1, n - 1));
    auto* box = (Box6*)dalloc(sizeof(Box6) * (size_t)(2 * n));
    auto* nodes = (ar_wide_node*)dalloc(sizeof(ar_wide_node) * (size_t)node_cap);
    auto* slots = (ar_prim_slot*)dalloc(sizeof(ar_prim_slot) * (size_t)n);
    auto* qa = (int2*)dalloc(sizeof(int2) * (size_t)node_cap);
    auto* qb = (int2*)dalloc(sizeof(int2) * (size_t)node_cap);
    auto* counters = (int*)dalloc(4 * sizeof(int));  // nodes, slots, next queue, error word
    for (void* p : bufs)
        if (!p)
        {
            cleanup();
            return "GPU BVH build: out of device memory";
        }
    cudaError_t e = cudaMemcpyAsync(dprims, prims.data(), sizeof(arbvh::PrimInput) * n, cudaMemcpyHostToDevice, s);
    const unsigned int init_bounds[6] = {0xffffffffu, 0xffffffffu, 0xffffffffu, 0u, 0u, 0u};
    if (e == cudaSuccess) e = cudaMemcpyAsync(bounds, init_bounds, sizeof(init_bounds), cudaMemcpyHostToDevice, s);
    const int grid = (n + 255) / 256;
    if (e == cudaSuccess)
    {
        k_centroid_bounds<<<std::min(grid, 1024), 256, 0, s>>>(dprims, n, bounds);
        k_morton<<<grid, 256, 0, s>>>(dprims, n, bounds, k0, v0);
        e = cudaGetLastError();
    }
    // 63-bit codes: eight 8-bit passes (the last one sees 7 bits)
    unsigned long long *ka = k0, *kb = k1;
    unsigned int *va = v0, *vb = v1;
    for (int pass = 0; pass < 8 && e == cudaSuccess; ++pass)
    {
        const int shift = 8 * pass;
        k_sort_hist<<<nblocks, kSortBlock, 0, s>>>(ka, n, shift, hist, nblocks);
        k_sort_scan<<<1, 1024, 0, s>>>(hist, 256 * nblocks);
        k_sort_scatter<<<nblocks, kSortBlock, 0, s>>>(ka, va, n, shift, hist, nblocks, kb, vb);
        e = cudaGetLastError();
        std::swap(ka, kb);
        std::swap(va, vb);
    }
    if (e == cudaSuccess) e = cudaMemsetAsync(flag, 0, sizeof(int) * (size_t)std::max(1, n - 1), s);
    if (e == cudaSuccess && n > 1)
    {
        k_radix_tree<<<(n - 1 + 255) / 256, 256, 0, s>>>(ka, n, child, parent, range);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess)
    {
        k_boxes<<<grid, 256, 0, s>>>(dprims, va, n, child, parent, box, flag);
        e = cudaGetLastError();
    }
    // collapse, level by level; the root is wide node 0 over binary node 0
    // (or the single leaf when n == 1)
    // the root: internal node 0, or leaf n - 1 = 0 when n == 1
    const int2 q0 = make_int2(0, 0);
    const int init_counters[4] = {1, 0, 0, 0};
    if (e == cudaSuccess) e = cudaMemcpyAsync(qa, &q0, sizeof(int2), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(counters, init_counters, sizeof(init_counters), cudaMemcpyHostToDevice, s);
    CollapseArgs ca{dprims, va, n, child, range, box, nodes, slots, &counters[0], &counters[1], node_cap};
    int nq = 1, depth = 0;
    while (e == cudaSuccess && nq > 0)
    {
        ++depth;
        e = cudaMemsetAsync(&counters[2], 0, sizeof(int), s);
        if (e != cudaSuccess) break;
        k_collapse<<<(nq + 127) / 128, 128, 0, s>>>(ca, qa, nq, qb, &counters[2], (unsigned int*)&counters[3]);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaMemcpyAsync(&nq, &counters[2], sizeof(int), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        std::swap(qa, qb);
        if (depth > 4096) break;
    }
    int host_counters[4] = {0, 0, 0, 0};
    if (e == cudaSuccess) e = cudaMemcpyAsync(host_counters, counters, sizeof(host_counters), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e == cudaSuccess && host_counters[3] != 0)
    {
        cleanup();
        return "GPU BVH build: node capacity exceeded";
    }
    if (e == cudaSuccess && host_counters[1] != n)
    {
        cleanup();
        return "GPU BVH build: primitive count mismatch";
    }
    if (e == cudaSuccess)
    {
        out.nodes.resize(host_counters[0]);
        out.slots.resize(n);
        e = cudaMemcpyAsync(out.nodes.data(), nodes, sizeof(ar_wide_node) * out.nodes.size(), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(out.slots.data(), slots, sizeof(ar_prim_slot) * (size_t)n, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    }
    Box6 rb{};
    if (e == cudaSuccess) e = cudaMemcpy(&rb, n > 1 ? &box[0] : &box[n - 1], sizeof(Box6), cudaMemcpyDeviceToHost);
    cleanup();
    if (e != cudaSuccess) return std::string("GPU BVH build: ") + cudaGetErrorString(e);
    for (int k = 0; k < 3; ++k)
    {
        out.root_lo[k] = rb.lo[k];
        out.root_hi[k] = rb.hi[k];
    }
    out.depth = depth;
    return "";
}
} // namespace ar
