// Host BVH builder: binned SAH binary tree, collapsed into 8-wide nodes with
// 8-bit quantized child boxes (layout in ar_bvh.h).
//
// The reference builds a binary binned-SAH BVH on the host (12 bins, longest
// centroid axis, leaves of up to 8 objects; core/bvh/bvh.cuh:142-422).  Hit
// results do not depend on the tree, so this builder is free to pick a layout
// for the GPU: 16 bins on all three axes, leaves of up to 3 primitives, parallel
// subtree builds, then a greedy largest-area-first collapse to width 8 with
// children placed in direction-octant slots for sort-free near-first traversal.
#include "ar_bvh_build.h"

#include <algorithm>
#include <atomic>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <future>
#include <thread>

namespace arbvh
{
namespace
{
struct Box
{
    float lo[3], hi[3];
    void reset()
    {
        for (int k = 0; k < 3; ++k)
        {
            lo[k] = FLT_MAX;
            hi[k] = -FLT_MAX;
        }
    }
    void grow(const Box& b)
    {
        for (int k = 0; k < 3; ++k)
        {
            lo[k] = std::min(lo[k], b.lo[k]);
            hi[k] = std::max(hi[k], b.hi[k]);
        }
    }
    void grow_pt(const float* p)
    {
        for (int k = 0; k < 3; ++k)
        {
            lo[k] = std::min(lo[k], p[k]);
            hi[k] = std::max(hi[k], p[k]);
        }
    }
    double area() const
    {
        const double dx = std::max(0.0, (double)hi[0] - lo[0]);
        const double dy = std::max(0.0, (double)hi[1] - lo[1]);
        const double dz = std::max(0.0, (double)hi[2] - lo[2]);
        return 2.0 * (dx * dy + dy * dz + dz * dx);
    }
};

struct BNode
{
    Box box;
    int left = -1, right = -1;
    int start = 0, count = 0;  // leaf when count > 0
};

constexpr int kBins = 16;
constexpr int kMaxLeaf = 3;
constexpr int kParallelCutoff = 1 << 15;

struct Builder
{
    const std::vector<Box>& pbox;
    std::vector<float> cent;  // 3 per prim
    std::vector<uint32_t> order;
    std::vector<BNode> nodes;     // preallocated to the 2N-1 upper bound
    std::atomic<int> next_node{1};

    explicit Builder(const std::vector<Box>& b) : pbox(b) {}

    int alloc_nodes(int n) { return next_node.fetch_add(n); }

    // builds the subtree for order[start, end) into node `self`
    void build(int self, int start, int end)
    {
        Box bounds, cb;
        bounds.reset();
        cb.reset();
        for (int i = start; i < end; ++i)
        {
            bounds.grow(pbox[order[i]]);
            cb.grow_pt(&cent[3 * (size_t)order[i]]);
        }
        const int n = end - start;
        int mid = -1;
        double best_cost = DBL_MAX;
        int best_axis = -1, best_split = -1;
        for (int axis = 0; axis < 3; ++axis)
        {
            const float cmin = cb.lo[axis], cmax = cb.hi[axis];
            if (!(cmax > cmin)) continue;
            const double scale = kBins / ((double)cmax - cmin);
            Box bb[kBins];
            int bc[kBins];
            for (int b = 0; b < kBins; ++b)
            {
                bb[b].reset();
                bc[b] = 0;
            }
            for (int i = start; i < end; ++i)
            {
                const uint32_t p = order[i];
                int b = (int)(((double)cent[3 * (size_t)p + axis] - cmin) * scale);
                b = std::min(std::max(b, 0), kBins - 1);
                bb[b].grow(pbox[p]);
                ++bc[b];
            }
            double la[kBins], ra[kBins];
            int lc[kBins], rc[kBins];
            Box acc;
            acc.reset();
            int cnt = 0;
            for (int b = 0; b < kBins; ++b)
            {
                if (bc[b]) acc.grow(bb[b]);
                cnt += bc[b];
                la[b] = cnt ? acc.area() : 0.0;
                lc[b] = cnt;
            }
            acc.reset();
            cnt = 0;
            for (int b = kBins - 1; b >= 0; --b)
            {
                if (bc[b]) acc.grow(bb[b]);
                cnt += bc[b];
                ra[b] = cnt ? acc.area() : 0.0;
                rc[b] = cnt;
            }
            for (int b = 0; b < kBins - 1; ++b)
            {
                if (lc[b] == 0 || rc[b + 1] == 0) continue;
                const double c = la[b] * lc[b] + ra[b + 1] * rc[b + 1];
                if (c < best_cost)
                {
                    best_cost = c;
                    best_axis = axis;
                    best_split = b;
                }
            }
        }
        const double parea = std::max(bounds.area(), 1e-30);
        const double split_cost = 1.0 + best_cost / parea;
        if (n <= kMaxLeaf && (best_axis < 0 || (double)n <= split_cost))
        {
            nodes[self].box = bounds;
            nodes[self].start = start;
            nodes[self].count = n;
            return;
        }
        if (best_axis >= 0)
        {
            const float cmin = cb.lo[best_axis], cmax = cb.hi[best_axis];
            const double scale = kBins / ((double)cmax - cmin);
            auto it = std::partition(order.begin() + start, order.begin() + end, [&](uint32_t p) {
                int b = (int)(((double)cent[3 * (size_t)p + best_axis] - cmin) * scale);
                b = std::min(std::max(b, 0), kBins - 1);
                return b <= best_split;
            });
            mid = (int)(it - order.begin());
        }
        if (mid <= start || mid >= end)
        {
            // identical centroids: split the index range in half
            mid = start + n / 2;
        }
        const int kids = alloc_nodes(2);
        nodes[self].box = bounds;
        nodes[self].left = kids;
        nodes[self].right = kids + 1;
        nodes[self].count = 0;
        if (n > kParallelCutoff)
        {
            auto f = std::async(std::launch::async, [&, kids, start, mid] { build(kids, start, mid); });
            build(kids + 1, mid, end);
            f.get();
        }
        else
        {
            build(kids, start, mid);
            build(kids + 1, mid, end);
        }
    }
};

struct Collapser
{
    const std::vector<BNode>& bn;
    const std::vector<uint32_t>& order;
    const std::vector<PrimInput>& prims;
    WideBVH& out;
    int max_depth = 0;

    // fills wide node `wi` from binary node `b`
    void emit(int wi, int b, int depth)
    {
        max_depth = std::max(max_depth, depth);
        std::vector<int> ch;
        if (bn[b].count > 0) ch.push_back(b);
        else
        {
            ch.push_back(bn[b].left);
            ch.push_back(bn[b].right);
        }
        while ((int)ch.size() < AR_BVH_WIDTH)
        {
            int pick = -1;
            double best = -1.0;
            for (int i = 0; i < (int)ch.size(); ++i)
            {
                if (bn[ch[i]].count > 0) continue;
                const double a = bn[ch[i]].box.area();
                if (a > best)
                {
                    best = a;
                    pick = i;
                }
            }
            if (pick < 0) break;
            const int c = ch[pick];
            ch[pick] = bn[c].left;
            ch.push_back(bn[c].right);
        }
        // node bounds and centroid
        Box nb;
        nb.reset();
        for (int c : ch) nb.grow(bn[c].box);
        double nc[3];
        for (int k = 0; k < 3; ++k) nc[k] = 0.5 * ((double)nb.lo[k] + nb.hi[k]);
        // octant slot assignment: greedy on alignment with slot directions
        struct Cand
        {
            double cost;
            int c, s;
        };
        std::vector<Cand> cands;
        for (int i = 0; i < (int)ch.size(); ++i)
        {
            const Box& cb = bn[ch[i]].box;
            double off[3];
            for (int k = 0; k < 3; ++k) off[k] = 0.5 * ((double)cb.lo[k] + cb.hi[k]) - nc[k];
            for (int s = 0; s < 8; ++s)
            {
                double c = 0.0;
                for (int k = 0; k < 3; ++k) c += ((s >> k) & 1) ? off[k] : -off[k];
                cands.push_back({c, i, s});
            }
        }
        std::stable_sort(cands.begin(), cands.end(), [](const Cand& a, const Cand& b) { return a.cost > b.cost; });
        int slot_of[8];
        int child_in_slot[8];
        for (int i = 0; i < 8; ++i)
        {
            slot_of[i] = -1;
            child_in_slot[i] = -1;
        }
        for (const Cand& c : cands)
        {
            if (slot_of[c.c] >= 0 || child_in_slot[c.s] >= 0) continue;
            slot_of[c.c] = c.s;
            child_in_slot[c.s] = c.c;
        }
        ar_wide_node node;
        std::memset(&node, 0, sizeof(node));
        // empty slots: an inverted box (low 255, high 0) that no ray meets
        std::memset(node.qlo, 0xff, sizeof(node.qlo));
        node.px = nb.lo[0];
        node.py = nb.lo[1];
        node.pz = nb.lo[2];
        float scale[3];
        const float p[3] = {nb.lo[0], nb.lo[1], nb.lo[2]};
        for (int k = 0; k < 3; ++k)
        {
            const double ext = (double)nb.hi[k] - nb.lo[k];
            int e = -126;
            if (ext > 0.0)
            {
                e = (int)std::ceil(std::log2(ext / 255.0));
                while (std::ldexp(255.0, e) < ext) ++e;
                e = std::max(-126, std::min(127, e));
            }
            node.e[k] = (uint8_t)(e + 127);
            scale[k] = (float)std::ldexp(1.0, e);
        }
        // internal children are stored in slot order at child_base
        int n_int = 0;
        for (int s = 0; s < 8; ++s)
        {
            const int ci = child_in_slot[s];
            if (ci >= 0 && bn[ch[ci]].count == 0) ++n_int;
        }
        const uint32_t child_base = (uint32_t)out.nodes.size();
        out.nodes.resize(out.nodes.size() + n_int);
        const uint32_t prim_base = (uint32_t)out.slots.size();
        node.child_base = child_base;
        node.prim_base = prim_base;
        int rank = 0;
        int off = 0;
        std::vector<std::pair<int, int>> recurse;
        for (int s = 0; s < 8; ++s)
        {
            const int ci = child_in_slot[s];
            if (ci < 0) continue;
            const BNode& c = bn[ch[ci]];
            for (int k = 0; k < 3; ++k)
            {
                double ql = std::floor(((double)c.box.lo[k] - p[k]) / scale[k]);
                double qh = std::ceil(((double)c.box.hi[k] - p[k]) / scale[k]);
                ql = std::min(std::max(ql, 0.0), 255.0);
                qh = std::min(std::max(qh, 0.0), 255.0);
                node.qlo[k][s] = (uint8_t)ql;
                node.qhi[k][s] = (uint8_t)qh;
            }
            if (c.count == 0)
            {
                node.imask |= (uint8_t)(1u << s);
                node.meta[s] = (uint8_t)(0x80u | (uint32_t)rank);
                recurse.push_back({(int)(child_base + rank), ch[ci]});
                ++rank;
            }
            else
            {
                node.meta[s] = (uint8_t)(((uint32_t)c.count << 5) | (uint32_t)off);
                for (int j = 0; j < c.count; ++j)
                {
                    const PrimInput& pi = prims[order[c.start + j]];
                    ar_prim_slot sl;
                    std::memset(&sl, 0, sizeof(sl));
                    uint32_t tag = pi.id | (pi.kind << AR_PRIM_KIND_SHIFT);
                    if (pi.kind == AR_PRIM_KIND_TRI)
                    {
                        for (int k = 0; k < 3; ++k)
                        {
                            sl.a[k] = pi.v[k];
                            sl.b[k] = pi.v[3 + k];
                            sl.c[k] = pi.v[6 + k];
                        }
                    }
                    std::memcpy(&sl.a[3], &tag, 4);
                    out.slots.push_back(sl);
                }
                off += c.count;
            }
        }
        out.nodes[wi] = node;
        for (auto& r : recurse) emit(r.first, r.second, depth + 1);
    }
};
} // namespace

bool build_wide_bvh(const std::vector<PrimInput>& prims, WideBVH& out, std::string* err)
{
    out.nodes.clear();
    out.slots.clear();
    out.depth = 0;
    if (prims.empty()) return true;
    if (prims.size() >= (size_t)AR_PRIM_ID_MASK)
    {
        if (err) *err = "too many primitives for 30-bit ids";
        return false;
    }
    std::vector<Box> pbox(prims.size());
    for (size_t i = 0; i < prims.size(); ++i)
    {
        for (int k = 0; k < 3; ++k)
        {
            pbox[i].lo[k] = prims[i].lo[k];
            pbox[i].hi[k] = prims[i].hi[k];
            if (!(pbox[i].lo[k] <= pbox[i].hi[k]))
            {
                if (err) *err = "primitive with invalid (NaN or inverted) bounds";
                return false;
            }
        }
    }
    Builder b(pbox);
    b.cent.resize(3 * prims.size());
    b.order.resize(prims.size());
    for (size_t i = 0; i < prims.size(); ++i)
    {
        b.order[i] = (uint32_t)i;
        for (int k = 0; k < 3; ++k) b.cent[3 * i + k] = 0.5f * (pbox[i].lo[k] + pbox[i].hi[k]);
    }
    b.nodes.resize(2 * prims.size() + 1);
    b.build(0, 0, (int)prims.size());
    b.nodes.resize(b.next_node.load());
    out.nodes.reserve(b.nodes.size() / 3 + 16);
    out.slots.reserve(prims.size());
    out.nodes.resize(1);
    Collapser c{b.nodes, b.order, prims, out};
    c.emit(0, 0, 1);
    out.depth = c.max_depth;
    for (int k = 0; k < 3; ++k)
    {
        out.root_lo[k] = b.nodes[0].box.lo[k];
        out.root_hi[k] = b.nodes[0].box.hi[k];
    }
    return true;
}
} // namespace arbvh
