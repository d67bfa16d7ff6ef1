// Device traversal of the 8-wide compressed BVH (layout: ar_bvh.h).
//
// One ray per thread; the traversal stack holds node groups (child base +
// bitmask of the still-unvisited hit children, in the ray's octant order), so
// its depth is bounded by the tree depth (AR_TRAV_STACK entries, checked at
// build time) and it stays in registers / L1-resident local memory.
//
// Closest hit keeps the reference's acceptance window [tmin, tmax)
// (core/render/intersection.cuh:73) and resolves exact ties in t to the
// smallest primitive id, so the answer is independent of traversal order.
// Any hit returns the first primitive with t in [tmin, tmax)
// (core/render/intersection.cuh:254-261).
#pragma once
#include "ar_bvh.h"
#include "ar_geom.h"
#include "ar_sdf.h"
#include "ar_sdf_obj.h"
#include "ar_shade.h"

#define AR_TRAV_STACK 40

namespace ar
{
struct TravScene
{
    const uint4* __restrict__ nodes;       // 5 uint4 per node
    const float4* __restrict__ slots;      // 3 float4 per primitive slot
    const Object* __restrict__ objects;    // analytic object table, indexed by primitive id
    const float4* __restrict__ sdf_params; // SDF objects: field parameters, indexed by primitive id
    const SdfVolume* __restrict__ sdf_vols;  // the SDF volume cache
    int sdf_vol_count;
    int node_count;
    SdfUnion sdf;                          // the smooth-union SDF object (count 0: none); not in the BVH
    int sdf_id;                            // its primitive id
};

// hit slot of the SDF object (marched after the BVH traversal)
#define AR_SLOT_SDF (-2)

// SDF march tolerance for a ray starting at intersect_eps-sized offsets (SDF_EPS, core/config.cuh:74)
AR_HD float sdf_eps(float tmin) { return 0.5f * fmaxf(tmin, 1.0e-3f); }

struct TravResult
{
    float t;
    int slot;  // primitive slot index, -1 on miss
    int id;    // primitive id, -1 on miss
};

// The traversal is compiled for the device and, for the CPU test suite, for
// the host; these shims are the only difference.
#if defined(__CUDA_ARCH__)
#define AR_LDG(p) __ldg(p)
#define AR_FFS(x) __ffs(x)
#define AR_POPC(x) __popc(x)
#define AR_F2U(x) __float_as_uint(x)
#define AR_U2F(x) __uint_as_float(x)
#define AR_ATOMIC_OR(p, v) atomicOr((p), (v))
#define AR_ATOMIC_ADD64(p, v) atomicAdd((p), (v))
#else
#define AR_ATOMIC_OR(p, v) (*(p) |= (v))
#define AR_ATOMIC_ADD64(p, v) (*(p) += (v))
#define AR_LDG(p) (*(p))
#define AR_FFS(x) __builtin_ffs((int)(x))
#define AR_POPC(x) __builtin_popcount(x)
#define AR_F2U(x) arm_detail::float_to_bits(x)
#define AR_U2F(x) arm_detail::bits_to_float(x)
#endif

AR_HD uint32_t byte_of(uint32_t lo_word, uint32_t hi_word, int s)
{
    const uint32_t w = (s < 4) ? lo_word : hi_word;
    return (w >> (8 * (s & 3))) & 0xffu;
}

// the field of SDF object `id` (Object.pad: kind, volume index)
AR_HD SdfObjField sdf_obj_field(const TravScene& sc, const Object& ob, int id)
{
    SdfObjField f;
    f.kind = ob.pad[0];
    f.prm = sc.sdf_params[id];
    const int vi = ob.pad[1];
    f.vol = (f.kind == AR_SDF_OBJ_VOLUME && vi >= 0 && vi < sc.sdf_vol_count) ? &sc.sdf_vols[vi] : nullptr;
    return f;
}

// Intersects one primitive slot; returns t (or -1 on miss) and the id.
// Sdf: the slot may hold an SDF object (the SDF objects' own BVH), marched
// with tolerance sdf_eps (SDF_EPS of the ray's depth); the main BVH holds no
// SDF objects, so its traversal is compiled without the march.
template <bool Sdf = false>
AR_HD float prim_hit(const TravScene& sc, int slot, const RayShear& sh, V3 o, V3 d, int* id_out, float tmin,
                     float sdf_eps = 0.0f)
{
    const float4 a = AR_LDG(&sc.slots[3 * (size_t)slot + 0]);
    const uint32_t tag = AR_F2U(a.w);
    const uint32_t kind = tag >> AR_PRIM_KIND_SHIFT;
    const int id = (int)(tag & AR_PRIM_ID_MASK);
    *id_out = id;
    if (kind == AR_PRIM_KIND_TRI)
    {
        const float4 b = AR_LDG(&sc.slots[3 * (size_t)slot + 1]);
        const float4 c = AR_LDG(&sc.slots[3 * (size_t)slot + 2]);
        float t, b0, b1, b2;
        if (tri_intersect(sh, o, v3(a.x, a.y, a.z), v3(b.x, b.y, b.z), v3(c.x, c.y, c.z), &t, &b0, &b1, &b2)) return t;
        return -1.0f;
    }
    (void)tmin;
    const Object ob = sc.objects[id];
    if (kind == AR_PRIM_KIND_SDF)
    {
        if (!Sdf) return -1.0f;
        return sdf_obj_hit(sdf_obj_field(sc, ob, id), ob.center, ob.extent, ob.w2o, o, d, sdf_eps, nullptr);
    }
    Hit h;
    h.hit = false;
    const bool ok = (kind == AR_PRIM_KIND_BOX) ? intersect_box(o, d, ob, &h, false) : intersect_sphere(o, d, ob, &h, false);
    return ok ? h.dist : -1.0f;
}

// Interval slab test of child slot sl of a wide node (words w0..w4) for a
// packet of rays that share the origin o and the direction octant oct, whose
// inverse direction components lie in [inv_lo, inv_hi] (inv_abs: the larger
// magnitude per axis).  Each plane's offset from the origin, c = p + q 2^e - o,
// times the packet's extreme inverses bounds every ray's t at that plane; the
// lowest near-plane t and the highest far-plane t, widened by 2^-19 of the
// largest magnitude involved (the rounding of c, of the products and of each
// ray's reciprocal stays below 2^-22 of it), give a test that rejects the
// child only if no ray of the packet meets its box in [tmin, tlim].  Empty
// slots (neither internal nor a leaf with primitives) are never met.
AR_HD bool packet_child_meets(const uint4& w0, const uint4& w1, const uint4& w2, const uint4& w3, const uint4& w4,
                              int sl, V3 o, uint32_t oct, V3 inv_lo, V3 inv_hi, V3 inv_abs, float tmin, float tlim)
{
    const uint32_t imask = w0.w >> 24;
    const bool internal = (imask >> sl) & 1u;
    if (!internal && (byte_of(w1.z, w1.w, sl) >> 5) == 0u) return false;
    const float px = AR_U2F(w0.x), py = AR_U2F(w0.y), pz = AR_U2F(w0.z);
    const float sx = AR_U2F((w0.w & 0xffu) << 23);
    const float sy = AR_U2F(((w0.w >> 8) & 0xffu) << 23);
    const float sz = AR_U2F(((w0.w >> 16) & 0xffu) << 23);
    const float bx = px - o.x, by = py - o.y, bz = pz - o.z;
    const float clx = fmaf((float)byte_of(w2.x, w2.y, sl), sx, bx);
    const float chx = fmaf((float)byte_of(w3.z, w3.w, sl), sx, bx);
    const float cly = fmaf((float)byte_of(w2.z, w2.w, sl), sy, by);
    const float chy = fmaf((float)byte_of(w4.x, w4.y, sl), sy, by);
    const float clz = fmaf((float)byte_of(w3.x, w3.y, sl), sz, bz);
    const float chz = fmaf((float)byte_of(w4.z, w4.w, sl), sz, bz);
    const float cnx = (oct & 1u) ? chx : clx, cfx = (oct & 1u) ? clx : chx;
    const float cny = (oct & 2u) ? chy : cly, cfy = (oct & 2u) ? cly : chy;
    const float cnz = (oct & 4u) ? chz : clz, cfz = (oct & 4u) ? clz : chz;
    const float ex = (fabsf(bx) + 256.0f * sx) * inv_abs.x * 0x1p-19f;
    const float ey = (fabsf(by) + 256.0f * sy) * inv_abs.y * 0x1p-19f;
    const float ez = (fabsf(bz) + 256.0f * sz) * inv_abs.z * 0x1p-19f;
    const float tnx = fminf(cnx * inv_lo.x, cnx * inv_hi.x) - ex;
    const float tny = fminf(cny * inv_lo.y, cny * inv_hi.y) - ey;
    const float tnz = fminf(cnz * inv_lo.z, cnz * inv_hi.z) - ez;
    const float tfx = fmaxf(cfx * inv_lo.x, cfx * inv_hi.x) + ex;
    const float tfy = fmaxf(cfy * inv_lo.y, cfy * inv_hi.y) + ey;
    const float tfz = fmaxf(cfz * inv_lo.z, cfz * inv_hi.z) + ez;
    const float tn = fmaxf(fmaxf(tnx, tny), fmaxf(tnz, tmin));
    const float tf = fminf(fminf(tfx, tfy), fminf(tfz, tlim));
    return !(tn > tf);  // a NaN (0 x inf) on either side keeps the child
}

// error bits written to the context's device status word
#define AR_DEVERR_STACK 1u
#define AR_DEVERR_QUEUE 2u

// Traversal of one ray as a resumable state: init() sets it up, each step()
// visits one node (box tests of its children, the primitives of the hit
// leaves, the next node from the children or the stack) and returns false once
// the traversal is over.  The persistent wavefront kernels interleave steps of
// many rays per lane (refilling lanes whose ray finished); traverse() runs one
// ray to completion.  Either way a ray performs the same operations in the
// same order.
template <bool AnyHit, bool Sdf = false>
struct TravState
{
    V3 o, d, inv;
    RayShear sh;
    uint32_t oct;
    float tmin, tmax;
    TravResult res;
    int node;
    int sp;
    uint32_t n_visits, n_tests;
    float sdf_eps;                 // Sdf: march tolerance of SDF objects
    uint2* stack;                  // AR_TRAV_STACK node groups, owned by the caller: kept out of
                                   // the struct so its scalars stay in registers

    AR_HD void init(const TravScene& sc, V3 o_, V3 d_, float tmin_, float tmax_, uint2* stack_)
    {
        stack = stack_;
        o = o_;
        d = d_;
        tmin = tmin_;
        tmax = tmax_;
        res.t = tmax_;
        res.slot = -1;
        res.id = -1;
        sh = make_shear(d_);
        inv = v3(inv_safe(d_.x), inv_safe(d_.y), inv_safe(d_.z));
        oct = (d_.x < 0.0f ? 1u : 0u) | (d_.y < 0.0f ? 2u : 0u) | (d_.z < 0.0f ? 4u : 0u);
        sp = 0;
        node = sc.node_count > 0 ? 0 : -2;  // -2: nothing to traverse
        n_visits = 0;
        n_tests = 0;
        sdf_eps = 0.0f;
    }

    // continues from a result found elsewhere (the main BVH's hit for the SDF
    // objects' BVH): closer hits or equal t with a smaller id replace it
    AR_HD void start_from(TravResult r, float sdf_eps_)
    {
        res = r;
        sdf_eps = sdf_eps_;
    }

    AR_HD TravResult result() const
    {
        TravResult r = res;
        if (r.slot < 0) r.t = tmax;
        return r;
    }

    AR_HD bool step(const TravScene& sc, unsigned int* err)
    {
        if (node == -2) return false;
        if (node >= 0)
        {
            ++n_visits;
            const uint4* np = sc.nodes + 5 * (size_t)node;
            const uint4 w0 = AR_LDG(np + 0);
            const uint4 w1 = AR_LDG(np + 1);
            const uint4 w2 = AR_LDG(np + 2);
            const uint4 w3 = AR_LDG(np + 3);
            const uint4 w4 = AR_LDG(np + 4);
            const float px = AR_U2F(w0.x), py = AR_U2F(w0.y), pz = AR_U2F(w0.z);
            const float sx = AR_U2F((w0.w & 0xffu) << 23);
            const float sy = AR_U2F(((w0.w >> 8) & 0xffu) << 23);
            const float sz = AR_U2F(((w0.w >> 16) & 0xffu) << 23);
            const uint32_t imask = w0.w >> 24;
            const uint32_t child_base = w1.x;
            const uint32_t prim_base = w1.y;
            // Per axis the plane p + q 2^e is met at t(q) = q A + B with
            // A = 2^e / d (exact: a power of two times the reciprocal) and
            // B = (p - o) / d.  Each child plane costs one fused multiply-add;
            // E = 2^-21 (|B| + 255 |A|) bounds every rounding of B, of the
            // reciprocal and of the fused evaluation (at most about 5.2 ulp of
            // |B| + 255 |A|), so near planes move down and far planes up by E
            // and the test never rejects a box the ray meets.  Overflow gives
            // NaN or an infinity on the permissive side, which fminf / fmaxf
            // then ignore.  The near plane of each axis is the low one when
            // the direction is positive (octant bit clear): no min / max pairs.
            const float ax = sx * inv.x, ay = sy * inv.y, az = sz * inv.z;
            const float bx = (px - o.x) * inv.x, by = (py - o.y) * inv.y, bz = (pz - o.z) * inv.z;
            const float ex = (fabsf(bx) + 255.0f * fabsf(ax)) * 0x1p-21f;
            const float ey = (fabsf(by) + 255.0f * fabsf(ay)) * 0x1p-21f;
            const float ez = (fabsf(bz) + 255.0f * fabsf(az)) * 0x1p-21f;
            const float bnx = bx - ex, bfx = bx + ex, bny = by - ey, bfy = by + ey, bnz = bz - ez, bfz = bz + ez;
            const bool fx = oct & 1u, fy = oct & 2u, fz = oct & 4u;
            const uint32_t nx0 = fx ? w3.z : w2.x, nx1 = fx ? w3.w : w2.y, fx0 = fx ? w2.x : w3.z, fx1 = fx ? w2.y : w3.w;
            const uint32_t ny0 = fy ? w4.x : w2.z, ny1 = fy ? w4.y : w2.w, fy0 = fy ? w2.z : w4.x, fy1 = fy ? w2.w : w4.y;
            const uint32_t nz0 = fz ? w4.z : w3.x, nz1 = fz ? w4.w : w3.y, fz0 = fz ? w3.x : w4.z, fz1 = fz ? w3.y : w4.w;
            const float tlim = res.t;
            uint32_t hit_int = 0, hit_leaf = 0;
#pragma unroll
            for (int s = 0; s < 8; ++s)
            {
                const float tnx = fmaf((float)byte_of(nx0, nx1, s), ax, bnx);
                const float tny = fmaf((float)byte_of(ny0, ny1, s), ay, bny);
                const float tnz = fmaf((float)byte_of(nz0, nz1, s), az, bnz);
                const float tfx = fmaf((float)byte_of(fx0, fx1, s), ax, bfx);
                const float tfy = fmaf((float)byte_of(fy0, fy1, s), ay, bfy);
                const float tfz = fmaf((float)byte_of(fz0, fz1, s), az, bfz);
                const float tn = fmaxf(fmaxf(tnx, tny), fmaxf(tnz, tmin));
                const float tf = fminf(fminf(tfx, tfy), fminf(tfz, tlim));
                if (tn <= tf)
                {
                    const uint32_t bit = 1u << ((uint32_t)s ^ oct);
                    if (imask & (1u << s)) hit_int |= bit;
                    else hit_leaf |= bit;
                }
            }
            while (hit_leaf)
            {
                const uint32_t i = AR_FFS(hit_leaf) - 1;
                hit_leaf &= hit_leaf - 1;
                const int s = (int)(i ^ oct);
                const uint32_t meta = byte_of(w1.z, w1.w, s);
                const int cnt = (int)(meta >> 5);
                const int first = (int)(prim_base + (meta & 31u));
                for (int k = 0; k < cnt; ++k)
                {
                    int id;
                    ++n_tests;
                    const float t = prim_hit<Sdf>(sc, first + k, sh, o, d, &id, tmin, sdf_eps);
                    if (!(t >= tmin)) continue;  // also rejects misses (-1)
                    if (AnyHit)
                    {
                        if (t < res.t)
                        {
                            res.t = t;
                            res.slot = first + k;
                            res.id = id;
                            node = -2;
                            return false;
                        }
                    }
                    else if (t < res.t || (t == res.t && res.id >= 0 && id < res.id))
                    {
                        res.t = t;
                        res.slot = first + k;
                        res.id = id;
                    }
                }
            }
            node = -1;
            if (hit_int)
            {
                const uint32_t i = AR_FFS(hit_int) - 1;
                hit_int &= hit_int - 1;
                const uint32_t s = i ^ oct;
                node = (int)(child_base + AR_POPC(imask & ((1u << s) - 1u)));
                if (hit_int)
                {
                    if (sp < AR_TRAV_STACK) stack[sp++] = make_uint2(child_base, hit_int | (imask << 8));
                    else if (err) AR_ATOMIC_OR(err, AR_DEVERR_STACK);
                }
                return true;
            }
        }
        if (sp == 0)
        {
            node = -2;
            return false;
        }
        // the top group gives its nearest child; the group stays while children remain
        const uint2 e = stack[sp - 1];
        uint32_t m = e.y & 0xffu;
        const uint32_t im = e.y >> 8;
        const uint32_t i = AR_FFS(m) - 1;
        m &= m - 1;
        const uint32_t s = i ^ oct;
        node = (int)(e.x + AR_POPC(im & ((1u << s) - 1u)));
        if (m) stack[sp - 1].y = m | (im << 8);
        else --sp;
        return true;
    }
};

// Slots of hits outside the main BVH (PathState::hit_slot)
#define AR_SLOT_SOLO (-3)          // a ray inside an SDF object, resolved by the SDF pass
#define AR_SLOT_SDFOBJ_BASE (-4)   // SDF object hit: AR_SLOT_SDFOBJ_BASE - (slot in the SDF objects' BVH)

// The SDF objects' BVH from a result found in the main BVH: closest hit
// (equal t: the smaller id wins, as in one traversal over both) or any hit.
// Returns the raw result: a different id than `start` means an SDF object won,
// and res.slot then indexes this BVH's slots.  Out of line: the march lives here.
template <bool AnyHit>
AR_SDFOBJ_CALL TravResult sdf_bvh_trace(const TravScene sc, V3 o, V3 d, float tmin, float tmax, float sdf_eps,
                                        TravResult start)
{
    if (sc.node_count <= 0) return start;
    TravState<AnyHit, true> st;
    uint2 stk[AR_TRAV_STACK];
    st.init(sc, o, d, tmin, tmax, stk);
    st.start_from(start, sdf_eps);
    while (st.step(sc, nullptr))
    {
    }
    return st.res;
}

template <bool AnyHit>
AR_HD TravResult traverse_impl(const TravScene& sc, V3 o, V3 d, float tmin, float tmax,
                                                    unsigned int* err, uint32_t& n_visits, uint32_t& n_tests)
{
    TravState<AnyHit> st;
    uint2 stk[AR_TRAV_STACK];
    st.init(sc, o, d, tmin, tmax, stk);
    while (st.step(sc, err))
    {
    }
    n_visits = st.n_visits;
    n_tests = st.n_tests;
    return st.result();
}

// stats (optional): [0] += node visits, [1] += primitive tests
template <bool AnyHit>
AR_HD TravResult traverse(const TravScene& sc, V3 o, V3 d, float tmin, float tmax,
                                               unsigned int* err, unsigned long long* stats = nullptr)
{
    uint32_t n_visits = 0, n_tests = 0;
    TravResult res = traverse_impl<AnyHit>(sc, o, d, tmin, tmax, err, n_visits, n_tests);
    if (stats)
    {
        AR_ATOMIC_ADD64(&stats[0], (unsigned long long)n_visits);
        AR_ATOMIC_ADD64(&stats[1], (unsigned long long)n_tests);
    }
    return res;
}
} // namespace ar
