// Wide (8-ary) compressed BVH: layout shared by the host builder and the
// device traversal.
//
// Node: 80 bytes = five 16-byte words, fetched with ld.global.v4 so a warp
// reads whole nodes in 128-byte segments.
//   w0: origin p.xyz (f32) | exponents ex, ey, ez (u8, biased 127) | internal-child mask (u8)
//   w1: child_base (u32) | prim_base (u32) | meta[0..7] (u8)
//   w2: qlo_x[8], qlo_y[8]      w3: qlo_z[8], qhi_x[8]      w4: qhi_y[8], qhi_z[8]
// A child box decodes as p + q * 2^(e-127) per axis (exact conservative bounds).
// meta[i]: 0 = empty slot (its box is inverted, qlo 255 and qhi 0: no ray meets it);
//          0x80 | r = internal child stored at child_base + r;
//          (n << 5) | off = leaf with n (1..3) primitive slots at prim_base + off.
// Children sit in slots chosen by the direction of their centroid from the
// node's centroid (slot bit k set = +axis k), so a ray whose direction-sign
// octant is o visits slots in the order i ^ o, i = 0..7: near first, no sort.
//
// Primitive slot: three float4.  Triangles: (v0, id) (v1, 0) (v2, 0).
// Analytic objects (boxes, spheres): (0, id | kind << 30) with the geometry in
// the object table.  id is the scene primitive index reported to callers.
#pragma once
#include <stdint.h>

#define AR_BVH_WIDTH 8
#define AR_PRIM_KIND_SHIFT 30
#define AR_PRIM_KIND_TRI 0u
#define AR_PRIM_KIND_BOX 1u
#define AR_PRIM_KIND_SPHERE 2u
#define AR_PRIM_KIND_SDF 3u
#define AR_PRIM_ID_MASK 0x3fffffffu

struct ar_wide_node
{
    float px, py, pz;
    uint8_t e[3];
    uint8_t imask;
    uint32_t child_base;
    uint32_t prim_base;
    uint8_t meta[8];
    uint8_t qlo[3][8];
    uint8_t qhi[3][8];
};
static_assert(sizeof(ar_wide_node) == 80, "wide node must be 80 bytes");

struct ar_prim_slot
{
    float a[4], b[4], c[4];
};
static_assert(sizeof(ar_prim_slot) == 48, "primitive slot must be 48 bytes");
