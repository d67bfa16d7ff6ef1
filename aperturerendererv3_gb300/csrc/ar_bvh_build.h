// Host-side BVH build interface (implementation in bvh_build.cpp).
#pragma once
#include <mutex>
#include <string>
#include <vector>

#include "ar_bvh.h"

namespace arbvh
{
struct PrimInput
{
    float lo[3], hi[3];
    float v[9];      // triangle vertices (triangles only)
    uint32_t id;     // scene primitive index
    uint32_t kind;   // AR_PRIM_KIND_*
};

struct WideBVH
{
    std::vector<ar_wide_node> nodes;
    std::vector<ar_prim_slot> slots;
    float root_lo[3] = {0, 0, 0}, root_hi[3] = {0, 0, 0};
    int depth = 0;
};

bool build_wide_bvh(const std::vector<PrimInput>& prims, WideBVH& out, std::string* err);
} // namespace arbvh
