// sah.cuh — host interface of the CPU SAH BVH builder (sah.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "rt_internal.cuh"

namespace rt {

struct SahTree {
    std::vector<uint32_t> order;   // slot -> triangle (order before the build)
    std::vector<float4> nodes;     // device node layout: 4 float4 per interior node
    BvhHeader hdr;
    uint32_t interior_nodes = 0;
    uint32_t max_interior_depth = 0;
};

// The reference's CPU SAH BVH over N triangles (idx, 3 per triangle, into V
// float4 positions) in their current order, subtrees built on `threads`
// host threads.  0 on success, -1 for invalid input, -2 when an interior
// node would lie deeper than the traversal's 32-entry stack reaches.
int sah_build(const float4* pos, uint32_t V, const uint32_t* idx, uint32_t N, int threads,
              SahTree* out);

}  // namespace rt
