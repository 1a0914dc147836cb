// lbvh.cuh — host interface of the LBVH builder kernels (lbvh.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "rt_internal.cuh"

namespace rt {

struct LbvhArgs {
    uint32_t n;               // triangles
    int depth;                // Morton bits (1..32)
    int min_leaf;             // reference bvh_min_leaf_size
    int num_sms;
    const float4* pos;        // vertex positions
    // triangle data in the order before this build, and its sorted copy
    const uint32_t* idx_in;
    const uint32_t* map_in;
    const uint32_t* orig_in;
    uint32_t* idx_out;
    uint32_t* map_out;
    uint32_t* orig_out;
    // sort buffers
    uint32_t* keys_unsorted;  // Morton key per triangle (order before the build)
    uint32_t* vals0;          // 0..n-1
    uint32_t* keys1;
    uint32_t* vals1;
    uint32_t* keys_sorted;
    uint32_t* vals_sorted;    // sorted slot -> triangle (order before the build)
    // outputs
    float4* tris;             // 3 float4 per sorted triangle
    float4* leafbox;          // 2 float4 per sorted triangle
    float4* nodes;            // 4 float4 per radix-tree node (n - 1)
    BvhHeader* hdr;
    uint32_t* scratch;        // lbvh_scratch_bytes(n, passes)
    uint32_t* status;         // device status word (RT_DEV_* bits)
};

size_t lbvh_scratch_bytes(uint32_t n, int passes);
// Byte offset of the emit's item buffers in a scene's build scratch (of
// lbvh_scratch_bytes(n, 4) bytes); the many-scene build uses them too.
size_t lbvh_emit_offset(uint32_t n);
// mangle (src/kernel/mangler.cl:12-32) over V vertices, in place (animate.cu).
cudaError_t launch_mangle(float4* pos, float4* nrm, uint32_t V, float arg, float height,
                          cudaStream_t s);
cudaError_t lbvh_build(const LbvhArgs& a, cudaStream_t s);
cudaError_t lbvh_refit(const LbvhArgs& a, cudaStream_t s);
// The triangle data (indices, materials, ids, triangle records, leaf boxes)
// of a.*_in rearranged into a.*_out by `order` (slot -> triangle), as the
// LBVH build does with its sorted permutation.
cudaError_t lbvh_permute(const LbvhArgs& a, const uint32_t* order, cudaStream_t s);

// Stable LSD radix sort of (key, value) pairs on the low key_bits bits with
// caller-provided scratch (radix_scratch_words words) and temporaries of n
// pairs; passes alternate between out and tmp so that the last lands in out.
size_t radix_scratch_words(uint32_t n, int passes);
// Self-test of the device timeout path: a radix-pass tile whose predecessor
// never publishes, in a zeroed buffer of wait_probe_words() words; sets
// RT_DEV_TIMEOUT in *status.
size_t wait_probe_words();
cudaError_t wait_probe(uint32_t* buf, uint32_t* status, cudaStream_t s);
int radix_tile_size();
cudaError_t radix_sort_pairs(const uint32_t* kin, const uint32_t* vin, uint32_t* kout,
                             uint32_t* vout, uint32_t* ktmp, uint32_t* vtmp, uint32_t n,
                             int key_bits, uint32_t* scratch, uint32_t* status, int num_sms,
                             cudaStream_t s);

}  // namespace rt
