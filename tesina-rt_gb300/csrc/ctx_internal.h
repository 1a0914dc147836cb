// ctx_internal.h — the rt_ctx structure shared by the C-ABI translation units.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include <map>
#include <mutex>

#include "../../include/rt_cuda.h"
#include "rt_internal.cuh"

struct rt_ctx {
    int device = 0;
    int num_sms = 0;
    int render_blocks_per_sm = 1;
    cudaStream_t stream = nullptr;
    uint32_t* d_status = nullptr;        // RT_DEV_* bits
    uint32_t* d_work = nullptr;          // work counter of launches on `stream`
    // work counters of launches on other streams, one per stream: launches
    // on one stream are ordered, so a counter is never shared by two
    // running kernels
    std::map<cudaStream_t, uint32_t*> work_by_stream;
    // fixed-point sums of the pooled render variants, per stream, with the
    // pixel count each holds (stream-ordered allocations)
    std::map<cudaStream_t, std::pair<uint32_t*, size_t>> accum_by_stream;
    std::mutex work_mu;
    // rt_gen_secondary block offsets, per stream, with their size in bytes
    // (stream-ordered allocations)
    std::map<cudaStream_t, std::pair<uint32_t*, size_t>> sec_by_stream;
    // rt_render_host / rt_render_host_async, per stream: a stream for the
    // normal upload beside the build and the events that fork and join it,
    // the device image and counters, pinned staging for the counters and the
    // status word (read back without blocking the host), and the frame that
    // waits for rt_render_host_wait
    struct HostRender {
        cudaStream_t side = nullptr;
        cudaEvent_t fork = nullptr, join = nullptr;
        uint8_t* d_out = nullptr;
        size_t out_cap = 0;
        rt_render_stats* d_stats = nullptr;
        struct Stage {
            rt_render_stats stats;
            uint32_t status;
        }* h_stage = nullptr;
        rt_render_stats* user_stats = nullptr;
        bool pending = false;
    };
    std::map<cudaStream_t, HostRender> host_by_stream;
    float inv1e6 = 1.0f / 1e6f;
    // until the autotuner or the caller picks one: the pooled kernel
    // (variant 8, k_render_pool<128, 6>) at full residency
    rt_render_config render_cfg = {8, 0, 32, 32};
    int variant_occupancy[rt::kMaxRenderVariants] = {0};   // resident blocks per SM per variant
    int variant_carveout[rt::kMaxRenderVariants];          // shared-memory carveout set (%), -1 unset
    int smem_per_sm = 0;                            // bytes of shared memory an SM offers
    int instance_occupancy[3] = {0, 0, 0};          // k_render_instances<0 / 4 / 6> blocks per SM
    std::map<uint64_t, rt_render_config> tuned;     // autotuner cache by workload class
};

// Scene state: geometry, the double-buffered triangle order (the build's
// permute writes the other half, `cur` flips) and the build products.
struct rt_scene {
    uint32_t V = 0, N = 0, M = 0;
    uint32_t capV = 0, capN = 0, capM = 0;
    float4* d_pos = nullptr;
    float4* d_nrm = nullptr;
    uint32_t* d_idx[2] = {nullptr, nullptr};
    uint32_t* d_map[2] = {nullptr, nullptr};
    uint32_t* d_orig[2] = {nullptr, nullptr};
    int cur = 0;                     // which of the [2] buffers holds the current order
    rt_material* d_mats = nullptr;
    rt_lights lights;
    // build products
    uint32_t* d_keys_unsorted = nullptr;
    uint32_t* d_vals0 = nullptr;
    uint32_t* d_keys1 = nullptr;
    uint32_t* d_vals1 = nullptr;
    uint32_t* d_keys_sorted = nullptr;
    uint32_t* d_vals_sorted = nullptr;
    float4* d_tris = nullptr;
    float4* d_leafbox = nullptr;
    float4* d_nodes = nullptr;
    rt::BvhHeader* d_hdr = nullptr;
    uint32_t* d_scratch = nullptr;
    size_t scratch_bytes = 0;
    uint32_t buildN = 0;             // capacity of the build buffers
    bool built = false;
    bool refracts = false;           // some material has refractive_index > 0
    bool sah = false;                // the tree came from rt_bvh_build_sah (no refit)
    int depth = 30, min_leaf = 1;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // Order of the rt_* calls on this scene across streams: the completion
    // of the last call that wrote it, and of the reading calls since, one
    // event per stream (the last slot absorbs further streams).
    struct Reader {
        cudaStream_t stream;
        cudaEvent_t ev;
    };
    cudaEvent_t ev_write = nullptr;
    cudaStream_t write_stream = nullptr;
    bool write_recorded = false;
    Reader readers[4] = {};
    int n_readers = 0;
    // stream-ordered allocation (served scenes): buffers come from `pool` in
    // the order of `pool_stream`; nullptr = cudaMalloc
    cudaMemPool_t pool = nullptr;
    cudaStream_t pool_stream = nullptr;
};

namespace rt {
// Records the message returned by rt_last_error() and returns code.
int32_t set_error(int32_t code, const char* fmt, ...);
// Allocates (or keeps) the build buffers for the scene's triangle count.
int32_t scene_ensure_build(rt_scene* s);
// Device view of the scene's current (sorted) order.
SceneView scene_view(const rt_scene* s);
// The persistent-kernel work counter for launches on stream s (nullptr if it
// cannot be allocated).
uint32_t* work_counter(rt_ctx* c, cudaStream_t s);
// Gives a new, empty scene a memory pool: its buffers are allocated and freed
// in the order of `stream`, which must carry its uploads and builds.
void scene_use_pool(rt_scene* s, cudaMemPool_t pool, cudaStream_t stream);
// Frees the work counter and the render sums of stream s (before the stream
// is destroyed).
void release_work_counter(rt_ctx* c, cudaStream_t s);
// Render sums (3 x uint32 per pixel) for launches on stream s, at least
// `pixels` long; grown in stream order.  nullptr if it cannot be allocated.
uint32_t* accum_buffer(rt_ctx* c, cudaStream_t s, size_t pixels);
// rt_gen_secondary scratch for launches on stream s, at least `bytes` long;
// grown in stream order.  nullptr if it cannot be allocated.
uint32_t* sec_scratch(rt_ctx* c, cudaStream_t s, size_t bytes);
// Per-scene ordering across streams: calls on one scene behave as on one
// in-order queue.  Writers (upload, build, refit) wait for every earlier call
// on other streams; readers (trace, render) for the last writer.
cudaError_t scene_write_begin(rt_scene* s, cudaStream_t cs);
cudaError_t scene_write_end(rt_scene* s, cudaStream_t cs);
cudaError_t scene_read_begin(rt_scene* s, cudaStream_t cs);
cudaError_t scene_read_end(rt_scene* s, cudaStream_t cs);
// Host wait for the scene's last writer (and its readers too when `all`).
cudaError_t scene_host_wait(rt_scene* s, bool all);
}  // namespace rt
