// ctx_internal.h — the rt_ctx structure shared by the C-ABI translation units.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include <map>

#include "../../include/rt_cuda.h"

struct rt_ctx {
    int device = 0;
    int num_sms = 0;
    int render_blocks_per_sm = 1;
    cudaStream_t stream = nullptr;
    uint32_t* d_status = nullptr;        // RT_DEV_* bits
    uint32_t* d_work = nullptr;          // persistent-kernel work counters
    uint32_t* d_sec_scratch = nullptr;   // rt_gen_secondary block offsets
    size_t sec_scratch_bytes = 0;
    uint8_t* d_out = nullptr;            // rt_render_host image staging
    size_t d_out_cap = 0;
    rt_render_stats* d_stats = nullptr;  // rt_render_host counters
    float inv1e6 = 1.0f / 1e6f;
    rt_render_config render_cfg = {4, 0, 32, 32};   // variant (128 threads, 8 blocks/SM)
    int variant_occupancy[16] = {0};                // resident blocks per SM per variant
    std::map<uint64_t, rt_render_config> tuned;     // autotuner cache by workload class
};

namespace rt {
// Records the message returned by rt_last_error() and returns code.
int32_t set_error(int32_t code, const char* fmt, ...);
}  // namespace rt
