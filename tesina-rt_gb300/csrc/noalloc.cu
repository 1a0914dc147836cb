// noalloc.cu — rt_sort_pairs_noalloc: the stable radix sort of the LBVH
// builder (the same k_onesweep passes) for callers that must not allocate.
//
// Some callers cannot allocate device memory at the moment they need a sort:
// a host application that has already handed its whole HBM budget to its
// own pool (a renderer's resident-scene arena, a serving process whose
// admission control accounts for every byte), or a frame loop that cannot
// afford the implicit synchronisation a cudaMalloc / cudaFree may cause.
// For them this entry point keeps its scratch in a fixed array in device
// memory that is part of the library itself: nothing is allocated per call.
//
// Limits and sharing rules:
//   - at most RT_NOALLOC_MAX_PAIRS pairs per call; larger calls fail with
//     RT_ERR_INVALID and leave the outputs untouched;
//   - the array (about 9 MiB) is reserved on every GPU that loads the
//     library, for the life of the process;
//   - all calls on a device share the one array, whichever rt_ctx they come
//     from: calls that overlap on the GPU (different streams or contexts, or
//     different host threads without ordering) race and corrupt each other's
//     results.  Serialize them on one stream, or order them with events;
//   - a device-side failure (a look-back wait that gave up) does not change
//     the return code: it sets RT_DEV_TIMEOUT in the context's status, which
//     rt_device_status reads after the caller synchronises;
//   - the first call on a device looks up the array's device address
//     (cudaGetSymbolAddress) and caches it; make that first call before
//     any stream capture begins.
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>

#include "../../include/rt_cuda.h"
#include "ctx_internal.h"
#include "lbvh.cuh"

namespace {

constexpr uint32_t kMaxPairs = RT_NOALLOC_MAX_PAIRS;
constexpr uint32_t kTile = 4096;                         // keys per k_onesweep tile
constexpr size_t kTiles = (kMaxPairs + kTile - 1) / kTile;
// hist[4*256] | tile counters[4] | lookback[4 passes * tiles * 256] | padding
constexpr size_t kControlWords = ((4 * 256 + 4 + 4 * kTiles * 256) + 63) / 64 * 64;
// + keys / values of the intermediate passes
constexpr size_t kScratchWords = kControlWords + 2 * (size_t)kMaxPairs;

// The scratch: part of the library's device image, never allocated per call.
static __device__ __align__(256) uint32_t g_noalloc_scratch[kScratchWords];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
uint32_t* g_scratch_ptr[kMaxDevices] = {nullptr};

// Device address of the array on the current device (looked up once per
// device; the host-side symbol itself is not a device address).
int32_t scratch_for_device(int dev, uint32_t** out) {
    if (dev < 0 || dev >= kMaxDevices)
        return rt::set_error(RT_ERR_INVALID, "rt_sort_pairs_noalloc: device %d out of range", dev);
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return rt::set_error(RT_ERR_CUDA, "rt_sort_pairs_noalloc: cudaGetSymbolAddress: %s",
                                 cudaGetErrorString(e));
        g_scratch_ptr[dev] = static_cast<uint32_t*>(p);
    }
    *out = g_scratch_ptr[dev];
    return RT_OK;
}

// True when the byte range of an output, [p, p + 4n), meets an input's or
// the other output's.  A pass that runs out of place reads one pair of
// arrays while it writes the other, so any overlap corrupts the result
// (with an odd pass count the first pass writes the outputs while it still
// reads the inputs).
bool overlapping(const uint32_t* ki, const uint32_t* vi, const uint32_t* ko, const uint32_t* vo,
                 uint32_t n) {
    const uintptr_t len = 4 * (uintptr_t)n;
    auto meet = [len](const uint32_t* a, const uint32_t* b) {
        const uintptr_t x = (uintptr_t)a, y = (uintptr_t)b;
        return x < y + len && y < x + len;
    };
    return meet(ko, ki) || meet(ko, vi) || meet(vo, ki) || meet(vo, vi) || meet(ko, vo);
}

}  // namespace

extern "C" RT_API int32_t rt_sort_pairs_noalloc(rt_ctx* ctx, const uint32_t* d_keys_in,
                                                const uint32_t* d_vals_in, uint32_t* d_keys_out,
                                                uint32_t* d_vals_out, uint32_t n, int32_t key_bits,
                                                rt_stream stream) {
    if (!ctx) return rt::set_error(RT_ERR_INVALID, "rt_sort_pairs_noalloc: null context");
    if (n > kMaxPairs)
        return rt::set_error(RT_ERR_INVALID,
                             "rt_sort_pairs_noalloc: %u pairs exceed the fixed scratch limit of "
                             "%u pairs (RT_NOALLOC_MAX_PAIRS)",
                             n, kMaxPairs);
    if (key_bits < 1 || key_bits > 32)
        return rt::set_error(RT_ERR_INVALID, "rt_sort_pairs_noalloc: key_bits %d outside [1, 32]",
                             key_bits);
    if (n > 0 && (!d_keys_in || !d_vals_in || !d_keys_out || !d_vals_out))
        return rt::set_error(RT_ERR_INVALID, "rt_sort_pairs_noalloc: null buffer");
    if (n > 0 && overlapping(d_keys_in, d_vals_in, d_keys_out, d_vals_out, n))
        return rt::set_error(RT_ERR_INVALID,
                             "rt_sort_pairs_noalloc: an output overlaps an input or the other output");
    int cur = -1;
    cudaError_t e = cudaGetDevice(&cur);
    if (e != cudaSuccess) return rt::set_error(RT_ERR_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
    if (cur != ctx->device) {
        e = cudaSetDevice(ctx->device);
        if (e != cudaSuccess)
            return rt::set_error(RT_ERR_CUDA, "cudaSetDevice: %s", cudaGetErrorString(e));
    }
    if (rt::radix_tile_size() != (int)kTile)
        return rt::set_error(RT_ERR, "rt_sort_pairs_noalloc: tile size mismatch");
    uint32_t* scratch = nullptr;
    int32_t r = scratch_for_device(ctx->device, &scratch);
    if (r) return r;
    cudaStream_t s = stream ? (cudaStream_t)stream : ctx->stream;
    uint32_t* ktmp = scratch + kControlWords;
    uint32_t* vtmp = ktmp + kMaxPairs;
    // radix_sort_pairs clears the histogram, tile counters and look-back
    // words it uses (cudaMemsetAsync) before its first pass.
    e = rt::radix_sort_pairs(d_keys_in, d_vals_in, d_keys_out, d_vals_out, ktmp, vtmp, n, key_bits,
                             scratch, ctx->d_status, ctx->num_sms, s);
    if (e != cudaSuccess)
        return rt::set_error(RT_ERR_CUDA, "rt_sort_pairs_noalloc: %s", cudaGetErrorString(e));
    return RT_OK;
}
