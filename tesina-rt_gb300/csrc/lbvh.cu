// lbvh.cu — LBVH construction of one scene for sm_103a.
//
// Stages (the reference's BVHBuilder::build_lbvh, src/rt/bvh-builder.cpp:201-741):
//   k_bounds        per-triangle AABB (build_primitive_bbox, bvh-builder.cl:100-130)
//                   reduced to the scene AABB (max_local_bbox, :318-391) with
//                   order-free integer min/max atomics;
//   k_morton_hist   morton_encode (:181-252) fused with the digit histograms of
//                   every radix pass;
//   k_onesweep      stable LSD radix pass, 8-bit digits, warp-level
//                   ballot ranking and decoupled look-back with a
//                   bounded spin (replaces the bitonic network of
//                   bvh-builder-sort.cl and bvh-builder.cpp:361-454);
//   k_emit_level0_permute
//                   rearrange_indices / rearrange_map (:49-72) and the
//                   triangle records used by traversal, fused with level 0 of
//                   the emit, which joins the triangles with their AABBs
//                   still in registers;
//   k_emit_level    bottom-up build of the radix tree (Apetrei's
//                   agglomerative formulation of Karras' tree), collapsed to
//                   the reference's leaf rule (find_middle, :484-552), with
//                   every AABB (build_leaf_bbox / build_node_bbox, :262-311)
//                   computed on the way up; a few launches whose warps join
//                   runs of 32 items (level 0 over 512 triangles per block,
//                   then over what 8 blocks left).
//   k_permute       the permutation alone, storing leaf AABBs (the stage-wise
//                   entry point); k_refit_leaves the leaf AABBs of the
//                   existing order (refit).
// The per-element work lives in lbvh_dev.cuh, shared with the many-scene
// persistent build of batch.cu.
#include <cuda_runtime.h>
#include <stdint.h>
#include <mutex>

#include "lbvh.cuh"
#include "lbvh_dev.cuh"
#include "rt_internal.cuh"

// The full build's level-0 emit performs the permutation itself (1), or a
// separate k_permute stores the leaf AABBs for it (0).
#ifndef RT_EMIT_PERMUTE
#define RT_EMIT_PERMUTE 1
#endif
// The first radix pass makes the values 0..n-1 itself (1) instead of reading
// them from a buffer k_morton_hist fills (0).
#ifndef RT_SORT_IOTA
#define RT_SORT_IOTA 1
#endif
constexpr bool kIotaVals = RT_SORT_IOTA != 0;
// Digit width of the build's radix passes: 8 (four passes for 30-bit keys)
// or 10 (three).  The pair sort entry points always use 8.
#ifndef RT_SORT_BITS
#define RT_SORT_BITS 8
#endif
constexpr int kBuildBits = RT_SORT_BITS;
constexpr int kBuildRadix = 1 << kBuildBits;
constexpr int kMaxBuildPasses = (32 + kBuildBits - 1) / kBuildBits;
static_assert(kBuildBits == 8 || kBuildBits == 10, "build digit width");

namespace rt {

// Programmatic dependent launch.  The build's kernels after the first are
// launched while their predecessor still runs (launch_dep); each waits at
// its start for the predecessor grid to finish and its writes to be visible
// (griddepcontrol.wait, which returns at once for a kernel launched without
// the dependency), then lets its own successor launch.  It hides the
// launches' latency: the mid-scale build took 0.2752-0.2772 ms against
// 0.2802 ms without it, the 17.7 M-triangle build 2.584-2.589 against
// 2.604-2.605 ms (three alternating runs each, one box).
__device__ __forceinline__ void pdl_enter() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

template <typename... KArgs, typename... Args>
static cudaError_t launch_dep(void (*kern)(KArgs...), unsigned grid, unsigned block, size_t smem,
                              cudaStream_t s, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kern, args...);
}

__global__ void __launch_bounds__(256) k_bounds(const float4* __restrict__ pos,
                                                const uint32_t* __restrict__ idx, uint32_t n,
                                                uint32_t* __restrict__ bounds) {
    pdl_enter();
    float lo[3] = {1e37f, 1e37f, 1e37f}, hi[3] = {-1e37f, -1e37f, -1e37f};
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float tl[3], th[3];
        tri_aabb(pos, idx, i, tl, th);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            lo[c] = fminf(lo[c], tl[c]);
            hi[c] = fmaxf(hi[c], th[c]);
        }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            lo[c] = fminf(lo[c], __shfl_xor_sync(0xffffffffu, lo[c], off));
            hi[c] = fmaxf(hi[c], __shfl_xor_sync(0xffffffffu, hi[c], off));
        }
    __shared__ float s[8][6];
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0)
        for (int c = 0; c < 3; ++c) {
            s[w][c] = lo[c];
            s[w][3 + c] = hi[c];
        }
    __syncthreads();
    if (threadIdx.x < 3) {
        const int c = threadIdx.x;
        float a = s[0][c], b = s[0][3 + c];
        for (int k = 1; k < (int)(blockDim.x >> 5); ++k) {
            a = fminf(a, s[k][c]);
            b = fmaxf(b, s[k][3 + c]);
        }
        atomicMin(&bounds[c], f2o(a));
        atomicMax(&bounds[3 + c], f2o(b));
    }
}

__global__ void __launch_bounds__(256) k_morton_hist(const float4* __restrict__ pos,
                                                     const uint32_t* __restrict__ idx, uint32_t n,
                                                     const uint32_t* __restrict__ bounds, int depth,
                                                     int passes, uint32_t* __restrict__ keys,
                                                     uint32_t* __restrict__ vals,
                                                     uint32_t* __restrict__ hist) {
    pdl_enter();
    __shared__ uint32_t sh[kMaxBuildPasses][kBuildRadix];
    for (int i = threadIdx.x; i < kMaxBuildPasses * kBuildRadix; i += blockDim.x) (&sh[0][0])[i] = 0;
    __syncthreads();
    const MortonParams P = morton_params(bounds, depth);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float lo[3], hi[3];
        tri_aabb(pos, idx, i, lo, hi);
        const uint32_t code = morton_code(P, lo, hi);
        keys[i] = code;
        if (vals) vals[i] = i;
        for (int p = 0; p < passes; ++p)
            atomicAdd(&sh[p][(code >> (kBuildBits * p)) & (uint32_t)(kBuildRadix - 1)], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < passes * kBuildRadix; i += blockDim.x) {
        const uint32_t v = (&sh[0][0])[i];
        if (v) atomicAdd(&hist[i], v);
    }
}

// Digit histograms of every radix pass over plain keys (the sort without the
// fused Morton stage).
__global__ void __launch_bounds__(256) k_radix_hist(const uint32_t* __restrict__ keys, uint32_t n,
                                                    int passes, uint32_t* __restrict__ hist) {
    __shared__ uint32_t sh[4][256];
    for (int i = threadIdx.x; i < 4 * 256; i += blockDim.x) (&sh[0][0])[i] = 0;
    __syncthreads();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t code = __ldg(&keys[i]);
        for (int p = 0; p < passes; ++p) atomicAdd(&sh[p][(code >> (8 * p)) & 255u], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < passes * 256; i += blockDim.x) {
        const uint32_t v = (&sh[0][0])[i];
        if (v) atomicAdd(&hist[i], v);
    }
}

// One radix pass of BITS-bit digits; dynamic shared memory of
// sizeof(SortSmemT<SORT_ITEMS, BITS>).  MINB tiles resident per SM bound the
// registers: a pass whose tiles all fit in one wave at 2 per SM runs the
// MINB = 2 instance (126 registers, 7 % faster per mid-scale build), a longer
// one RT_SORT_MINB (3, 80 registers: the third tile hides latency).
template <int BITS, int MINB>
__global__ void __launch_bounds__(SORT_THREADS, MINB) k_onesweep(
    const uint32_t* __restrict__ kin, const uint32_t* __restrict__ vin, uint32_t* __restrict__ kout,
    uint32_t* __restrict__ vout, uint32_t n, int shift, const uint32_t* __restrict__ hist,
    uint32_t* __restrict__ lookback, uint32_t* __restrict__ tile_ctr, uint32_t* __restrict__ status) {
    pdl_enter();
    extern __shared__ __align__(16) unsigned char sort_smem[];
    auto& S = *reinterpret_cast<SortSmemT<SORT_ITEMS, BITS>*>(sort_smem);
    if (threadIdx.x == 0) S.tile = atomicAdd(tile_ctr, 1u);   // tiles in launch order
    __syncthreads();
    onesweep_tile<SORT_ITEMS, LB_SPIN_LIMIT, BITS>(S, S.tile, kin, vin, kout, vout, n, shift, hist,
                                                   lookback, status);
}
template <int BITS>
constexpr size_t onesweep_smem() { return sizeof(SortSmemT<SORT_ITEMS, BITS>); }

constexpr int kOneWaveMinB = 2;
// The instance for a pass of `tiles` tiles on `sms` SMs.
template <int BITS>
static auto onesweep_kernel(size_t tiles, int sms) {
    return tiles <= (size_t)kOneWaveMinB * (size_t)sms ? k_onesweep<BITS, kOneWaveMinB>
                                                       : k_onesweep<BITS, RT_SORT_MINB>;
}

// Self-test of the look-back timeout: one block sorts tile 1 of a pass
// whose tile 0 is never launched, so its look-back word stays unpublished;
// with a spin limit of 1,024 polls the wait gives up at once.
constexpr uint32_t kProbeSpinLimit = 1024;
__global__ void __launch_bounds__(SORT_THREADS, 1) k_onesweep_wait_probe(
    const uint32_t* __restrict__ kin, const uint32_t* __restrict__ vin, uint32_t* __restrict__ kout,
    uint32_t* __restrict__ vout, uint32_t n, const uint32_t* __restrict__ hist,
    uint32_t* __restrict__ lookback, uint32_t* __restrict__ status) {
    __shared__ SortSmem S;
    onesweep_tile<SORT_ITEMS, kProbeSpinLimit>(S, 1, kin, vin, kout, vout, n, 0, hist, lookback,
                                               status);
}

__global__ void __launch_bounds__(256) k_permute(uint32_t n, PermuteIO P,
                                                  float4* __restrict__ leafbox) {
    pdl_enter();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        permute_one(i, P, leafbox);
}

// Per-triangle AABBs of the current vertex positions in the existing sorted
// order (refit_lbvh, bvh-builder.cpp:743-790) plus fresh triangle records.
__global__ void __launch_bounds__(256) k_refit_leaves(uint32_t n, const uint32_t* __restrict__ idx,
                                                      const float4* __restrict__ pos,
                                                      float4* __restrict__ tris,
                                                      float4* __restrict__ leafbox) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t a = __ldg(&idx[3 * (size_t)i]), b = __ldg(&idx[3 * (size_t)i + 1]),
                       c = __ldg(&idx[3 * (size_t)i + 2]);
        const float4 p0 = __ldg(&pos[a]), p1 = __ldg(&pos[b]), p2 = __ldg(&pos[c]);
        tris[3 * (size_t)i] = make_float4(p0.x, p0.y, p0.z, 0.f);
        tris[3 * (size_t)i + 1] = make_float4(p1.x - p0.x, p1.y - p0.y, p1.z - p0.z, 0.f);
        tris[3 * (size_t)i + 2] = make_float4(p2.x - p0.x, p2.y - p0.y, p2.z - p0.z, 0.f);
        float lo[3], hi[3];
        tri_aabb(pos, idx, i, lo, hi);
        leafbox[2 * (size_t)i] = make_float4(lo[0], lo[1], lo[2], 0.f);
        leafbox[2 * (size_t)i + 1] = make_float4(hi[0], hi[1], hi[2], 0.f);
    }
}

// One level of the emit (emit_level), one block per run of items; blocks
// are kept to a register budget that lets RT_EMIT_MINB0 (level 0) or
// RT_EMIT_MINB1 (above) of them share an SM.
template <int C>
__global__ void __launch_bounds__(C, C == EMIT_C0 ? RT_EMIT_MINB0 : RT_EMIT_MINB1) k_emit_level(
    uint32_t n, const uint32_t* __restrict__ skeys, const float4* __restrict__ leafbox,
    const EmitItem* __restrict__ in, const uint32_t* __restrict__ in_count, uint32_t n_in,
    EmitItem* __restrict__ out, uint32_t* __restrict__ out_count, float4* __restrict__ nodes,
    int min_leaf, uint32_t leave, BvhHeader* __restrict__ hdr, uint32_t* __restrict__ status) {
    pdl_enter();
    extern __shared__ __align__(16) unsigned char emit_smem[];
    auto& S = *reinterpret_cast<EmitSmem<C>*>(emit_smem);
    emit_level<C>(S, blockIdx.x, n, skeys, leafbox, in, in_count, n_in, out, out_count, nodes,
                  min_leaf, leave, hdr, status);
}

// Level 0 of a full build: each block first permutes its own triangles
// (index buffer, material map, upload ids, triangle records) and joins them
// with their boxes still in registers, so no leaf AABB goes through memory.
__global__ void __launch_bounds__(EMIT_C0, RT_EMIT_MINB0) k_emit_level0_permute(
    uint32_t n, const uint32_t* __restrict__ skeys, PermuteIO P, EmitItem* __restrict__ out,
    uint32_t* __restrict__ out_count, float4* __restrict__ nodes, int min_leaf, uint32_t leave,
    BvhHeader* __restrict__ hdr, uint32_t* __restrict__ status) {
    pdl_enter();
    extern __shared__ __align__(16) unsigned char emit_smem[];
    auto& S = *reinterpret_cast<EmitSmem<EMIT_C0>*>(emit_smem);
    emit_level<EMIT_C0, true>(S, blockIdx.x, n, skeys, nullptr, nullptr, nullptr, 0, out,
                              out_count, nodes, min_leaf, leave, hdr, status, P);
}

static size_t sort_scratch_bytes(uint32_t n, int passes) {
    const size_t tiles = ((size_t)n + SORT_TILE - 1) / SORT_TILE;
    return (sizeof(uint32_t) * (8 + (size_t)kMaxBuildPasses * kBuildRadix + 4 +
                                (size_t)passes * tiles * kBuildRadix) + 255) & ~(size_t)255;
}

static size_t emit_scratch_bytes(uint32_t n) { return emit_buffers_bytes(n); }

// The emit's levels: level 0 over triangles, then levels over the items left
// by EMIT_GROUP blocks each until a single block reaches the root.  Item
// buffers alternate: A holds level 0, 2, ... and B level 1, 3, ....  With
// `perm`, level 0 also performs the permutation (k_emit_level0_permute);
// without, it reads the leaf AABBs a previous launch stored.
// The shared-memory opt-ins of the kernels with dynamic shared memory (a
// property of the kernel on each device), once per device.
static cudaError_t setup_kernels() {
    static std::mutex mu;
    static uint64_t done = 0;   // devices 0..63 set up
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lk(mu);
    if (dev < 64 && ((done >> dev) & 1)) return cudaSuccess;
    auto opt_in = [&](const void* f, size_t bytes) {
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    };
    opt_in((const void*)k_emit_level<EMIT_C0>, sizeof(EmitSmem<EMIT_C0>));
    opt_in((const void*)k_emit_level0_permute, sizeof(EmitSmem<EMIT_C0>));
    opt_in((const void*)k_emit_level<EMIT_C1>, sizeof(EmitSmem<EMIT_C1>));
    opt_in((const void*)k_onesweep<8, kOneWaveMinB>, onesweep_smem<8>());
    opt_in((const void*)k_onesweep<8, RT_SORT_MINB>, onesweep_smem<8>());
    opt_in((const void*)k_onesweep<kBuildBits, kOneWaveMinB>, onesweep_smem<kBuildBits>());
    opt_in((const void*)k_onesweep<kBuildBits, RT_SORT_MINB>, onesweep_smem<kBuildBits>());
    if (e != cudaSuccess) return e;
    if (dev < 64) done |= 1ull << dev;
    return cudaSuccess;
}

static cudaError_t launch_emit(const LbvhArgs& a, uint8_t* emit_scratch, cudaStream_t s,
                               const PermuteIO* perm = nullptr) {
    const uint32_t n = a.n;
    if (cudaError_t e0 = setup_kernels()) return e0;
    const uint32_t nb0 = emit_blocks0(n);
    const EmitBuffers B = emit_buffers(n, emit_scratch);
    cudaError_t e =
        perm ? launch_dep(k_emit_level0_permute, nb0, EMIT_C0, sizeof(EmitSmem<EMIT_C0>), s, n,
                          (const uint32_t*)a.keys_sorted, *perm, B.items[0], B.counts[0], a.nodes,
                          a.min_leaf, emit_leave(0, nb0), a.hdr, a.status)
             : launch_dep(k_emit_level<EMIT_C0>, nb0, EMIT_C0, sizeof(EmitSmem<EMIT_C0>), s, n,
                          (const uint32_t*)a.keys_sorted, (const float4*)a.leafbox,
                          (const EmitItem*)nullptr, (const uint32_t*)nullptr, 0u, B.items[0],
                          B.counts[0], a.nodes, a.min_leaf, emit_leave(0, nb0), a.hdr, a.status);
    if (e) return e;
    uint32_t n_in = nb0;
    int src = 0;
    while (n_in > 1) {
        const uint32_t g = emit_next_level(n_in);
        e = launch_dep(k_emit_level<EMIT_C1>, g, EMIT_C1, sizeof(EmitSmem<EMIT_C1>), s, n,
                       (const uint32_t*)a.keys_sorted, (const float4*)a.leafbox,
                       (const EmitItem*)B.items[src], (const uint32_t*)B.counts[src], n_in,
                       B.items[src ^ 1], B.counts[src ^ 1], a.nodes, a.min_leaf, emit_leave(1, g),
                       a.hdr, a.status);
        if (e) return e;
        n_in = g;
        src ^= 1;
    }
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// host launchers
// ---------------------------------------------------------------------------

static int grid_for(uint32_t n, int threads, int max_blocks) {
    int64_t b = ((int64_t)n + threads - 1) / threads;
    if (b < 1) b = 1;
    if (b > max_blocks) b = max_blocks;
    return (int)b;
}

size_t lbvh_scratch_bytes(uint32_t n, int passes) {
    return sort_scratch_bytes(n, passes) + emit_scratch_bytes(n);
}

size_t lbvh_emit_offset(uint32_t n) { return sort_scratch_bytes(n, kMaxBuildPasses); }

cudaError_t lbvh_build(const LbvhArgs& a, cudaStream_t s) {
    const uint32_t n = a.n;
    const int passes = (a.depth + kBuildBits - 1) / kBuildBits;
    const size_t tiles = ((size_t)n + SORT_TILE - 1) / SORT_TILE;
    // scratch: bounds[8] | hist[passes max * radix] | tile_ctr[4] |
    // lookback[passes * tiles * radix]
    uint32_t* bounds = a.scratch;
    uint32_t* hist = bounds + 8;
    uint32_t* tile_ctr = hist + kMaxBuildPasses * kBuildRadix;
    uint32_t* lookback = tile_ctr + 4;
    cudaError_t e = setup_kernels();
    if (e) return e;
    e = cudaMemsetAsync(a.scratch, 0, sort_scratch_bytes(n, passes), s);
    if (e) return e;
    // bounds init: lo = ordered(+big) via 0xFF.. (max), hi = 0 (min)
    e = cudaMemsetAsync(bounds, 0xff, 3 * sizeof(uint32_t), s);
    if (e) return e;
    const int sms = a.num_sms;
    k_bounds<<<grid_for(n, 256, sms * 8), 256, 0, s>>>(a.pos, a.idx_in, n, bounds);
    e = launch_dep(k_morton_hist, grid_for(n, 256, sms * 8), 256, 0, s, a.pos, a.idx_in, n,
                   bounds, a.depth, passes, a.keys_unsorted, kIotaVals ? nullptr : a.vals0, hist);
    if (e) return e;
    const uint32_t* kin = a.keys_unsorted;
    const uint32_t* vin = kIotaVals ? nullptr : a.vals0;
    uint32_t* kbuf[2] = {a.keys1, a.keys_sorted};
    uint32_t* vbuf[2] = {a.vals1, a.vals_sorted};
    for (int p = 0; p < passes; ++p) {
        // the last pass always lands in keys_sorted / vals_sorted
        const int dst = ((passes - 1 - p) & 1) ? 0 : 1;
        e = launch_dep(onesweep_kernel<kBuildBits>(tiles, sms), (unsigned)tiles, SORT_THREADS,
                       onesweep_smem<kBuildBits>(), s, kin, vin, kbuf[dst], vbuf[dst], n,
                       kBuildBits * p, (const uint32_t*)(hist + kBuildRadix * p),
                       lookback + (size_t)p * tiles * kBuildRadix, tile_ctr + p, a.status);
        if (e) return e;
        kin = kbuf[dst];
        vin = vbuf[dst];
    }
    const PermuteIO P{a.vals_sorted, a.idx_in,  a.map_in,   a.orig_in, a.pos,
                      a.idx_out,     a.map_out, a.orig_out, a.tris};
#if RT_EMIT_PERMUTE
    return launch_emit(a, reinterpret_cast<uint8_t*>(a.scratch) + lbvh_emit_offset(n), s, &P);
#else
    e = launch_dep(k_permute, grid_for(n, 256, sms * 16), 256, 0, s, n, P, a.leafbox);
    if (e) return e;
    return launch_emit(a, reinterpret_cast<uint8_t*>(a.scratch) + lbvh_emit_offset(n), s);
#endif
}

size_t radix_scratch_words(uint32_t n, int passes) {
    const size_t tiles = ((size_t)n + SORT_TILE - 1) / SORT_TILE;
    return 4 * 256 + 4 + (size_t)passes * tiles * 256;
}

int radix_tile_size() { return SORT_TILE; }

size_t wait_probe_words() { return (size_t)2 * SORT_TILE * 4 + 256 + 2 * 256; }

cudaError_t wait_probe(uint32_t* buf, uint32_t* status, cudaStream_t s) {
    // buf: keys | vals | kout | vout (2 tiles each) | hist[256] | lookback[2 * 256]
    const uint32_t n = 2 * SORT_TILE;
    uint32_t* keys = buf;
    uint32_t* vals = keys + n;
    uint32_t* kout = vals + n;
    uint32_t* vout = kout + n;
    uint32_t* hist = vout + n;
    uint32_t* lookback = hist + 256;
    cudaError_t e = cudaMemsetAsync(buf, 0, sizeof(uint32_t) * wait_probe_words(), s);
    if (e) return e;
    k_radix_hist<<<1, 256, 0, s>>>(keys, n, 1, hist);
    k_onesweep_wait_probe<<<1, SORT_THREADS, 0, s>>>(keys, vals, kout, vout, n, hist, lookback,
                                                     status);
    return cudaGetLastError();
}

cudaError_t radix_sort_pairs(const uint32_t* kin, const uint32_t* vin, uint32_t* kout,
                             uint32_t* vout, uint32_t* ktmp, uint32_t* vtmp, uint32_t n,
                             int key_bits, uint32_t* scratch, uint32_t* status, int num_sms,
                             cudaStream_t s) {
    const int passes = (key_bits + 7) / 8;
    const size_t tiles = ((size_t)n + SORT_TILE - 1) / SORT_TILE;
    uint32_t* hist = scratch;
    uint32_t* tile_ctr = hist + 4 * 256;
    uint32_t* lookback = tile_ctr + 4;
    cudaError_t e = setup_kernels();
    if (e) return e;
    e = cudaMemsetAsync(scratch, 0, sizeof(uint32_t) * radix_scratch_words(n, passes), s);
    if (e) return e;
    if (n == 0) return cudaSuccess;
    k_radix_hist<<<grid_for(n, 256, num_sms * 8), 256, 0, s>>>(kin, n, passes, hist);
    const uint32_t* ki = kin;
    const uint32_t* vi = vin;
    for (int p = 0; p < passes; ++p) {
        const bool to_out = ((passes - 1 - p) & 1) == 0;
        uint32_t* ko = to_out ? kout : ktmp;
        uint32_t* vo = to_out ? vout : vtmp;
        onesweep_kernel<8>(tiles, num_sms)<<<(unsigned)tiles, SORT_THREADS, onesweep_smem<8>(), s>>>(
            ki, vi, ko, vo, n, 8 * p, hist + 256 * p, lookback + (size_t)p * tiles * 256,
            tile_ctr + p, status);
        ki = ko;
        vi = vo;
    }
    return cudaGetLastError();
}

cudaError_t lbvh_permute(const LbvhArgs& a, const uint32_t* order, cudaStream_t s) {
    const PermuteIO P{order,     a.idx_in,  a.map_in,   a.orig_in, a.pos,
                      a.idx_out, a.map_out, a.orig_out, a.tris};
    k_permute<<<grid_for(a.n, 256, a.num_sms * 16), 256, 0, s>>>(a.n, P, a.leafbox);
    return cudaGetLastError();
}

cudaError_t lbvh_refit(const LbvhArgs& a, cudaStream_t s) {
    const uint32_t n = a.n;
    k_refit_leaves<<<grid_for(n, 256, a.num_sms * 16), 256, 0, s>>>(n, a.idx_out, a.pos, a.tris,
                                                                    a.leafbox);
    // the emit is deterministic in the sorted keys, so rerunning it on the
    // same keys reproduces the same topology with the new boxes
    return launch_emit(a, reinterpret_cast<uint8_t*>(a.scratch) + lbvh_emit_offset(n), s);
}

}  // namespace rt
