// lbvh_dev.cuh — device-side stages of the LBVH build, shared by the
// one-scene kernels (lbvh.cu) and the persistent many-scene kernel
// (batch.cu).  Each function works on one scene whose arrays are passed
// already offset to that scene, so the same code serves both.
//
// Reference: BVHBuilder::build_lbvh (src/rt/bvh-builder.cpp:201-741) and
// src/kernel/bvh-builder.cl (citations per function).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "rt_internal.cuh"

namespace rt {

#ifndef RT_SORT_VEC_LOADS
#define RT_SORT_VEC_LOADS 1   // whole tiles staged in shared memory: 0 no, 1 by 128-bit loads, 2 by bulk copy
#endif
#ifndef RT_SORT_MINB
#define RT_SORT_MINB 3   // radix tiles resident per SM (register budget)
#endif
constexpr int SORT_THREADS = 256;
constexpr int SORT_WARPS = SORT_THREADS / 32;
#ifndef RT_SORT_ITEMS
#define RT_SORT_ITEMS 16   // keys per thread of a radix tile
#endif
constexpr int SORT_ITEMS = RT_SORT_ITEMS;
constexpr int SORT_TILE = SORT_THREADS * SORT_ITEMS;   // 4096 keys per tile
constexpr uint32_t LB_AGG = 1u << 30, LB_PREFIX = 2u << 30, LB_MASK = (1u << 30) - 1;
constexpr uint32_t LB_SPIN_LIMIT = 1u << 22;
// Look-back words read per round trip.  A poll that meets an unpublished
// word reads its whole window again, so a wide window costs more in polls
// than it saves in round trips: 2 to 6 words measured best (32 words: a
// build of 17.7 M triangles 7 % slower; a sleep between polls changed
// nothing).
#ifndef RT_LB_WINDOW
#define RT_LB_WINDOW 4
#endif
constexpr int LB_WINDOW = RT_LB_WINDOW;

// float <-> order-preserving uint32 (min/max of the integers == fmin/fmax of
// the floats for non-NaN values).
__device__ __forceinline__ uint32_t f2o(float f) {
    uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float o2f(uint32_t o) {
    uint32_t u = (o & 0x80000000u) ? (o & 0x7fffffffu) : ~o;
    return __uint_as_float(u);
}

// Relaxed GPU-scope accesses: coherent in L2, no ordering of other memory.
// For words that carry their whole message (the radix look-back's flag and
// count).
__device__ __forceinline__ uint32_t ld_relaxed(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed(uint32_t* p, uint32_t v) {
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// A shared-memory mbarrier and the 1-D bulk copy (the TMA engine without a
// tensor map) that completes on it.
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_inval(uint64_t* bar) {
    asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_addr(bar)) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
                 "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok) : "r"(smem_addr(bar)), "r"(parity) : "memory");
    return ok != 0;
}
// global -> shared, `bytes` a multiple of 16, both addresses 16-byte aligned
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
        ::"r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(bar)) : "memory");
}
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
constexpr uint32_t BULK_WAIT_LIMIT = 1u << 22;   // polls of a bulk copy's mbarrier
// atomicAdd with acquire-release ordering at GPU scope: the caller's earlier
// writes are visible to whoever reads the counter's new value, and the
// caller sees everything released by earlier adders.
__device__ __forceinline__ uint32_t atomic_add_acq_rel(uint32_t* p, uint32_t v) {
    uint32_t old;
    asm volatile("atom.add.acq_rel.gpu.global.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v)
                 : "memory");
    return old;
}

// build_primitive_bbox (bvh-builder.cl:100-130) of one triangle.
__device__ __forceinline__ void tri_aabb(const float4* __restrict__ pos,
                                         const uint32_t* __restrict__ idx, uint32_t i,
                                         float lo[3], float hi[3]) {
    const uint32_t a = __ldg(&idx[3 * (size_t)i]), b = __ldg(&idx[3 * (size_t)i + 1]),
                   c = __ldg(&idx[3 * (size_t)i + 2]);
    const float4 p0 = __ldg(&pos[a]), p1 = __ldg(&pos[b]), p2 = __ldg(&pos[c]);
    hi[0] = fmaxf(fmaxf(p0.x, p1.x), p2.x);
    hi[1] = fmaxf(fmaxf(p0.y, p1.y), p2.y);
    hi[2] = fmaxf(fmaxf(p0.z, p1.z), p2.z);
    lo[0] = fminf(fminf(p0.x, p1.x), p2.x);
    lo[1] = fminf(fminf(p0.y, p1.y), p2.y);
    lo[2] = fminf(fminf(p0.z, p1.z), p2.z);
}

// Per-scene constants of morton_encode (bvh-builder.cl:181-252).
struct MortonParams {
    float glo[3], inv[3];
    float scale;          // pow(2, ceil(depth / 3.0))
    int depth, offset;    // offset = depth % 3 ? 3 - depth % 3 : 0
};

__device__ __forceinline__ MortonParams morton_params(const uint32_t* bounds, int depth) {
    MortonParams m;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        m.glo[c] = o2f(bounds[c]);
        const float ghi = o2f(bounds[3 + c]);
        m.inv[c] = 1.0f / (ghi - m.glo[c]);
    }
    m.scale = (float)(1u << ((depth + 2) / 3));
    m.depth = depth;
    m.offset = depth % 3 ? 3 - (depth % 3) : 0;
    return m;
}

// Spreads the low 21 bits of v to every third bit (bit t to bit 3t): the
// mask-and-shift bit interleave ("magic numbers") of Morton encoders.
__device__ __forceinline__ uint64_t spread3(uint64_t v) {
    v &= 0x1fffffull;
    v = (v | (v << 32)) & 0x1f00000000ffffull;
    v = (v | (v << 16)) & 0x1f0000ff0000ffull;
    v = (v | (v << 8)) & 0x100f00f00f00f00full;
    v = (v | (v << 4)) & 0x10c30c30c30c30c3ull;
    v = (v | (v << 2)) & 0x1249249249249249ull;
    return v;
}

// morton_encode's bit loop takes, for code bit b (b < depth), bit (b+off)/3
// of the slice of axis (b+off+1) % 3.  With j = b + off, that is the
// interleave I whose bit j is bit j/3 of axis (j+1) % 3 (y, z, x for
// j = 0, 1, 2 mod 3), shifted down by off; the slices keep their low
// ceil(depth/3) bits (a slice of 2^ceil(depth/3), from a centroid at the
// upper bound, contributes nothing).
__device__ __forceinline__ uint32_t morton_code(const MortonParams& P, const float lo[3],
                                                const float hi[3]) {
    uint32_t m[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float center = (hi[k] + lo[k]) * 0.5f;
        float slice = (center - P.glo[k]) * P.inv[k];
        slice = fmaxf(0.0f, fminf(1.0f, slice));
        slice *= P.scale;
        m[k] = (uint32_t)slice;   // truncation
    }
    const int bits = (P.depth + 2) / 3;
    const uint32_t keep = (1u << bits) - 1u;
    const uint64_t I = spread3(m[1] & keep) | (spread3(m[2] & keep) << 1) |
                       (spread3(m[0] & keep) << 2);
    const uint64_t code = I >> P.offset;
    return P.depth >= 32 ? (uint32_t)code : (uint32_t)code & ((1u << P.depth) - 1u);
}

// Exclusive scan of one value per thread over a 256-thread block.
__device__ __forceinline__ uint32_t block_excl_scan_256(uint32_t v, uint32_t* s_warp) {
    const int l = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (l >= o) x += y;
    }
    if (l == 31) s_warp[w] = x;
    __syncthreads();
    if (w == 0) {
        uint32_t t = l < SORT_WARPS ? s_warp[l] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, t, o);
            if (l >= o) t += y;
        }
        if (l < SORT_WARPS) s_warp[l] = t;
    }
    __syncthreads();
    const uint32_t warp_base = w ? s_warp[w - 1] : 0;
    __syncthreads();
    return warp_base + x - v;
}

// Phase marks of a radix tile (k = 0..6), for timing harnesses; none by default.
#ifndef RT_SORT_MARK
#define RT_SORT_MARK(k)
#endif

template <int ITEMS, int BITS = 8>
struct __align__(16) SortSmemT {
    static constexpr int RADIX = 1 << BITS;
    uint32_t keys[SORT_THREADS * ITEMS];
    uint32_t vals[SORT_THREADS * ITEMS];
    uint32_t whist[SORT_WARPS][RADIX];
    uint32_t goff[RADIX];
    uint32_t lstart[RADIX];
    uint64_t bar;   // the bulk tile load's mbarrier
    uint32_t scan[SORT_WARPS];
    uint32_t tile;
};
using SortSmem = SortSmemT<SORT_ITEMS>;

// One tile of a stable LSD radix pass (BITS-bit digit at `shift`; each
// thread owns 2^BITS / SORT_THREADS consecutive digits): warp-striped loads,
// ballot ranking in index order, decoupled look-back over the earlier tiles
// of the same sequence, shared-memory staging and a coalesced scatter.  Must
// be called by all SORT_THREADS threads of a block; a tile holds
// SORT_THREADS * ITEMS keys.  A null `vin` stands for the values 0, 1, 2, ...
// (the first pass of a build).  A look-back that polls an unpublished word
// more than SPIN_LIMIT times gives up: it sets RT_DEV_TIMEOUT in *status and
// goes on with the counts it has, so every block ends; the tile's writes
// then stay inside [0, n), since a partial prefix only lowers the scatter
// offsets, which start at the digit's global offset.  `hist` holds the
// pass's 2^BITS digit counts, `lookback` 2^BITS words per tile.
template <int ITEMS = SORT_ITEMS, uint32_t SPIN_LIMIT = LB_SPIN_LIMIT, int BITS = 8>
__device__ __forceinline__ void onesweep_tile(SortSmemT<ITEMS, BITS>& S, uint32_t tile,
                                              const uint32_t* __restrict__ kin,
                                              const uint32_t* __restrict__ vin,
                                              uint32_t* __restrict__ kout,
                                              uint32_t* __restrict__ vout, uint32_t n, int shift,
                                              const uint32_t* __restrict__ hist,
                                              uint32_t* __restrict__ lookback,
                                              uint32_t* __restrict__ status) {
    constexpr int RADIX = 1 << BITS;
    constexpr int DPT = RADIX / SORT_THREADS;   // digits per thread
    constexpr uint32_t DMASK = (uint32_t)RADIX - 1u;
    static_assert(DPT >= 1 && RADIX % SORT_THREADS == 0, "digits per thread");
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    RT_SORT_MARK(0);
    for (int i = tid; i < SORT_WARPS * RADIX; i += SORT_THREADS) (&S.whist[0][0])[i] = 0;
    __syncthreads();
    const size_t base = (size_t)tile * (SORT_THREADS * ITEMS);
    const uint32_t lanemask_lt = (1u << lane) - 1u;

    uint32_t k[ITEMS], v[ITEMS], rank[ITEMS];
#if RT_SORT_VEC_LOADS
    // a whole, 16-byte aligned tile: 128-bit loads into shared memory, then
    // the warp-striped layout the ranking needs from there
    const bool vec = base + (size_t)(SORT_THREADS * ITEMS) <= n &&
                     ((reinterpret_cast<uintptr_t>(kin) | reinterpret_cast<uintptr_t>(vin)) & 15u) == 0;
    static_assert(ITEMS % 4 == 0, "whole 128-bit words per thread");
    if (vec) {
#if RT_SORT_VEC_LOADS == 2
        // one bulk copy per array, completing on the tile's mbarrier
        constexpr uint32_t TB = SORT_THREADS * ITEMS * 4;
        if (tid == 0) {
            mbar_init(&S.bar);
            fence_proxy_async_smem();   // earlier generic accesses of the buffers come first
            mbar_arrive_expect_tx(&S.bar, vin ? 2 * TB : TB);
            bulk_load(S.keys, kin + base, TB, &S.bar);
            if (vin) bulk_load(S.vals, vin + base, TB, &S.bar);
        }
        __syncthreads();   // the barrier is initialised before anyone polls it
        uint32_t polls = 0;
        while (!mbar_try_wait(&S.bar, 0) && ++polls < BULK_WAIT_LIMIT) {
        }
        if (polls >= BULK_WAIT_LIMIT) {
            atomicOr(status, RT_DEV_TIMEOUT);
            while (!mbar_try_wait(&S.bar, 0) && ++polls < 2 * BULK_WAIT_LIMIT) {
            }
        }
#else
        const uint4* k4 = reinterpret_cast<const uint4*>(kin + base);
        const uint4* v4 = reinterpret_cast<const uint4*>(vin + base);
#pragma unroll
        for (int j = 0; j < ITEMS / 4; ++j) {
            const int e = j * SORT_THREADS + tid;
            reinterpret_cast<uint4*>(S.keys)[e] = __ldcs(&k4[e]);
            if (vin) reinterpret_cast<uint4*>(S.vals)[e] = __ldcs(&v4[e]);
        }
        __syncthreads();
#endif
#pragma unroll
        for (int j = 0; j < ITEMS; ++j) {
            const int e = warp * (ITEMS * 32) + j * 32 + lane;
            k[j] = S.keys[e];
            v[j] = vin ? S.vals[e] : (uint32_t)(base + e);
        }
    } else
#endif
#pragma unroll
    for (int j = 0; j < ITEMS; ++j) {
        const size_t g = base + (size_t)warp * (ITEMS * 32) + j * 32 + lane;
        const bool ok = g < n;
        k[j] = ok ? __ldcs(&kin[g]) : 0xffffffffu;
        v[j] = ok ? (vin ? __ldcs(&vin[g]) : (uint32_t)g) : 0u;
    }
#pragma unroll
    for (int j = 0; j < ITEMS; ++j) {
        const size_t g = base + (size_t)warp * (ITEMS * 32) + j * 32 + lane;
        const bool ok = g < n;
        const uint32_t d = (k[j] >> shift) & DMASK;
        // lanes holding the same digit: one ballot per digit bit (a fixed
        // cost, where a match instruction grows with the distinct digits)
        uint32_t peers = __ballot_sync(0xffffffffu, ok);
#pragma unroll
        for (int b = 0; b < BITS; ++b) {
            const uint32_t bit = __ballot_sync(0xffffffffu, (d >> b) & 1u);
            peers &= ((d >> b) & 1u) ? bit : ~bit;
        }
        uint32_t prev = 0;
        if (ok) prev = S.whist[warp][d];
        __syncwarp();
        if (ok) {
            rank[j] = prev + __popc(peers & lanemask_lt);
            const int leader = __ffs(peers) - 1;
            if (lane == leader) S.whist[warp][d] = prev + __popc(peers);
        }
        __syncwarp();
    }
    __syncthreads();

    RT_SORT_MARK(1);
    // this thread's digits: tid * DPT .. tid * DPT + DPT - 1
    const uint32_t dgt0 = (uint32_t)tid * DPT;
    uint32_t cnt[DPT], lstart[DPT];
    uint32_t tsum = 0;
#pragma unroll
    for (int q = 0; q < DPT; ++q) {
        uint32_t c = 0;
#pragma unroll
        for (int w = 0; w < SORT_WARPS; ++w) {
            const uint32_t x = S.whist[w][dgt0 + q];
            S.whist[w][dgt0 + q] = c;
            c += x;
        }
        cnt[q] = c;
        lstart[q] = tsum;
        tsum += c;
    }
    uint32_t* my = &lookback[(size_t)tile * RADIX + dgt0];
#pragma unroll
    for (int q = 0; q < DPT; ++q)   // as early as the counts are known
        st_relaxed(my + q, (tile == 0 ? LB_PREFIX : LB_AGG) | cnt[q]);
    const uint32_t lbase = block_excl_scan_256(tsum, S.scan);
#pragma unroll
    for (int q = 0; q < DPT; ++q) {
        lstart[q] += lbase;
        S.lstart[dgt0 + q] = lstart[q];
    }
    __syncthreads();
    // the tile in digit order in shared memory (frees the registers of the
    // keys for the look-back's window)
#pragma unroll
    for (int j = 0; j < ITEMS; ++j) {
        const size_t g = base + (size_t)warp * (ITEMS * 32) + j * 32 + lane;
        if (g < n) {
            const uint32_t d = (k[j] >> shift) & DMASK;
            const uint32_t p = S.lstart[d] + S.whist[warp][d] + rank[j];
            S.keys[p] = k[j];
            S.vals[p] = v[j];
        }
    }
    // Decoupled look-back.  Each word holds its whole message (flag and
    // count), so relaxed accesses suffice; the words of LB_WINDOW earlier
    // tiles are read per round trip and summed nearest first, for each digit
    // up to its first inclusive prefix, and for all of them up to the first
    // tile that has not published a digit still open.
    RT_SORT_MARK(2);
    uint32_t excl[DPT];
#pragma unroll
    for (int q = 0; q < DPT; ++q) excl[q] = 0;
    if (tile > 0) {
        constexpr uint32_t ALL = (1u << DPT) - 1u;
        uint32_t open = ALL;   // digits without an inclusive prefix yet
        int64_t p = (int64_t)tile - 1;
        uint32_t spins = 0;
        for (;;) {
            uint32_t w[LB_WINDOW][DPT];
#pragma unroll
            for (int t = 0; t < LB_WINDOW; ++t)   // tile 0 is always a prefix: p - t < 0 is never summed
#pragma unroll
                for (int q = 0; q < DPT; ++q)
                    w[t][q] = p - t >= 0 ? ld_relaxed(&lookback[(size_t)(p - t) * RADIX + dgt0 + q])
                                         : LB_PREFIX;
            int used = 0;
            bool wait = false;
#pragma unroll
            for (int t = 0; t < LB_WINDOW; ++t) {
                if (open && !wait) {
                    bool miss = false;
#pragma unroll
                    for (int q = 0; q < DPT; ++q)
                        miss |= ((open >> q) & 1u) && (w[t][q] & ~LB_MASK) == 0u;
                    if (miss) {
                        wait = true;
                    } else {
#pragma unroll
                        for (int q = 0; q < DPT; ++q)
                            if ((open >> q) & 1u) {
                                excl[q] += w[t][q] & LB_MASK;
                                if ((w[t][q] & ~LB_MASK) == LB_PREFIX) open &= ~(1u << q);
                            }
                        ++used;
                    }
                }
            }
            if (!open) break;
            p -= used;
            if (wait && ++spins > SPIN_LIMIT) {
                atomicOr(status, RT_DEV_TIMEOUT);
                break;
            }
        }
#pragma unroll
        for (int q = 0; q < DPT; ++q) st_relaxed(my + q, LB_PREFIX | (excl[q] + cnt[q]));
    }
    RT_SORT_MARK(3);
    uint32_t h[DPT], hsum = 0;
#pragma unroll
    for (int q = 0; q < DPT; ++q) {
        h[q] = hsum;
        hsum += __ldg(&hist[dgt0 + q]);
    }
    const uint32_t gbase = block_excl_scan_256(hsum, S.scan);
#pragma unroll
    for (int q = 0; q < DPT; ++q) S.goff[dgt0 + q] = gbase + h[q] + excl[q] - lstart[q];
    __syncthreads();
    RT_SORT_MARK(4);
    const uint32_t valid_n = (uint32_t)min((size_t)(SORT_THREADS * ITEMS), (size_t)n - base);
    for (uint32_t i = tid; i < valid_n; i += SORT_THREADS) {
        const uint32_t key = S.keys[i];
        const uint32_t d = (key >> shift) & DMASK;
        const uint32_t dst = S.goff[d] + i;
        if (dst < n) {   // always, unless a wait gave up (RT_DEV_TIMEOUT)
            kout[dst] = key;
            vout[dst] = S.vals[i];
        }
    }
    __syncthreads();   // the shared buffers are reused by the next tile
#if RT_SORT_VEC_LOADS == 2
    if (vec && tid == 0) mbar_inval(&S.bar);
#endif
    RT_SORT_MARK(5);
}

// rearrange_indices / rearrange_map (bvh-builder.cl:49-72) of sorted slot i,
// plus the traversal's triangle record; returns the triangle's AABB
// (build_leaf_bbox's min / max of the three vertices).
struct PermuteIO {
    const uint32_t* vals;       // sorted slot -> triangle in the order before the build
    const uint32_t* idx_old;
    const uint32_t* map_old;
    const uint32_t* orig_old;
    const float4* pos;
    uint32_t* idx_new;
    uint32_t* map_new;
    uint32_t* orig_new;
    float4* tris;
};

__device__ __forceinline__ void permute_tri(uint32_t i, const PermuteIO& P, float4& lo, float4& hi) {
    const uint32_t o = __ldg(&P.vals[i]);
    const uint32_t a = __ldg(&P.idx_old[3 * (size_t)o]), b = __ldg(&P.idx_old[3 * (size_t)o + 1]),
                   c = __ldg(&P.idx_old[3 * (size_t)o + 2]);
    P.idx_new[3 * (size_t)i] = a;
    P.idx_new[3 * (size_t)i + 1] = b;
    P.idx_new[3 * (size_t)i + 2] = c;
    P.map_new[i] = __ldg(&P.map_old[o]);
    P.orig_new[i] = __ldg(&P.orig_old[o]);
    const float4 p0 = __ldg(&P.pos[a]), p1 = __ldg(&P.pos[b]), p2 = __ldg(&P.pos[c]);
    P.tris[3 * (size_t)i] = make_float4(p0.x, p0.y, p0.z, 0.f);
    P.tris[3 * (size_t)i + 1] = make_float4(p1.x - p0.x, p1.y - p0.y, p1.z - p0.z, 0.f);
    P.tris[3 * (size_t)i + 2] = make_float4(p2.x - p0.x, p2.y - p0.y, p2.z - p0.z, 0.f);
    hi.x = fmaxf(fmaxf(p0.x, p1.x), p2.x);
    hi.y = fmaxf(fmaxf(p0.y, p1.y), p2.y);
    hi.z = fmaxf(fmaxf(p0.z, p1.z), p2.z);
    lo.x = fminf(fminf(p0.x, p1.x), p2.x);
    lo.y = fminf(fminf(p0.y, p1.y), p2.y);
    lo.z = fminf(fminf(p0.z, p1.z), p2.z);
    lo.w = hi.w = 0.f;
}

// permute_tri with the leaf AABB stored for a later emit (the many-scene
// build and any caller of k_permute).
__device__ __forceinline__ void permute_one(uint32_t i, const PermuteIO& P,
                                            float4* __restrict__ leafbox) {
    float4 lo, hi;
    permute_tri(i, P, lo, hi);
    leafbox[2 * (size_t)i] = lo;
    leafbox[2 * (size_t)i + 1] = hi;
}

// delta(i): highest differing bit between sorted keys i and i+1, with the
// index appended so that equal keys still order (Karras' augmentation).
__device__ __forceinline__ uint64_t delta(const uint32_t* __restrict__ k, uint32_t i) {
    const uint32_t x = __ldg(&k[i]) ^ __ldg(&k[i + 1]);
    return ((uint64_t)x << 32) | (uint64_t)(i ^ (i + 1));
}


// ---------------------------------------------------------------------------
// Multi-level emit + refit, warp-synchronous.  The tree is built bottom-up
// in a few launches ("levels").  Within a block, runs of consecutive items
// are joined by warps: a warp holds up to 32 consecutive items, one per lane
// (at level 0 the items are the sorted triangles).  warp_join writes in one
// step every node whose range lies inside the warp's items: the levels of
// the boundaries between items, as seven ballots, give each node's range and
// parent, and sparse tables in shared memory give its children's boxes.  A
// run whose parent lies outside the warp's items is left over; the block
// gathers the leftovers of its warps in order and joins them again, at most
// 32 per warp, until one warp holds them all or no node inside the block is
// left.  What is left then has its parent outside the block and becomes an
// item of the next level, which gathers the items of EMIT_GROUP blocks,
// until one block reaches the root.  A block leaves at most EMIT_FMAX items:
// they hang off the chains of nodes crossing its two ends, each at most 64
// deep (32 key bits + 32 index bits).
//
// The tree is the binary radix tree of the sorted keys (Karras), collapsed
// to the reference's leaf rule: a node [L, R] is an interior node of the
// reference's tree iff R - L + 1 >= min_leaf + 3 (find_middle's unsigned test
// last - first - 1 <= min_leaf, bvh-builder.cl:501) and its keys are not all
// equal (the bit loop of :515-525); otherwise it is a leaf, or part of one.
// The reference's split (highest differing bit, first index with the bit
// set) is the radix tree's split, so both trees have the same ranges.  With
// d[j] the augmented delta of the boundary before item j of a chunk and d[c]
// the boundary after its last item (D(-1) = D(n-1) = max), a run j..b is a
// left child iff d[b+1] < d[j];
// its parent stays in the chunk iff max d[b+2..c] > d[b+1] (the parent's
// range ends at the first boundary above d[b+1]); a right child's parent
// stays iff max d[0..j-1] > d[j].  Above the leftovers of a chunk, the
// boundaries between consecutive items are exactly the splits of the
// remaining nodes (a node's inner boundaries all lie below its end
// boundaries), so chunks and levels compose.
// ---------------------------------------------------------------------------
constexpr int EMIT_FMAX = 128;   // items a block may leave
#ifndef RT_EMIT_GROUP
#define RT_EMIT_GROUP 8
#endif
constexpr int EMIT_GROUP = RT_EMIT_GROUP;   // blocks of one level gathered by a block of the next

#ifndef RT_EMIT_C0
#define RT_EMIT_C0 512
#endif
#ifndef RT_EMIT_MINB0
#define RT_EMIT_MINB0 3
#endif
#ifndef RT_EMIT_MINB1
#define RT_EMIT_MINB1 1
#endif
#ifndef RT_EMIT_LEAVE0
#define RT_EMIT_LEAVE0 128u   // runs a level-0 block may leave unjoined
#endif
#ifndef RT_EMIT_LEAVE1
#define RT_EMIT_LEAVE1 64u    // the same above level 0
#endif
constexpr int EMIT_C0 = RT_EMIT_C0;                // triangles per level-0 block
constexpr int EMIT_C1 = EMIT_GROUP * EMIT_FMAX;    // items per block above level 0

// Blocks of level 0 of an n-triangle scene, and of the level above nb blocks.
__host__ __device__ __forceinline__ uint32_t emit_blocks0(uint32_t n) {
    return (n + EMIT_C0 - 1) / EMIT_C0;
}
__host__ __device__ __forceinline__ uint32_t emit_next_level(uint32_t nb) {
    return (nb + EMIT_GROUP - 1) / EMIT_GROUP;
}
// Runs a block of a level with `blocks` blocks may leave unjoined (a level of
// one block is the root's and joins everything).
__host__ __device__ __forceinline__ uint32_t emit_leave(int level, uint32_t blocks) {
    return blocks > 1 ? (level == 0 ? RT_EMIT_LEAVE0 : RT_EMIT_LEAVE1) : 32u;
}

// An item: leaf range, keys at its ends, box, ref / count, and the augmented
// delta of the boundary before it.
struct __align__(16) EmitItem {
    uint32_t l, r, kl, kr;
    float lo[3], hi[3];
    int32_t ref, cnt;
    uint64_t db;
    uint32_t pad[2];
};

// A scene's emit items in its emit scratch `base`: level 0 writes buffer A,
// level 1 B, level 2 A, ...; A holds up to EMIT_FMAX items per level-0 block,
// B per level-1 block, then the item counts of A and of B.
struct EmitBuffers {
    EmitItem* items[2];
    uint32_t* counts[2];
};
__host__ __device__ __forceinline__ EmitBuffers emit_buffers(uint32_t n, uint8_t* base) {
    const uint32_t nb0 = emit_blocks0(n), nb1 = emit_next_level(nb0);
    EmitBuffers b;
    b.items[0] = reinterpret_cast<EmitItem*>(base);
    b.items[1] = b.items[0] + (size_t)nb0 * EMIT_FMAX;
    b.counts[0] = reinterpret_cast<uint32_t*>(b.items[1] + (size_t)nb1 * EMIT_FMAX);
    b.counts[1] = b.counts[0] + nb0;
    return b;
}
__host__ __device__ __forceinline__ size_t emit_buffers_bytes(uint32_t n) {
    const size_t blocks = (size_t)emit_blocks0(n) + emit_next_level(emit_blocks0(n));
    return blocks * EMIT_FMAX * sizeof(EmitItem) + ((blocks * sizeof(uint32_t) + 255) & ~(size_t)255);
}

struct WarpItem {
    uint32_t l, r, kl, kr;
    float lox, loy, loz, hix, hiy, hiz;
    int32_t ref, cnt;
    uint64_t db;
};

__device__ __forceinline__ uint64_t delta_or_max(const uint32_t* __restrict__ k, int64_t i,
                                                 uint32_t n) {
    return (i < 0 || i >= (int64_t)n - 1) ? ~0ull : delta(k, (uint32_t)i);
}

__device__ __forceinline__ void item_to_reg(const EmitItem& e, WarpItem& w) {
    w.l = e.l; w.r = e.r; w.kl = e.kl; w.kr = e.kr;
    w.lox = e.lo[0]; w.loy = e.lo[1]; w.loz = e.lo[2];
    w.hix = e.hi[0]; w.hiy = e.hi[1]; w.hiz = e.hi[2];
    w.ref = e.ref; w.cnt = e.cnt; w.db = e.db;
}

__device__ __forceinline__ void reg_to_item(const WarpItem& w, EmitItem& e) {
    e.l = w.l; e.r = w.r; e.kl = w.kl; e.kr = w.kr;
    e.lo[0] = w.lox; e.lo[1] = w.loy; e.lo[2] = w.loz;
    e.hi[0] = w.hix; e.hi[1] = w.hiy; e.hi[2] = w.hiz;
    e.ref = w.ref; e.cnt = w.cnt; e.db = w.db;
}

// Shared scratch of one warp for warp_join, 2048 bytes: the space of the 32
// list items the warp's chunk takes.  st is a sparse table of one axis of
// the items' boxes (level t at start i: min / max over items i .. i+2^t-1);
// the arrays hold the items' ranges, end keys and references.  At the end
// the first 1536 bytes hand the runs left over to the lanes they start at.
struct __align__(16) WarpScratch {
    float2 st[5][32];
    uint32_t il[32], ir[32], ikl[32], ikr[32];
    int32_t iref[32], icnt[32];
};
static_assert(sizeof(WarpScratch) == 32 * sizeof(EmitItem), "scratch aliases 32 items");

// Level of a boundary delta: its highest set bit (the radix tree's level),
// 64 for the virtual boundaries before the first and after the last
// triangle.  Two boundaries of one level always have a higher one between
// them, so the nearest boundary above another one is the same by level as
// by delta, and levels order every pair of boundaries the tree compares.
__device__ __forceinline__ uint32_t delta_level(uint64_t x) {
    return x == ~0ull ? 64u : 63u - (uint32_t)__clzll(x);
}

// Lanes of `valid` whose level (bit planes P, most significant last) is
// above L.
__device__ __forceinline__ uint32_t levels_above(uint32_t L, const uint32_t P[7], uint32_t valid) {
    uint32_t gt = 0u, eq = valid;
#pragma unroll
    for (int t = 6; t >= 0; --t) {
        if ((L >> t) & 1u) {
            eq &= P[t];
        } else {
            gt |= eq & P[t];
            eq &= ~P[t];
        }
    }
    return gt;
}

__device__ __forceinline__ uint32_t level_at(uint32_t k, const uint32_t P[7]) {
    uint32_t L = 0u;
#pragma unroll
    for (int t = 0; t < 7; ++t) L |= ((P[t] >> k) & 1u) << t;
    return L;
}

// The lane of the highest boundary in the non-empty mask m (unique: two of
// one level have a higher one between them).
__device__ __forceinline__ uint32_t top_level(uint32_t m, const uint32_t P[7]) {
#pragma unroll
    for (int t = 6; t >= 0; --t) {
        const uint32_t c = m & P[t];
        if (c) m = c;
    }
    return (uint32_t)__ffs(m) - 1u;
}

// min / max of one axis over items a..b (a <= b, b - a < 31) from the table.
__device__ __forceinline__ float2 axis_range(const WarpScratch& W, uint32_t a, uint32_t b) {
    const uint32_t t = 31u - (uint32_t)__clz(b - a + 1u);
    const float2 u = W.st[t][a], v = W.st[t][b + 1u - (1u << t)];
    return make_float2(fminf(u.x, v.x), fmaxf(u.y, v.y));
}

// Joins the items of lanes 0..cnt-1 of the warp (all 32 lanes call it):
// every node whose range lies inside these items is written out, and the
// runs left over (maximal subtrees whose parent lies outside) stay, each in
// the lane of its first item (true for those lanes, `it` holding the run); a
// run that reaches [0, n-1] writes the header instead.  `edge` is the
// boundary after the last item.  With d[j] the boundary before item j, the
// node split at boundary j spans from the nearest higher boundary on its
// left to the one on its right, and its parent is split at the lower of
// those two.  All of it comes from bit planes of the boundary levels, with
// no rounds; the children's boxes come from sparse tables of the item boxes.
// fminf / fmaxf order -0 below +0 and skip NaN whatever the operand order,
// so any grouping of a range gives the bits of the bottom-up merge.
__device__ __forceinline__ bool warp_join(WarpItem& it, uint32_t cnt, uint64_t edge, uint32_t n,
                                          int min_leaf, float4* __restrict__ nodes,
                                          WarpScratch& W, BvhHeader* __restrict__ hdr) {
    const uint32_t lane = threadIdx.x & 31u;
    const unsigned FULL = 0xffffffffu;
    if (cnt == 0u) return false;
    const bool item = lane < cnt;
    __syncwarp();   // the lanes have read their items out of this space
    if (item) {
        W.il[lane] = it.l;
        W.ir[lane] = it.r;
        W.ikl[lane] = it.kl;
        W.ikr[lane] = it.kr;
        W.iref[lane] = it.ref;
        W.icnt[lane] = it.cnt;
    }
    // --- topology, from the levels of the boundaries
    // the node split at boundary j = lane (1 <= j < cnt), when it lies
    // inside: left child items A..j-1 (split at lsplit's right end), right
    // child j..B (split at rsplit's)
    bool local = false, out = false;
    uint32_t A = lane, B = lane, lsplit = 0u, rsplit = 0u;
    {
        const uint32_t lev = item ? delta_level(it.db) : 0u;
        uint32_t P[7];
#pragma unroll
        for (int t = 0; t < 7; ++t) P[t] = __ballot_sync(FULL, item && ((lev >> t) & 1u));
        const uint32_t valid = cnt >= 32u ? FULL : ((1u << cnt) - 1u);
        const uint32_t edge_lev = delta_level(edge);
        if (item && lane >= 1u) {
            const uint32_t gt = levels_above(lev, P, valid);
            const uint32_t lm = gt & ((1u << lane) - 1u);
            const uint32_t rm = gt & ~((2u << lane) - 1u);
            if (lm != 0u && (rm != 0u || edge_lev > lev)) {
                local = true;
                A = 31u - (uint32_t)__clz(lm);
                B = rm ? (uint32_t)__ffs(rm) - 2u : cnt - 1u;
                const uint32_t lin = ((1u << lane) - 1u) & ~((2u << A) - 1u);   // A+1..j-1
                const uint32_t rin = ((2u << B) - 1u) & ~((2u << lane) - 1u);   // j+1..B
                lsplit = lin ? top_level(lin, P) - 1u : 0u;
                rsplit = rin ? top_level(rin, P) - 1u : 0u;
            }
        }
        const uint32_t LM = __ballot_sync(FULL, local);
        // the part of this lane whose parent may lie outside (items A..B:
        // its node if local, else its item) and whether it does
        if (item) {
            const uint32_t la = level_at(A, P);
            const uint32_t lb = B + 1u < cnt ? level_at(B + 1u, P) : edge_lev;
            const uint32_t p = lb < la ? B + 1u : A;   // the parent's split
            out = p == 0u || p >= cnt || !((LM >> p) & 1u);
        }
    }
    // --- boxes: the children's for a local node, the item's otherwise
    float llo[3], lhi[3], rlo[3], rhi[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float vlo = k == 0 ? it.lox : (k == 1 ? it.loy : it.loz);
        const float vhi = k == 0 ? it.hix : (k == 1 ? it.hiy : it.hiz);
        __syncwarp();   // the previous axis' queries are done
        if (item) W.st[0][lane] = make_float2(vlo, vhi);
#pragma unroll
        for (int t = 1; t < 5; ++t) {
            __syncwarp();
            const uint32_t h = 1u << (t - 1);
            if (lane + 2u * h <= cnt) {
                const float2 u = W.st[t - 1][lane], v = W.st[t - 1][lane + h];
                W.st[t][lane] = make_float2(fminf(u.x, v.x), fmaxf(u.y, v.y));
            }
        }
        __syncwarp();
        llo[k] = vlo;
        lhi[k] = vhi;
        rlo[k] = vlo;
        rhi[k] = vhi;
        if (local) {
            const float2 l = axis_range(W, A, lane - 1u), r = axis_range(W, lane, B);
            llo[k] = l.x; lhi[k] = l.y;
            rlo[k] = r.x; rhi[k] = r.y;
        }
    }
    // reference and leaf count of items a..b as one node (split at the
    // right end of item `split`) or as the item itself
    auto ref_of = [&](uint32_t a, uint32_t b, uint32_t split, int32_t& ref, int32_t& c) {
        if (a == b) {
            ref = W.iref[a];
            c = W.icnt[a];
            return;
        }
        const uint32_t L = W.il[a], count = W.ir[b] - L + 1u;
        const bool interior = count >= (uint32_t)min_leaf + 3u && W.ikl[a] != W.ikr[b];
        ref = interior ? (int32_t)W.ir[split] : (int32_t)L;
        c = interior ? 0 : (int32_t)count;
    };
    if (local) {
        int32_t lref, lcnt, rref, rcnt;
        ref_of(A, lane - 1u, lsplit, lref, lcnt);
        ref_of(lane, B, rsplit, rref, rcnt);
        float4* np = nodes + 4 * (size_t)W.ir[lane - 1u];
        np[0] = make_float4(llo[0], llo[1], llo[2], lhi[0]);
        np[1] = make_float4(lhi[1], lhi[2], rlo[0], rlo[1]);
        np[2] = make_float4(rlo[2], rhi[0], rhi[1], rhi[2]);
        np[3] = make_float4(__int_as_float(lref), __int_as_float(rref), __int_as_float(lcnt),
                            __int_as_float(rcnt));
    }
    float4 q0, q1, q2;
    if (out) {
        int32_t eref, ecnt;
        ref_of(A, B, lane - 1u, eref, ecnt);
        const float lx = local ? fminf(llo[0], rlo[0]) : llo[0],
                    ly = local ? fminf(llo[1], rlo[1]) : llo[1],
                    lz = local ? fminf(llo[2], rlo[2]) : llo[2];
        const float hx = local ? fmaxf(lhi[0], rhi[0]) : lhi[0],
                    hy = local ? fmaxf(lhi[1], rhi[1]) : lhi[1],
                    hz = local ? fmaxf(lhi[2], rhi[2]) : lhi[2];
        const uint32_t gl = W.il[A], gr = W.ir[B];
        if (gl == 0u && gr == n - 1u) {   // the root
            hdr->root_ref = eref;
            hdr->root_cnt = ecnt;
            hdr->n_tris = n;
            hdr->root_lo = make_float4(lx, ly, lz, 0.f);
            hdr->root_hi = make_float4(hx, hy, hz, 0.f);
            out = false;
        }
        q0 = make_float4(__uint_as_float(gl), __uint_as_float(gr), __uint_as_float(W.ikl[A]),
                         __uint_as_float(W.ikr[B]));
        q1 = make_float4(lx, ly, lz, hx);
        q2 = make_float4(hy, hz, __int_as_float(eref), __int_as_float(ecnt));
    }
    // hand each run left over to the lane of its first item
    const uint32_t keep = __reduce_or_sync(FULL, out ? (1u << A) : 0u);
    float4* stage = reinterpret_cast<float4*>(&W);
    __syncwarp();   // every read of the scratch is done
    if (out) {
        stage[A] = q0;
        stage[32 + A] = q1;
        stage[64 + A] = q2;
    }
    __syncwarp();
    const bool mine = (keep >> lane) & 1u;
    if (mine) {
        q0 = stage[lane];
        q1 = stage[32 + lane];
        q2 = stage[64 + lane];
        it.l = __float_as_uint(q0.x);
        it.r = __float_as_uint(q0.y);
        it.kl = __float_as_uint(q0.z);
        it.kr = __float_as_uint(q0.w);
        it.lox = q1.x; it.loy = q1.y; it.loz = q1.z; it.hix = q1.w;
        it.hiy = q2.x; it.hiz = q2.y;
        it.ref = __float_as_int(q2.z);
        it.cnt = __float_as_int(q2.w);   // it.db stays: the run starts at this lane
    }
    __syncwarp();   // the staged runs are read before the space is reused
    return mine;
}

// Shared state of one emit block: the items left over by its warps, in order.
template <int C>
struct EmitSmem {
    union {
        EmitItem list[C];
        WarpScratch scratch[C / 32];   // warp w's: list[32w .. 32w+31]
    };
    uint32_t wcount[C / 32], woff[C / 32 + 1];
    uint64_t edge;   // boundary after the block's last item
};

// Gathers, in order, the runs still held by the warps' lanes into S.list and
// returns their number.  Call with all C threads; `keep` marks held runs.
template <int C>
__device__ __forceinline__ uint32_t gather_runs(EmitSmem<C>& S, const WarpItem& it, bool keep) {
    const uint32_t lane = threadIdx.x & 31u, w = threadIdx.x >> 5;
    const unsigned bal = __ballot_sync(0xffffffffu, keep);
    if (lane == 0) S.wcount[w] = __popc(bal);
    __syncthreads();   // also: every warp has read its chunk of S.list
    if (w == 0) {
        const uint32_t v = lane < (uint32_t)(C / 32) ? S.wcount[lane] : 0u;
        uint32_t x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t u = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= (uint32_t)o) x += u;
        }
        if (lane < (uint32_t)(C / 32)) S.woff[lane] = x - v;
        if (lane == 31) S.woff[C / 32] = x;
    }
    __syncthreads();
    if (keep) reg_to_item(it, S.list[S.woff[w] + __popc(bal & ((1u << lane) - 1u))]);
    const uint32_t m = S.woff[C / 32];
    __syncthreads();
    return m;
}

// One level of the emit for block `blk` (C threads = C / 32 warps).  Level 0
// (in == null): the items are triangles blk*C .. blk*C+C-1; otherwise the
// items left by blocks blk*EMIT_GROUP .. of the previous level (in_count[k]
// items at in[k * EMIT_FMAX]).  Leaves the block's own items at
// out[blk * EMIT_FMAX] and their number in out_count[blk].  The block stops
// joining once `leave` runs or fewer are left (leave <= EMIT_FMAX; 32: join
// down to one warp's runs, as the root's level must).
//
// With PERMUTE, level 0 performs the permutation of its own triangles
// (permute_tri with `perm`) and keeps their boxes in registers; `leafbox` is
// then unused.
template <int C, bool PERMUTE = false>
__device__ __forceinline__ void emit_level(EmitSmem<C>& S, uint32_t blk, uint32_t n,
                                           const uint32_t* __restrict__ skeys,
                                           const float4* __restrict__ leafbox,
                                           const EmitItem* __restrict__ in,
                                           const uint32_t* __restrict__ in_count,
                                           uint32_t n_in, EmitItem* __restrict__ out,
                                           uint32_t* __restrict__ out_count,
                                           float4* __restrict__ nodes, int min_leaf,
                                           uint32_t leave, BvhHeader* __restrict__ hdr,
                                           uint32_t* __restrict__ status,
                                           const PermuteIO& perm = PermuteIO{}) {
    static_assert(C % 32 == 0 && C >= EMIT_FMAX, "block size");
    const uint32_t t = threadIdx.x, lane = t & 31u, w = t >> 5;
    WarpItem it;
    bool keep;
    uint32_t m;
    if (!in) {
        // level 0: warp w joins triangles b0 + 32w ..
        const uint32_t b0 = blk * (uint32_t)C, i = b0 + t;
        const uint32_t w0 = b0 + 32u * w;
        const uint32_t cnt = w0 < n ? min(32u, n - w0) : 0u;
        const bool have = i < n;
        const uint32_t k = have ? __ldg(&skeys[i]) : 0u;
        uint32_t kprev = __shfl_up_sync(0xffffffffu, k, 1);
        if (lane == 0 && have && i > 0) kprev = __ldg(&skeys[i - 1]);
        it.l = it.r = i;
        it.kl = it.kr = k;
        it.db = (!have || i == 0) ? ~0ull
                                  : (((uint64_t)(kprev ^ k) << 32) | (uint64_t)((i - 1) ^ i));
        float4 lo = make_float4(0.f, 0.f, 0.f, 0.f), hi = lo;
        if (have) {
            if constexpr (PERMUTE) {
                permute_tri(i, perm, lo, hi);
            } else {
                lo = leafbox[2 * (size_t)i];
                hi = leafbox[2 * (size_t)i + 1];
            }
        }
        it.lox = lo.x; it.loy = lo.y; it.loz = lo.z;
        it.hix = hi.x; it.hiy = hi.y; it.hiz = hi.z;
        it.ref = (int32_t)i;
        it.cnt = 1;
        const uint64_t edge = cnt ? delta_or_max(skeys, (int64_t)w0 + cnt - 1, n) : 0ull;
        if (n == 1) {
            if (t == 0) {
                hdr->root_ref = 0;
                hdr->root_cnt = 1;
                hdr->n_tris = 1;
                hdr->root_lo = lo;
                hdr->root_hi = hi;
            }
            if (t == 0 && out_count) out_count[blk] = 0;
            return;
        }
        if (t == 0) S.edge = delta_or_max(skeys, (int64_t)min(b0 + (uint32_t)C, n) - 1, n);
        keep = warp_join(it, cnt, edge, n, min_leaf, nodes, S.scratch[w], hdr);
        m = gather_runs<C>(S, it, keep);
    } else {
        // the items left by EMIT_GROUP blocks of the previous level, in order
        if (w == 0) {
            const uint32_t k = blk * EMIT_GROUP + lane;
            const uint32_t v = (lane < (uint32_t)EMIT_GROUP && k < n_in)
                                   ? min(__ldg(&in_count[k]), (uint32_t)EMIT_FMAX) : 0u;
            uint32_t x = v;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t u = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= (uint32_t)o) x += u;
            }
            if (lane < (uint32_t)EMIT_GROUP) S.woff[lane] = x - v;
            if (lane == 31) S.woff[EMIT_GROUP] = x;
        }
        __syncthreads();
        m = S.woff[EMIT_GROUP];
        for (uint32_t e = t; e < m; e += C) {
            int g = 0;
            while (g + 1 < EMIT_GROUP && S.woff[g + 1] <= e) ++g;
            S.list[e] = in[(size_t)(blk * EMIT_GROUP + g) * EMIT_FMAX + (e - S.woff[g])];
        }
        __syncthreads();   // the last item may have been copied by another thread
        if (t == 0 && m) S.edge = delta_or_max(skeys, (int64_t)S.list[m - 1].r, n);
        __syncthreads();
    }
    // Join the gathered runs in chunks of at most 32, one chunk per warp,
    // until one warp holds them all or none can be joined inside the block.
    // A pass joins only nodes that lie inside one chunk, so passes alternate
    // between chunks aligned at multiples of 32 and chunks shifted by 16: if
    // a node inside the block is left, so is one whose two children are
    // adjacent runs, and those share a chunk in one of the two layouts.  Two
    // passes in a row without a join therefore mean that every run left has
    // its parent outside the block.
    uint32_t stalls = 0;
    for (uint32_t pass = 0;; ++pass) {
        if (m <= leave && leave > 32u) {
            // few enough to be items of the next level as they are: the
            // next level joins them (a block's passes get longer and emptier
            // as its runs thin out)
            for (uint32_t e = t; e < m; e += (uint32_t)C) out[(size_t)blk * EMIT_FMAX + e] = S.list[e];
            if (t == 0 && out_count) out_count[blk] = m;
            return;
        }
        if (m <= 32u) {
            if (w == 0) {
                const uint32_t cnt = m;
                if (lane < cnt) item_to_reg(S.list[lane], it);
                keep = warp_join(it, cnt, S.edge, n, min_leaf, nodes, S.scratch[0], hdr);
                const unsigned bal = __ballot_sync(0xffffffffu, keep);
                if (keep) reg_to_item(it, out[(size_t)blk * EMIT_FMAX + __popc(bal & ((1u << lane) - 1u))]);
                if (lane == 0 && out_count) out_count[blk] = __popc(bal);
            }
            return;
        }
        if (stalls >= 2u || pass >= 2u * (uint32_t)C + 4u) {
            if (stalls < 2u && t == 0) atomicOr(status, RT_DEV_BADINDEX);
            // every run left has its parent outside the block: all of them,
            // in order, are items of the next level
            const uint32_t nf = min(m, (uint32_t)EMIT_FMAX);
            for (uint32_t e = t; e < nf; e += (uint32_t)C) out[(size_t)blk * EMIT_FMAX + e] = S.list[e];
            if (t == 0) {
                if (m > (uint32_t)EMIT_FMAX) atomicOr(status, RT_DEV_OVERFLOW);
                if (out_count) out_count[blk] = nf;
            }
            return;
        }
        // chunk w is [0, off) for w == 0, else [off + 32(w-1), off + 32w)
        const uint32_t off = ((pass & 1u) && m + 16u <= (uint32_t)C) ? 16u : 32u;
        const uint32_t c0 = w == 0 ? 0u : off + 32u * (w - 1u);
        const uint32_t c1 = min(m, off + 32u * w);
        const uint32_t cnt = c0 < m ? c1 - c0 : 0u;
        if (lane < cnt) item_to_reg(S.list[c0 + lane], it);
        const uint64_t edge = c1 < m ? S.list[c1].db : S.edge;
        __syncthreads();   // the chunks are read: the list space becomes the warps' scratch
        keep = warp_join(it, cnt, edge, n, min_leaf, nodes, S.scratch[w], hdr);
        const uint32_t m_new = gather_runs<C>(S, it, keep);
        stalls = m_new == m ? stalls + 1u : 0u;
        m = m_new;
    }
}


}  // namespace rt
