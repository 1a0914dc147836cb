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

constexpr int SORT_THREADS = 256;
constexpr int SORT_WARPS = SORT_THREADS / 32;
constexpr int SORT_ITEMS = 16;
constexpr int SORT_TILE = SORT_THREADS * SORT_ITEMS;   // 4096 keys per tile
constexpr uint32_t LB_AGG = 1u << 30, LB_PREFIX = 2u << 30, LB_MASK = (1u << 30) - 1;
constexpr uint32_t LB_SPIN_LIMIT = 1u << 22;

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

__device__ __forceinline__ uint32_t ld_acquire(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(uint32_t* p, uint32_t v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
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

__device__ __forceinline__ uint32_t morton_code(const MortonParams& P, const float lo[3],
                                                const float hi[3]) {
    uint32_t m[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float center = (hi[k] + lo[k]) * 0.5f;
        float slice = (center - P.glo[k]) * P.inv[k];
        slice = fmaxf(0.0f, fminf(1.0f, slice));
        slice *= P.scale;
        m[k] = (uint32_t)slice;   // truncation; slice == 2^k keeps only out-of-range bits
    }
    uint32_t code = 0;
    int axis = (P.offset + 1) % 3;
#pragma unroll
    for (int bit = 0; bit < 32; ++bit) {
        if (bit < P.depth) {
            const int src = (bit + P.offset) / 3;
            const uint32_t mv = axis == 0 ? m[0] : (axis == 1 ? m[1] : m[2]);
            code |= ((mv >> src) & 1u) << bit;
            axis = axis == 2 ? 0 : axis + 1;
        }
    }
    return code;
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

template <int ITEMS>
struct SortSmemT {
    uint32_t keys[SORT_THREADS * ITEMS];
    uint32_t vals[SORT_THREADS * ITEMS];
    uint32_t whist[SORT_WARPS][256];
    uint32_t goff[256];
    uint32_t lstart[256];
    uint32_t scan[SORT_WARPS];
    uint32_t tile;
};
using SortSmem = SortSmemT<SORT_ITEMS>;

// One tile of a stable LSD radix pass (8-bit digit at `shift`): warp-striped
// loads, __match_any_sync ranking in index order, decoupled look-back over
// the earlier tiles of the same sequence, shared-memory staging and a
// coalesced scatter.  Must be called by all SORT_THREADS threads of a block;
// a tile holds SORT_THREADS * ITEMS keys.
template <int ITEMS = SORT_ITEMS>
__device__ __forceinline__ void onesweep_tile(SortSmemT<ITEMS>& S, uint32_t tile,
                                              const uint32_t* __restrict__ kin,
                                              const uint32_t* __restrict__ vin,
                                              uint32_t* __restrict__ kout,
                                              uint32_t* __restrict__ vout, uint32_t n, int shift,
                                              const uint32_t* __restrict__ hist,
                                              uint32_t* __restrict__ lookback,
                                              uint32_t* __restrict__ status) {
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    for (int i = tid; i < SORT_WARPS * 256; i += SORT_THREADS) (&S.whist[0][0])[i] = 0;
    __syncthreads();
    const size_t base = (size_t)tile * (SORT_THREADS * ITEMS);
    const uint32_t lanemask_lt = (1u << lane) - 1u;

    uint32_t k[ITEMS], v[ITEMS], rank[ITEMS];
#pragma unroll
    for (int j = 0; j < ITEMS; ++j) {
        const size_t g = base + (size_t)warp * (ITEMS * 32) + j * 32 + lane;
        const bool ok = g < n;
        k[j] = ok ? __ldcs(&kin[g]) : 0xffffffffu;
        v[j] = ok ? __ldcs(&vin[g]) : 0u;
    }
#pragma unroll
    for (int j = 0; j < ITEMS; ++j) {
        const size_t g = base + (size_t)warp * (ITEMS * 32) + j * 32 + lane;
        const bool ok = g < n;
        const uint32_t d = (k[j] >> shift) & 255u;
        const uint32_t valid = __ballot_sync(0xffffffffu, ok);
        uint32_t peers = 0, prev = 0;
        if (ok) {
            peers = __match_any_sync(valid, d);
            prev = S.whist[warp][d];
        }
        __syncwarp();
        if (ok) {
            rank[j] = prev + __popc(peers & lanemask_lt);
            const int leader = __ffs(peers) - 1;
            if (lane == leader) S.whist[warp][d] = prev + __popc(peers);
        }
        __syncwarp();
    }
    __syncthreads();

    const uint32_t dgt = tid;   // 256 threads <-> 256 digits
    uint32_t cnt = 0;
#pragma unroll
    for (int w = 0; w < SORT_WARPS; ++w) {
        const uint32_t c = S.whist[w][dgt];
        S.whist[w][dgt] = cnt;
        cnt += c;
    }
    uint32_t* my = &lookback[(size_t)tile * 256 + dgt];
    uint32_t excl = 0;
    if (tile == 0) {
        st_release(my, LB_PREFIX | cnt);
    } else {
        st_release(my, LB_AGG | cnt);
        int64_t p = (int64_t)tile - 1;
        uint32_t spins = 0;
        while (p >= 0) {
            const uint32_t s = ld_acquire(&lookback[(size_t)p * 256 + dgt]);
            const uint32_t flag = s & ~LB_MASK;
            if (flag == 0) {
                if (++spins > LB_SPIN_LIMIT) {
                    atomicOr(status, RT_DEV_TIMEOUT);
                    break;
                }
                continue;
            }
            excl += s & LB_MASK;
            if (flag == LB_PREFIX) break;
            --p;
        }
        st_release(my, LB_PREFIX | (excl + cnt));
    }
    const uint32_t gstart = block_excl_scan_256(__ldg(&hist[dgt]), S.scan);
    const uint32_t lstart = block_excl_scan_256(cnt, S.scan);
    S.goff[dgt] = gstart + excl - lstart;
    S.lstart[dgt] = lstart;
    __syncthreads();
#pragma unroll
    for (int j = 0; j < ITEMS; ++j) {
        const size_t g = base + (size_t)warp * (ITEMS * 32) + j * 32 + lane;
        if (g < n) {
            const uint32_t d = (k[j] >> shift) & 255u;
            const uint32_t p = S.lstart[d] + S.whist[warp][d] + rank[j];
            S.keys[p] = k[j];
            S.vals[p] = v[j];
        }
    }
    __syncthreads();
    const uint32_t valid_n = (uint32_t)min((size_t)(SORT_THREADS * ITEMS), (size_t)n - base);
    for (uint32_t i = tid; i < valid_n; i += SORT_THREADS) {
        const uint32_t key = S.keys[i];
        const uint32_t d = (key >> shift) & 255u;
        const uint32_t dst = S.goff[d] + i;
        kout[dst] = key;
        vout[dst] = S.vals[i];
    }
    __syncthreads();   // the shared buffers are reused by the next tile
}

// rearrange_indices / rearrange_map (bvh-builder.cl:49-72) of sorted slot i,
// plus the traversal's triangle record and the leaf AABB.
__device__ __forceinline__ void permute_one(uint32_t i, const uint32_t* __restrict__ vals,
                                            const uint32_t* __restrict__ idx_old,
                                            const uint32_t* __restrict__ map_old,
                                            const uint32_t* __restrict__ orig_old,
                                            const float4* __restrict__ pos,
                                            uint32_t* __restrict__ idx_new,
                                            uint32_t* __restrict__ map_new,
                                            uint32_t* __restrict__ orig_new,
                                            float4* __restrict__ tris,
                                            float4* __restrict__ leafbox) {
    const uint32_t o = __ldg(&vals[i]);
    const uint32_t a = __ldg(&idx_old[3 * (size_t)o]), b = __ldg(&idx_old[3 * (size_t)o + 1]),
                   c = __ldg(&idx_old[3 * (size_t)o + 2]);
    idx_new[3 * (size_t)i] = a;
    idx_new[3 * (size_t)i + 1] = b;
    idx_new[3 * (size_t)i + 2] = c;
    map_new[i] = __ldg(&map_old[o]);
    orig_new[i] = __ldg(&orig_old[o]);
    const float4 p0 = __ldg(&pos[a]), p1 = __ldg(&pos[b]), p2 = __ldg(&pos[c]);
    tris[3 * (size_t)i] = make_float4(p0.x, p0.y, p0.z, 0.f);
    tris[3 * (size_t)i + 1] = make_float4(p1.x - p0.x, p1.y - p0.y, p1.z - p0.z, 0.f);
    tris[3 * (size_t)i + 2] = make_float4(p2.x - p0.x, p2.y - p0.y, p2.z - p0.z, 0.f);
    float4 lo, hi;
    hi.x = fmaxf(fmaxf(p0.x, p1.x), p2.x);
    hi.y = fmaxf(fmaxf(p0.y, p1.y), p2.y);
    hi.z = fmaxf(fmaxf(p0.z, p1.z), p2.z);
    lo.x = fminf(fminf(p0.x, p1.x), p2.x);
    lo.y = fminf(fminf(p0.y, p1.y), p2.y);
    lo.z = fminf(fminf(p0.z, p1.z), p2.z);
    lo.w = hi.w = 0.f;
    leafbox[2 * (size_t)i] = lo;
    leafbox[2 * (size_t)i + 1] = hi;
}

// delta(i): highest differing bit between sorted keys i and i+1, with the
// index appended so that equal keys still order (Karras' augmentation).
__device__ __forceinline__ uint64_t delta(const uint32_t* __restrict__ k, uint32_t i) {
    const uint32_t x = __ldg(&k[i]) ^ __ldg(&k[i + 1]);
    return ((uint64_t)x << 32) | (uint64_t)(i ^ (i + 1));
}

// Bottom-up emit + refit from sorted triangle i of an n-triangle scene: the
// thread climbs while it is the second child to arrive.  A radix-tree node
// [L, R] is an interior node of the reference's tree iff R - L + 1 >=
// min_leaf + 3 (find_middle's unsigned test last - first - 1 <= min_leaf,
// bvh-builder.cl:501) and its keys are not all equal (the bit loop of
// :515-525); otherwise it is a leaf, or part of one.  The reference's split
// (highest differing bit, first index with the bit set) is the radix tree's
// split, so both trees have the same ranges.
__device__ __forceinline__ void emit_climb(uint32_t i, uint32_t n,
                                           const uint32_t* __restrict__ skeys,
                                           const float4* __restrict__ leafbox,
                                           float4* __restrict__ nodes, uint32_t* __restrict__ flags,
                                           uint32_t* __restrict__ rangeL,
                                           uint32_t* __restrict__ rangeR, int min_leaf,
                                           BvhHeader* __restrict__ hdr) {
    float4 lo = leafbox[2 * (size_t)i], hi = leafbox[2 * (size_t)i + 1];
    if (n == 1) {
        hdr->root_ref = 0;
        hdr->root_cnt = 1;
        hdr->n_tris = 1;
        hdr->root_lo = lo;
        hdr->root_hi = hi;
        return;
    }
    uint32_t l = i, r = i;
    int32_t ref = (int32_t)i, cnt = 1;
    for (;;) {
        bool is_left;
        uint32_t p;
        if (l == 0 || (r != n - 1 && delta(skeys, r) < delta(skeys, l - 1))) {
            p = r;
            is_left = true;
        } else {
            p = l - 1;
            is_left = false;
        }
        float* rec = reinterpret_cast<float*>(nodes + 4 * (size_t)p);
        int* rec_i = reinterpret_cast<int*>(nodes + 4 * (size_t)p + 3);
        if (is_left) {
            nodes[4 * (size_t)p] = make_float4(lo.x, lo.y, lo.z, hi.x);
            *reinterpret_cast<float2*>(rec + 4) = make_float2(hi.y, hi.z);
            rec_i[0] = ref;
            rec_i[2] = cnt;
            rangeL[p] = l;
        } else {
            *reinterpret_cast<float2*>(rec + 6) = make_float2(lo.x, lo.y);
            nodes[4 * (size_t)p + 2] = make_float4(lo.z, hi.x, hi.y, hi.z);
            rec_i[1] = ref;
            rec_i[3] = cnt;
            rangeR[p] = r;
        }
        if (atomic_add_acq_rel(&flags[p], 1u) == 0) return;   // the sibling finishes p
        const float4 n0 = __ldcg(&nodes[4 * (size_t)p]);
        const float4 n1 = __ldcg(&nodes[4 * (size_t)p + 1]);
        const float4 n2 = __ldcg(&nodes[4 * (size_t)p + 2]);
        const uint32_t L = is_left ? l : __ldcg(&rangeL[p]);
        const uint32_t R = is_left ? __ldcg(&rangeR[p]) : r;
        // merge_bbox(left, right): lo = fmin(left.lo, right.lo), hi = fmax(...)
        lo = make_float4(fminf(n0.x, n1.z), fminf(n0.y, n1.w), fminf(n0.z, n2.x), 0.f);
        hi = make_float4(fmaxf(n0.w, n2.y), fmaxf(n1.x, n2.z), fmaxf(n1.y, n2.w), 0.f);
        const uint32_t count = R - L + 1;
        const bool interior =
            count >= (uint32_t)min_leaf + 3u && __ldg(&skeys[L]) != __ldg(&skeys[R]);
        if (interior) {
            ref = (int32_t)p;
            cnt = 0;
        } else {
            ref = (int32_t)L;
            cnt = (int32_t)count;
        }
        l = L;
        r = R;
        if (L == 0 && R == n - 1) {
            hdr->root_ref = ref;
            hdr->root_cnt = cnt;
            hdr->n_tris = n;
            hdr->root_lo = lo;
            hdr->root_hi = hi;
            return;
        }
    }
}

// ---------------------------------------------------------------------------
// Chunked emit + refit.  A block takes the C sorted triangles [b0, b1] and
// starts one climber per triangle, as emit_climb does.  While a climber's
// parent lies wholly inside the chunk, the node is assembled in shared memory
// (each child writes its half, as in emit_climb), the arrival counter is a
// shared atomic and the keys come from a shared copy, so that climb touches
// no global memory; the chunk's nodes are written out at the end with
// coalesced stores.  Only nodes whose range crosses a chunk boundary (about
// depth x n / C of them) use the global records and counters of emit_climb.
// The tree is the same: which climber finishes a node never changes it.
//
// Whether the parent stays inside is known before arriving.  With D(k) the
// augmented delta of boundary k (D(-1) = D(n-1) = max), a left child [l, r]
// has parent p = r whose range ends at the first k > r with D(k) > D(r), so
// the parent is inside iff max D(r+1..b1) > D(r); a right child's parent
// p = l-1 is inside iff max D(b0-1..l-2) > D(l-1).  Both children of a node
// get the same answer from the chunk's prefix and suffix maxima of D.
// ---------------------------------------------------------------------------
template <int C>
struct EmitSmem {
    uint64_t d[C + 1];     // D(b0 - 1 + j)
    uint64_t pre[C + 1];   // max D(b0 - 1 .. b0 - 1 + j)
    uint64_t suf[C + 1];   // max D(b0 - 1 + j .. b1)
    float4 node[C][4];     // nodes p = b0 + q, in the global layout
    uint32_t key[C];       // sorted keys b0..b1
    uint32_t bound[2][C];  // left child's l, right child's r
    uint32_t flag[C];      // arrivals at node b0 + q
};

__device__ __forceinline__ uint64_t delta_or_max(const uint32_t* __restrict__ k, int64_t i,
                                                 uint32_t n) {
    return (i < 0 || i >= (int64_t)n - 1) ? ~0ull : delta(k, (uint32_t)i);
}

// Inclusive max-scan over the block (C threads, one value each).
template <int C>
__device__ __forceinline__ uint64_t block_max_scan(uint64_t v, uint64_t* s_warp) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint64_t u = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v = v > u ? v : u;
    }
    if (lane == 31) s_warp[w] = v;
    __syncthreads();
    if (w == 0) {
        uint64_t x = lane < C / 32 ? s_warp[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint64_t u = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x = x > u ? x : u;
        }
        if (lane < C / 32) s_warp[lane] = x;
    }
    __syncthreads();
    if (w > 0) {
        const uint64_t u = s_warp[w - 1];
        v = v > u ? v : u;
    }
    __syncthreads();   // s_warp is reused by the next scan
    return v;
}

// One child's half of node record `rec` (the layout emit_climb writes).
__device__ __forceinline__ void write_half(float4* rec, bool is_left, float4 lo, float4 hi,
                                           int32_t ref, int32_t cnt) {
    float* f = reinterpret_cast<float*>(rec);
    int* ri = reinterpret_cast<int*>(rec + 3);
    if (is_left) {
        rec[0] = make_float4(lo.x, lo.y, lo.z, hi.x);
        *reinterpret_cast<float2*>(f + 4) = make_float2(hi.y, hi.z);
        ri[0] = ref;
        ri[2] = cnt;
    } else {
        *reinterpret_cast<float2*>(f + 6) = make_float2(lo.x, lo.y);
        rec[2] = make_float4(lo.z, hi.x, hi.y, hi.z);
        ri[1] = ref;
        ri[3] = cnt;
    }
}

template <int C>
__device__ __forceinline__ void emit_chunk(EmitSmem<C>& S, uint64_t* s_warp, uint32_t b0,
                                           uint32_t n, const uint32_t* __restrict__ skeys,
                                           const float4* __restrict__ leafbox,
                                           float4* __restrict__ nodes,
                                           uint32_t* __restrict__ flags,
                                           uint32_t* __restrict__ rangeL,
                                           uint32_t* __restrict__ rangeR, int min_leaf,
                                           BvhHeader* __restrict__ hdr,
                                           uint32_t* __restrict__ status) {
    const uint32_t t = threadIdx.x;
    const uint32_t b1 = min(b0 + (uint32_t)C - 1u, n - 1u);
    const uint32_t m = b1 - b0 + 1;   // D entries 0..m cover boundaries b0-1..b1
    // boundaries, their prefix maxima and (by a reversed scan) suffix maxima
    const uint64_t dt = t <= m ? delta_or_max(skeys, (int64_t)b0 - 1 + t, n) : 0ull;
    const uint64_t dC = m == (uint32_t)C ? delta_or_max(skeys, (int64_t)b0 - 1 + C, n) : 0ull;
    S.d[t] = dt;
    if (t == 0) S.d[C] = dC;
    S.flag[t] = 0;
    if (t < m) S.key[t] = __ldg(&skeys[b0 + t]);
    const uint64_t pf = block_max_scan<C>(dt, s_warp);
    S.pre[t] = pf;
    const uint32_t tr = (uint32_t)C - 1u - t;   // reversed position
    const uint64_t dr = tr <= m ? delta_or_max(skeys, (int64_t)b0 - 1 + tr, n) : 0ull;
    uint64_t sf = block_max_scan<C>(dr, s_warp);
    sf = sf > dC ? sf : dC;
    S.suf[tr] = sf;
    if (t == (uint32_t)C - 1u) {
        S.pre[C] = pf > dC ? pf : dC;
        S.suf[C] = dC;
    }
    __syncthreads();
    const uint32_t i = b0 + t;
    float4 lo = make_float4(0.f, 0.f, 0.f, 0.f), hi = lo;
    bool climbing = i < n;
    if (climbing) {
        lo = leafbox[2 * (size_t)i];
        hi = leafbox[2 * (size_t)i + 1];
    }
    if (climbing && n == 1) {
        hdr->root_ref = 0;
        hdr->root_cnt = 1;
        hdr->n_tris = 1;
        hdr->root_lo = lo;
        hdr->root_hi = hi;
        climbing = false;
    }
    uint32_t l = i, r = i;
    int32_t ref = (int32_t)i, cnt = 1;
    bool local = true;
    while (climbing) {
        uint64_t dl, dr2;   // D(l-1), D(r)
        if (local) {
            dl = S.d[l - b0];
            dr2 = S.d[r - b0 + 1];
        } else {
            dl = delta_or_max(skeys, (int64_t)l - 1, n);
            dr2 = delta_or_max(skeys, (int64_t)r, n);
        }
        const bool is_left = dr2 < dl;
        const uint32_t p = is_left ? r : l - 1;
        if (local)
            local = is_left ? (r < b1 && S.suf[r - b0 + 2] > dr2)
                            : (l > b0 && S.pre[l - b0 - 1] > dl);
        float4 n0, n1, n2;
        uint32_t L, R, kL, kR;
        if (local) {
            const uint32_t q = p - b0;
            write_half(S.node[q], is_left, lo, hi, ref, cnt);
            S.bound[is_left ? 0 : 1][q] = is_left ? l : r;
            __threadfence_block();
            if (atomicAdd(&S.flag[q], 1u) == 0) break;   // the sibling finishes p
            __threadfence_block();
            n0 = S.node[q][0];
            n1 = S.node[q][1];
            n2 = S.node[q][2];
            L = is_left ? l : S.bound[0][q];
            R = is_left ? S.bound[1][q] : r;
            kL = L >= b0 && L <= b1 ? S.key[L - b0] : 0u;
            kR = R >= b0 && R <= b1 ? S.key[R - b0] : 0u;
        } else {
            write_half(nodes + 4 * (size_t)p, is_left, lo, hi, ref, cnt);
            if (is_left)
                rangeL[p] = l;
            else
                rangeR[p] = r;
            if (atomic_add_acq_rel(&flags[p], 1u) == 0) break;
            n0 = __ldcg(&nodes[4 * (size_t)p]);
            n1 = __ldcg(&nodes[4 * (size_t)p + 1]);
            n2 = __ldcg(&nodes[4 * (size_t)p + 2]);
            L = is_left ? l : __ldcg(&rangeL[p]);
            R = is_left ? __ldcg(&rangeR[p]) : r;
            kL = L < n ? __ldg(&skeys[L]) : 0u;
            kR = R < n ? __ldg(&skeys[R]) : 0u;
        }
        // every step must strictly widen the range; anything else is a
        // broken invariant, reported instead of climbing on
        if (L > l || R < r || R - L <= r - l || R >= n) {
            atomicOr(status, RT_DEV_BADINDEX);
            break;
        }
        // merge_bbox(left, right) = fmin / fmax of the two boxes of the record
        lo = make_float4(fminf(n0.x, n1.z), fminf(n0.y, n1.w), fminf(n0.z, n2.x), 0.f);
        hi = make_float4(fmaxf(n0.w, n2.y), fmaxf(n1.x, n2.z), fmaxf(n1.y, n2.w), 0.f);
        const uint32_t count = R - L + 1;
        const bool interior = count >= (uint32_t)min_leaf + 3u && kL != kR;
        ref = interior ? (int32_t)p : (int32_t)L;
        cnt = interior ? 0 : (int32_t)count;
        l = L;
        r = R;
        if (L == 0 && R == n - 1) {
            hdr->root_ref = ref;
            hdr->root_cnt = cnt;
            hdr->n_tris = n;
            hdr->root_lo = lo;
            hdr->root_hi = hi;
            break;
        }
    }
    // the chunk's nodes that were joined here (both children arrived)
    __syncthreads();
    for (uint32_t e = t; e < 4u * (uint32_t)C; e += (uint32_t)C) {
        const uint32_t q = e >> 2;
        if (q + 1 < m && S.flag[q] == 2u) nodes[4 * ((size_t)b0 + q) + (e & 3u)] = S.node[q][e & 3u];
    }
}

// K climbs of emit_climb advanced in lockstep by one thread: one release
// fence before the K arrival counters are bumped and one acquire fence before
// the winners read their siblings, instead of one ordering point per climber
// and level.  Used where few threads must cover many triangles (the
// persistent many-scene build).  Climbers are the triangles first..first+K-1
// of one scene (those >= n are idle).
template <int K>
__device__ __forceinline__ void emit_climb_multi(uint32_t first, uint32_t n,
                                                 const uint32_t* __restrict__ skeys,
                                                 const float4* __restrict__ leafbox,
                                                 float4* __restrict__ nodes,
                                                 uint32_t* __restrict__ flags,
                                                 uint32_t* __restrict__ rangeL,
                                                 uint32_t* __restrict__ rangeR, int min_leaf,
                                                 BvhHeader* __restrict__ hdr) {
    if (n == 1) {
        if (first == 0) emit_climb(0, 1, skeys, leafbox, nodes, flags, rangeL, rangeR, min_leaf, hdr);
        return;
    }
    uint32_t l[K], r[K], p[K];
    int32_t ref[K], cnt[K];
    float4 lo[K], hi[K];
    bool alive[K], left[K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const uint32_t i = first + k;
        alive[k] = i < n;
        l[k] = r[k] = i;
        ref[k] = (int32_t)i;
        cnt[k] = 1;
        if (alive[k]) {
            lo[k] = leafbox[2 * (size_t)i];
            hi[k] = leafbox[2 * (size_t)i + 1];
        }
    }
    for (;;) {
        bool any = false;
#pragma unroll
        for (int k = 0; k < K; ++k) {
            if (!alive[k]) continue;
            any = true;
            if (l[k] == 0 || (r[k] != n - 1 && delta(skeys, r[k]) < delta(skeys, l[k] - 1))) {
                p[k] = r[k];
                left[k] = true;
            } else {
                p[k] = l[k] - 1;
                left[k] = false;
            }
            float* rec = reinterpret_cast<float*>(nodes + 4 * (size_t)p[k]);
            int* rec_i = reinterpret_cast<int*>(nodes + 4 * (size_t)p[k] + 3);
            if (left[k]) {
                nodes[4 * (size_t)p[k]] = make_float4(lo[k].x, lo[k].y, lo[k].z, hi[k].x);
                *reinterpret_cast<float2*>(rec + 4) = make_float2(hi[k].y, hi[k].z);
                rec_i[0] = ref[k];
                rec_i[2] = cnt[k];
                rangeL[p[k]] = l[k];
            } else {
                *reinterpret_cast<float2*>(rec + 6) = make_float2(lo[k].x, lo[k].y);
                nodes[4 * (size_t)p[k] + 2] = make_float4(lo[k].z, hi[k].x, hi[k].y, hi[k].z);
                rec_i[1] = ref[k];
                rec_i[3] = cnt[k];
                rangeR[p[k]] = r[k];
            }
        }
        if (!any) return;
        __threadfence();   // release every record written above
#pragma unroll
        for (int k = 0; k < K; ++k)
            if (alive[k] && atomicAdd(&flags[p[k]], 1u) == 0) alive[k] = false;
        __threadfence();   // acquire the siblings' records
#pragma unroll
        for (int k = 0; k < K; ++k) {
            if (!alive[k]) continue;
            const size_t q = p[k];
            const float4 n0 = __ldcg(&nodes[4 * q]);
            const float4 n1 = __ldcg(&nodes[4 * q + 1]);
            const float4 n2 = __ldcg(&nodes[4 * q + 2]);
            const uint32_t L = left[k] ? l[k] : __ldcg(&rangeL[q]);
            const uint32_t R = left[k] ? __ldcg(&rangeR[q]) : r[k];
            lo[k] = make_float4(fminf(n0.x, n1.z), fminf(n0.y, n1.w), fminf(n0.z, n2.x), 0.f);
            hi[k] = make_float4(fmaxf(n0.w, n2.y), fmaxf(n1.x, n2.z), fmaxf(n1.y, n2.w), 0.f);
            const uint32_t count = R - L + 1;
            const bool interior =
                count >= (uint32_t)min_leaf + 3u && __ldg(&skeys[L]) != __ldg(&skeys[R]);
            ref[k] = interior ? (int32_t)q : (int32_t)L;
            cnt[k] = interior ? 0 : (int32_t)count;
            l[k] = L;
            r[k] = R;
            if (L == 0 && R == n - 1) {
                hdr->root_ref = ref[k];
                hdr->root_cnt = cnt[k];
                hdr->n_tris = n;
                hdr->root_lo = lo[k];
                hdr->root_hi = hi[k];
                alive[k] = false;
            }
        }
    }
}

}  // namespace rt
