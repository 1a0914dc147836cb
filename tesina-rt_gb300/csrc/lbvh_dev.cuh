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
// Multi-level emit + refit, warp-synchronous.  The tree is built bottom-up
// in a few launches ("levels").  Within a block, runs of consecutive items
// are joined by warps: a warp holds up to 32 consecutive items, one per lane
// (at level 0 the items are the sorted triangles).  Each lane owns the run
// of items that starts at it; in a round, a run that is a left child (its
// parent's split is its right boundary) takes over the run that starts at
// the next lane if that run is the matching right child, writes the 64-byte
// node (left half its own, right half the sibling's, shuffled across) and
// carries on with the merged box; the absorbed lane drops out.  No shared
// memory, barrier or fence is involved.  A run whose parent lies outside the
// warp's items is left over; the block gathers the leftovers of its warps in
// order and joins them again, at most 32 per warp, until one warp holds them
// all or no node inside the block is left.  What is left then has its parent
// outside the block and becomes an item of the next level, which gathers the items of EMIT_GROUP blocks, until one
// block reaches the root.  A block leaves at most EMIT_FMAX items: they hang
// off the chains of nodes crossing its two ends, each at most 64 deep (32
// key bits + 32 index bits).
//
// The tree is the one of emit_climb.  With d[j] the augmented delta of the
// boundary before item j of a chunk and d[c] the boundary after its last
// item (D(-1) = D(n-1) = max), a run j..b is a left child iff d[b+1] < d[j];
// its parent stays in the chunk iff max d[b+2..c] > d[b+1] (the parent's
// range ends at the first boundary above d[b+1]); a right child's parent
// stays iff max d[0..j-1] > d[j].  Above the leftovers of a chunk, the
// boundaries between consecutive items are exactly the splits of the
// remaining nodes (a node's inner boundaries all lie below its end
// boundaries), so chunks and levels compose.
// ---------------------------------------------------------------------------
constexpr int EMIT_FMAX = 128;   // items a block may leave
constexpr int EMIT_GROUP = 8;    // blocks of one level gathered by a block of the next

// An item: leaf range, keys at its ends, box, ref / count, and the augmented
// delta of the boundary before it.
struct __align__(16) EmitItem {
    uint32_t l, r, kl, kr;
    float lo[3], hi[3];
    int32_t ref, cnt;
    uint64_t db;
    uint32_t pad[2];
};

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

// Joins the items of lanes 0..cnt-1 of the warp (all 32 lanes call it) whose
// parents lie inside these items; `edge` is the boundary after the last item.
// Returns true for a lane that still holds a run afterwards (its parent is
// outside).  A run that reaches [0, n-1] writes the header instead.
__device__ __forceinline__ bool warp_join(WarpItem& it, uint32_t cnt, uint64_t edge, uint32_t n,
                                          int min_leaf, float4* __restrict__ nodes,
                                          BvhHeader* __restrict__ hdr,
                                          uint32_t* __restrict__ status) {
    const uint32_t lane = threadIdx.x & 31u;
    const unsigned FULL = 0xffffffffu;
    bool on = lane < cnt;
    // prefix maxima of d[0..lane] and suffix maxima of d[lane..cnt]
    const uint64_t dv = on ? it.db : 0ull;
    uint64_t pre = dv, suf = dv;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint64_t u = __shfl_up_sync(FULL, pre, o);
        const uint64_t w = __shfl_down_sync(FULL, suf, o);
        if (lane >= (uint32_t)o) pre = pre > u ? pre : u;
        if (lane + (uint32_t)o < 32u) suf = suf > w ? suf : w;
    }
    suf = suf > edge ? suf : edge;
    const uint64_t pre_left = __shfl_up_sync(FULL, pre, 1);   // max d[0..lane-1]
    uint32_t bl = lane;   // lane of the run's last item
    for (int round = 0;; ++round) {
        const uint32_t nb = bl + 1u;   // first lane after the run
        const uint32_t src = nb < 32u ? nb : 31u;
        const uint64_t dnext = __shfl_sync(FULL, it.db, src);
        const uint32_t s2 = nb + 1u < 32u ? nb + 1u : 31u;
        const uint64_t sufn = __shfl_sync(FULL, suf, s2);
        const uint64_t dR = nb < cnt ? dnext : edge;
        const bool is_left = dR < it.db;
        const uint64_t far = nb + 1u < cnt ? sufn : edge;   // max d[bl+2..cnt]
        const bool inside = is_left ? (nb < cnt && far > dR) : (lane > 0 && pre_left > it.db);
        // the run at lane nb is the matching right child when it is a right
        // child whose parent is inside (its parent is then this run's split)
        const bool ready_right = on && !is_left && inside;
        const bool partner = __shfl_sync(FULL, ready_right, src) && nb < cnt;
        const bool absorb = on && is_left && inside && partner;
        const uint32_t p_bl = __shfl_sync(FULL, bl, src);
        const uint32_t p_r = __shfl_sync(FULL, it.r, src);
        const uint32_t p_kr = __shfl_sync(FULL, it.kr, src);
        const float plx = __shfl_sync(FULL, it.lox, src), ply = __shfl_sync(FULL, it.loy, src),
                    plz = __shfl_sync(FULL, it.loz, src);
        const float phx = __shfl_sync(FULL, it.hix, src), phy = __shfl_sync(FULL, it.hiy, src),
                    phz = __shfl_sync(FULL, it.hiz, src);
        const int32_t p_ref = __shfl_sync(FULL, it.ref, src), p_cnt = __shfl_sync(FULL, it.cnt, src);
        const uint32_t gone = __reduce_or_sync(FULL, absorb ? (1u << src) : 0u);
        if (gone == 0u) break;
        if (round >= 64) {   // deeper than any tree of 64-bit augmented keys
            if (lane == 0) atomicOr(status, RT_DEV_BADINDEX);
            break;
        }
        if (absorb) {
            const uint32_t p = it.r;   // global node index: the split
            float4* np = nodes + 4 * (size_t)p;
            np[0] = make_float4(it.lox, it.loy, it.loz, it.hix);
            np[1] = make_float4(it.hiy, it.hiz, plx, ply);
            np[2] = make_float4(plz, phx, phy, phz);
            np[3] = make_float4(__int_as_float(it.ref), __int_as_float(p_ref),
                                __int_as_float(it.cnt), __int_as_float(p_cnt));
            // merge_bbox(left, right): fmin / fmax, left operand first
            it.lox = fminf(it.lox, plx); it.loy = fminf(it.loy, ply); it.loz = fminf(it.loz, plz);
            it.hix = fmaxf(it.hix, phx); it.hiy = fmaxf(it.hiy, phy); it.hiz = fmaxf(it.hiz, phz);
            it.r = p_r;
            it.kr = p_kr;
            bl = p_bl;
            const uint32_t count = it.r - it.l + 1;
            const bool interior = count >= (uint32_t)min_leaf + 3u && it.kl != it.kr;
            it.ref = interior ? (int32_t)p : (int32_t)it.l;
            it.cnt = interior ? 0 : (int32_t)count;
            if (it.l == 0 && it.r == n - 1) {
                hdr->root_ref = it.ref;
                hdr->root_cnt = it.cnt;
                hdr->n_tris = n;
                hdr->root_lo = make_float4(it.lox, it.loy, it.loz, 0.f);
                hdr->root_hi = make_float4(it.hix, it.hiy, it.hiz, 0.f);
                on = false;
            }
        }
        if ((gone >> lane) & 1u) on = false;
    }
    return on;
}

// Shared state of one emit block: the items left over by its warps, in order.
template <int C>
struct EmitSmem {
    EmitItem list[C];
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
// out[blk * EMIT_FMAX] and their number in out_count[blk].
template <int C>
__device__ __forceinline__ void emit_level(EmitSmem<C>& S, uint32_t blk, uint32_t n,
                                           const uint32_t* __restrict__ skeys,
                                           const float4* __restrict__ leafbox,
                                           const EmitItem* __restrict__ in,
                                           const uint32_t* __restrict__ in_count,
                                           uint32_t n_in, EmitItem* __restrict__ out,
                                           uint32_t* __restrict__ out_count,
                                           float4* __restrict__ nodes, int min_leaf,
                                           BvhHeader* __restrict__ hdr,
                                           uint32_t* __restrict__ status) {
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
            lo = leafbox[2 * (size_t)i];
            hi = leafbox[2 * (size_t)i + 1];
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
        keep = warp_join(it, cnt, edge, n, min_leaf, nodes, hdr, status);
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
        if (m <= 32u) {
            if (w == 0) {
                const uint32_t cnt = m;
                if (lane < cnt) item_to_reg(S.list[lane], it);
                keep = warp_join(it, cnt, S.edge, n, min_leaf, nodes, hdr, status);
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
        keep = warp_join(it, cnt, edge, n, min_leaf, nodes, hdr, status);
        const uint32_t m_new = gather_runs<C>(S, it, keep);
        stalls = m_new == m ? stalls + 1u : 0u;
        m = m_new;
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
