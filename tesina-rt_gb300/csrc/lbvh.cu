// lbvh.cu — LBVH construction for sm_103a.
//
// Stages (the reference's BVHBuilder::build_lbvh, src/rt/bvh-builder.cpp:201-741):
//   k_bounds        per-triangle AABB (build_primitive_bbox, bvh-builder.cl:100-130)
//                   reduced to the scene AABB (max_local_bbox, :318-391) with
//                   order-free integer min/max atomics;
//   k_morton_hist   morton_encode (:181-252) fused with the digit histograms of
//                   every radix pass;
//   k_onesweep      stable LSD radix pass, 8-bit digits, warp-level
//                   __match_any_sync ranking and decoupled look-back with a
//                   bounded spin (replaces the bitonic network of
//                   bvh-builder-sort.cl and bvh-builder.cpp:361-454);
//   k_permute       rearrange_indices / rearrange_map (:49-72) fused with the
//                   triangle records used by traversal and the leaf AABBs;
//   k_emit_refit    one bottom-up pass that builds the radix tree (Apetrei's
//                   agglomerative formulation of Karras' tree), collapses it
//                   to the reference's leaf rule (find_middle, :484-552) and
//                   computes every AABB (build_leaf_bbox / build_node_bbox,
//                   :262-311) on the way up.
#include <cuda_runtime.h>
#include <stdint.h>

#include "lbvh.cuh"
#include "rt_internal.cuh"

namespace rt {

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

// ---------------------------------------------------------------------------
// scene AABB
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_bounds(const float4* __restrict__ pos,
                                                const uint32_t* __restrict__ idx, uint32_t n,
                                                uint32_t* __restrict__ bounds) {
    float lo[3] = {1e37f, 1e37f, 1e37f}, hi[3] = {-1e37f, -1e37f, -1e37f};
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t a = __ldg(&idx[3 * (size_t)i]), b = __ldg(&idx[3 * (size_t)i + 1]),
                       c = __ldg(&idx[3 * (size_t)i + 2]);
        const float4 p0 = __ldg(&pos[a]), p1 = __ldg(&pos[b]), p2 = __ldg(&pos[c]);
        lo[0] = fminf(lo[0], fminf(fminf(p0.x, p1.x), p2.x));
        lo[1] = fminf(lo[1], fminf(fminf(p0.y, p1.y), p2.y));
        lo[2] = fminf(lo[2], fminf(fminf(p0.z, p1.z), p2.z));
        hi[0] = fmaxf(hi[0], fmaxf(fmaxf(p0.x, p1.x), p2.x));
        hi[1] = fmaxf(hi[1], fmaxf(fmaxf(p0.y, p1.y), p2.y));
        hi[2] = fmaxf(hi[2], fmaxf(fmaxf(p0.z, p1.z), p2.z));
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

// ---------------------------------------------------------------------------
// Morton codes + radix histograms
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_morton_hist(const float4* __restrict__ pos,
                                                     const uint32_t* __restrict__ idx, uint32_t n,
                                                     const uint32_t* __restrict__ bounds, int depth,
                                                     int passes, uint32_t* __restrict__ keys,
                                                     uint32_t* __restrict__ vals,
                                                     uint32_t* __restrict__ hist) {
    __shared__ uint32_t sh[4][256];
    for (int i = threadIdx.x; i < 4 * 256; i += blockDim.x) (&sh[0][0])[i] = 0;
    __syncthreads();
    const float glo[3] = {o2f(bounds[0]), o2f(bounds[1]), o2f(bounds[2])};
    const float ghi[3] = {o2f(bounds[3]), o2f(bounds[4]), o2f(bounds[5])};
    float inv[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) inv[c] = 1.0f / (ghi[c] - glo[c]);
    const int bits_per_axis = (depth + 2) / 3;                  // ceil(depth / 3)
    const float scale = (float)(1u << bits_per_axis);          // pow(2, ceil(depth/3.0))
    const int offset = depth % 3 ? 3 - (depth % 3) : 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t a = __ldg(&idx[3 * (size_t)i]), b = __ldg(&idx[3 * (size_t)i + 1]),
                       c = __ldg(&idx[3 * (size_t)i + 2]);
        const float4 p0 = __ldg(&pos[a]), p1 = __ldg(&pos[b]), p2 = __ldg(&pos[c]);
        const float P[3][3] = {{p0.x, p0.y, p0.z}, {p1.x, p1.y, p1.z}, {p2.x, p2.y, p2.z}};
        uint32_t m[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            float h = P[0][k], l = P[0][k];
            h = fmaxf(h, P[1][k]);
            h = fmaxf(h, P[2][k]);
            l = fminf(l, P[1][k]);
            l = fminf(l, P[2][k]);
            float center = (h + l) * 0.5f;
            float slice = (center - glo[k]) * inv[k];
            slice = fmaxf(0.0f, fminf(1.0f, slice));
            slice *= scale;
            m[k] = (uint32_t)slice;   // truncation; slice == 2^k keeps only out-of-range bits
        }
        uint32_t code = 0;
        int axis = (offset + 1) % 3;
#pragma unroll
        for (int bit = 0; bit < 32; ++bit) {
            if (bit < depth) {
                const int src = (bit + offset) / 3;
                const uint32_t mv = axis == 0 ? m[0] : (axis == 1 ? m[1] : m[2]);
                code |= ((mv >> src) & 1u) << bit;
                axis = axis == 2 ? 0 : axis + 1;
            }
        }
        keys[i] = code;
        vals[i] = i;
        for (int p = 0; p < passes; ++p) atomicAdd(&sh[p][(code >> (8 * p)) & 255u], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < passes * 256; i += blockDim.x) {
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

// ---------------------------------------------------------------------------
// Onesweep radix pass
// ---------------------------------------------------------------------------
constexpr int SORT_THREADS = 256;
constexpr int SORT_WARPS = SORT_THREADS / 32;
constexpr int SORT_ITEMS = 16;
constexpr int SORT_TILE = SORT_THREADS * SORT_ITEMS;   // 4096 keys per tile
constexpr uint32_t LB_AGG = 1u << 30, LB_PREFIX = 2u << 30, LB_MASK = (1u << 30) - 1;
constexpr uint32_t LB_SPIN_LIMIT = 1u << 22;

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

__global__ void __launch_bounds__(SORT_THREADS) k_onesweep(
    const uint32_t* __restrict__ kin, const uint32_t* __restrict__ vin, uint32_t* __restrict__ kout,
    uint32_t* __restrict__ vout, uint32_t n, int shift, const uint32_t* __restrict__ hist,
    uint32_t* __restrict__ lookback, uint32_t* __restrict__ tile_ctr, uint32_t* __restrict__ status) {
    __shared__ uint32_t s_keys[SORT_TILE];
    __shared__ uint32_t s_vals[SORT_TILE];
    __shared__ uint32_t s_whist[SORT_WARPS][256];
    __shared__ uint32_t s_goff[256];
    __shared__ uint32_t s_lstart[256];
    __shared__ uint32_t s_scan[SORT_WARPS];
    __shared__ uint32_t s_tile;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (tid == 0) s_tile = atomicAdd(tile_ctr, 1u);
    for (int i = tid; i < SORT_WARPS * 256; i += SORT_THREADS) (&s_whist[0][0])[i] = 0;
    __syncthreads();
    const uint32_t tile = s_tile;
    const size_t base = (size_t)tile * SORT_TILE;
    const uint32_t lanemask_lt = (1u << lane) - 1u;

    // warp-striped load: warp w owns [base + w*512, base + (w+1)*512)
    uint32_t k[SORT_ITEMS], v[SORT_ITEMS], rank[SORT_ITEMS];
#pragma unroll
    for (int j = 0; j < SORT_ITEMS; ++j) {
        const size_t g = base + (size_t)warp * (SORT_ITEMS * 32) + j * 32 + lane;
        const bool ok = g < n;
        k[j] = ok ? __ldcs(&kin[g]) : 0xffffffffu;
        v[j] = ok ? __ldcs(&vin[g]) : 0u;
    }
    // stable warp-level ranking with __match_any_sync
#pragma unroll
    for (int j = 0; j < SORT_ITEMS; ++j) {
        const size_t g = base + (size_t)warp * (SORT_ITEMS * 32) + j * 32 + lane;
        const bool ok = g < n;
        const uint32_t d = (k[j] >> shift) & 255u;
        const uint32_t valid = __ballot_sync(0xffffffffu, ok);
        uint32_t peers = 0, prev = 0;
        if (ok) {
            peers = __match_any_sync(valid, d);
            prev = s_whist[warp][d];
        }
        __syncwarp();
        if (ok) {
            rank[j] = prev + __popc(peers & lanemask_lt);
            const int leader = __ffs(peers) - 1;
            if (lane == leader) s_whist[warp][d] = prev + __popc(peers);
        }
        __syncwarp();
    }
    __syncthreads();

    // per-digit: exclusive offsets of each warp, tile count
    const uint32_t dgt = tid;   // 256 threads <-> 256 digits
    uint32_t cnt = 0;
#pragma unroll
    for (int w = 0; w < SORT_WARPS; ++w) {
        const uint32_t c = s_whist[w][dgt];
        s_whist[w][dgt] = cnt;
        cnt += c;
    }
    // decoupled look-back over earlier tiles for this digit
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
    // global digit start (exclusive scan of the pass histogram)
    const uint32_t gstart = block_excl_scan_256(__ldg(&hist[dgt]), s_scan);
    const uint32_t lstart = block_excl_scan_256(cnt, s_scan);
    s_goff[dgt] = gstart + excl - lstart;
    s_lstart[dgt] = lstart;
    __syncthreads();

    // scatter into shared memory in digit order
#pragma unroll
    for (int j = 0; j < SORT_ITEMS; ++j) {
        const size_t g = base + (size_t)warp * (SORT_ITEMS * 32) + j * 32 + lane;
        if (g < n) {
            const uint32_t d = (k[j] >> shift) & 255u;
            const uint32_t p = s_lstart[d] + s_whist[warp][d] + rank[j];
            s_keys[p] = k[j];
            s_vals[p] = v[j];
        }
    }
    __syncthreads();
    const uint32_t valid_n = (uint32_t)min((size_t)SORT_TILE, (size_t)n - base);
    for (uint32_t i = tid; i < valid_n; i += SORT_THREADS) {
        const uint32_t key = s_keys[i];
        const uint32_t d = (key >> shift) & 255u;
        const uint32_t dst = s_goff[d] + i;
        kout[dst] = key;
        vout[dst] = s_vals[i];
    }
}

// ---------------------------------------------------------------------------
// permutation of the triangle data into sorted order
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_permute(
    uint32_t n, const uint32_t* __restrict__ vals, const uint32_t* __restrict__ idx_old,
    const uint32_t* __restrict__ map_old, const uint32_t* __restrict__ orig_old,
    const float4* __restrict__ pos, uint32_t* __restrict__ idx_new, uint32_t* __restrict__ map_new,
    uint32_t* __restrict__ orig_new, float4* __restrict__ tris, float4* __restrict__ leafbox) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
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
}

// ---------------------------------------------------------------------------
// bottom-up emit + refit
// ---------------------------------------------------------------------------
// delta(i): highest differing bit between sorted keys i and i+1, with the
// index appended so that equal keys still order (Karras' augmentation).
__device__ __forceinline__ uint64_t delta(const uint32_t* __restrict__ k, uint32_t i) {
    const uint32_t x = __ldg(&k[i]) ^ __ldg(&k[i + 1]);
    return ((uint64_t)x << 32) | (uint64_t)(i ^ (i + 1));
}

// One thread per sorted triangle climbs while it is the second child to
// arrive.  A radix-tree node [L, R] is an interior node of the reference's
// tree iff R - L + 1 >= min_leaf + 3 (find_middle's unsigned test
// last - first - 1 <= min_leaf, bvh-builder.cl:501) and its keys are not all
// equal (the bit loop of :515-525); otherwise it is a leaf, or part of one.
// The reference's split (highest differing bit, first index with the bit
// set) is the radix tree's split, so both trees have the same ranges.
__global__ void __launch_bounds__(256) k_emit_refit(uint32_t n, const uint32_t* __restrict__ skeys,
                                                    const float4* __restrict__ leafbox,
                                                    float4* __restrict__ nodes,
                                                    uint32_t* __restrict__ flags,
                                                    uint32_t* __restrict__ rangeL,
                                                    uint32_t* __restrict__ rangeR, int min_leaf,
                                                    BvhHeader* __restrict__ hdr) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
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
        // second arrival: both children of p are in its record
        const float4 n0 = __ldcg(&nodes[4 * (size_t)p]);
        const float4 n1 = __ldcg(&nodes[4 * (size_t)p + 1]);
        const float4 n2 = __ldcg(&nodes[4 * (size_t)p + 2]);
        const uint32_t L = is_left ? l : __ldcg(&rangeL[p]);
        const uint32_t R = is_left ? __ldcg(&rangeR[p]) : r;
        // merge_bbox(left, right): lo = fmin(left.lo, right.lo), hi = fmax(...)
        lo = make_float4(fminf(n0.x, n1.z), fminf(n0.y, n1.w), fminf(n0.z, n2.x), 0.f);
        hi = make_float4(fmaxf(n0.w, n2.y), fmaxf(n1.x, n2.z), fmaxf(n1.y, n2.w), 0.f);
        const uint32_t count = R - L + 1;
        const bool interior = count >= (uint32_t)min_leaf + 3u && __ldg(&skeys[L]) != __ldg(&skeys[R]);
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

}  // namespace rt

// ---------------------------------------------------------------------------
// host launchers
// ---------------------------------------------------------------------------
namespace rt {

static int grid_for(uint32_t n, int threads, int max_blocks) {
    int64_t b = ((int64_t)n + threads - 1) / threads;
    if (b < 1) b = 1;
    if (b > max_blocks) b = max_blocks;
    return (int)b;
}

size_t lbvh_scratch_bytes(uint32_t n, int passes) {
    const size_t tiles = ((size_t)n + SORT_TILE - 1) / SORT_TILE;
    return sizeof(uint32_t) * (8 + 4 * 256 + 4 + (size_t)passes * tiles * 256);
}

cudaError_t lbvh_build(const LbvhArgs& a, cudaStream_t s) {
    const uint32_t n = a.n;
    const int passes = (a.depth + 7) / 8;
    const size_t tiles = ((size_t)n + SORT_TILE - 1) / SORT_TILE;
    // scratch: bounds[8] | hist[4*256] | tile_ctr[4] | lookback[passes*tiles*256]
    uint32_t* bounds = a.scratch;
    uint32_t* hist = bounds + 8;
    uint32_t* tile_ctr = hist + 4 * 256;
    uint32_t* lookback = tile_ctr + 4;
    cudaError_t e;
    e = cudaMemsetAsync(a.scratch, 0, lbvh_scratch_bytes(n, passes), s);
    if (e) return e;
    // bounds init: lo = ordered(+big) via 0xFF.. (max), hi = 0 (min)
    e = cudaMemsetAsync(bounds, 0xff, 3 * sizeof(uint32_t), s);
    if (e) return e;
    const int sms = a.num_sms;
    k_bounds<<<grid_for(n, 256, sms * 8), 256, 0, s>>>(a.pos, a.idx_in, n, bounds);
    k_morton_hist<<<grid_for(n, 256, sms * 8), 256, 0, s>>>(a.pos, a.idx_in, n, bounds, a.depth,
                                                            passes, a.keys_unsorted, a.vals0, hist);
    const uint32_t* kin = a.keys_unsorted;
    const uint32_t* vin = a.vals0;
    uint32_t* kbuf[2] = {a.keys1, a.keys_sorted};
    uint32_t* vbuf[2] = {a.vals1, a.vals_sorted};
    for (int p = 0; p < passes; ++p) {
        // the last pass always lands in keys_sorted / vals_sorted
        const int dst = ((passes - 1 - p) & 1) ? 0 : 1;
        k_onesweep<<<(unsigned)tiles, SORT_THREADS, 0, s>>>(kin, vin, kbuf[dst], vbuf[dst], n, 8 * p,
                                                          hist + 256 * p, lookback + (size_t)p * tiles * 256,
                                                          tile_ctr + p, a.status);
        kin = kbuf[dst];
        vin = vbuf[dst];
    }
    k_permute<<<grid_for(n, 256, sms * 16), 256, 0, s>>>(n, a.vals_sorted, a.idx_in, a.map_in,
                                                         a.orig_in, a.pos, a.idx_out, a.map_out,
                                                         a.orig_out, a.tris, a.leafbox);
    if (n > 1) {
        e = cudaMemsetAsync(a.flags, 0, sizeof(uint32_t) * (n - 1), s);
        if (e) return e;
    }
    k_emit_refit<<<(n + 255) / 256, 256, 0, s>>>(n, a.keys_sorted, a.leafbox, a.nodes, a.flags,
                                                 a.rangeL, a.rangeR, a.min_leaf, a.hdr);
    return cudaGetLastError();
}

size_t radix_scratch_words(uint32_t n, int passes) {
    const size_t tiles = ((size_t)n + SORT_TILE - 1) / SORT_TILE;
    return 4 * 256 + 4 + (size_t)passes * tiles * 256;
}

int radix_tile_size() { return SORT_TILE; }

cudaError_t radix_sort_pairs(const uint32_t* kin, const uint32_t* vin, uint32_t* kout,
                             uint32_t* vout, uint32_t* ktmp, uint32_t* vtmp, uint32_t n,
                             int key_bits, uint32_t* scratch, uint32_t* status, int num_sms,
                             cudaStream_t s) {
    const int passes = (key_bits + 7) / 8;
    const size_t tiles = ((size_t)n + SORT_TILE - 1) / SORT_TILE;
    uint32_t* hist = scratch;
    uint32_t* tile_ctr = hist + 4 * 256;
    uint32_t* lookback = tile_ctr + 4;
    cudaError_t e = cudaMemsetAsync(scratch, 0, sizeof(uint32_t) * radix_scratch_words(n, passes), s);
    if (e) return e;
    if (n == 0) return cudaSuccess;
    k_radix_hist<<<grid_for(n, 256, num_sms * 8), 256, 0, s>>>(kin, n, passes, hist);
    const uint32_t* ki = kin;
    const uint32_t* vi = vin;
    for (int p = 0; p < passes; ++p) {
        const bool to_out = ((passes - 1 - p) & 1) == 0;
        uint32_t* ko = to_out ? kout : ktmp;
        uint32_t* vo = to_out ? vout : vtmp;
        k_onesweep<<<(unsigned)tiles, SORT_THREADS, 0, s>>>(ki, vi, ko, vo, n, 8 * p, hist + 256 * p,
                                                          lookback + (size_t)p * tiles * 256,
                                                          tile_ctr + p, status);
        ki = ko;
        vi = vo;
    }
    return cudaGetLastError();
}

cudaError_t lbvh_refit(const LbvhArgs& a, cudaStream_t s) {
    const uint32_t n = a.n;
    k_refit_leaves<<<grid_for(n, 256, a.num_sms * 16), 256, 0, s>>>(n, a.idx_out, a.pos, a.tris,
                                                                    a.leafbox);
    if (n > 1) {
        cudaError_t e = cudaMemsetAsync(a.flags, 0, sizeof(uint32_t) * (n - 1), s);
        if (e) return e;
    }
    // the climb is deterministic in the sorted keys, so rerunning it on the
    // same keys reproduces the same topology with the new boxes
    k_emit_refit<<<(n + 255) / 256, 256, 0, s>>>(n, a.keys_sorted, a.leafbox, a.nodes, a.flags,
                                                 a.rangeL, a.rangeR, a.min_leaf, a.hdr);
    return cudaGetLastError();
}

}  // namespace rt
