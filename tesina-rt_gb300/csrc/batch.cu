// batch.cu — many scenes and many images per launch.
//
// rt_batch_build builds the LBVHs of every distinct scene of a batch in ONE
// persistent cooperative launch: the stages of BVHBuilder::build_lbvh
// (src/rt/bvh-builder.cpp:201-741) run over the concatenated triangle index
// space of all scenes, separated by grid-wide barriers; the radix passes use
// per-scene histograms and look-back regions, so each scene is sorted on its
// own while all scenes' tiles share the machine.  Results land in each
// scene's own buffers, exactly as a one-scene build would write them.
//
// rt_batch_render renders every view of the batch in ONE persistent launch:
// warps fetch chunks of the concatenated pixel space of all images and trace
// the same rays as rt_render (trace_dev.cuh), either one pixel path per lane
// (k_render_batch, used by the request loop) or with reflection rays pooled
// per warp (k_render_batch_pool, used by rt_batch).
//
// rt_batch_capture records build + render in a CUDA graph that
// rt_batch_replay relaunches.
#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <vector>
#include <mutex>

#include "../../include/rt_cuda.h"
#include "batch.cuh"
#include "lbvh_dev.cuh"
#include "rt_internal.cuh"
#include "trace_dev.cuh"

namespace cg = cooperative_groups;

// The unpooled many-view kernel (the server's) with the two-phase
// traversal (1) or the plain loop (0, measured faster there: 1047 against
// 982 Mrays/s of served capacity); the pooled kernel always uses the
// two-phase loop (4 % faster on the 64 soups).
#ifndef RT_WW_SERVED
#define RT_WW_SERVED 0
#endif

namespace rt {

constexpr int kMaxBatchScenes = 1024;
// Keys per thread of the batched radix tiles: 8 (2048-key tiles) keeps the
// persistent kernel at <= 64 registers, i.e. 4 resident blocks per SM, which
// doubles the threads available to the latency-bound emit stage.
constexpr int kBatchItems = 8;

__device__ __forceinline__ unsigned long long globaltimer() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}

// Stage timestamps for profiling (block 0, thread 0, after each barrier).
__device__ __forceinline__ void stamp(const BatchBuildArgs& A, int k) {
    if (A.stage_ns && blockIdx.x == 0 && threadIdx.x == 0) A.stage_ns[k] = globaltimer();
}

// Scene index of global element g (offsets ascending, off[count] = total).
__device__ __forceinline__ int find_segment(const uint32_t* off, int count, uint32_t g) {
    int lo = 0, hi = count - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (off[mid] <= g)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

__global__ void __launch_bounds__(SORT_THREADS, 4) k_batch_build(BatchBuildArgs A) {
    cg::grid_group grid = cg::this_grid();
    __shared__ SortSmemT<kBatchItems> S;
    __shared__ uint32_t s_toff[kMaxBatchScenes + 1];
    __shared__ uint32_t s_tileoff[kMaxBatchScenes + 1];
    __shared__ uint32_t s_hist[4][256];
    __shared__ float s_red[SORT_WARPS][6];
    __shared__ int s_cur;
    const int nsc = A.count;
    for (int i = threadIdx.x; i <= nsc; i += blockDim.x) {
        s_toff[i] = A.tri_off[i];
        s_tileoff[i] = A.tile_off[i];
    }
    __syncthreads();
    const uint32_t total = s_toff[nsc];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t nblk = gridDim.x;
    const uint32_t gtid = blockIdx.x * blockDim.x + tid, gthreads = nblk * blockDim.x;
    stamp(A, 0);

    // ---- stage 0: initialise bounds, histograms, look-back, arrival flags ---
    for (uint32_t i = gtid; i < (uint32_t)nsc * 8; i += gthreads)
        A.scenes[i >> 3].bounds[i & 7] = (i & 7) < 3 ? 0xffffffffu : 0u;
    for (uint32_t i = gtid; i < (uint32_t)nsc * 1024; i += gthreads)
        A.scenes[i >> 10].hist[i & 1023] = 0;
    for (int sc = 0; sc < nsc; ++sc) {
        const BatchScene& B = A.scenes[sc];
        const size_t words = (size_t)B.passes * (s_tileoff[sc + 1] - s_tileoff[sc]) * 256;
        for (size_t i = gtid; i < words; i += gthreads) B.lookback[i] = 0;
    }
    if (gtid < 4) A.tile_ctr[gtid] = 0;
    grid.sync();
    stamp(A, 1);

    // ---- stage 1: scene AABBs (steps of 256 consecutive triangles) ----------
    for (uint32_t step = blockIdx.x; (size_t)step * SORT_THREADS < total; step += nblk) {
        const uint32_t g = step * SORT_THREADS + tid;
        const bool ok = g < total;
        int s = ok ? find_segment(s_toff, nsc, g) : -1;
        float lo[3] = {1e37f, 1e37f, 1e37f}, hi[3] = {-1e37f, -1e37f, -1e37f};
        if (ok) {
            const BatchScene& B = A.scenes[s];
            tri_aabb(B.pos, B.idx_in, g - s_toff[s], lo, hi);
        }
        const uint32_t last = min(total - 1, step * SORT_THREADS + SORT_THREADS - 1);
        const int s0 = find_segment(s_toff, nsc, step * SORT_THREADS);
        const int s1 = find_segment(s_toff, nsc, last);
        if (s0 == s1) {   // the whole step is one scene: block reduction, 6 atomics
#pragma unroll
            for (int off = 16; off > 0; off >>= 1)
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    lo[c] = fminf(lo[c], __shfl_xor_sync(0xffffffffu, lo[c], off));
                    hi[c] = fmaxf(hi[c], __shfl_xor_sync(0xffffffffu, hi[c], off));
                }
            if (lane == 0)
                for (int c = 0; c < 3; ++c) {
                    s_red[warp][c] = lo[c];
                    s_red[warp][3 + c] = hi[c];
                }
            __syncthreads();
            if (tid < 3) {
                float a = s_red[0][tid], b = s_red[0][3 + tid];
                for (int k = 1; k < SORT_WARPS; ++k) {
                    a = fminf(a, s_red[k][tid]);
                    b = fmaxf(b, s_red[k][3 + tid]);
                }
                atomicMin(&A.scenes[s0].bounds[tid], f2o(a));
                atomicMax(&A.scenes[s0].bounds[3 + tid], f2o(b));
            }
            __syncthreads();
        } else if (ok) {   // a scene boundary inside the step: per-triangle atomics
            for (int c = 0; c < 3; ++c) {
                atomicMin(&A.scenes[s].bounds[c], f2o(lo[c]));
                atomicMax(&A.scenes[s].bounds[3 + c], f2o(hi[c]));
            }
        }
    }
    grid.sync();
    stamp(A, 2);

    // ---- stage 2: Morton codes + per-scene digit histograms ------------------
    // Each block walks a contiguous range of steps, keeping the histogram of
    // the scene it is in and flushing it when the scene changes.
    {
        const uint32_t nsteps = (total + SORT_THREADS - 1) / SORT_THREADS;
        const uint32_t per = (nsteps + nblk - 1) / nblk;
        const uint32_t st0 = blockIdx.x * per, st1 = min(nsteps, st0 + per);
        for (int i = tid; i < 4 * 256; i += blockDim.x) (&s_hist[0][0])[i] = 0;
        if (tid == 0) s_cur = -1;
        __syncthreads();
        for (uint32_t step = st0; step < st1; ++step) {
            const uint32_t g = step * SORT_THREADS + tid;
            const bool ok = g < total;
            const uint32_t last = min(total - 1, step * SORT_THREADS + SORT_THREADS - 1);
            const int s0 = find_segment(s_toff, nsc, step * SORT_THREADS);
            const int s1 = find_segment(s_toff, nsc, last);
            const bool single = s0 == s1;
            if (single && s0 != s_cur) {   // flush the previous scene's histogram
                if (s_cur >= 0) {
                    const BatchScene& P = A.scenes[s_cur];
                    for (int i = tid; i < P.passes * 256; i += blockDim.x) {
                        const uint32_t v = (&s_hist[0][0])[i];
                        if (v) atomicAdd(&P.hist[i], v);
                    }
                }
                __syncthreads();
                for (int i = tid; i < 4 * 256; i += blockDim.x) (&s_hist[0][0])[i] = 0;
                if (tid == 0) s_cur = s0;
                __syncthreads();
            }
            if (ok) {
                const int s = single ? s0 : find_segment(s_toff, nsc, g);
                const BatchScene& B = A.scenes[s];
                const uint32_t li = g - s_toff[s];
                float lo[3], hi[3];
                tri_aabb(B.pos, B.idx_in, li, lo, hi);
                const MortonParams P = morton_params(B.bounds, B.depth);
                const uint32_t code = morton_code(P, lo, hi);
                B.keys_unsorted[li] = code;
                for (int p = 0; p < B.passes; ++p) {
                    const uint32_t d = (code >> (8 * p)) & 255u;
                    if (single)
                        atomicAdd(&s_hist[p][d], 1u);
                    else
                        atomicAdd(&B.hist[p * 256 + d], 1u);
                }
            }
            __syncthreads();
        }
        if (s_cur >= 0) {
            const BatchScene& P = A.scenes[s_cur];
            for (int i = tid; i < P.passes * 256; i += blockDim.x) {
                const uint32_t v = (&s_hist[0][0])[i];
                if (v) atomicAdd(&P.hist[i], v);
            }
        }
    }
    grid.sync();
    stamp(A, 3);

    // ---- stage 3: radix passes; tiles of all scenes share the grid ----------
    const uint32_t total_tiles = s_tileoff[nsc];
    for (int p = 0; p < A.passes; ++p) {
        for (;;) {
            if (tid == 0) S.tile = atomicAdd(&A.tile_ctr[p], 1u);   // global tile order
            __syncthreads();
            const uint32_t t = S.tile;
            __syncthreads();
            if (t >= total_tiles) break;
            const int s = find_segment(s_tileoff, nsc, t);
            const BatchScene& B = A.scenes[s];
            const uint32_t lt = t - s_tileoff[s];
            const int dst = ((B.passes - 1 - p) & 1) ? 0 : 1;   // last pass -> sorted
            const uint32_t* kin = p == 0 ? B.keys_unsorted : (dst ? B.keys1 : B.keys_sorted);
            // the first pass makes the identity values itself
            const uint32_t* vin = p == 0 ? nullptr : (dst ? B.vals1 : B.vals_sorted);
            uint32_t* kout = dst ? B.keys_sorted : B.keys1;
            uint32_t* vout = dst ? B.vals_sorted : B.vals1;
            const uint32_t ntiles_s = s_tileoff[s + 1] - s_tileoff[s];
            onesweep_tile<kBatchItems>(S, lt, kin, vin, kout, vout, B.n, 8 * p, B.hist + 256 * p,
                          B.lookback + (size_t)p * ntiles_s * 256, A.status);
        }
        grid.sync();
        if (p == A.passes - 1) stamp(A, 4);
    }

    // the permutation into sorted order happens in level 0 of the emit
    stamp(A, 5);
    // ---- stage 5: the emit, level by level (k_batch_emit launches) ---------
}

// One level of the emit over every scene that still has blocks at it: the
// one-scene emit's blocks (emit_level, the same items, buffers and leave
// rule), with block j of the launch taken by the scene whose range of the
// level's blocks holds j.  The C == EMIT_C0 instance is level 0.
static_assert(EMIT_C0 != EMIT_C1, "k_batch_emit tells level 0 by its block size");
template <int C>
__global__ void __launch_bounds__(C, C == EMIT_C0 ? RT_EMIT_MINB0 : RT_EMIT_MINB1) k_batch_emit(
    const BatchScene* __restrict__ scenes, int count, int level, const uint32_t* __restrict__ off,
    uint32_t* __restrict__ status) {
    extern __shared__ __align__(16) unsigned char emit_smem[];
    auto& S = *reinterpret_cast<EmitSmem<C>*>(emit_smem);
    const int s = find_segment(off, count, blockIdx.x);
    const BatchScene& B = scenes[s];
    const uint32_t job = blockIdx.x - off[s];
    const EmitBuffers E = emit_buffers(B.n, B.emit);
    uint32_t n_in = emit_blocks0(B.n);   // blocks of the level below
    if constexpr (C == EMIT_C0) {
        // level 0 permutes its triangles into sorted order and joins them
        // with their AABBs in registers (as k_emit_level0_permute)
        const PermuteIO P{B.vals_sorted, B.idx_in,  B.map_in,   B.orig_in, B.pos,
                          B.idx_out,     B.map_out, B.orig_out, B.tris};
        emit_level<C, true>(S, job, B.n, B.keys_sorted, nullptr, nullptr, nullptr, 0, E.items[0],
                            E.counts[0], B.nodes, B.min_leaf, emit_leave(0, n_in), B.hdr, status,
                            P);
    } else {
        for (int l = 2; l <= level; ++l) n_in = emit_next_level(n_in);
        const int src = (level - 1) & 1;
        emit_level<C>(S, job, B.n, B.keys_sorted, nullptr, E.items[src], E.counts[src], n_in,
                      E.items[src ^ 1], E.counts[src ^ 1], B.nodes, B.min_leaf,
                      emit_leave(level, emit_next_level(n_in)), B.hdr, status);
    }
}

__global__ void k_batch_stamp(unsigned long long* t) { *t = globaltimer(); }

// ---------------------------------------------------------------------------
// many-image render
// ---------------------------------------------------------------------------
// REFR: each pixel's ray tree, refracted rays included (scenes with
// refracting materials).
template <int THREADS, int MINB, bool REFR = false>
__global__ void __launch_bounds__(THREADS, MINB) k_render_batch(BatchRenderArgs A) {
    __shared__ uint32_t s_poff[kMaxBatchViews + 1];
    for (int i = threadIdx.x; i <= A.count; i += blockDim.x) s_poff[i] = A.pix_off[i];
    __syncthreads();
    const uint32_t total = s_poff[A.count];
    const int lane = threadIdx.x & 31;
    uint32_t n_prim = 0, n_sec = 0, n_shadow = 0, n_hits = 0;
    for (;;) {
        uint32_t base0 = 0;
        if (lane == 0) base0 = atomicAdd(A.work_counter, (unsigned)A.chunk);
        base0 = __shfl_sync(0xffffffffu, base0, 0);
        if (base0 >= total) break;
        for (uint32_t base = base0; base < base0 + A.chunk && base < total; base += 32) {
            const uint32_t g = base + lane;
            // the view of the warp's first pixel; lanes past its end look their own up
            const int v0 = find_segment(s_poff, A.count, base);
            const bool same = g < s_poff[v0 + 1];
            if (g < total) {
                const int v = same ? v0 : find_segment(s_poff, A.count, g);
                const BatchView& V = A.views[v];
                const int local = (int)(g - s_poff[v]);
                int x, y;
                pixel_of(warp_tile_order(local, V.width, V.height), V.width, V.height, 32, x, y);
                const BvhHeader H = *V.scene.hdr;
                const PixelResult pr = render_pixel<RT_WW_SERVED, REFR>(
                    V.scene, H, *V.lights, V.cam, x, y, V.width, V.height, V.max_bounces, A.status);
                ++n_prim;
                n_sec += pr.secondary;
                n_shadow += pr.shadow;
                n_hits += pr.hits;
                uchar4 px;
                px.x = to_unorm8(pr.r, A.inv1e6);
                px.y = to_unorm8(pr.g, A.inv1e6);
                px.z = to_unorm8(pr.b, A.inv1e6);
                px.w = 255;
                reinterpret_cast<uchar4*>(A.rgba)[(size_t)V.rgba_offset + V.width * y + x] = px;
            }
        }
    }
    if (A.stats) {
        n_prim = __reduce_add_sync(0xffffffffu, n_prim);
        n_sec = __reduce_add_sync(0xffffffffu, n_sec);
        n_shadow = __reduce_add_sync(0xffffffffu, n_shadow);
        n_hits = __reduce_add_sync(0xffffffffu, n_hits);
        if (lane == 0) {
            atomicAdd((unsigned long long*)&A.stats->primary_rays, (unsigned long long)n_prim);
            atomicAdd((unsigned long long*)&A.stats->secondary_rays, (unsigned long long)n_sec);
            atomicAdd((unsigned long long*)&A.stats->shadow_rays, (unsigned long long)n_shadow);
            atomicAdd((unsigned long long*)&A.stats->hits, (unsigned long long)n_hits);
        }
    }
}

// ---------------------------------------------------------------------------
// k_render_batch_pool: the rays of k_render_batch scheduled as in
// k_render_pool (trace.cu): warp tiles of primary rays, dense (hit, light)
// shadow tasks, and a per-warp pool of reflection rays traced 32 at a time,
// whichever views and pixels they belong to.  Fixed-point contributions are
// summed into A.accum (3 per pixel of the launch's concatenated pixel space,
// integer sums being independent of order) and k_batch_fb writes RGBA8 at
// each view's offset afterwards.  Bit-identical to k_render_batch.
// ---------------------------------------------------------------------------
// MAXB > 0: scenes with refracting materials, as k_render_pool_refr
// (trace.cu) follows them: a hit continues its reflected and refracted rays,
// the pool is taken from the top and holds 32 (MAXB + 2) rays, enough for
// views of up to MAXB bounces; a push past it raises RT_DEV_OVERFLOW.
namespace {
template <int BPOOL>
struct WarpPoolB {
    float ro[3][BPOOL], rd[3][BPOOL], rc[BPOOL];
    int rv[BPOOL], rai[BPOOL], rbounce[BPOOL];   // view, sum index, bounce
    float hp[3][32], hn[3][32], hd[3][32], hc[32];
    int hid[32], hv[32], hai[32], hbounce[32], hoff[33];
    unsigned hmask[32];
    unsigned char hinv[32];
    uint8_t task[32 * RT_MAX_LIGHTS];   // shadow tasks that need a ray
    int pool_n;
};
}  // namespace

template <int THREADS, int MINB, int MAXB = 0>
__global__ void __launch_bounds__(THREADS, MINB) k_render_batch_pool(BatchRenderArgs A) {
    constexpr int BPOOL = MAXB ? 32 * (MAXB + 2) : 64;
    __shared__ uint32_t s_poff[kMaxBatchViews + 1];
    __shared__ WarpPoolB<BPOOL> sQ[THREADS / 32];
    for (int i = threadIdx.x; i <= A.count; i += blockDim.x) s_poff[i] = A.pix_off[i];
    const int lane = threadIdx.x & 31;
    WarpPoolB<BPOOL>& Q = sQ[threadIdx.x >> 5];
    if (lane == 0) Q.pool_n = 0;
    __syncthreads();
    const uint32_t total = s_poff[A.count];
    const unsigned lt = (1u << lane) - 1u;
    uint32_t n_prim = 0, n_sec = 0, n_shadow = 0, n_hits = 0;
    bool tiles = true;
    for (;;) {
        const int pn = Q.pool_n;
        bool have = false;
        f3 o = mk3(0.f, 0.f, 0.f), d = o;
        float c = 1.0f, tmin = 0.0f, tmax = 1e36f;
        int v = 0, ai = 0, bounce = 0;
        if (pn >= 32 || (!tiles && pn > 0)) {
            const int k = min(32, pn);
            const int j = pn - k + lane;
            have = lane < k;
            if (have) {
                o = mk3(Q.ro[0][j], Q.ro[1][j], Q.ro[2][j]);
                d = mk3(Q.rd[0][j], Q.rd[1][j], Q.rd[2][j]);
                c = Q.rc[j];
                v = Q.rv[j];
                ai = Q.rai[j];
                bounce = Q.rbounce[j];
                tmin = 0.0001f;
                tmax = 1e37f;
            }
            __syncwarp();
            if (lane == 0) Q.pool_n = pn - k;
        } else if (tiles) {
            uint32_t base = 0;
            if (lane == 0) base = atomicAdd(A.work_counter, 32u);
            base = __shfl_sync(0xffffffffu, base, 0);
            if (base >= total) {
                tiles = false;
                continue;
            }
            const uint32_t g = base + lane;
            const int v0 = find_segment(s_poff, A.count, base);
            have = g < total;
            if (have) {
                v = g < s_poff[v0 + 1] ? v0 : find_segment(s_poff, A.count, g);
                const BatchView& V = A.views[v];
                int x, y;
                pixel_of(warp_tile_order((int)(g - s_poff[v]), V.width, V.height), V.width,
                         V.height, 32, x, y);
                ai = (int)s_poff[v] + V.width * y + x;
                o = mk3(V.cam.pos[0], V.cam.pos[1], V.cam.pos[2]);
                d = primary_dir(V.cam, x, y, V.width, V.height, 0.0f, 0.0f);
                ++n_prim;
            }
        } else {
            break;
        }
        bool hit_ok = false;
        Hit hit{-1, 0.f, 0.f, 0.f};
        if (have) {
            const BatchView& V = A.views[v];
            const BvhHeader H = *V.scene.hdr;
            const TRay r = make_tray(o, d, mk3(1.0f / d.x, 1.0f / d.y, 1.0f / d.z), tmin);
            hit = closest_hit_ww(V.scene, H, r, tmax, A.status);
            hit_ok = hit.id >= 0;
        }
        const unsigned hm = __ballot_sync(0xffffffffu, hit_ok);
        const int nh = __popc(hm);
        int nl = 0;
        if (hit_ok) {
            const int k = __popc(hm & lt);
            const HitInfo hi = complete_hit(A.views[v].scene, o, d, hit);
            Q.hp[0][k] = hi.hp.x; Q.hp[1][k] = hi.hp.y; Q.hp[2][k] = hi.hp.z;
            Q.hn[0][k] = hi.n.x; Q.hn[1][k] = hi.n.y; Q.hn[2][k] = hi.n.z;
            Q.hd[0][k] = d.x; Q.hd[1][k] = d.y; Q.hd[2][k] = d.z;
            Q.hc[k] = c;
            Q.hid[k] = hit.id;
            Q.hv[k] = v;
            Q.hai[k] = ai;
            Q.hbounce[k] = bounce;
            Q.hinv[k] = hi.inverse_n;
            Q.hmask[k] = 0u;
            nl = A.views[v].lights->count;
        }
        // shadow tasks: hit k owns tasks hoff[k] .. hoff[k+1]-1 (one per light)
        int ex = nl;
#pragma unroll
        for (int s = 1; s < 32; s <<= 1) {
            const int u = __shfl_up_sync(0xffffffffu, ex, s);
            if (lane >= s) ex += u;
        }
        const int ntask = __shfl_sync(0xffffffffu, ex, 31);
        if (hit_ok) Q.hoff[__popc(hm & lt)] = ex - nl;
        if (lane == 0) Q.hoff[nh] = ntask;
        __syncwarp();
        // the tasks whose light adds nothing are settled without a ray
        // (light_vanishes); the others are listed densely (hit | light << 5)
        // and traced 32 at a time
        int nt = 0;
        for (int t0 = 0; t0 < ntask; t0 += 32) {
            const int t = t0 + lane;
            bool nd = false;
            int lo = 0, l = 0;
            if (t < ntask) {
                int hi2 = nh - 1;   // the hit whose tasks contain t
                while (lo < hi2) {
                    const int mid = (lo + hi2 + 1) >> 1;
                    if (Q.hoff[mid] <= t)
                        lo = mid;
                    else
                        hi2 = mid - 1;
                }
                l = t - Q.hoff[lo];
                const BatchView& V = A.views[Q.hv[lo]];
                nd = !light_vanishes(V.lights->light[l],
                                     V.scene.mats[__ldg(&V.scene.map[Q.hid[lo]])],
                                     mk3(Q.hp[0][lo], Q.hp[1][lo], Q.hp[2][lo]),
                                     mk3(Q.hn[0][lo], Q.hn[1][lo], Q.hn[2][lo]),
                                     mk3(Q.hd[0][lo], Q.hd[1][lo], Q.hd[2][lo]));
            }
            const unsigned bm = __ballot_sync(0xffffffffu, nd);
            if (nd) Q.task[nt + __popc(bm & lt)] = (uint8_t)(lo | (l << 5));
            nt += __popc(bm);
        }
        __syncwarp();
        for (int i = lane; i < nt; i += 32) {
            const int e = Q.task[i], lo = e & 31, l = e >> 5;
            const BatchView& V = A.views[Q.hv[lo]];
            const BvhHeader H = *V.scene.hdr;
            const f3 p = mk3(Q.hp[0][lo], Q.hp[1][lo], Q.hp[2][lo]);
            if (occluded<true>(V.scene, H, V.lights->light[l], p, A.status))
                atomicOr(&Q.hmask[lo], 1u << l);
        }
        __syncwarp();
        bool push = false, push_t = false;
        f3 np = mk3(0.f, 0.f, 0.f), nd = np, td = np;
        float nc = 0.f, tc = 0.f;
        int nv = 0, nai = 0, nbounce = 0;
        if (lane < nh) {
            const int k = lane;
            const BatchView& V = A.views[Q.hv[k]];
            const f3 p = mk3(Q.hp[0][k], Q.hp[1][k], Q.hp[2][k]);
            const f3 n = mk3(Q.hn[0][k], Q.hn[1][k], Q.hn[2][k]);
            const f3 dk = mk3(Q.hd[0][k], Q.hd[1][k], Q.hd[2][k]);
            const float ck = Q.hc[k];
            const rt_material mat = V.scene.mats[__ldg(&V.scene.map[Q.hid[k]])];
            const uint3 col = shade_hit(*V.lights, mat, p, n, dk, ck, Q.hmask[k]);
            const int ak = Q.hai[k];
            if (col.x | col.y | col.z) {   // a zero colour adds nothing
                atomicAdd(&A.accum[3 * (size_t)ak], col.x);
                atomicAdd(&A.accum[3 * (size_t)ak + 1], col.y);
                atomicAdd(&A.accum[3 * (size_t)ak + 2], col.z);
            }
            ++n_hits;
            n_shadow += (uint32_t)V.lights->count;
            const int bk = Q.hbounce[k];
            if (bk < V.max_bounces) {
                float R = 1.0f;
                if (MAXB > 0 && mat.refractive_index > 0.0f &&
                    refract_ray(dk, n, Q.hinv[k] != 0, mat.refractive_index, R, td)) {
                    tc = ck * mat.reflectiveness * (1.0f - R);
                    push_t = true;
                }
                if (mat.reflectiveness > 0.0f) {
                    reflect_ray(dk, n, nd);
                    nc = ck * mat.reflectiveness * R;
                    push = true;
                }
                np = p;
                nv = Q.hv[k];
                nai = ak;
                nbounce = bk + 1;
            }
        }
        const unsigned pm = __ballot_sync(0xffffffffu, push);
        const unsigned pt = MAXB > 0 ? __ballot_sync(0xffffffffu, push_t) : 0u;
        const int pbase = Q.pool_n;
        if (push) {
            const int j = pbase + __popc(pm & lt);
            if (MAXB == 0 || j < BPOOL) {
                Q.ro[0][j] = np.x; Q.ro[1][j] = np.y; Q.ro[2][j] = np.z;
                Q.rd[0][j] = nd.x; Q.rd[1][j] = nd.y; Q.rd[2][j] = nd.z;
                Q.rc[j] = nc;
                Q.rv[j] = nv;
                Q.rai[j] = nai;
                Q.rbounce[j] = nbounce;
                ++n_sec;
            } else {
                atomicOr(A.status, RT_DEV_OVERFLOW);
            }
        }
        if (MAXB > 0 && push_t) {
            const int j = pbase + __popc(pm) + __popc(pt & lt);
            if (j < BPOOL) {
                Q.ro[0][j] = np.x; Q.ro[1][j] = np.y; Q.ro[2][j] = np.z;
                Q.rd[0][j] = td.x; Q.rd[1][j] = td.y; Q.rd[2][j] = td.z;
                Q.rc[j] = tc;
                Q.rv[j] = nv;
                Q.rai[j] = nai;
                Q.rbounce[j] = nbounce;
                ++n_sec;
            } else {
                atomicOr(A.status, RT_DEV_OVERFLOW);
            }
        }
        __syncwarp();
        if (lane == 0) Q.pool_n = min(BPOOL, pbase + __popc(pm) + __popc(pt));
        __syncwarp();
    }
    if (A.stats) {
        n_prim = __reduce_add_sync(0xffffffffu, n_prim);
        n_sec = __reduce_add_sync(0xffffffffu, n_sec);
        n_shadow = __reduce_add_sync(0xffffffffu, n_shadow);
        n_hits = __reduce_add_sync(0xffffffffu, n_hits);
        if (lane == 0) {
            atomicAdd((unsigned long long*)&A.stats->primary_rays, (unsigned long long)n_prim);
            atomicAdd((unsigned long long*)&A.stats->secondary_rays, (unsigned long long)n_sec);
            atomicAdd((unsigned long long*)&A.stats->shadow_rays, (unsigned long long)n_shadow);
            atomicAdd((unsigned long long*)&A.stats->hits, (unsigned long long)n_hits);
        }
    }
}

// RGBA8 of the pooled sums: pixel i of the launch belongs to view v and goes
// to rgba[v.rgba_offset + i - pix_off[v]].
__global__ void k_batch_fb(BatchRenderArgs A) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.total) return;
    const int v = find_segment(A.pix_off, A.count, i);
    uchar4 o;
    o.x = to_unorm8(A.accum[3 * (size_t)i], A.inv1e6);
    o.y = to_unorm8(A.accum[3 * (size_t)i + 1], A.inv1e6);
    o.z = to_unorm8(A.accum[3 * (size_t)i + 2], A.inv1e6);
    o.w = 255;
    reinterpret_cast<uchar4*>(A.rgba)[(size_t)A.views[v].rgba_offset + (i - A.pix_off[v])] = o;
}

struct BatchRenderVariant {
    int threads, min_blocks;
    void (*fn)(BatchRenderArgs);
    bool pooled;
    bool refract;      // follows refracted rays
    int max_bounces;   // deepest view it holds (0: any)
};
// Variant 0 serves the request loop (many short launches, where the unpooled
// kernel measured faster); rt_batch takes the first pooled one (one large
// launch, where the pool keeps lanes busy).
static const BatchRenderVariant kBatchVariants[] = {
    {128, 8, k_render_batch<128, 8>, false},
    {128, 6, k_render_batch_pool<128, 6>, true},
    {256, 4, k_render_batch<256, 4>, false},
    {128, 6, k_render_batch<128, 6>, false},
    {128, 8, k_render_batch_pool<128, 8>, true},
    {128, 6, k_render_batch<128, 6, true>, false, true},
    {128, 5, k_render_batch_pool<128, 5, 4>, true, true, 4},
    {128, 4, k_render_batch_pool<128, 4, 6>, true, true, 6},
};

int batch_render_variant_count() { return (int)(sizeof(kBatchVariants) / sizeof(kBatchVariants[0])); }

int batch_render_variant_info(int v, int* threads, const void** fn) {
    if (v < 0 || v >= batch_render_variant_count()) return -1;
    if (threads) *threads = kBatchVariants[v].threads;
    if (fn) *fn = (const void*)kBatchVariants[v].fn;
    return 0;
}

bool batch_render_variant_pooled(int v) {
    return v >= 0 && v < batch_render_variant_count() && kBatchVariants[v].pooled;
}

bool batch_render_variant_refracts(int v) {
    return v >= 0 && v < batch_render_variant_count() && kBatchVariants[v].refract;
}

int batch_refract_variant(bool pooled, int max_bounces) {
    int best = -1;
    for (int v = 0; v < batch_render_variant_count(); ++v) {
        const BatchRenderVariant& k = kBatchVariants[v];
        if (!k.refract || k.pooled != pooled) continue;
        if (k.max_bounces != 0 && max_bounces > k.max_bounces) continue;
        if (best < 0 || (k.max_bounces != 0 && (kBatchVariants[best].max_bounces == 0 ||
                                                k.max_bounces < kBatchVariants[best].max_bounces)))
            best = v;
    }
    return best;
}

cudaError_t launch_batch_render(const BatchRenderArgs& a, int variant, int grid, cudaStream_t s) {
    if (variant < 0 || variant >= batch_render_variant_count()) return cudaErrorInvalidValue;
    const bool pooled = kBatchVariants[variant].pooled;
    if (pooled) {
        if (!a.accum) return cudaErrorInvalidValue;
        cudaError_t e = cudaMemsetAsync(a.accum, 0, 3 * sizeof(uint32_t) * (size_t)a.total, s);
        if (e != cudaSuccess) return e;
    }
    kBatchVariants[variant].fn<<<grid, kBatchVariants[variant].threads, 0, s>>>(a);
    if (pooled && a.total) k_batch_fb<<<(a.total + 255) / 256, 256, 0, s>>>(a);
    return cudaGetLastError();
}

const void* batch_build_kernel() { return (const void*)k_batch_build; }
int batch_build_threads() { return SORT_THREADS; }
int batch_max_scenes() { return kMaxBatchScenes; }
int sort_tile_size() { return SORT_THREADS * kBatchItems; }

cudaError_t launch_batch_build(const BatchBuildArgs& a, int grid, cudaStream_t s) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(SORT_THREADS);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaError_t e = cudaLaunchKernelEx(&cfg, k_batch_build, a);
    if (e != cudaSuccess) return e;
    {
        // the shared-memory opt-in is a property of the kernel on each device
        static std::mutex mu;
        static uint64_t done = 0;   // devices 0..63 set up
        int dev = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (e != cudaSuccess) return e;
        std::lock_guard<std::mutex> lk(mu);
        if (dev >= 64 || !((done >> dev) & 1)) {
            e = cudaFuncSetAttribute(k_batch_emit<EMIT_C0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)sizeof(EmitSmem<EMIT_C0>));
            if (e == cudaSuccess)
                e = cudaFuncSetAttribute(k_batch_emit<EMIT_C1>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)sizeof(EmitSmem<EMIT_C1>));
            if (e != cudaSuccess) return e;
            if (dev < 64) done |= 1ull << dev;
        }
    }
    for (int L = 0; L < a.emit_levels; ++L) {
        if (a.emit_jobs[L] == 0) continue;
        const uint32_t* off = a.emit_off + (size_t)L * (a.count + 1);
        if (L == 0)
            k_batch_emit<EMIT_C0><<<a.emit_jobs[L], EMIT_C0, sizeof(EmitSmem<EMIT_C0>), s>>>(
                a.scenes, a.count, L, off, a.status);
        else
            k_batch_emit<EMIT_C1><<<a.emit_jobs[L], EMIT_C1, sizeof(EmitSmem<EMIT_C1>), s>>>(
                a.scenes, a.count, L, off, a.status);
    }
    if (a.stage_ns) k_batch_stamp<<<1, 1, 0, s>>>(a.stage_ns + 6);
    return cudaGetLastError();
}

}  // namespace rt
