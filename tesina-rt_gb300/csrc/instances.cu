// instances.cu — multi-root (instanced) scenes: the reference's trace_multi /
// shadow_trace_multi (src/kernel/trace-bvh.cl:420-463, :84-181;
// src/kernel/shadow-trace-bvh.cl:317-373) with its BVHRoot records
// (src/rt/scene.cpp:595-703), rendered by one persistent kernel.
//
// An instance is a built scene (its LBVH, triangles, materials) under a
// row-major 4x4 transform and its inverse, given by the caller as the
// reference's objects give them.  Per ray and instance: the ray goes into the
// object's space through the inverse (with the homogeneous divide of
// multiply_point / multiply_vector), is traversed with the scene's own
// closest_hit, and the hit's distance is measured again in world space
// (distance from the origin to the hit point taken back through the
// transform); the nearest wins, the first instance on a tie.  The hit
// normal is the object-space normal through the transform, not renormalised.
// Shadow rays test every instance; a spot light's cone test leaves the point
// lit, as in shadow_trace_multi (the single-root kernel treats it as shadow).
// Refracting scenes are not taken (rt_render renders those).
#include <cuda_runtime.h>
#include <stdint.h>

#include <new>
#include <cstring>
#include <vector>

#include "../../include/rt_cuda.h"
#include "ctx_internal.h"
#include "rt_internal.cuh"
#include "trace.cuh"
#include "trace_dev.cuh"

namespace rt {

struct InstanceRoot {
    SceneView scene;
    float tr[16], trinv[16];
};

struct InstanceArgs {
    const InstanceRoot* roots;
    const float4* cull;       // per root: world box lo, hi (padded; infinite = never culled)
    int count;
    rt_lights lights;
    rt_camera cam;
    int width, height, max_bounces;
    uint32_t* accum;          // 3 fixed-point sums per pixel, zeroed before the launch
    rt_render_stats* stats;
    uint32_t* work_counter;
    uint32_t* status;
    float inv1e6;
};

// M (v, w): four products summed left to right per row, then divided by the
// fourth row's value when |w'| > 1e-26.
__device__ __forceinline__ f3 mat_apply(const float* M, f3 v, float w) {
    float r[4];
#pragma unroll
    for (int k = 0; k < 4; ++k)
        r[k] = M[4 * k] * v.x + M[4 * k + 1] * v.y + M[4 * k + 2] * v.z + M[4 * k + 3] * w;
    if (fabsf(r[3]) > 1e-26f) {
        const float d = r[3];
        r[0] = r[0] / d;
        r[1] = r[1] / d;
        r[2] = r[2] / d;
    }
    return mk3(r[0], r[1], r[2]);
}

// World-space box of each root, for culling only: the eight corners of the
// root box moved by the root's transform, padded for rounding.  A projective
// transform, or one that gives non-finite corners, gets an infinite box.
// Skipping a root the ray cannot reach changes no result: each root's hit is
// a function of that root and the ray alone.
__global__ void k_instance_boxes(const InstanceRoot* roots, int count, float4* cull) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const InstanceRoot& R = roots[i];
    const BvhHeader H = *R.scene.hdr;
    const float* M = R.tr;
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    bool ok = M[12] == 0.0f && M[13] == 0.0f && M[14] == 0.0f && M[15] == 1.0f;
    float big = 0.0f;
    for (int c = 0; c < 8 && ok; ++c) {
        const float x = (c & 1) ? H.root_hi.x : H.root_lo.x;
        const float y = (c & 2) ? H.root_hi.y : H.root_lo.y;
        const float z = (c & 4) ? H.root_hi.z : H.root_lo.z;
        for (int k = 0; k < 3; ++k) {
            const float v = M[4 * k] * x + M[4 * k + 1] * y + M[4 * k + 2] * z + M[4 * k + 3];
            if (!isfinite(v)) ok = false;
            lo[k] = fminf(lo[k], v);
            hi[k] = fmaxf(hi[k], v);
            big = fmaxf(big, fabsf(v));
        }
    }
    if (!ok || H.n_tris == 0) {
        cull[2 * i] = make_float4(-INFINITY, -INFINITY, -INFINITY, 0.0f);
        cull[2 * i + 1] = make_float4(INFINITY, INFINITY, INFINITY, 0.0f);
        return;
    }
    const float pad = 1e-4f * big + 1e-30f;
    cull[2 * i] = make_float4(lo[0] - pad, lo[1] - pad, lo[2] - pad, 0.0f);
    cull[2 * i + 1] = make_float4(hi[0] + pad, hi[1] + pad, hi[2] + pad, 0.0f);
}

// Entry parameter of the ray o + t d (t >= 0) into the box, or -1 when it
// misses.  NaN slabs (a zero direction component on a box face) constrain
// nothing, so the test can only keep roots, never drop one it would reach.
__device__ __forceinline__ float cull_enter(const float4* cull, int i, f3 o, f3 inv) {
    const float4 lo = __ldg(&cull[2 * i]), hi = __ldg(&cull[2 * i + 1]);
    const float ax = (lo.x - o.x) * inv.x, bx = (hi.x - o.x) * inv.x;
    const float ay = (lo.y - o.y) * inv.y, by = (hi.y - o.y) * inv.y;
    const float az = (lo.z - o.z) * inv.z, bz = (hi.z - o.z) * inv.z;
    const float t0 = fmaxf(fmaxf(fmaxf(fminf(ax, bx), fminf(ay, by)), fminf(az, bz)), 0.0f);
    const float t1 = fminf(fminf(fmaxf(ax, bx), fmaxf(ay, by)), fmaxf(az, bz));
    return t0 > t1 ? -1.0f : t0;
}

#ifndef RT_INST_NEAR
#define RT_INST_NEAR 1   // visit a group's roots near to far (0: in index order)
#endif

struct MultiHit {
    Hit h;        // id local to the instance's scene; t in world space
    int root;
};

__device__ __forceinline__ Hit root_closest(const InstanceRoot& R, f3 o, f3 d, float tmin,
                                            float tmax, uint32_t* status) {
    const f3 td = mat_apply(R.trinv, d, 0.0f);
    const f3 to = mat_apply(R.trinv, o, 1.0f);
    const TRay tr = make_tray(to, td, mk3(1.0f / td.x, 1.0f / td.y, 1.0f / td.z), tmin);
    const BvhHeader H = *R.scene.hdr;
    Hit h = closest_hit(R.scene, H, tr, tmax, status);
    if (h.id >= 0) {
        const f3 hp = mat_apply(R.tr, add(to, muls(td, h.t)), 1.0f);
        const f3 dv = sub(hp, o);
        h.t = sqrtf(dot(dv, dv));
    }
    return h;
}

// The reference keeps the first root (in index order) of least world t.  Each
// root's hit depends only on that root and the ray, so the roots are visited
// in groups of 32, near to far by box entry within a group, and a root is
// taken when nearer, or as near and of lower index; the visit stops once the
// next entry lies beyond the best hit.  The result is the reference's as long
// as no world t is NaN (no order then): a NaN t reruns the reference's own
// loop, every root in index order.
__device__ __forceinline__ MultiHit closest_multi(const InstanceArgs& A, f3 o, f3 d, float tmin,
                                                  float tmax) {
    MultiHit best;
    const f3 inv = mk3(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
    // world hit t is a distance: a root entered at parameter e is no nearer
    // than e |d| (slack for rounding)
    const float dlen = sqrtf(dot(d, d)) * 0.999f;
    float ent[32];
    bool seq = false, again;
    do {
        again = false;
        best = MultiHit{{-1, 0.f, 0.f, 0.f}, -1};
        for (int g = 0; g < A.count && !again; g += 32) {
            const int m = min(32, A.count - g);
            uint32_t live = 0;
            for (int j = 0; j < m; ++j) {
                const float e = seq ? 0.0f : cull_enter(A.cull, g + j, o, inv);
                ent[j] = e;
                if (seq || (e >= 0.0f && !(best.h.id >= 0 && e * dlen > best.h.t)))
                    live |= 1u << j;
            }
            while (live) {
                int jm = __ffs(live) - 1;
                float em = ent[jm];
                for (uint32_t r = live & (live - 1); RT_INST_NEAR && r && !seq; r &= r - 1) {
                    const int j = __ffs(r) - 1;
                    if (ent[j] < em) {
                        em = ent[j];
                        jm = j;
                    }
                }
                live &= ~(1u << jm);
                if (!seq && best.h.id >= 0 && em * dlen > best.h.t) {
                    if (RT_INST_NEAR) break;   // the rest of the group enters later still
                    continue;
                }
                const int i = g + jm;
                const Hit h = root_closest(A.roots[i], o, d, tmin, tmax, A.status);
                if (!seq && h.id >= 0 && isnan(h.t)) {
                    seq = again = true;
                    break;
                }
                if (h.id >= 0 &&
                    (best.h.id < 0 || h.t < best.h.t || (h.t == best.h.t && i < best.root))) {
                    best.h = h;
                    best.root = i;
                }
            }
        }
    } while (again);
    return best;
}

__device__ __forceinline__ bool occluded_multi(const InstanceArgs& A, const rt_light& L, f3 hp) {
    f3 dir;
    if (L.type == RT_DIR_L) {
        dir = neg(mk3(L.dir[0], L.dir[1], L.dir[2]));
    } else if (L.type == RT_SPOT_L) {
        dir = normalize(sub(mk3(L.pos[0], L.pos[1], L.pos[2]), hp));
        if (dot(dir, mk3(L.dir[0], L.dir[1], L.dir[2])) < L.angle) return false;
    } else if (L.type == RT_POINT_L) {
        dir = normalize(sub(mk3(L.pos[0], L.pos[1], L.pos[2]), hp));
    } else {
        return false;
    }
    const f3 inv = mk3(1.0f / dir.x, 1.0f / dir.y, 1.0f / dir.z);
    for (int i = 0; i < A.count; ++i) {
        if (cull_enter(A.cull, i, hp, inv) < 0.0f) continue;
        const InstanceRoot& R = A.roots[i];
        const f3 td = mat_apply(R.trinv, dir, 0.0f);
        const f3 to = mat_apply(R.trinv, hp, 1.0f);
        const TRay tr = make_tray(to, td, mk3(1.0f / td.x, 1.0f / td.y, 1.0f / td.z), 0.01f);
        const BvhHeader H = *R.scene.hdr;
        if (any_hit(R.scene, H, tr, 1e37f, A.status)) return true;
    }
    return false;
}

// Surface of a multi-root hit: world point o + d t, the interpolated normal of
// the instance's mesh moved by its transform (not renormalised), turned
// against the ray.
__device__ __forceinline__ void multi_surface(const InstanceArgs& A, const MultiHit& mh, f3 o, f3 d,
                                              f3& hp, f3& n, bool& inverse_n) {
    const SceneView& S = A.roots[mh.root].scene;
    hp = add(o, muls(d, mh.h.t));
    const uint32_t* ix = S.idx + 3 * (size_t)mh.h.id;
    const f3 n0 = normalize(ld3(__ldg(&S.nrm[__ldg(ix)])));
    const f3 n1 = normalize(ld3(__ldg(&S.nrm[__ldg(ix + 1)])));
    const f3 n2 = normalize(ld3(__ldg(&S.nrm[__ldg(ix + 2)])));
    const float w = 1.0f - (mh.h.u + mh.h.v);
    n = normalize(add(add(muls(n0, w), muls(n2, mh.h.v)), muls(n1, mh.h.u)));
    n = mat_apply(A.roots[mh.root].tr, n, 0.0f);
    inverse_n = dot(n, d) > 0.0f;
    if (inverse_n) n = muls(n, -1.0f);
}

// k_render_instances: the rays of the reference's multi-root render
// (primary, then reflections up to max_bounces; one shadow ray per hit and
// light), scheduled as in the single-root pooled kernel: a warp traces 32
// primary rays of a pixel tile together, the hits' shadow rays as a dense
// list of (hit, light) tasks, and the continuing paths' reflection rays from
// a pool in shared memory, 32 at a time whichever pixels they belong to.
// Contributions are fixed-point sums per pixel (independent of order), so
// the image is the one the per-pixel loop gives.
// MAXB > 0: meshes with refracting materials: a hit continues its reflected
// and refracted rays (as k_render_pool_refr does), the pool is taken from the
// top and holds 32 (MAXB + 2) rays, enough for frames of up to MAXB bounces;
// a push past it raises RT_DEV_OVERFLOW instead of writing.
namespace {
template <int IPOOL>
struct InstPool {
    float ro[3][IPOOL], rd[3][IPOOL], rc[IPOOL];
    int rpix[IPOOL], rbounce[IPOOL];
    float hp[3][32], hn[3][32], hd[3][32], hc[32];
    int hid[32], hroot[32], hpix[32], hbounce[32];
    unsigned hmask[32];
    unsigned char hinv[32];
    uint8_t task[32 * RT_MAX_LIGHTS];   // shadow tasks that need a ray
    int pool_n;
};
}  // namespace

#ifndef RT_INST_MINB
#define RT_INST_MINB 6
#endif
template <int MAXB>
__global__ void __launch_bounds__(128, MAXB == 6 ? 5 : RT_INST_MINB) k_render_instances(InstanceArgs A) {
    constexpr int IPOOL = MAXB ? 32 * (MAXB + 2) : 64;   // reflections only: < 32 left + 32 new
    __shared__ InstanceArgs sA;
    __shared__ InstPool<IPOOL> sQ[4];
    if (threadIdx.x == 0) sA = A;
    const int lane = threadIdx.x & 31;
    InstPool<IPOOL>& Q = sQ[threadIdx.x >> 5];
    if (lane == 0) Q.pool_n = 0;
    __syncthreads();
    const int pixels = sA.width * sA.height;
    const unsigned lt = (1u << lane) - 1u;
    uint64_t n_sec = 0, n_shadow = 0, n_hits = 0, n_prim = 0;
    bool tiles = true;
    for (;;) {
        const int pn = Q.pool_n;
        bool have = false;
        f3 o = mk3(0.f, 0.f, 0.f), d = o;
        float c = 1.0f, tmin = 0.0f, tmax = 1e36f;
        int pix = 0, bounce = 0;
        if (pn >= 32 || (!tiles && pn > 0)) {
            const int k = min(32, pn);
            const int j = pn - k + lane;
            have = lane < k;
            if (have) {
                o = mk3(Q.ro[0][j], Q.ro[1][j], Q.ro[2][j]);
                d = mk3(Q.rd[0][j], Q.rd[1][j], Q.rd[2][j]);
                c = Q.rc[j];
                pix = Q.rpix[j];
                bounce = Q.rbounce[j];
                tmin = 0.0001f;
                tmax = 1e37f;
            }
            __syncwarp();
            if (lane == 0) Q.pool_n = pn - k;
        } else if (tiles) {
            int base = 0;
            if (lane == 0) base = (int)atomicAdd(sA.work_counter, 32u);
            base = __shfl_sync(0xffffffffu, base, 0);
            if (base >= pixels) {
                tiles = false;
                continue;
            }
            const int gid = base + lane;
            have = gid < pixels;
            if (have) {
                int x, y;
                pixel_of(warp_tile_order(gid, sA.width, sA.height), sA.width, sA.height, 32, x, y);
                pix = sA.width * y + x;
                o = mk3(sA.cam.pos[0], sA.cam.pos[1], sA.cam.pos[2]);
                d = primary_dir(sA.cam, x, y, sA.width, sA.height, 0.0f, 0.0f);
                ++n_prim;
            }
        } else {
            break;
        }
        MultiHit mh{{-1, 0.f, 0.f, 0.f}, -1};
        if (have) mh = closest_multi(sA, o, d, tmin, tmax);
        const bool hit_ok = mh.h.id >= 0;
        const unsigned hm = __ballot_sync(0xffffffffu, hit_ok);
        const int nh = __popc(hm);
        if (hit_ok) {
            const int k = __popc(hm & lt);
            f3 hp, n;
            bool inv;
            multi_surface(sA, mh, o, d, hp, n, inv);
            Q.hinv[k] = inv;
            Q.hp[0][k] = hp.x; Q.hp[1][k] = hp.y; Q.hp[2][k] = hp.z;
            Q.hn[0][k] = n.x; Q.hn[1][k] = n.y; Q.hn[2][k] = n.z;
            Q.hd[0][k] = d.x; Q.hd[1][k] = d.y; Q.hd[2][k] = d.z;
            Q.hc[k] = c;
            Q.hid[k] = mh.h.id;
            Q.hroot[k] = mh.root;
            Q.hpix[k] = pix;
            Q.hbounce[k] = bounce;
            Q.hmask[k] = 0u;
        }
        __syncwarp();
        const int nl = sA.lights.count;
        shadow_tasks(   // light-major, as k_render_pool
            nh, nl, Q.task,
            [&](int k, int l) {
                const SceneView& Sk = sA.roots[Q.hroot[k]].scene;
                return !light_vanishes(sA.lights.light[l], Sk.mats[__ldg(&Sk.map[Q.hid[k]])],
                                       mk3(Q.hp[0][k], Q.hp[1][k], Q.hp[2][k]),
                                       mk3(Q.hn[0][k], Q.hn[1][k], Q.hn[2][k]),
                                       mk3(Q.hd[0][k], Q.hd[1][k], Q.hd[2][k]));
            },
            [&](int k, int l) {
                if (occluded_multi(sA, sA.lights.light[l], mk3(Q.hp[0][k], Q.hp[1][k], Q.hp[2][k])))
                    atomicOr(&Q.hmask[k], 1u << l);
            });
        __syncwarp();
        bool push = false, push_t = false;
        f3 np = mk3(0.f, 0.f, 0.f), nd = np, td = np;
        float nc = 0.f, tc = 0.f;
        int npix = 0, nbounce = 0;
        if (lane < nh) {
            const int k = lane;
            const f3 p = mk3(Q.hp[0][k], Q.hp[1][k], Q.hp[2][k]);
            const f3 n = mk3(Q.hn[0][k], Q.hn[1][k], Q.hn[2][k]);
            const f3 dk = mk3(Q.hd[0][k], Q.hd[1][k], Q.hd[2][k]);
            const float ck = Q.hc[k];
            const SceneView& S = sA.roots[Q.hroot[k]].scene;
            const rt_material mat = S.mats[__ldg(&S.map[Q.hid[k]])];
            const uint3 col = shade_hit(sA.lights, mat, p, n, dk, ck, Q.hmask[k]);
            const int pk = Q.hpix[k];
            if (col.x | col.y | col.z) {   // a zero colour adds nothing
                atomicAdd(&sA.accum[3 * (size_t)pk], col.x);
                atomicAdd(&sA.accum[3 * (size_t)pk + 1], col.y);
                atomicAdd(&sA.accum[3 * (size_t)pk + 2], col.z);
            }
            ++n_hits;
            n_shadow += (uint32_t)nl;
            const int bk = Q.hbounce[k];
            if (bk < sA.max_bounces) {
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
                npix = pk;
                nbounce = bk + 1;
            }
        }
        const unsigned pm = __ballot_sync(0xffffffffu, push);
        const unsigned pt = MAXB > 0 ? __ballot_sync(0xffffffffu, push_t) : 0u;
        const int pbase = Q.pool_n;
        if (push) {
            const int j = pbase + __popc(pm & lt);
            if (MAXB == 0 || j < IPOOL) {
                Q.ro[0][j] = np.x; Q.ro[1][j] = np.y; Q.ro[2][j] = np.z;
                Q.rd[0][j] = nd.x; Q.rd[1][j] = nd.y; Q.rd[2][j] = nd.z;
                Q.rc[j] = nc;
                Q.rpix[j] = npix;
                Q.rbounce[j] = nbounce;
                ++n_sec;
            } else {
                atomicOr(sA.status, RT_DEV_OVERFLOW);
            }
        }
        if (MAXB > 0 && push_t) {
            const int j = pbase + __popc(pm) + __popc(pt & lt);
            if (j < IPOOL) {
                Q.ro[0][j] = np.x; Q.ro[1][j] = np.y; Q.ro[2][j] = np.z;
                Q.rd[0][j] = td.x; Q.rd[1][j] = td.y; Q.rd[2][j] = td.z;
                Q.rc[j] = tc;
                Q.rpix[j] = npix;
                Q.rbounce[j] = nbounce;
                ++n_sec;
            } else {
                atomicOr(sA.status, RT_DEV_OVERFLOW);
            }
        }
        __syncwarp();
        if (lane == 0) Q.pool_n = min(IPOOL, pbase + __popc(pm) + __popc(pt));
        __syncwarp();
    }
    if (sA.stats) {
        n_prim = __reduce_add_sync(0xffffffffu, (unsigned)n_prim);
        n_sec = __reduce_add_sync(0xffffffffu, (unsigned)n_sec);
        n_shadow = __reduce_add_sync(0xffffffffu, (unsigned)n_shadow);
        n_hits = __reduce_add_sync(0xffffffffu, (unsigned)n_hits);
        if (lane == 0) {
            atomicAdd((unsigned long long*)&sA.stats->primary_rays, (unsigned long long)n_prim);
            atomicAdd((unsigned long long*)&sA.stats->secondary_rays, (unsigned long long)n_sec);
            atomicAdd((unsigned long long*)&sA.stats->shadow_rays, (unsigned long long)n_shadow);
            atomicAdd((unsigned long long*)&sA.stats->hits, (unsigned long long)n_hits);
        }
    }
}

}  // namespace rt

struct rt_instances {
    std::vector<rt_scene*> scenes;
    std::vector<int32_t> inst_scene;
    std::vector<float> tr, trinv;
    rt_lights lights;
    rt::InstanceRoot* d_roots = nullptr;
    float4* d_cull = nullptr;          // 2 float4 per root, rewritten before each render
    std::vector<rt::SceneView> views;  // the scenes' buffers as the roots name them
    cudaEvent_t ev_render = nullptr;   // after the last render that read d_roots
    cudaStream_t render_stream = nullptr;
    bool rendered = false;
};

namespace {

#define fail rt::set_error

#define CU(call)                                                                              \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess)                                                                \
            return fail(RT_ERR_CUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_),  \
                        __FILE__, __LINE__);                                                  \
    } while (0)

// Rewrites the device roots on stream s once every earlier render that read
// them has finished, and returns when the copy is done.
int32_t upload_roots(rt_instances* I, cudaStream_t s) {
    if (I->rendered) CU(cudaStreamWaitEvent(s, I->ev_render, 0));
    I->views.resize(I->scenes.size());
    for (size_t k = 0; k < I->scenes.size(); ++k) I->views[k] = rt::scene_view(I->scenes[k]);
    std::vector<rt::InstanceRoot> roots(I->inst_scene.size());
    for (size_t i = 0; i < roots.size(); ++i) {
        roots[i].scene = I->views[I->inst_scene[i]];
        for (int k = 0; k < 16; ++k) {
            roots[i].tr[k] = I->tr[16 * i + k];
            roots[i].trinv[k] = I->trinv[16 * i + k];
        }
    }
    CU(cudaMemcpyAsync(I->d_roots, roots.data(), sizeof(rt::InstanceRoot) * roots.size(),
                       cudaMemcpyHostToDevice, s));
    CU(cudaStreamSynchronize(s));
    return RT_OK;
}

}  // namespace

extern "C" {

int32_t rt_instances_create(rt_ctx* c, rt_scene* const* scenes, int32_t scene_count,
                            const int32_t* inst_scene, const float* tr, const float* tr_inv,
                            int32_t count, const rt_lights* lights, rt_instances** out) {
    if (!c || !scenes || !inst_scene || !tr || !tr_inv || !lights || !out)
        return fail(RT_ERR_INVALID, "rt_instances_create: null argument");
    if (scene_count < 1 || count < 1 || count > 65536)
        return fail(RT_ERR_INVALID, "rt_instances_create: %d scenes, %d instances", scene_count,
                    count);
    if (lights->count < 1 || lights->count > RT_MAX_LIGHTS)
        return fail(RT_ERR_INVALID, "rt_instances_create: light count %d", lights->count);
    for (int k = 0; k < scene_count; ++k) {
        if (!scenes[k] || !scenes[k]->built)
            return fail(RT_ERR_NOT_BUILT, "rt_instances_create: scene %d has no BVH", k);
    }
    for (int i = 0; i < count; ++i)
        if (inst_scene[i] < 0 || inst_scene[i] >= scene_count)
            return fail(RT_ERR_INVALID, "rt_instances_create: instance %d names scene %d", i,
                        inst_scene[i]);
    rt_instances* I = new (std::nothrow) rt_instances();
    if (!I) return fail(RT_ERR_OOM, "rt_instances_create: host allocation failed");
    I->scenes.assign(scenes, scenes + scene_count);
    I->inst_scene.assign(inst_scene, inst_scene + count);
    I->tr.assign(tr, tr + 16 * (size_t)count);
    I->trinv.assign(tr_inv, tr_inv + 16 * (size_t)count);
    I->lights = *lights;
    if (cudaMalloc(&I->d_roots, sizeof(rt::InstanceRoot) * (size_t)count) != cudaSuccess ||
        cudaMalloc(&I->d_cull, 2 * sizeof(float4) * (size_t)count) != cudaSuccess) {
        cudaGetLastError();
        cudaFree(I->d_roots);
        delete I;
        return fail(RT_ERR_OOM, "rt_instances_create: device allocation failed");
    }
    const int32_t r = upload_roots(I, c->stream);
    if (r) {
        cudaFree(I->d_roots);
        cudaFree(I->d_cull);
        delete I;
        return r;
    }
    *out = I;
    return RT_OK;
}

int32_t rt_instances_set_transforms(rt_ctx* c, rt_instances* I, const float* tr,
                                    const float* tr_inv) {
    if (!c || !I || !tr || !tr_inv) return fail(RT_ERR_INVALID, "rt_instances_set_transforms: null");
    I->tr.assign(tr, tr + I->tr.size());
    I->trinv.assign(tr_inv, tr_inv + I->trinv.size());
    return upload_roots(I, c->stream);
}

int32_t rt_instances_render(rt_ctx* c, rt_instances* I, const rt_camera* cam, int32_t w, int32_t h,
                            int32_t max_bounces, uint8_t* rgba, uint32_t* img,
                            rt_render_stats* stats, rt_stream stream) {
    if (!c || !I || !cam || !rgba) return fail(RT_ERR_INVALID, "rt_instances_render: null argument");
    if (w <= 0 || h <= 0 || (int64_t)w * h > (1ll << 30) || max_bounces < 0 || max_bounces > 64)
        return fail(RT_ERR_INVALID, "rt_instances_render: bad size or depth");
    bool refracts = false;
    for (rt_scene* s : I->scenes) {
        if (!s->built) return fail(RT_ERR_NOT_BUILT, "rt_instances_render: a scene has no BVH");
        refracts = refracts || s->refracts;
    }
    // glass: both rays of a hit share the warp's pool, sized by the depth
    int kind = 0;
    void (*kern)(rt::InstanceArgs) = rt::k_render_instances<0>;
    if (refracts) {
        if (max_bounces > 6)
            return fail(RT_ERR_INVALID, "rt_instances_render: instance sets with refracting "
                        "materials render up to 6 bounces (%d asked)", max_bounces);
        kind = max_bounces <= 4 ? 1 : 2;
        kern = kind == 1 ? rt::k_render_instances<4> : rt::k_render_instances<6>;
    }
    cudaStream_t cs = stream ? (cudaStream_t)stream : c->stream;
    if (!I->ev_render) CU(cudaEventCreateWithFlags(&I->ev_render, cudaEventDisableTiming));
    uint32_t* work = rt::work_counter(c, cs);
    if (!work) return fail(RT_ERR_OOM, "rt_instances_render: work counter");
    CU(cudaMemsetAsync(work, 0, sizeof(uint32_t), cs));
    rt::InstanceArgs A;
    A.roots = I->d_roots;
    A.cull = I->d_cull;
    A.count = (int)I->inst_scene.size();
    A.lights = I->lights;
    A.cam = *cam;
    A.width = w;
    A.height = h;
    A.max_bounces = max_bounces;
    const size_t px = (size_t)w * h;
    A.accum = img ? img : rt::accum_buffer(c, cs, px);
    if (!A.accum) return fail(RT_ERR_OOM, "rt_instances_render: pixel sums");
    A.stats = stats;
    A.work_counter = work;
    A.status = c->d_status;
    A.inv1e6 = c->inv1e6;
    int& occ = c->instance_occupancy[kind];   // per context: its device's residency
    if (occ <= 0) {
        int b = 0;
        CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kern, 128, 0));
        occ = b > 0 ? b : 1;
    }
    int64_t grid = (int64_t)c->num_sms * occ;
    const int64_t useful = ((int64_t)px + 127) / 128;   // one 32-pixel tile per warp
    if (grid > useful) grid = useful;
    for (size_t k = 0; k < I->scenes.size(); ++k) {
        // a rebuild may have moved a scene's sorted buffers: name the new ones
        const rt::SceneView v = rt::scene_view(I->scenes[k]);
        if (std::memcmp(&v, &I->views[k], sizeof v) != 0) {
            const int32_t r = upload_roots(I, cs);
            if (r) return r;
            break;
        }
    }
    for (rt_scene* s : I->scenes) CU(rt::scene_read_begin(s, cs));
    // renders of one instance set share its cull boxes: they run in call order
    if (I->rendered && I->render_stream != cs) CU(cudaStreamWaitEvent(cs, I->ev_render, 0));
    rt::k_instance_boxes<<<(unsigned)((A.count + 127) / 128), 128, 0, cs>>>(I->d_roots, A.count,
                                                                            I->d_cull);
    CU(cudaMemsetAsync(A.accum, 0, 3 * sizeof(uint32_t) * px, cs));
    kern<<<(unsigned)grid, 128, 0, cs>>>(A);
    CU(cudaGetLastError());
    CU(rt::launch_fb_copy(A.accum, rgba, px, c->inv1e6, cs));
    for (rt_scene* s : I->scenes) CU(rt::scene_read_end(s, cs));
    CU(cudaEventRecord(I->ev_render, cs));
    I->render_stream = cs;
    I->rendered = true;
    return RT_OK;
}

int32_t rt_instances_destroy(rt_ctx* c, rt_instances* I) {
    if (!I) return RT_OK;
    if (c) cudaStreamSynchronize(c->stream);
    if (I->ev_render) {
        cudaEventSynchronize(I->ev_render);
        cudaEventDestroy(I->ev_render);
    }
    cudaFree(I->d_roots);
    cudaFree(I->d_cull);
    delete I;
    return RT_OK;
}

}  // extern "C"
