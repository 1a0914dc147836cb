// trace.cu — one-scene traversal, shading and ray-generation kernels for
// sm_103a (the device functions are in trace_dev.cuh).
#include <cuda_runtime.h>
#include <stdint.h>

#include "rt_internal.cuh"
#include "trace.cuh"
#include "trace_dev.cuh"

namespace rt {

// ---------------------------------------------------------------------------
// fused per-pixel Whitted path (Renderer::render_to_framebuffer, one pixel
// per lane, persistent warps fetching 32 pixels at a time)
// ---------------------------------------------------------------------------
template <int THREADS, int MINB, bool REFR = false>
__global__ void __launch_bounds__(THREADS, MINB) k_render(RenderArgs a) {
    const SceneView S = a.scene;
    __shared__ BvhHeader sH;
    __shared__ rt_lights sL;
    if (threadIdx.x == 0) sH = *S.hdr;
    for (int i = threadIdx.x; i < (int)(sizeof(rt_lights) / 4); i += blockDim.x)
        reinterpret_cast<uint32_t*>(&sL)[i] = reinterpret_cast<const uint32_t*>(&a.lights)[i];
    __syncthreads();
    const BvhHeader& H = sH;
    const int lane = threadIdx.x & 31;
    const int pixels = a.width * a.height;
    uint64_t n_sec = 0, n_shadow = 0, n_hits = 0, n_prim = 0;
    const int chunk = a.chunk;   // pixels a warp takes per fetch (multiple of 32)
    for (;;) {
        int base0 = 0;
        if (lane == 0) base0 = (int)atomicAdd(a.work_counter, (unsigned)chunk);
        base0 = __shfl_sync(0xffffffffu, base0, 0);
        if (base0 >= pixels) break;
        for (int base = base0; base < base0 + chunk && base < pixels; base += 32) {
        const int gid = base + lane;
        if (gid < pixels) {
            int x, y;
            pixel_of(warp_tile_order(gid, a.width, a.height), a.width, a.height, 32, x, y);
            const PixelResult pr = render_pixel<false, REFR>(S, H, sL, a.cam, x, y, a.width,
                                                             a.height, a.max_bounces, a.status);
            const uint32_t acc_r = pr.r, acc_g = pr.g, acc_b = pr.b;
            ++n_prim;
            n_sec += pr.secondary;
            n_shadow += pr.shadow;
            n_hits += pr.hits;
            const int pix = a.width * y + x;
            if (a.image_rgb) {
                a.image_rgb[3 * (size_t)pix] = acc_r;
                a.image_rgb[3 * (size_t)pix + 1] = acc_g;
                a.image_rgb[3 * (size_t)pix + 2] = acc_b;
            }
            uchar4 px;
            px.x = to_unorm8(acc_r, a.inv1e6);
            px.y = to_unorm8(acc_g, a.inv1e6);
            px.z = to_unorm8(acc_b, a.inv1e6);
            px.w = 255;
            reinterpret_cast<uchar4*>(a.rgba)[pix] = px;
        }
        }
    }
    if (a.stats) {
        n_prim = __reduce_add_sync(0xffffffffu, (unsigned)n_prim);
        n_sec = __reduce_add_sync(0xffffffffu, (unsigned)n_sec);
        n_shadow = __reduce_add_sync(0xffffffffu, (unsigned)n_shadow);
        n_hits = __reduce_add_sync(0xffffffffu, (unsigned)n_hits);
        if (lane == 0) {
            atomicAdd((unsigned long long*)&a.stats->primary_rays, (unsigned long long)n_prim);
            atomicAdd((unsigned long long*)&a.stats->secondary_rays, (unsigned long long)n_sec);
            atomicAdd((unsigned long long*)&a.stats->shadow_rays, (unsigned long long)n_shadow);
            atomicAdd((unsigned long long*)&a.stats->hits, (unsigned long long)n_hits);
        }
    }
}

// ---------------------------------------------------------------------------
// k_render_pool: the same rays as k_render, scheduled so that a warp's lanes
// stay busy.  A warp takes a tile of 32 pixels and traces their primary rays
// together (coherent); the hits' shadow rays are traced as a dense list of
// (hit, light) tasks; each hit is shaded and, if the path continues, its
// reflection ray goes into the warp's pool in shared memory, which is traced
// 32 rays at a time whichever pixels they come from.  A pixel's fixed-point
// contributions are added into its accumulator (integer sums do not depend
// on order) and k_fb_copy turns the sums into RGBA8 afterwards.  Every ray is
// traversed and shaded exactly as in render_pixel, so the image is
// bit-identical to k_render's.
// ---------------------------------------------------------------------------
namespace {
constexpr int POOL = 64;   // reflection rays a warp can hold: < 32 left + 32 new

struct WarpPool {
    float ro[3][POOL], rd[3][POOL], rc[POOL];   // pooled rays: origin, direction, contribution
    int rpix[POOL], rbounce[POOL];
    float hp[3][32], hn[3][32], hd[3][32], hc[32];   // hits of the current step
    int hid[32], hpix[32], hbounce[32];
    unsigned hmask[32];
    uint8_t task[32 * RT_MAX_LIGHTS];   // shadow tasks that need a ray
    int pool_n;
};
}  // namespace

template <int THREADS, int MINB>
__global__ void __launch_bounds__(THREADS, MINB) k_render_pool(RenderArgs a) {
    const SceneView S = a.scene;
    __shared__ BvhHeader sH;
    __shared__ rt_lights sL;
    __shared__ WarpPool sQ[THREADS / 32];
    if (threadIdx.x == 0) sH = *S.hdr;
    for (int i = threadIdx.x; i < (int)(sizeof(rt_lights) / 4); i += blockDim.x)
        reinterpret_cast<uint32_t*>(&sL)[i] = reinterpret_cast<const uint32_t*>(&a.lights)[i];
    const int lane = threadIdx.x & 31;
    WarpPool& Q = sQ[threadIdx.x >> 5];
    if (lane == 0) Q.pool_n = 0;
    __syncthreads();
    const BvhHeader& H = sH;
    const int pixels = a.width * a.height;
    const unsigned lt = (1u << lane) - 1u;
    uint64_t n_sec = 0, n_shadow = 0, n_hits = 0, n_prim = 0;
    bool tiles = true;
    for (;;) {
        const int pn = Q.pool_n;
        // 1. rays to trace: a full batch from the pool, else a new tile
        //    of primary rays, else what is left in the pool
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
            if (lane == 0) base = (int)atomicAdd(a.work_counter, 32u);
            base = __shfl_sync(0xffffffffu, base, 0);
            if (base >= pixels) {
                tiles = false;
                continue;
            }
            const int gid = base + lane;
            have = gid < pixels;
            if (have) {
                int x, y;
                pixel_of(warp_tile_order(gid, a.width, a.height), a.width, a.height, 32, x, y);
                pix = a.width * y + x;
                o = mk3(a.cam.pos[0], a.cam.pos[1], a.cam.pos[2]);
                d = primary_dir(a.cam, x, y, a.width, a.height, 0.0f, 0.0f);
                ++n_prim;
            }
        } else {
            break;
        }
        // 2. closest hits; the hits are listed in the warp's hit slots
        bool hit_ok = false;
        Hit hit{-1, 0.f, 0.f, 0.f};
        if (have) {
            const TRay r = make_tray(o, d, mk3(1.0f / d.x, 1.0f / d.y, 1.0f / d.z), tmin);
            hit = closest_hit(S, H, r, tmax, a.status);
            hit_ok = hit.id >= 0;
        }
        const unsigned hm = __ballot_sync(0xffffffffu, hit_ok);
        const int nh = __popc(hm);
        if (hit_ok) {
            const int k = __popc(hm & lt);
            const HitInfo hi = complete_hit(S, o, d, hit);
            Q.hp[0][k] = hi.hp.x; Q.hp[1][k] = hi.hp.y; Q.hp[2][k] = hi.hp.z;
            Q.hn[0][k] = hi.n.x; Q.hn[1][k] = hi.n.y; Q.hn[2][k] = hi.n.z;
            Q.hd[0][k] = d.x; Q.hd[1][k] = d.y; Q.hd[2][k] = d.z;
            Q.hc[k] = c;
            Q.hid[k] = hit.id;
            Q.hpix[k] = pix;
            Q.hbounce[k] = bounce;
            Q.hmask[k] = 0u;
        }
        __syncwarp();
        // 3. shadow rays of every hit and light, 32 at a time
        const int nl = sL.count;
        // light-major (shadow_tasks): neighbouring lanes trace toward the same
        // light from neighbouring hits (coherent paths: 3 % faster on the
        // mid-scale frame with 2 lights, 10 % on the stress pose with 3, than
        // a hit's lights on neighbouring lanes); the tasks that need a ray
        // are traced densely
        shadow_tasks(
            nh, nl, Q.task,
            [&](int k, int l) {
                return !light_vanishes(sL.light[l], S.mats[__ldg(&S.map[Q.hid[k]])],
                                       mk3(Q.hp[0][k], Q.hp[1][k], Q.hp[2][k]),
                                       mk3(Q.hn[0][k], Q.hn[1][k], Q.hn[2][k]),
                                       mk3(Q.hd[0][k], Q.hd[1][k], Q.hd[2][k]));
            },
            [&](int k, int l) {
                if (occluded(S, H, sL.light[l], mk3(Q.hp[0][k], Q.hp[1][k], Q.hp[2][k]), a.status))
                    atomicOr(&Q.hmask[k], 1u << l);
            });
        __syncwarp();
        // 4. shading; continuing paths put their reflection ray into the pool
        bool push = false;
        f3 np = mk3(0.f, 0.f, 0.f), nd = np;
        float nc = 0.f;
        int npix = 0, nbounce = 0;
        if (lane < nh) {
            const int k = lane;
            const f3 p = mk3(Q.hp[0][k], Q.hp[1][k], Q.hp[2][k]);
            const f3 n = mk3(Q.hn[0][k], Q.hn[1][k], Q.hn[2][k]);
            const f3 dk = mk3(Q.hd[0][k], Q.hd[1][k], Q.hd[2][k]);
            const float ck = Q.hc[k];
            const rt_material mat = S.mats[__ldg(&S.map[Q.hid[k]])];
            const uint3 col = shade_hit(sL, mat, p, n, dk, ck, Q.hmask[k]);
            const int pk = Q.hpix[k];
            if (col.x | col.y | col.z) {   // a zero colour adds nothing
                atomicAdd(&a.accum[3 * (size_t)pk], col.x);
                atomicAdd(&a.accum[3 * (size_t)pk + 1], col.y);
                atomicAdd(&a.accum[3 * (size_t)pk + 2], col.z);
            }
            ++n_hits;
            n_shadow += (uint32_t)nl;
            const int bk = Q.hbounce[k];
            if (bk != a.max_bounces && mat.reflectiveness > 0.0f) {
                reflect_ray(dk, n, nd);
                np = p;
                nc = ck * mat.reflectiveness * 1.0f;
                npix = pk;
                nbounce = bk + 1;
                push = true;
                ++n_sec;
            }
        }
        const unsigned pm = __ballot_sync(0xffffffffu, push);
        const int pbase = Q.pool_n;
        if (push) {
            const int j = pbase + __popc(pm & lt);
            Q.ro[0][j] = np.x; Q.ro[1][j] = np.y; Q.ro[2][j] = np.z;
            Q.rd[0][j] = nd.x; Q.rd[1][j] = nd.y; Q.rd[2][j] = nd.z;
            Q.rc[j] = nc;
            Q.rpix[j] = npix;
            Q.rbounce[j] = nbounce;
        }
        __syncwarp();
        if (lane == 0) Q.pool_n = pbase + __popc(pm);
        __syncwarp();
    }
    if (a.stats) {
        n_prim = __reduce_add_sync(0xffffffffu, (unsigned)n_prim);
        n_sec = __reduce_add_sync(0xffffffffu, (unsigned)n_sec);
        n_shadow = __reduce_add_sync(0xffffffffu, (unsigned)n_shadow);
        n_hits = __reduce_add_sync(0xffffffffu, (unsigned)n_hits);
        if (lane == 0) {
            atomicAdd((unsigned long long*)&a.stats->primary_rays, (unsigned long long)n_prim);
            atomicAdd((unsigned long long*)&a.stats->secondary_rays, (unsigned long long)n_sec);
            atomicAdd((unsigned long long*)&a.stats->shadow_rays, (unsigned long long)n_shadow);
            atomicAdd((unsigned long long*)&a.stats->hits, (unsigned long long)n_hits);
        }
    }
}

// ---------------------------------------------------------------------------
// k_render_pool_refr: k_render_pool for scenes with refracting materials.  A
// hit may continue two rays (the refracted one, contribution * reflectiveness
// * (1 - R), and the reflected one, * R, as generate_secondary_rays_disc
// makes them), and both go into the warp's pool.  The pool is taken from the
// top (last in, first out), so it holds at most 32 (max_bounces + 2) rays;
// it is sized for max_bounces <= MAXB (deeper frames use a larger pool or
// the ray-tree variant) and a push beyond it raises RT_DEV_OVERFLOW instead
// of writing.  Sums are integers, so the image is the ray-tree variant's.
// ---------------------------------------------------------------------------
namespace {
template <int RPOOL>
struct RefrPool {
    float ro[3][RPOOL], rd[3][RPOOL], rc[RPOOL];
    int rpix[RPOOL], rbounce[RPOOL];
    float hp[3][32], hn[3][32], hd[3][32], hc[32];
    int hid[32], hpix[32], hbounce[32];
    unsigned hmask[32];
    unsigned char hinv[32];
    uint8_t task[32 * RT_MAX_LIGHTS];   // shadow tasks that need a ray
    int pool_n;
};
}  // namespace

template <int THREADS, int MINB, int MAXB>
__global__ void __launch_bounds__(THREADS, MINB) k_render_pool_refr(RenderArgs a) {
    constexpr int RPOOL = 32 * (MAXB + 2);
    const SceneView S = a.scene;
    __shared__ BvhHeader sH;
    __shared__ rt_lights sL;
    __shared__ RefrPool<RPOOL> sQ[THREADS / 32];
    if (threadIdx.x == 0) sH = *S.hdr;
    for (int i = threadIdx.x; i < (int)(sizeof(rt_lights) / 4); i += blockDim.x)
        reinterpret_cast<uint32_t*>(&sL)[i] = reinterpret_cast<const uint32_t*>(&a.lights)[i];
    const int lane = threadIdx.x & 31;
    RefrPool<RPOOL>& Q = sQ[threadIdx.x >> 5];
    if (lane == 0) Q.pool_n = 0;
    __syncthreads();
    const BvhHeader& H = sH;
    const int pixels = a.width * a.height;
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
            if (lane == 0) base = (int)atomicAdd(a.work_counter, 32u);
            base = __shfl_sync(0xffffffffu, base, 0);
            if (base >= pixels) {
                tiles = false;
                continue;
            }
            const int gid = base + lane;
            have = gid < pixels;
            if (have) {
                int x, y;
                pixel_of(warp_tile_order(gid, a.width, a.height), a.width, a.height, 32, x, y);
                pix = a.width * y + x;
                o = mk3(a.cam.pos[0], a.cam.pos[1], a.cam.pos[2]);
                d = primary_dir(a.cam, x, y, a.width, a.height, 0.0f, 0.0f);
                ++n_prim;
            }
        } else {
            break;
        }
        bool hit_ok = false;
        Hit hit{-1, 0.f, 0.f, 0.f};
        if (have) {
            const TRay r = make_tray(o, d, mk3(1.0f / d.x, 1.0f / d.y, 1.0f / d.z), tmin);
            hit = closest_hit(S, H, r, tmax, a.status);
            hit_ok = hit.id >= 0;
        }
        const unsigned hm = __ballot_sync(0xffffffffu, hit_ok);
        const int nh = __popc(hm);
        if (hit_ok) {
            const int k = __popc(hm & lt);
            const HitInfo hi = complete_hit(S, o, d, hit);
            Q.hp[0][k] = hi.hp.x; Q.hp[1][k] = hi.hp.y; Q.hp[2][k] = hi.hp.z;
            Q.hn[0][k] = hi.n.x; Q.hn[1][k] = hi.n.y; Q.hn[2][k] = hi.n.z;
            Q.hd[0][k] = d.x; Q.hd[1][k] = d.y; Q.hd[2][k] = d.z;
            Q.hc[k] = c;
            Q.hid[k] = hit.id;
            Q.hpix[k] = pix;
            Q.hbounce[k] = bounce;
            Q.hinv[k] = hi.inverse_n;
            Q.hmask[k] = 0u;
        }
        __syncwarp();
        const int nl = sL.count;
        shadow_tasks(
            nh, nl, Q.task,
            [&](int k, int l) {
                return !light_vanishes(sL.light[l], S.mats[__ldg(&S.map[Q.hid[k]])],
                                       mk3(Q.hp[0][k], Q.hp[1][k], Q.hp[2][k]),
                                       mk3(Q.hn[0][k], Q.hn[1][k], Q.hn[2][k]),
                                       mk3(Q.hd[0][k], Q.hd[1][k], Q.hd[2][k]));
            },
            [&](int k, int l) {
                if (occluded(S, H, sL.light[l], mk3(Q.hp[0][k], Q.hp[1][k], Q.hp[2][k]), a.status))
                    atomicOr(&Q.hmask[k], 1u << l);
            });
        __syncwarp();
        // shading; the continuing rays of each hit: reflected, refracted
        bool push_r = false, push_t = false;
        f3 np = mk3(0.f, 0.f, 0.f), nd = np, td = np;
        float nc = 0.f, tc = 0.f;
        int npix = 0, nbounce = 0;
        if (lane < nh) {
            const int k = lane;
            const f3 p = mk3(Q.hp[0][k], Q.hp[1][k], Q.hp[2][k]);
            const f3 n = mk3(Q.hn[0][k], Q.hn[1][k], Q.hn[2][k]);
            const f3 dk = mk3(Q.hd[0][k], Q.hd[1][k], Q.hd[2][k]);
            const float ck = Q.hc[k];
            const rt_material mat = S.mats[__ldg(&S.map[Q.hid[k]])];
            const uint3 col = shade_hit(sL, mat, p, n, dk, ck, Q.hmask[k]);
            const int pk = Q.hpix[k];
            if (col.x | col.y | col.z) {   // a zero colour adds nothing
                atomicAdd(&a.accum[3 * (size_t)pk], col.x);
                atomicAdd(&a.accum[3 * (size_t)pk + 1], col.y);
                atomicAdd(&a.accum[3 * (size_t)pk + 2], col.z);
            }
            ++n_hits;
            n_shadow += (uint32_t)nl;
            const int bk = Q.hbounce[k];
            if (bk < a.max_bounces) {
                float R = 1.0f;
                if (mat.refractive_index > 0.0f &&
                    refract_ray(dk, n, Q.hinv[k] != 0, mat.refractive_index, R, td)) {
                    tc = ck * mat.reflectiveness * (1.0f - R);
                    push_t = true;
                }
                if (mat.reflectiveness > 0.0f) {
                    reflect_ray(dk, n, nd);
                    nc = ck * mat.reflectiveness * R;
                    push_r = true;
                }
                np = p;
                npix = pk;
                nbounce = bk + 1;
            }
        }
        const unsigned pr = __ballot_sync(0xffffffffu, push_r);
        const unsigned pt = __ballot_sync(0xffffffffu, push_t);
        const int pbase = Q.pool_n;
        if (push_r) {
            const int j = pbase + __popc(pr & lt);
            if (j < RPOOL) {
                Q.ro[0][j] = np.x; Q.ro[1][j] = np.y; Q.ro[2][j] = np.z;
                Q.rd[0][j] = nd.x; Q.rd[1][j] = nd.y; Q.rd[2][j] = nd.z;
                Q.rc[j] = nc;
                Q.rpix[j] = npix;
                Q.rbounce[j] = nbounce;
                ++n_sec;
            } else {
                atomicOr(a.status, RT_DEV_OVERFLOW);
            }
        }
        if (push_t) {
            const int j = pbase + __popc(pr) + __popc(pt & lt);
            if (j < RPOOL) {
                Q.ro[0][j] = np.x; Q.ro[1][j] = np.y; Q.ro[2][j] = np.z;
                Q.rd[0][j] = td.x; Q.rd[1][j] = td.y; Q.rd[2][j] = td.z;
                Q.rc[j] = tc;
                Q.rpix[j] = npix;
                Q.rbounce[j] = nbounce;
                ++n_sec;
            } else {
                atomicOr(a.status, RT_DEV_OVERFLOW);
            }
        }
        __syncwarp();
        if (lane == 0) Q.pool_n = min(RPOOL, pbase + __popc(pr) + __popc(pt));
        __syncwarp();
    }
    if (a.stats) {
        n_prim = __reduce_add_sync(0xffffffffu, (unsigned)n_prim);
        n_sec = __reduce_add_sync(0xffffffffu, (unsigned)n_sec);
        n_shadow = __reduce_add_sync(0xffffffffu, (unsigned)n_shadow);
        n_hits = __reduce_add_sync(0xffffffffu, (unsigned)n_hits);
        if (lane == 0) {
            atomicAdd((unsigned long long*)&a.stats->primary_rays, (unsigned long long)n_prim);
            atomicAdd((unsigned long long*)&a.stats->secondary_rays, (unsigned long long)n_sec);
            atomicAdd((unsigned long long*)&a.stats->shadow_rays, (unsigned long long)n_shadow);
            atomicAdd((unsigned long long*)&a.stats->hits, (unsigned long long)n_hits);
        }
    }
}

// ---------------------------------------------------------------------------
// stage-wise kernels on reference-layout buffers
// ---------------------------------------------------------------------------
__global__ void k_gen_primary(rt_camera cam, int w, int h, int q, const rt_pixel_sample* ps,
                              size_t count, size_t offset, rt_sample* out) {
    const size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (k >= count) return;
    const int gid = (int)(offset + k);
    const int pixels = w * h;
    rt_pixel_sample p = {0.f, 0.f, 1.f};
    if (ps) p = ps[gid / pixels];
    int x, y;
    pixel_of(gid, w, h, q, x, y);
    const f3 d = primary_dir(cam, x, y, w, h, p.ox, p.oy);
    rt_sample s;
    s.ray.ori[0] = cam.pos[0];
    s.ray.ori[1] = cam.pos[1];
    s.ray.ori[2] = cam.pos[2];
    s.ray.ori[3] = 0.f;
    s.ray.dir[0] = d.x;
    s.ray.dir[1] = d.y;
    s.ray.dir[2] = d.z;
    s.ray.dir[3] = 0.f;
    s.ray.inv_dir[0] = 1.0f / d.x;
    s.ray.inv_dir[1] = 1.0f / d.y;
    s.ray.inv_dir[2] = 1.0f / d.z;
    s.ray.inv_dir[3] = 0.f;
    s.ray.tmin = 0.0f;
    s.ray.tmax = 1e36f;
    s.ray._pad[0] = s.ray._pad[1] = 0.f;
    s.pixel = w * y + x;
    s.contribution = p.contribution;
    s._pad[0] = s._pad[1] = 0;
    out[k] = s;
}

__device__ __forceinline__ f3 f3_of(const float* v) { return mk3(v[0], v[1], v[2]); }

__global__ void __launch_bounds__(128) k_trace(SceneView S, const rt_sample* __restrict__ smp,
                                               int n, rt_hit* __restrict__ hits,
                                               uint32_t* status) {
    __shared__ BvhHeader sH;
    if (threadIdx.x == 0) sH = *S.hdr;
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const rt_ray& ray = smp[i].ray;
    const f3 o = f3_of(ray.ori), d = f3_of(ray.dir);
    const TRay r = make_tray(o, d, f3_of(ray.inv_dir), ray.tmin);
    const Hit h = closest_hit(S, sH, r, ray.tmax, status);
    if (h.id < 0) {
        hits[i].hit = 0;
        return;
    }
    const HitInfo hi = complete_hit(S, o, d, h);
    rt_hit out;
    out.hit = 1;
    out.shadow_hit = hits[i].shadow_hit;
    out.inverse_n = hi.inverse_n;
    out.reserved = 0;
    out.t = h.t;
    out.id = h.id;
    out._pad0 = 0.f;
    out.uv[0] = out.uv[1] = 0.f;
    out._pad1[0] = out._pad1[1] = 0.f;
    out.n[0] = hi.n.x;
    out.n[1] = hi.n.y;
    out.n[2] = hi.n.z;
    out.n[3] = 0.f;
    out.hit_point[0] = hi.hp.x;
    out.hit_point[1] = hi.hp.y;
    out.hit_point[2] = hi.hp.z;
    out.hit_point[3] = 0.f;
    hits[i] = out;
}

__global__ void __launch_bounds__(128) k_shadow(SceneView S, rt_lights Ls, int n,
                                                rt_hit* __restrict__ hits, uint32_t* status) {
    __shared__ BvhHeader sH;
    if (threadIdx.x == 0) sH = *S.hdr;
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (!hits[i].hit) return;
    const f3 hp = f3_of(hits[i].hit_point);
    uint32_t mask = 0;
    for (int l = 0; l < Ls.count; ++l)
        if (occluded(S, sH, Ls.light[l], hp, status)) mask |= 1u << l;
    hits[i].shadow_hit = (uint8_t)mask;
}

__global__ void k_shade(SceneView S, rt_lights Ls, const rt_sample* __restrict__ smp,
                        const rt_hit* __restrict__ hits, int n, uint32_t* __restrict__ image) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const rt_hit& h = hits[i];
    if (!h.hit) return;
    const rt_material mat = S.mats[__ldg(&S.map[h.id])];
    const uint3 c = shade_hit(Ls, mat, f3_of(h.hit_point), f3_of(h.n), f3_of(smp[i].ray.dir),
                              smp[i].contribution, h.shadow_hit);
    uint32_t* px = image + 3 * (size_t)smp[i].pixel;
    atomicAdd(px, c.x);
    atomicAdd(px + 1, c.y);
    atomicAdd(px + 2, c.z);
}

// Secondary generation (the reference's mark / scan / generate of
// generate_secondary_rays_disc): flags -> per-block counts -> block offsets
// -> emit, in input order.  Reflected rays take the first slots, refracted
// rays the slots after all of them; a ray whose slot is at or beyond max_out
// is dropped, and a hit whose refracted slot is beyond it keeps R = 1 for its
// reflected ray, as in the kernel.
__device__ __forceinline__ void sec_flags(const SceneView& S, const rt_sample& smp, const rt_hit& h,
                                          bool& refl, bool& refr, rt_material& mat) {
    refl = refr = false;
    if (!h.hit) return;
    mat = S.mats[__ldg(&S.map[h.id])];
    refl = mat.reflectiveness > 0.0f;
    if (mat.refractive_index > 0.0f) {
        float R;
        f3 td;
        refr = refract_ray(f3_of(smp.ray.dir), f3_of(h.n), h.inverse_n != 0, mat.refractive_index,
                           R, td);
    }
}

// block_counts[b] = reflected rays of block b, block_counts[nb + b] =
// refracted ones; the scan over the 2 nb entries gives both slot bases.
__global__ void k_sec_count(SceneView S, const rt_sample* __restrict__ in,
                            const rt_hit* __restrict__ hits, int n,
                            uint32_t* __restrict__ block_counts) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    bool refl = false, refr = false;
    rt_material mat;
    if (i < n) sec_flags(S, in[i], hits[i], refl, refr, mat);
    const int cr = __syncthreads_count(refl);
    const int ct = __syncthreads_count(refr);
    if (threadIdx.x == 0) {
        block_counts[blockIdx.x] = (uint32_t)cr;
        block_counts[gridDim.x + blockIdx.x] = (uint32_t)ct;
    }
}

__global__ void k_sec_scan(uint32_t* __restrict__ block_counts, int nblocks, int max_out,
                           int32_t* __restrict__ d_count) {
    // single block, sequential chunks of 1024
    __shared__ uint32_t s[1024];
    __shared__ uint32_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int b0 = 0; b0 < nblocks; b0 += 1024) {
        const int i = b0 + threadIdx.x;
        const uint32_t v = i < nblocks ? block_counts[i] : 0;
        s[threadIdx.x] = v;
        __syncthreads();
        for (int off = 1; off < 1024; off <<= 1) {
            const uint32_t t = threadIdx.x >= (unsigned)off ? s[threadIdx.x - off] : 0;
            __syncthreads();
            s[threadIdx.x] += t;
            __syncthreads();
        }
        if (i < nblocks) block_counts[i] = carry + s[threadIdx.x] - v;
        __syncthreads();
        if (threadIdx.x == 0) carry += s[1023];
        __syncthreads();
    }
    if (threadIdx.x == 0) *d_count = (int32_t)min(carry, (uint32_t)max_out);
}

__device__ __forceinline__ rt_sample sec_sample(const rt_hit& h, f3 dir, int pixel,
                                                float contribution) {
    rt_sample o;
    o.ray.ori[0] = h.hit_point[0];
    o.ray.ori[1] = h.hit_point[1];
    o.ray.ori[2] = h.hit_point[2];
    o.ray.ori[3] = 0.f;
    o.ray.dir[0] = dir.x;
    o.ray.dir[1] = dir.y;
    o.ray.dir[2] = dir.z;
    o.ray.dir[3] = 0.f;
    o.ray.inv_dir[0] = 1.0f / dir.x;
    o.ray.inv_dir[1] = 1.0f / dir.y;
    o.ray.inv_dir[2] = 1.0f / dir.z;
    o.ray.inv_dir[3] = 0.f;
    o.ray.tmin = 0.0001f;
    o.ray.tmax = 1e37f;
    o.ray._pad[0] = o.ray._pad[1] = 0.f;
    o.pixel = pixel;
    o.contribution = contribution;
    o._pad[0] = o._pad[1] = 0;
    return o;
}

__global__ void k_sec_emit(SceneView S, const rt_sample* __restrict__ in,
                           const rt_hit* __restrict__ hits, int n,
                           const uint32_t* __restrict__ block_offsets, rt_sample* __restrict__ out,
                           int max_out) {
    __shared__ uint32_t warp_tot[2][32];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    bool refl = false, refr = false;
    rt_material mat;
    if (i < n) sec_flags(S, in[i], hits[i], refl, refr, mat);
    const unsigned bal_l = __ballot_sync(0xffffffffu, refl);
    const unsigned bal_t = __ballot_sync(0xffffffffu, refr);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) {
        warp_tot[0][w] = __popc(bal_l);
        warp_tot[1][w] = __popc(bal_t);
    }
    __syncthreads();
    if (!refl && !refr) return;
    uint32_t wl = 0, wt = 0;
    for (int k = 0; k < w; ++k) {
        wl += warp_tot[0][k];
        wt += warp_tot[1][k];
    }
    const uint32_t below = (1u << lane) - 1u;
    const uint32_t slot_l = block_offsets[blockIdx.x] + wl + __popc(bal_l & below);
    const uint32_t slot_t = block_offsets[gridDim.x + blockIdx.x] + wt + __popc(bal_t & below);
    const rt_hit& h = hits[i];
    const rt_sample& smp = in[i];
    float R = 1.0f;
    if (refr && slot_t < (uint32_t)max_out) {
        f3 td;
        refract_ray(f3_of(smp.ray.dir), f3_of(h.n), h.inverse_n != 0, mat.refractive_index, R, td);
        out[slot_t] = sec_sample(h, td, smp.pixel, smp.contribution * mat.reflectiveness * (1.0f - R));
    }
    if (refl && slot_l < (uint32_t)max_out) {
        f3 dir;
        reflect_ray(f3_of(smp.ray.dir), f3_of(h.n), dir);
        out[slot_l] = sec_sample(h, dir, smp.pixel, smp.contribution * mat.reflectiveness * R);
    }
}

__global__ void k_fb_copy(const uint32_t* __restrict__ img, uchar4* __restrict__ rgba, size_t px,
                          float inv1e6) {
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= px) return;
    uchar4 o;
    o.x = to_unorm8(img[3 * i], inv1e6);
    o.y = to_unorm8(img[3 * i + 1], inv1e6);
    o.z = to_unorm8(img[3 * i + 2], inv1e6);
    o.w = 255;
    rgba[i] = o;
}

// ---------------------------------------------------------------------------
// host launchers
// ---------------------------------------------------------------------------
static unsigned blocks(size_t n, int t) { return (unsigned)((n + t - 1) / t); }

// Kernel variants the autotuner chooses from: block size x minimum resident
// blocks per SM (which bounds the registers per thread).
struct RenderVariant {
    int threads, min_blocks;
    void (*fn)(RenderArgs);
    bool pooled;
    bool refract;     // follows the refracted rays of refracting materials
    int max_bounces;  // deepest frame it holds (0: any)
};
static const RenderVariant kVariants[] = {
    {64, 8, k_render<64, 8>, false},    {64, 12, k_render<64, 12>, false},
    {128, 4, k_render<128, 4>, false},  {128, 6, k_render<128, 6>, false},
    {128, 8, k_render<128, 8>, false},  {256, 2, k_render<256, 2>, false},
    {256, 3, k_render<256, 3>, false},  {256, 4, k_render<256, 4>, false},
    {128, 6, k_render_pool<128, 6>, true}, {128, 8, k_render_pool<128, 8>, true},
    {256, 3, k_render_pool<256, 3>, true}, {256, 4, k_render_pool<256, 4>, true},
    {128, 6, k_render<128, 6, true>, false, true},
    {128, 4, k_render_pool_refr<128, 4, 6>, true, true, 6},
    {128, 5, k_render_pool_refr<128, 5, 4>, true, true, 4},
};
constexpr int kNumVariants = sizeof(kVariants) / sizeof(kVariants[0]);
static_assert(kNumVariants <= kMaxRenderVariants, "per-variant context arrays");

int render_variant_count() { return kNumVariants; }

int render_variant_info(int v, int* threads, int* min_blocks, const void** fn) {
    if (v < 0 || v >= kNumVariants) return -1;
    if (threads) *threads = kVariants[v].threads;
    if (min_blocks) *min_blocks = kVariants[v].min_blocks;
    if (fn) *fn = (const void*)kVariants[v].fn;
    return 0;
}

bool render_variant_pooled(int v) { return v >= 0 && v < kNumVariants && kVariants[v].pooled; }

bool render_variant_refracts(int v) { return v >= 0 && v < kNumVariants && kVariants[v].refract; }

bool render_variant_fits(int v, int max_bounces) {
    if (v < 0 || v >= kNumVariants) return false;
    return kVariants[v].max_bounces == 0 || max_bounces <= kVariants[v].max_bounces;
}

int render_refract_variant(int max_bounces) {
    // the pooled variant with the smallest pool that holds the frame, else
    // the ray-tree walk
    int best = -1;
    for (int v = 0; v < kNumVariants; ++v) {
        if (!kVariants[v].refract || !render_variant_fits(v, max_bounces)) continue;
        if (best < 0 || (kVariants[v].pooled && (!kVariants[best].pooled ||
                                                 kVariants[v].max_bounces < kVariants[best].max_bounces)))
            best = v;
    }
    return best;
}

cudaError_t launch_render(const RenderArgs& a, int variant, int grid, cudaStream_t s) {
    if (variant < 0 || variant >= kNumVariants) return cudaErrorInvalidValue;
    const size_t px = (size_t)a.width * a.height;
    if (kVariants[variant].pooled) {
        if (!a.accum) return cudaErrorInvalidValue;
        cudaError_t e = cudaMemsetAsync(a.accum, 0, 3 * sizeof(uint32_t) * px, s);
        if (e != cudaSuccess) return e;
    }
    kVariants[variant].fn<<<grid, kVariants[variant].threads, 0, s>>>(a);
    if (kVariants[variant].pooled && px)
        k_fb_copy<<<blocks(px, 256), 256, 0, s>>>(a.accum, reinterpret_cast<uchar4*>(a.rgba), px,
                                                  a.inv1e6);
    return cudaGetLastError();
}

cudaError_t launch_gen_primary(const rt_camera& cam, int w, int h, int q, const rt_pixel_sample* ps,
                               size_t count, size_t offset, rt_sample* out, cudaStream_t s) {
    if (count == 0) return cudaSuccess;
    k_gen_primary<<<blocks(count, 256), 256, 0, s>>>(cam, w, h, q, ps, count, offset, out);
    return cudaGetLastError();
}

cudaError_t launch_trace(const SceneView& S, const rt_sample* smp, int n, rt_hit* hits,
                         uint32_t* status, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    k_trace<<<blocks(n, 128), 128, 0, s>>>(S, smp, n, hits, status);
    return cudaGetLastError();
}

cudaError_t launch_shadow(const SceneView& S, const rt_lights& L, int n, rt_hit* hits,
                          uint32_t* status, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    k_shadow<<<blocks(n, 128), 128, 0, s>>>(S, L, n, hits, status);
    return cudaGetLastError();
}

cudaError_t launch_shade(const SceneView& S, const rt_lights& L, const rt_sample* smp,
                         const rt_hit* hits, int n, uint32_t* image, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    k_shade<<<blocks(n, 128), 128, 0, s>>>(S, L, smp, hits, n, image);
    return cudaGetLastError();
}

cudaError_t launch_gen_secondary(const SceneView& S, const rt_sample* in, int n, const rt_hit* hits,
                                 rt_sample* out, int max_out, int32_t* d_count,
                                 uint32_t* block_scratch, cudaStream_t s) {
    if (n <= 0) return cudaMemsetAsync(d_count, 0, sizeof(int32_t), s);
    const int nb = (int)blocks(n, 256);
    k_sec_count<<<nb, 256, 0, s>>>(S, in, hits, n, block_scratch);
    k_sec_scan<<<1, 1024, 0, s>>>(block_scratch, 2 * nb, max_out, d_count);
    k_sec_emit<<<nb, 256, 0, s>>>(S, in, hits, n, block_scratch, out, max_out);
    return cudaGetLastError();
}

cudaError_t launch_fb_copy(const uint32_t* img, uint8_t* rgba, size_t px, float inv1e6,
                           cudaStream_t s) {
    if (px == 0) return cudaSuccess;
    k_fb_copy<<<blocks(px, 256), 256, 0, s>>>(img, reinterpret_cast<uchar4*>(rgba), px, inv1e6);
    return cudaGetLastError();
}

size_t gen_secondary_scratch_bytes(int n) { return sizeof(uint32_t) * (2 * blocks(n, 256) + 1); }

}  // namespace rt
