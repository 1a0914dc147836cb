// trace.cu — traversal, shading and ray generation for sm_103a.
//
// Device functions restate, in the reference's operation order:
//   closest_hit   trace_ray / leaf_hit / bbox_hit (src/kernel/trace-bvh.cl:247-417)
//   any_hit       trace_shadow_ray / leaf_hit_any (src/kernel/shadow-trace-bvh.cl:160-315)
//   complete_hit  complete_trace_info (trace-bvh.cl:190-245)
//   shade_hit     shade_sample (src/kernel/ray-shader.cl:116-333), untextured
//   reflect       generate_secondary_rays_disc reflection branch
//                 (src/kernel/secondary-ray-generator.cl:258-270)
//   primary_ray   generate_primary_rays (src/kernel/primary-ray-generator.cl:27-103)
//
// Traversal order is the reference's: depth first, near child first where
// near = left iff dot(dir, right.lo - left.lo) > 0 (trace-bvh.cl:391-409).
// Both child boxes are tested when their parent is visited; the far child is
// pushed with its entry distance A, and popped only if A <= the current tMax.
// Because tMax only shrinks, this accepts exactly the nodes the reference
// accepts when it tests the far child's box at pop time, so leaves are
// visited in the same order and equal-t ties resolve the same way.
#include <cuda_runtime.h>
#include <stdint.h>

#include "rt_internal.cuh"
#include "trace.cuh"

namespace rt {

constexpr int STACK = 32;

struct Hit {
    int32_t id;
    float t, u, v;
};

__device__ __forceinline__ void load_node(const float4* __restrict__ nodes, int32_t p, float4& n0,
                                          float4& n1, float4& n2, int4& n3) {
    const float4* q = nodes + 4 * (size_t)p;
    n0 = __ldg(q);
    n1 = __ldg(q + 1);
    n2 = __ldg(q + 2);
    n3 = __ldg(reinterpret_cast<const int4*>(q + 3));
}

__device__ __forceinline__ void leaf_closest(const SceneView& S, const TRay& r, int32_t start,
                                             int32_t cnt, Hit& best) {
    for (int32_t i = start; i < start + cnt; ++i) {
        float t, u, v;
        if (!mt(S.tris, (uint32_t)i, r.o, r.d, t, u, v)) continue;
        if (t <= best.t && t >= r.tmin) best = Hit{i, t, u, v};
    }
}

__device__ __forceinline__ bool leaf_any(const SceneView& S, const TRay& r, int32_t start,
                                         int32_t cnt, float tmax) {
    for (int32_t i = start; i < start + cnt; ++i) {
        float t, u, v;
        if (!mt(S.tris, (uint32_t)i, r.o, r.d, t, u, v)) continue;
        if (t < tmax && t > r.tmin) return true;
    }
    return false;
}

__device__ Hit closest_hit(const SceneView& S, const BvhHeader& H, const TRay& r, float tmax,
                           uint32_t* status) {
    Hit best{-1, tmax, 0.f, 0.f};
    float A;
    if (!slab(r, best.t, H.root_lo.x, H.root_lo.y, H.root_lo.z, H.root_hi.x, H.root_hi.y,
              H.root_hi.z, A))
        return best;
    if (H.root_cnt > 0) {
        leaf_closest(S, r, H.root_ref, H.root_cnt, best);
        return best;
    }
    int32_t st_ref[STACK], st_cnt[STACK];
    float st_a[STACK];
    int sp = 0;
    int32_t cur = H.root_ref;
    for (;;) {
        float4 n0, n1, n2;
        int4 n3;
        load_node(S.nodes, cur, n0, n1, n2, n3);
        // c0 = left: lo (n0.x, n0.y, n0.z) hi (n0.w, n1.x, n1.y)
        // c1 = right: lo (n1.z, n1.w, n2.x) hi (n2.y, n2.z, n2.w)
        const f3 dl = mk3(n1.z - n0.x, n1.w - n0.y, n2.x - n0.z);
        const bool left_first = dot(r.d, dl) > 0.0f;
        float a0, a1;
        const bool h0 = slab(r, best.t, n0.x, n0.y, n0.z, n0.w, n1.x, n1.y, a0);
        const bool h1 = slab(r, best.t, n1.z, n1.w, n2.x, n2.y, n2.z, n2.w, a1);
        const bool hf = left_first ? h0 : h1, hs = left_first ? h1 : h0;
        const int32_t rf = left_first ? n3.x : n3.y, rs = left_first ? n3.y : n3.x;
        const int32_t cf = left_first ? n3.z : n3.w, cs = left_first ? n3.w : n3.z;
        const float as = left_first ? a1 : a0;
        if (hs) {
            if (sp < STACK) {
                st_ref[sp] = rs;
                st_cnt[sp] = cs;
                st_a[sp] = as;
                ++sp;
            } else {
                atomicOr(status, RT_DEV_OVERFLOW);
            }
        }
        bool descend = false;
        if (hf) {
            if (cf > 0)
                leaf_closest(S, r, rf, cf, best);
            else {
                cur = rf;
                descend = true;
            }
        }
        if (descend) continue;
        // pop
        bool found = false;
        while (sp > 0) {
            --sp;
            if (!(st_a[sp] <= best.t)) continue;
            if (st_cnt[sp] > 0) {
                leaf_closest(S, r, st_ref[sp], st_cnt[sp], best);
                continue;
            }
            cur = st_ref[sp];
            found = true;
            break;
        }
        if (!found) return best;
    }
}

__device__ bool any_hit(const SceneView& S, const BvhHeader& H, const TRay& r, float tmax,
                        uint32_t* status) {
    if (!slab_shadow(r, tmax, H.root_lo.x, H.root_lo.y, H.root_lo.z, H.root_hi.x, H.root_hi.y,
                     H.root_hi.z))
        return false;
    if (H.root_cnt > 0) return leaf_any(S, r, H.root_ref, H.root_cnt, tmax);
    int32_t st_ref[STACK], st_cnt[STACK];
    int sp = 0;
    int32_t cur = H.root_ref;
    for (;;) {
        float4 n0, n1, n2;
        int4 n3;
        load_node(S.nodes, cur, n0, n1, n2, n3);
        const f3 dl = mk3(n1.z - n0.x, n1.w - n0.y, n2.x - n0.z);
        const bool left_first = dot(r.d, dl) > 0.0f;
        const bool h0 = slab_shadow(r, tmax, n0.x, n0.y, n0.z, n0.w, n1.x, n1.y);
        const bool h1 = slab_shadow(r, tmax, n1.z, n1.w, n2.x, n2.y, n2.z, n2.w);
        const bool hf = left_first ? h0 : h1, hs = left_first ? h1 : h0;
        const int32_t rf = left_first ? n3.x : n3.y, rs = left_first ? n3.y : n3.x;
        const int32_t cf = left_first ? n3.z : n3.w, cs = left_first ? n3.w : n3.z;
        if (hs) {
            if (sp < STACK) {
                st_ref[sp] = rs;
                st_cnt[sp] = cs;
                ++sp;
            } else {
                atomicOr(status, RT_DEV_OVERFLOW);
            }
        }
        if (hf) {
            if (cf > 0) {
                if (leaf_any(S, r, rf, cf, tmax)) return true;
            } else {
                cur = rf;
                continue;
            }
        }
        bool found = false;
        while (sp > 0) {
            --sp;
            if (st_cnt[sp] > 0) {
                if (leaf_any(S, r, st_ref[sp], st_cnt[sp], tmax)) return true;
                continue;
            }
            cur = st_ref[sp];
            found = true;
            break;
        }
        if (!found) return false;
    }
}

// Hit record of complete_trace_info.
struct HitInfo {
    f3 n, hp;
    uint8_t inverse_n;
};

__device__ __forceinline__ HitInfo complete_hit(const SceneView& S, f3 o, f3 d, const Hit& h) {
    HitInfo hi;
    hi.hp = add(o, muls(d, h.t));
    const uint32_t a = __ldg(&S.idx[3 * (size_t)h.id]), b = __ldg(&S.idx[3 * (size_t)h.id + 1]),
                   c = __ldg(&S.idx[3 * (size_t)h.id + 2]);
    const f3 n0 = normalize(ld3(__ldg(&S.nrm[a])));
    const f3 n1 = normalize(ld3(__ldg(&S.nrm[b])));
    const f3 n2 = normalize(ld3(__ldg(&S.nrm[c])));
    const float w = 1.0f - (h.u + h.v);
    f3 n = normalize(add(add(muls(n0, w), muls(n2, h.v)), muls(n1, h.u)));
    if (dot(n, d) > 0.0f) {
        hi.inverse_n = 1;
        n = neg(n);
    } else {
        hi.inverse_n = 0;
    }
    hi.n = n;
    return hi;
}

// Shadow ray of shadow_trace_single for one light (shadow-trace-bvh.cl:
// 375-418); point lights as spot lights without a cone.
__device__ __forceinline__ bool occluded(const SceneView& S, const BvhHeader& H, const rt_light& L,
                                         f3 hp, uint32_t* status) {
    f3 dir;
    if (L.type == RT_DIR_L) {
        dir = neg(mk3(L.dir[0], L.dir[1], L.dir[2]));
    } else if (L.type == RT_SPOT_L) {
        dir = normalize(sub(mk3(L.pos[0], L.pos[1], L.pos[2]), hp));
        if (dot(neg(dir), mk3(L.dir[0], L.dir[1], L.dir[2])) < L.angle) return true;
    } else if (L.type == RT_POINT_L) {
        dir = normalize(sub(mk3(L.pos[0], L.pos[1], L.pos[2]), hp));
    } else {
        return true;
    }
    const f3 inv = mk3(1.0f / dir.x, 1.0f / dir.y, 1.0f / dir.z);
    const TRay r = make_tray(hp, dir, inv, 0.01f);
    return any_hit(S, H, r, 1e37f, status);
}

// Local Whitted term of shade_sample, as the fixed-point increments that
// to_color_int + image[pixel] += produce (ray-shader.cl:101-109, 312-330).
__device__ __forceinline__ uint3 shade_hit(const rt_lights& Ls, const rt_material& mat, f3 hp, f3 n,
                                           f3 d, float contribution, uint32_t shadow_mask) {
    const f3 diffuse = mk3(mat.diffuse[0], mat.diffuse[1], mat.diffuse[2]);
    f3 val = mul(mk3(Ls.ambient[0], Ls.ambient[1], Ls.ambient[2]), diffuse);
    for (int l = 0; l < Ls.count; ++l) {
        const rt_light& L = Ls.light[l];
        f3 Ld, rgb = mk3(L.color[0], L.color[1], L.color[2]);
        float LD;
        if (L.type == RT_DIR_L) {
            Ld = mk3(L.dir[0], L.dir[1], L.dir[2]);
            LD = 1.0f;
        } else if (L.type == RT_SPOT_L) {
            Ld = normalize(sub(hp, mk3(L.pos[0], L.pos[1], L.pos[2])));
            LD = dot(Ld, mk3(L.dir[0], L.dir[1], L.dir[2])) - L.angle;
            LD /= 1.0f - L.angle;
            LD = clamp01(LD);
        } else {
            Ld = normalize(sub(hp, mk3(L.pos[0], L.pos[1], L.pos[2])));
            LD = 1.0f;
        }
        rgb = muls(rgb, LD);
        if (!((shadow_mask >> l) & 1u)) {
            const float dn = dot(d, n);
            const f3 rr = sub(d, muls(muls(n, 2.0f), dn));
            float cosL = clamp01(dot(n, neg(Ld)));
            cosL = cosL * cosL;
            float spec = clamp01(dot(rr, neg(Ld)));
            spec = spec * spec;
            spec = spec * spec;
            spec = spec * spec;
            spec *= cosL * mat.shininess;
            val = add(val, muls(mul(rgb, diffuse), cosL));
            val = add(val, muls(rgb, spec));
        }
    }
    val = muls(val, 1.0f - mat.reflectiveness);
    f3 f = muls(val, contribution);
    f = mk3(clamp01(f.x), clamp01(f.y), clamp01(f.z));
    return make_uint3((uint32_t)floorf(f.x * 1e6f), (uint32_t)floorf(f.y * 1e6f),
                      (uint32_t)floorf(f.z * 1e6f));
}

// Reflection ray (secondary-ray-generator.cl:258-270).
__device__ __forceinline__ void reflect_ray(f3 d_in, f3 n_in, f3& dir) {
    f3 d = neg(normalize(d_in));
    const f3 n = normalize(n_in);
    d = neg(d);
    dir = normalize(sub(d, muls(muls(n, 2.0f), dot(d, n))));
}

// Pixel of global id gid in the quad_size block order of generate_primary_rays.
__device__ __forceinline__ void pixel_of(int gid, int w, int h, int q, int& x, int& y) {
    const int pixels = w * h;
    const int i = gid % pixels;
    const int ba = q * q, xb = w / q, yb = h / q;
    const int block_rays = xb * yb * ba;
    const int right_rays = (w - xb * q) * h;
    if (i < block_rays) {
        const int block = i / ba, bp = i % ba;
        x = (block % xb) * q + bp % q;
        y = (block / xb) * q + bp / q;
    } else if (i < block_rays + right_rays) {
        const int sx = xb * q, slab_w = w - sx, ri = i - block_rays;
        x = sx + ri % slab_w;
        y = ri / slab_w;
    } else {
        const int sy = yb * q, slab_h = h - sy, ti = i - (block_rays + right_rays);
        x = ti / slab_h;
        y = sy + ti % slab_h;
    }
}

// Work order of the fused kernel: inside each full 32x32 block, the 32 pixels
// a warp takes form an 8x4 tile instead of one 32-pixel row (rays closer
// together).  Only the assignment of pixels to lanes changes; every pixel is
// still rendered exactly once.
__device__ __forceinline__ int warp_tile_order(int gid, int w, int h) {
    const int xb = w / 32, yb = h / 32;
    const int block_rays = xb * yb * 1024;
    if (gid >= block_rays) return gid;
    const int block = gid >> 10, bp = gid & 1023;
    const int t = bp >> 5, r = bp & 31;
    const int px = (t & 3) * 8 + (r & 7), py = (t >> 2) * 4 + (r >> 3);
    return (block << 10) + py * 32 + px;
}

__device__ __forceinline__ f3 primary_dir(const rt_camera& cam, int x, int y, int w, int h,
                                          float ox, float oy) {
    const float xn = (0.5f + (float)x + ox) / (float)w;
    const float yn = (0.5f + (float)y + oy) / (float)h;
    const float a = xn * 2.0f - 1.0f, b = yn * 2.0f - 1.0f;
    f3 d = add(add(mk3(cam.dir[0], cam.dir[1], cam.dir[2]),
                   muls(mk3(cam.right[0], cam.right[1], cam.right[2]), a)),
               muls(mk3(cam.up[0], cam.up[1], cam.up[2]), b));
    return normalize(d);
}

__device__ __forceinline__ uint8_t to_unorm8(uint32_t v, float inv1e6) {
    const float f = (float)v * inv1e6;
    return (uint8_t)__float2uint_rn(clamp01(f) * 255.0f);
}

// ---------------------------------------------------------------------------
// fused per-pixel Whitted path (Renderer::render_to_framebuffer, one pixel
// per lane, persistent warps fetching 32 pixels at a time)
// ---------------------------------------------------------------------------
template <int THREADS, int MINB>
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
            f3 o = mk3(a.cam.pos[0], a.cam.pos[1], a.cam.pos[2]);
            f3 d = primary_dir(a.cam, x, y, a.width, a.height, 0.0f, 0.0f);
            float tmin = 0.0f, tmax = 1e36f, contribution = 1.0f;
            uint32_t acc_r = 0, acc_g = 0, acc_b = 0;
            ++n_prim;
            for (int bounce = 0;; ++bounce) {
                const f3 inv = mk3(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
                const TRay r = make_tray(o, d, inv, tmin);
                const Hit h = closest_hit(S, H, r, tmax, a.status);
                if (h.id < 0) break;
                ++n_hits;
                const HitInfo hi = complete_hit(S, o, d, h);
                const rt_material mat = S.mats[__ldg(&S.map[h.id])];
                uint32_t mask = 0;
                for (int l = 0; l < sL.count; ++l)
                    if (occluded(S, H, sL.light[l], hi.hp, a.status)) mask |= 1u << l;
                n_shadow += (uint64_t)sL.count;
                const uint3 c = shade_hit(sL, mat, hi.hp, hi.n, d, contribution, mask);
                acc_r += c.x;
                acc_g += c.y;
                acc_b += c.z;
                if (bounce == a.max_bounces) break;
                if (!(mat.reflectiveness > 0.0f)) break;
                f3 nd;
                reflect_ray(d, hi.n, nd);
                contribution = contribution * mat.reflectiveness * 1.0f;
                o = hi.hp;
                d = nd;
                tmin = 0.0001f;
                tmax = 1e37f;
                ++n_sec;
            }
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

// Secondary generation: flags -> per-block counts -> block offsets -> emit,
// which keeps the input order (the reference's mark / scan / generate).
__device__ __forceinline__ bool wants_reflection(const SceneView& S, const rt_hit& h, float& refl) {
    if (!h.hit) return false;
    refl = S.mats[__ldg(&S.map[h.id])].reflectiveness;
    return refl > 0.0f;
}

__global__ void k_sec_count(SceneView S, const rt_hit* __restrict__ hits, int n,
                            uint32_t* __restrict__ block_counts) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    float refl;
    const bool f = i < n && wants_reflection(S, hits[i], refl);
    const int c = __syncthreads_count(f);
    if (threadIdx.x == 0) block_counts[blockIdx.x] = (uint32_t)c;
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

__global__ void k_sec_emit(SceneView S, const rt_sample* __restrict__ in,
                           const rt_hit* __restrict__ hits, int n,
                           const uint32_t* __restrict__ block_offsets, rt_sample* __restrict__ out,
                           int max_out) {
    __shared__ uint32_t warp_tot[32];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    float refl = 0.f;
    const bool f = i < n && wants_reflection(S, hits[i], refl);
    const unsigned bal = __ballot_sync(0xffffffffu, f);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) warp_tot[w] = __popc(bal);
    __syncthreads();
    uint32_t wbase = 0;
    for (int k = 0; k < w; ++k) wbase += warp_tot[k];
    if (!f) return;
    const uint32_t slot = block_offsets[blockIdx.x] + wbase + __popc(bal & ((1u << lane) - 1u));
    if (slot >= (uint32_t)max_out) return;
    const rt_hit& h = hits[i];
    const rt_sample& s = in[i];
    f3 dir;
    reflect_ray(f3_of(s.ray.dir), f3_of(h.n), dir);
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
    o.pixel = s.pixel;
    o.contribution = s.contribution * refl * 1.0f;
    o._pad[0] = o._pad[1] = 0;
    out[slot] = o;
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
};
static const RenderVariant kVariants[] = {
    {64, 8, k_render<64, 8>},    {64, 12, k_render<64, 12>},  {128, 4, k_render<128, 4>},
    {128, 6, k_render<128, 6>},  {128, 8, k_render<128, 8>},  {256, 2, k_render<256, 2>},
    {256, 3, k_render<256, 3>},  {256, 4, k_render<256, 4>},
};
constexpr int kNumVariants = sizeof(kVariants) / sizeof(kVariants[0]);

int render_variant_count() { return kNumVariants; }

int render_variant_info(int v, int* threads, int* min_blocks, const void** fn) {
    if (v < 0 || v >= kNumVariants) return -1;
    if (threads) *threads = kVariants[v].threads;
    if (min_blocks) *min_blocks = kVariants[v].min_blocks;
    if (fn) *fn = (const void*)kVariants[v].fn;
    return 0;
}

cudaError_t launch_render(const RenderArgs& a, int variant, int grid, cudaStream_t s) {
    if (variant < 0 || variant >= kNumVariants) return cudaErrorInvalidValue;
    kVariants[variant].fn<<<grid, kVariants[variant].threads, 0, s>>>(a);
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
    k_sec_count<<<nb, 256, 0, s>>>(S, hits, n, block_scratch);
    k_sec_scan<<<1, 1024, 0, s>>>(block_scratch, nb, max_out, d_count);
    k_sec_emit<<<nb, 256, 0, s>>>(S, in, hits, n, block_scratch, out, max_out);
    return cudaGetLastError();
}

cudaError_t launch_fb_copy(const uint32_t* img, uint8_t* rgba, size_t px, float inv1e6,
                           cudaStream_t s) {
    if (px == 0) return cudaSuccess;
    k_fb_copy<<<blocks(px, 256), 256, 0, s>>>(img, reinterpret_cast<uchar4*>(rgba), px, inv1e6);
    return cudaGetLastError();
}

size_t gen_secondary_scratch_bytes(int n) { return sizeof(uint32_t) * (blocks(n, 256) + 1); }

}  // namespace rt
