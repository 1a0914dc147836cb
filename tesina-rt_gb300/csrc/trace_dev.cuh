// trace_dev.cuh — device-side traversal, shading and ray generation shared by
// the one-scene kernels (trace.cu) and the many-scene render (batch.cu).
//
// Device functions restate, in the reference's operation order:
//   closest_hit   trace_ray / leaf_hit / bbox_hit (src/kernel/trace-bvh.cl:247-417)
//   any_hit       trace_shadow_ray / leaf_hit_any (src/kernel/shadow-trace-bvh.cl:160-315)
//   complete_hit  complete_trace_info (trace-bvh.cl:190-245)
//   shade_hit     shade_sample (src/kernel/ray-shader.cl:116-333), untextured
//   reflect_ray   generate_secondary_rays_disc reflection branch
//                 (src/kernel/secondary-ray-generator.cl:258-270)
//   primary_dir   generate_primary_rays (src/kernel/primary-ray-generator.cl:27-103)
//
// Traversal order is the reference's: depth first, near child first where
// near = left iff dot(dir, right.lo - left.lo) > 0 (trace-bvh.cl:391-409).
// Both child boxes are tested when their parent is visited; the far child is
// pushed with its entry distance A, and popped only if A <= the current tMax.
// Because tMax only shrinks, this accepts exactly the nodes the reference
// accepts when it tests the far child's box at pop time, so leaves are
// visited in the same order and equal-t ties resolve the same way.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "rt_internal.cuh"

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

// Traversal stack of the two-phase loop: node references with their leaf
// counts and (DIST) the entry distances the closest-hit search prunes by.
template <bool DIST>
struct TravStack {
    int32_t ref[STACK], cnt[STACK];
    float a[DIST ? STACK : 1];
    int sp = 0;
    __device__ __forceinline__ bool push(int32_t r, int32_t c, float d) {
        if (sp >= STACK) return false;
        ref[sp] = r;
        cnt[sp] = c;
        if (DIST) a[sp] = d;
        ++sp;
        return true;
    }
    // The next entry (DIST: the next whose entry distance is within tmax)
    // into cur / cur_cnt; cur = -1 when none is left.
    __device__ __forceinline__ void pop(float tmax, int32_t& cur, int32_t& cur_cnt) {
        cur = -1;
        while (sp > 0) {
            --sp;
            if (!DIST || a[sp] <= tmax) {
                cur = ref[sp];
                cur_cnt = cnt[sp];
                return;
            }
        }
    }
};

// Traversal in two phases per round (Aila & Laine's "while-while" loop with
// speculative traversal): a lane walks inner nodes, setting aside the first
// leaf it reaches and walking on, until every lane of the warp holds a leaf;
// then the lanes intersect their leaves.  Leaves are still intersected in
// the depth-first order above.  Nodes walked past a set-aside leaf are
// accepted against the tMax before that leaf; any of them the exact order
// would have dropped starts beyond the final tMax, so none of its triangles
// is accepted (t >= entry > tMax): the same hit, equal-t ties included.
static __device__ Hit closest_hit_ww(const SceneView& S, const BvhHeader& H, const TRay& r,
                                     float tmax, uint32_t* status) {
    Hit best{-1, tmax, 0.f, 0.f};
    float A;
    if (!slab(r, best.t, H.root_lo.x, H.root_lo.y, H.root_lo.z, H.root_hi.x, H.root_hi.y,
              H.root_hi.z, A))
        return best;
    if (H.root_cnt > 0) {
        leaf_closest(S, r, H.root_ref, H.root_cnt, best);
        return best;
    }
    TravStack<true> st;
    // the next node (inner: cnt 0, leaf: cnt > 0, none: ref < 0) and the
    // leaf set aside
    int32_t cur = H.root_ref, cur_cnt = 0, lf = -1, lf_cnt = 0;
    auto pop = [&]() { st.pop(best.t, cur, cur_cnt); };
    for (;;) {
        while (cur >= 0 && cur_cnt == 0) {
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
            if (hs && !st.push(left_first ? n3.y : n3.x, left_first ? n3.w : n3.z,
                               left_first ? a1 : a0))
                atomicOr(status, RT_DEV_OVERFLOW);
            if (hf) {
                cur = left_first ? n3.x : n3.y;
                cur_cnt = left_first ? n3.z : n3.w;
            } else {
                pop();
            }
            if (cur >= 0 && cur_cnt > 0 && lf < 0) {   // set the leaf aside, walk on
                lf = cur;
                lf_cnt = cur_cnt;
                pop();
            }
            if (__all_sync(__activemask(), lf >= 0)) break;
        }
        while (lf >= 0) {
            leaf_closest(S, r, lf, lf_cnt, best);
            lf = -1;
            if (cur >= 0 && cur_cnt > 0) {
                lf = cur;
                lf_cnt = cur_cnt;
                pop();
            }
        }
        if (cur < 0) return best;
    }
}

// Any hit ends the search, whatever the order: the same two-phase loop.
static __device__ bool any_hit_ww(const SceneView& S, const BvhHeader& H, const TRay& r, float tmax,
                                  uint32_t* status) {
    if (!slab_shadow(r, tmax, H.root_lo.x, H.root_lo.y, H.root_lo.z, H.root_hi.x, H.root_hi.y,
                     H.root_hi.z))
        return false;
    if (H.root_cnt > 0) return leaf_any(S, r, H.root_ref, H.root_cnt, tmax);
    TravStack<false> st;
    int32_t cur = H.root_ref, cur_cnt = 0, lf = -1, lf_cnt = 0;
    auto pop = [&]() { st.pop(0.f, cur, cur_cnt); };
    for (;;) {
        while (cur >= 0 && cur_cnt == 0) {
            float4 n0, n1, n2;
            int4 n3;
            load_node(S.nodes, cur, n0, n1, n2, n3);
            const f3 dl = mk3(n1.z - n0.x, n1.w - n0.y, n2.x - n0.z);
            const bool left_first = dot(r.d, dl) > 0.0f;
            const bool h0 = slab_shadow(r, tmax, n0.x, n0.y, n0.z, n0.w, n1.x, n1.y);
            const bool h1 = slab_shadow(r, tmax, n1.z, n1.w, n2.x, n2.y, n2.z, n2.w);
            const bool hf = left_first ? h0 : h1, hs = left_first ? h1 : h0;
            if (hs && !st.push(left_first ? n3.y : n3.x, left_first ? n3.w : n3.z, 0.f))
                atomicOr(status, RT_DEV_OVERFLOW);
            if (hf) {
                cur = left_first ? n3.x : n3.y;
                cur_cnt = left_first ? n3.z : n3.w;
            } else {
                pop();
            }
            if (cur >= 0 && cur_cnt > 0 && lf < 0) {
                lf = cur;
                lf_cnt = cur_cnt;
                pop();
            }
            if (__all_sync(__activemask(), lf >= 0)) break;
        }
        while (lf >= 0) {
            if (leaf_any(S, r, lf, lf_cnt, tmax)) return true;
            lf = -1;
            if (cur >= 0 && cur_cnt > 0) {
                lf = cur;
                lf_cnt = cur_cnt;
                pop();
            }
        }
        if (cur < 0) return false;
    }
}

static __device__ Hit closest_hit(const SceneView& S, const BvhHeader& H, const TRay& r, float tmax,
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

static __device__ bool any_hit(const SceneView& S, const BvhHeader& H, const TRay& r, float tmax,
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
// WW: the two-phase traversal (any_hit_ww) instead of any_hit.
template <bool WW = false>
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
    return WW ? any_hit_ww(S, H, r, 1e37f, status) : any_hit(S, H, r, 1e37f, status);
}

// Light direction (from the light toward the hit) and colour at a hit, as
// shade_sample computes them (ray-shader.cl:116-333; point lights without a
// cone).
__device__ __forceinline__ void light_at(const rt_light& L, f3 hp, f3& Ld, f3& rgb) {
    rgb = mk3(L.color[0], L.color[1], L.color[2]);
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
}

// The two terms shade_sample adds for light L when its shadow ray is not
// blocked (ray-shader.cl:312-330): diffuse rgb * diffuse * cosL and specular
// rgb * spec, with cosL = clamp(dot(n, -Ld))^2 and spec = clamp(dot(r,
// -Ld))^8 * cosL * shininess, r the incoming direction d reflected about n.
__device__ __forceinline__ void light_terms(const rt_light& L, const rt_material& mat, f3 hp, f3 n,
                                            f3 d, f3& dterm, f3& sterm) {
    f3 Ld, rgb;
    light_at(L, hp, Ld, rgb);
    const f3 diffuse = mk3(mat.diffuse[0], mat.diffuse[1], mat.diffuse[2]);
    const float dn = dot(d, n);
    const f3 rr = sub(d, muls(muls(n, 2.0f), dn));
    float cosL = clamp01(dot(n, neg(Ld)));
    cosL = cosL * cosL;
    float spec = clamp01(dot(rr, neg(Ld)));
    spec = spec * spec;
    spec = spec * spec;
    spec = spec * spec;
    spec *= cosL * mat.shininess;
    dterm = muls(mul(rgb, diffuse), cosL);
    sterm = muls(rgb, spec);
}

// True when light L adds nothing to the hit's colour whether or not its
// shadow ray is blocked: both terms of light_terms are zero (a light behind
// the surface, cosL = 0; a surface with no diffuse colour and no shininess,
// as the mirrors here; a black light).  Adding a zero term changes the sum
// at most in the sign of a zero, which floor(f * 1e6) to an integer
// removes, so skipping the shadow ray gives the same image; a NaN or
// infinite term is never skipped.  Only the fused renders skip; the
// stage-wise shadow pass reports every ray's result.
__device__ __forceinline__ bool light_vanishes(const rt_light& L, const rt_material& mat, f3 hp,
                                               f3 n, f3 d) {
    f3 dt, st;
    light_terms(L, mat, hp, n, d, dt, st);
    return dt.x == 0.0f && dt.y == 0.0f && dt.z == 0.0f && st.x == 0.0f && st.y == 0.0f &&
           st.z == 0.0f;
}

// The shadow tasks of a warp's nh hits (nh <= 32) and nl lights (nl <=
// RT_MAX_LIGHTS), in light-major order so that neighbouring lanes trace
// toward one light from neighbouring hits.  need(k, l) settles a task
// without a ray when it returns false (light_vanishes); the tasks that need
// a ray are listed densely in `list` (hit | light << 5, 32 * RT_MAX_LIGHTS
// bytes of the warp's shared memory) and trace(k, l) runs them 32 at a
// time, so a round of the warp traces 32 rays whatever was settled (against
// each lane taking the tasks of its own index: 1.5 % faster on the
// mid-scale frame, 4 % on the stress pose, equal on the small soup).  All 32
// lanes call it.
static_assert(RT_MAX_LIGHTS <= 8, "task list entries hold the light in 3 bits");
template <class Need, class Trace>
__device__ __forceinline__ void shadow_tasks(int nh, int nl, uint8_t* list, Need need, Trace trace) {
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    const int ntask = nh * nl;
    int nt = 0;
    for (int t0 = 0; t0 < ntask; t0 += 32) {
        const int t = t0 + lane;
        bool nd = false;
        int k = 0, l = 0;
        if (t < ntask) {
            l = t / nh;
            k = t - l * nh;
            nd = need(k, l);
        }
        const unsigned bm = __ballot_sync(0xffffffffu, nd);
        if (nd) list[nt + __popc(bm & lt)] = (uint8_t)(k | (l << 5));
        nt += __popc(bm);
    }
    __syncwarp();
    for (int i = lane; i < nt; i += 32) {
        const int e = list[i];
        trace(e & 31, e >> 5);
    }
}

// Local Whitted term of shade_sample, as the fixed-point increments that
// to_color_int + image[pixel] += produce (ray-shader.cl:101-109, 312-330).
__device__ __forceinline__ uint3 shade_hit(const rt_lights& Ls, const rt_material& mat, f3 hp, f3 n,
                                           f3 d, float contribution, uint32_t shadow_mask) {
    const f3 diffuse = mk3(mat.diffuse[0], mat.diffuse[1], mat.diffuse[2]);
    f3 val = mul(mk3(Ls.ambient[0], Ls.ambient[1], Ls.ambient[2]), diffuse);
    for (int l = 0; l < Ls.count; ++l) {
        if (!((shadow_mask >> l) & 1u)) {
            f3 dt, st;
            light_terms(Ls.light[l], mat, hp, n, d, dt, st);
            val = add(val, dt);
            val = add(val, st);
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

// pow(x, 5) of the Schlick term: the product in double precision, rounded to
// float once (the oracle evaluates it the same way; OpenCL allows pow 16 ulp).
__device__ __forceinline__ float pow5(float x) {
    const double p = (double)x;
    return (float)((((p * p) * p) * p) * p);
}

// Refraction branch of generate_secondary_rays_disc
// (secondary-ray-generator.cl:220-256): whether the refracted ray exists
// (k > 0), Schlick's factor R and the refracted direction.
__device__ __forceinline__ bool refract_ray(f3 d_in, f3 n_in, bool inverse_n, float ior, float& R,
                                            f3& dir) {
    const f3 d = neg(normalize(d_in));
    const f3 n = normalize(n_in);
    const float etai = inverse_n ? ior : 1.0f, etat = inverse_n ? 1.0f : ior;
    const float cosi = dot(d, n);
    const float rel_eta = etai / etat;
    const float w = rel_eta * cosi;
    float k = 1.0f + (w - rel_eta) * (w + rel_eta);
    if (!(k > 0.0f)) return false;
    float R0 = (etat - 1.0f) / (etat + 1.0f);
    R0 *= R0;
    R = R0 + (1.0f - R0) * pow5(1.0f - cosi);
    k = sqrtf(k);
    dir = normalize(sub(muls(n, w - k), muls(d, etai)));
    return true;
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


// Result of one pixel's Whitted path.
struct PixelResult {
    uint32_t r, g, b;
    uint32_t secondary, shadow, hits;
};

// The whole path of one pixel (Renderer::render_to_framebuffer's tile and
// bounce loops restricted to the pixel): primary ray, closest hit, one
// shadow ray per light, local shading, reflection ray while the material
// reflects and the bounce budget lasts.  Integer accumulation of the
// fixed-point contributions makes the sum independent of evaluation order.
// Pending secondary ray of a pixel's ray tree (refraction branches it).
struct PendingRay {
    f3 o, d;
    float contribution;
    int bounce;
};
constexpr int REFR_STACK = 16;   // pending rays per lane: one per level of the tree

// One pixel's Whitted rays: the primary ray and, up to max_bounces, the
// secondary rays of generate_secondary_rays_disc (a reflected ray with
// contribution * reflectiveness * R, and with REFR a refracted one with
// contribution * reflectiveness * (1 - R), R = Schlick's factor, 1 without
// refraction), each traced, shadowed and shaded as the reference's wavefront
// does.  The sums are integers, so the depth-first order of this tree walk
// gives the wavefront's image.  WW: the two-phase traversal.
template <bool WW = false, bool REFR = false>
__device__ __forceinline__ PixelResult render_pixel(const SceneView& S, const BvhHeader& H,
                                                    const rt_lights& L, const rt_camera& cam,
                                                    int x, int y, int w, int h, int max_bounces,
                                                    uint32_t* status) {
    PixelResult res = {0, 0, 0, 0, 0, 0};
    f3 o = mk3(cam.pos[0], cam.pos[1], cam.pos[2]);
    f3 d = primary_dir(cam, x, y, w, h, 0.0f, 0.0f);
    float tmin = 0.0f, tmax = 1e36f, contribution = 1.0f;
    PendingRay stack[REFR ? REFR_STACK : 1];
    int sp = 0;
    for (int bounce = 0;;) {
        bool next = false;
        const f3 inv = mk3(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
        const TRay r = make_tray(o, d, inv, tmin);
        const Hit hit = WW ? closest_hit_ww(S, H, r, tmax, status) : closest_hit(S, H, r, tmax, status);
        if (hit.id >= 0) {
            ++res.hits;
            const HitInfo hi = complete_hit(S, o, d, hit);
            const rt_material mat = S.mats[__ldg(&S.map[hit.id])];
            uint32_t mask = 0;
            for (int l = 0; l < L.count; ++l)
                if (!light_vanishes(L.light[l], mat, hi.hp, hi.n, d) &&
                    occluded<WW>(S, H, L.light[l], hi.hp, status))
                    mask |= 1u << l;
            res.shadow += (uint32_t)L.count;
            const uint3 c = shade_hit(L, mat, hi.hp, hi.n, d, contribution, mask);
            res.r += c.x;
            res.g += c.y;
            res.b += c.z;
            if (bounce < max_bounces) {
                float R = 1.0f;
                if (REFR && mat.refractive_index > 0.0f) {
                    f3 td;
                    if (refract_ray(d, hi.n, hi.inverse_n != 0, mat.refractive_index, R, td)) {
                        if (sp < REFR_STACK) {
                            stack[sp].o = hi.hp;
                            stack[sp].d = td;
                            stack[sp].contribution = contribution * mat.reflectiveness * (1.0f - R);
                            stack[sp].bounce = bounce + 1;
                            ++sp;
                        } else {
                            atomicOr(status, RT_DEV_OVERFLOW);
                        }
                    }
                }
                if (mat.reflectiveness > 0.0f) {
                    f3 nd;
                    reflect_ray(d, hi.n, nd);
                    contribution = contribution * mat.reflectiveness * R;
                    o = hi.hp;
                    d = nd;
                    tmin = 0.0001f;
                    tmax = 1e37f;
                    ++bounce;
                    ++res.secondary;
                    next = true;
                }
            }
        }
        if (next) continue;
        if (!REFR || sp == 0) break;
        --sp;   // the next refracted ray set aside
        o = stack[sp].o;
        d = stack[sp].d;
        contribution = stack[sp].contribution;
        bounce = stack[sp].bounce;
        tmin = 0.0001f;
        tmax = 1e37f;
        ++res.secondary;
    }
    return res;
}

}  // namespace rt
