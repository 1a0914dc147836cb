// render_refill.cuh — k_render_refill: the Whitted frame of k_render_pool with
// lane refill (Aila & Laine's dynamic ray fetch, applied to every kind of
// ray a frame traces).
//
// k_render_pool traces 32 rays per warp to completion before a lane takes
// new work, so a warp runs as long as its slowest ray while the finished
// lanes idle (about 11 of 32 lanes active per instruction on the mid-scale
// frame).  Here every lane carries one ray at a time, closest-hit or shadow,
// advanced one node visit per loop iteration by the same step function; when
// enough lanes have finished, the warp stops, completes their rays and hands
// the idle lanes new ones:
//   1. shadow tasks (hit slot, light) of hits that await their shadow rays;
//   2. reflection rays from the warp's pool;
//   3. new primary rays, from a 32-pixel tile the warp has claimed.
// A closest-hit ray holds a hit slot from its start; a hit keeps it until
// its last shadow task is done, when the lane that finished that task shades
// the hit, adds the fixed-point colour into the pixel's sums and puts the
// reflection ray (if the path goes on) into the pool.  Slots and pool share
// one bound: pool rays + slots in use <= NS, so neither can overflow and the
// pool always has a slot for each of its rays.
//
// Every ray is traversed exactly as closest_hit / any_hit traverse it (same
// box tests, near-first order, pruning and leaf acceptance), shaded by
// shade_hit from the same inputs, and the pixel sums are integers, so the
// image is bit-identical to k_render's.
#pragma once

namespace rt {
namespace refill {

constexpr int NS = 32;                      // hit slots per warp
constexpr int RING = NS * RT_MAX_LIGHTS;    // shadow tasks: at most NS hits x lights
static_assert((RING & (RING - 1)) == 0, "ring index by mask");
enum : int { IDLE = 0, CLOSEST = 1, SHADOW = 2 };

struct WarpState {
    // hit slots: hit point, normal, incoming direction, contribution,
    // triangle, pixel, bounce, shadow mask, shadow tasks outstanding
    float hp[3][NS], hn[3][NS], hd[3][NS], hc[NS];
    int hid[NS], hpix[NS], hbounce[NS];
    unsigned hmask[NS];
    int hpend[NS];
    int free_slot[NS];
    // pooled reflection rays: origin, direction, contribution, pixel, bounce
    float ro[3][NS], rd[3][NS], rc[NS];
    int rpix[NS], rbounce[NS];
    // shadow tasks: slot | light << 8
    int ring[RING];
};

// Traversal stack of one lane (closest-hit entries carry their entry
// distance for pruning; shadow entries ignore it).
struct LaneStack {
    int32_t ref[STACK], cnt[STACK];
    float a[STACK];
    int sp;
};

// One step of a lane's traversal: visit inner node `cur`, test its leaves in
// the near-first order (a near leaf at once, stacked leaves as they are
// popped), and stop at the next inner node to visit.  Returns true when the
// traversal is over (stack empty, or a shadow ray found an occluder, `occl`).
// The visits and leaf tests are closest_hit's and any_hit's, in their order.
__device__ __forceinline__ bool trav_step(const SceneView& S, const TRay& r, bool shadow,
                                          Hit& best, int32_t& cur, LaneStack& st, bool& occl,
                                          uint32_t* status) {
    float4 n0, n1, n2;
    int4 n3;
    load_node(S.nodes, cur, n0, n1, n2, n3);
    const f3 dl = mk3(n1.z - n0.x, n1.w - n0.y, n2.x - n0.z);
    const bool left_first = dot(r.d, dl) > 0.0f;
    float a0 = 0.f, a1 = 0.f;
    bool h0, h1;
    if (shadow) {
        h0 = slab_shadow(r, 1e37f, n0.x, n0.y, n0.z, n0.w, n1.x, n1.y);
        h1 = slab_shadow(r, 1e37f, n1.z, n1.w, n2.x, n2.y, n2.z, n2.w);
    } else {
        h0 = slab(r, best.t, n0.x, n0.y, n0.z, n0.w, n1.x, n1.y, a0);
        h1 = slab(r, best.t, n1.z, n1.w, n2.x, n2.y, n2.z, n2.w, a1);
    }
    const bool hf = left_first ? h0 : h1, hs = left_first ? h1 : h0;
    const int32_t rf = left_first ? n3.x : n3.y, rs = left_first ? n3.y : n3.x;
    const int32_t cf = left_first ? n3.z : n3.w, cs = left_first ? n3.w : n3.z;
    if (hs) {
        if (st.sp < STACK) {
            st.ref[st.sp] = rs;
            st.cnt[st.sp] = cs;
            st.a[st.sp] = left_first ? a1 : a0;
            ++st.sp;
        } else {
            atomicOr(status, RT_DEV_OVERFLOW);
        }
    }
    if (hf) {
        if (cf == 0) {
            cur = rf;
            return false;
        }
        if (shadow) {
            if (leaf_any(S, r, rf, cf, 1e37f)) {
                occl = true;
                return true;
            }
        } else {
            leaf_closest(S, r, rf, cf, best);
        }
    }
    while (st.sp > 0) {
        --st.sp;
        if (!shadow && !(st.a[st.sp] <= best.t)) continue;
        const int32_t c = st.cnt[st.sp], p = st.ref[st.sp];
        if (c == 0) {
            cur = p;
            return false;
        }
        if (shadow) {
            if (leaf_any(S, r, p, c, 1e37f)) {
                occl = true;
                return true;
            }
        } else {
            leaf_closest(S, r, p, c, best);
        }
    }
    return true;
}

}  // namespace refill

// REFILL_AT: the warp stops tracing to refill once this many lanes are idle.
template <int THREADS, int MINB, int REFILL_AT>
__global__ void __launch_bounds__(THREADS, MINB) k_render_refill(RenderArgs a) {
    using namespace refill;
    const SceneView S = a.scene;
    __shared__ BvhHeader sH;
    __shared__ rt_lights sL;
    __shared__ WarpState sW[THREADS / 32];
    if (threadIdx.x == 0) sH = *S.hdr;
    for (int i = threadIdx.x; i < (int)(sizeof(rt_lights) / 4); i += blockDim.x)
        reinterpret_cast<uint32_t*>(&sL)[i] = reinterpret_cast<const uint32_t*>(&a.lights)[i];
    const int lane = threadIdx.x & 31;
    WarpState& W = sW[threadIdx.x >> 5];
    W.free_slot[lane] = lane;   // NS == 32: one slot per lane to start
    __syncthreads();
    const BvhHeader& H = sH;
    const int pixels = a.width * a.height;
    const int nl = sL.count;
    const unsigned lt = (1u << lane) - 1u;
    uint64_t n_sec = 0, n_shadow = 0, n_hits = 0, n_prim = 0;

    // warp-uniform counters (every lane updates them identically)
    int free_n = NS, pool_n = 0;
    unsigned ring_head = 0, ring_tail = 0;
    int prim_next = 0, prim_end = 0;
    bool more_pixels = true;

    // lane state
    int kind = IDLE;
    bool done = false, occl = false;
    TRay r;
    r.o = r.d = r.inv = mk3(0.f, 0.f, 0.f);
    r.tmin = 0.f;
    Hit best{-1, 0.f, 0.f, 0.f};
    int32_t cur = 0;
    int slot = 0, light = 0;
    LaneStack st;
    st.sp = 0;

    for (;;) {
        // ---- refill the idle lanes ------------------------------------------
        const unsigned idle = __ballot_sync(0xffffffffu, kind == IDLE);
        if (idle) {
            const int n_idle = __popc(idle);
            const int rank = __popc(idle & lt);
            const int n_sh = min(n_idle, (int)(ring_tail - ring_head));
            int rem = n_idle - n_sh;
            const int n_pool = min(rem, pool_n);
            rem -= n_pool;
            // primaries: pool rays + slots in use stay within NS
            int n_prim_new = min(rem, NS - pool_n - (NS - free_n));
            if (n_prim_new > 0 && prim_next == prim_end && more_pixels) {
                int base = 0;
                if (lane == 0) base = (int)atomicAdd(a.work_counter, 32u);
                base = __shfl_sync(0xffffffffu, base, 0);
                if (base >= pixels) {
                    more_pixels = false;
                } else {
                    prim_next = base;
                    prim_end = min(base + 32, pixels);
                }
            }
            n_prim_new = min(n_prim_new, prim_end - prim_next);
            if (kind == IDLE) {
                if (rank < n_sh) {
                    // a shadow task: the shadow ray of occluded() for one light
                    const int e = W.ring[(ring_head + rank) & (RING - 1)];
                    slot = e & 0xff;
                    light = e >> 8;
                    kind = SHADOW;
                    done = false;
                    occl = false;
                    const rt_light& L = sL.light[light];
                    const f3 hp = mk3(W.hp[0][slot], W.hp[1][slot], W.hp[2][slot]);
                    f3 dir = mk3(0.f, 0.f, 0.f);
                    bool trace = true;
                    if (L.type == RT_DIR_L) {
                        dir = neg(mk3(L.dir[0], L.dir[1], L.dir[2]));
                    } else if (L.type == RT_SPOT_L) {
                        dir = normalize(sub(mk3(L.pos[0], L.pos[1], L.pos[2]), hp));
                        if (dot(neg(dir), mk3(L.dir[0], L.dir[1], L.dir[2])) < L.angle) trace = false;
                    } else if (L.type == RT_POINT_L) {
                        dir = normalize(sub(mk3(L.pos[0], L.pos[1], L.pos[2]), hp));
                    } else {
                        trace = false;
                    }
                    if (!trace) {
                        occl = true;
                        done = true;
                    } else {
                        r = make_tray(hp, dir, mk3(1.0f / dir.x, 1.0f / dir.y, 1.0f / dir.z), 0.01f);
                        if (!slab_shadow(r, 1e37f, H.root_lo.x, H.root_lo.y, H.root_lo.z,
                                         H.root_hi.x, H.root_hi.y, H.root_hi.z)) {
                            done = true;
                        } else if (H.root_cnt > 0) {
                            occl = leaf_any(S, r, H.root_ref, H.root_cnt, 1e37f);
                            done = true;
                        } else {
                            cur = H.root_ref;
                            st.sp = 0;
                        }
                    }
                } else if (rank < n_sh + n_pool + n_prim_new) {
                    // a closest-hit ray: a pooled reflection ray, else a primary
                    const int k = rank - n_sh;
                    slot = W.free_slot[free_n - 1 - k];
                    f3 o, d;
                    float tmin, tmax;
                    if (k < n_pool) {
                        const int j = pool_n - 1 - k;
                        o = mk3(W.ro[0][j], W.ro[1][j], W.ro[2][j]);
                        d = mk3(W.rd[0][j], W.rd[1][j], W.rd[2][j]);
                        W.hc[slot] = W.rc[j];
                        W.hpix[slot] = W.rpix[j];
                        W.hbounce[slot] = W.rbounce[j];
                        tmin = 0.0001f;
                        tmax = 1e37f;
                    } else {
                        const int gid = prim_next + (k - n_pool);
                        int x, y;
                        pixel_of(warp_tile_order(gid, a.width, a.height), a.width, a.height, 32,
                                 x, y);
                        o = mk3(a.cam.pos[0], a.cam.pos[1], a.cam.pos[2]);
                        d = primary_dir(a.cam, x, y, a.width, a.height, 0.0f, 0.0f);
                        W.hc[slot] = 1.0f;
                        W.hpix[slot] = a.width * y + x;
                        W.hbounce[slot] = 0;
                        tmin = 0.0f;
                        tmax = 1e36f;
                        ++n_prim;
                    }
                    kind = CLOSEST;
                    done = false;
                    r = make_tray(o, d, mk3(1.0f / d.x, 1.0f / d.y, 1.0f / d.z), tmin);
                    best = Hit{-1, tmax, 0.f, 0.f};
                    float A;
                    if (!slab(r, best.t, H.root_lo.x, H.root_lo.y, H.root_lo.z, H.root_hi.x,
                              H.root_hi.y, H.root_hi.z, A)) {
                        done = true;
                    } else if (H.root_cnt > 0) {
                        leaf_closest(S, r, H.root_ref, H.root_cnt, best);
                        done = true;
                    } else {
                        cur = H.root_ref;
                        st.sp = 0;
                    }
                }
            }
            ring_head += (unsigned)n_sh;
            pool_n -= n_pool;
            free_n -= n_pool + n_prim_new;
            prim_next += n_prim_new;
            __syncwarp();
        }
        if (!__any_sync(0xffffffffu, kind != IDLE)) {
            if (!more_pixels && pool_n == 0 && ring_head == ring_tail) break;
            continue;
        }

        // ---- traverse until enough lanes are finished ---------------------
        // (a finished ray must be completed; lanes idle for want of work do
        // not stop the others by themselves)
        for (;;) {
            if (kind != IDLE && !done) done = trav_step(S, r, kind == SHADOW, best, cur, st, occl,
                                                        a.status);
            const unsigned fin = __ballot_sync(0xffffffffu, kind == IDLE || done);
            const unsigned dm = __ballot_sync(0xffffffffu, kind != IDLE && done);
            if (fin == 0xffffffffu || (dm && __popc(fin) >= REFILL_AT)) break;
        }

        // ---- complete the finished rays -----------------------------------
        bool shade = false, release = false;
        // closest hits: the hit record, then its shadow tasks
        const bool hit_done = kind == CLOSEST && done && best.id >= 0;
        if (hit_done) {
            const HitInfo hi = complete_hit(S, r.o, r.d, best);
            W.hp[0][slot] = hi.hp.x; W.hp[1][slot] = hi.hp.y; W.hp[2][slot] = hi.hp.z;
            W.hn[0][slot] = hi.n.x; W.hn[1][slot] = hi.n.y; W.hn[2][slot] = hi.n.z;
            W.hd[0][slot] = r.d.x; W.hd[1][slot] = r.d.y; W.hd[2][slot] = r.d.z;
            W.hid[slot] = best.id;
            W.hmask[slot] = 0u;
            W.hpend[slot] = nl;
            ++n_hits;
            n_shadow += (uint32_t)nl;
            if (nl == 0) shade = true;
        }
        if (kind == CLOSEST && done && best.id < 0) release = true;
        const unsigned hm = __ballot_sync(0xffffffffu, hit_done);
        if (hit_done) {
            const unsigned base = ring_tail + (unsigned)(__popc(hm & lt) * nl);
            for (int l = 0; l < nl; ++l) W.ring[(base + (unsigned)l) & (RING - 1)] = slot | (l << 8);
        }
        ring_tail += (unsigned)(__popc(hm) * nl);
        __syncwarp();
        // shadow rays: the mask bit, and the hit's shading after its last one
        if (kind == SHADOW && done) {
            if (occl) atomicOr(&W.hmask[slot], 1u << light);
            if (atomicSub(&W.hpend[slot], 1) == 1) shade = true;
        }
        __syncwarp();
        bool push = false;
        f3 np = mk3(0.f, 0.f, 0.f), nd = np;
        float nc = 0.f;
        int npix = 0, nbounce = 0;
        if (shade) {
            const f3 p = mk3(W.hp[0][slot], W.hp[1][slot], W.hp[2][slot]);
            const f3 n = mk3(W.hn[0][slot], W.hn[1][slot], W.hn[2][slot]);
            const f3 dk = mk3(W.hd[0][slot], W.hd[1][slot], W.hd[2][slot]);
            const float ck = W.hc[slot];
            const rt_material mat = S.mats[__ldg(&S.map[W.hid[slot]])];
            const uint3 col = shade_hit(sL, mat, p, n, dk, ck, W.hmask[slot]);
            const int pk = W.hpix[slot];
            atomicAdd(&a.accum[3 * (size_t)pk], col.x);
            atomicAdd(&a.accum[3 * (size_t)pk + 1], col.y);
            atomicAdd(&a.accum[3 * (size_t)pk + 2], col.z);
            const int bk = W.hbounce[slot];
            if (bk != a.max_bounces && mat.reflectiveness > 0.0f) {
                reflect_ray(dk, n, nd);
                np = p;
                nc = ck * mat.reflectiveness * 1.0f;
                npix = pk;
                nbounce = bk + 1;
                push = true;
                ++n_sec;
            }
            release = true;
        }
        const unsigned pm = __ballot_sync(0xffffffffu, push);
        if (push) {
            const int j = pool_n + __popc(pm & lt);
            W.ro[0][j] = np.x; W.ro[1][j] = np.y; W.ro[2][j] = np.z;
            W.rd[0][j] = nd.x; W.rd[1][j] = nd.y; W.rd[2][j] = nd.z;
            W.rc[j] = nc;
            W.rpix[j] = npix;
            W.rbounce[j] = nbounce;
        }
        pool_n += __popc(pm);
        const unsigned fm = __ballot_sync(0xffffffffu, release);
        if (release) W.free_slot[free_n + __popc(fm & lt)] = slot;
        free_n += __popc(fm);
        if (done) {
            kind = IDLE;
            done = false;
        }
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

}  // namespace rt
