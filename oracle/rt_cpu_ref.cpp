/*
 * rt_cpu_ref.cpp — ORACLE (test infrastructure only; never part of the product).
 *
 * A CPU restatement of the reference's hot path, used by the tests as the
 * checker and by bench.py as the timed CPU baseline.  Nothing in the product
 * library links, loads or calls this file.
 *
 * It restates, in the reference's operation order and with IEEE single
 * precision and no FMA contraction (compile with -ffp-contract=off):
 *   LBVH build   src/kernel/bvh-builder.cl:100-130 (build_primitive_bbox),
 *                :318-391 + src/rt/bvh-builder.cpp:289-334 (global bbox),
 *                :181-252 (morton_encode), bvh-builder-sort.cl:9-232 +
 *                bvh-builder.cpp:361-454 (bitonic network, exact),
 *                bvh-builder.cl:49-97 (rearrange_*), :484-671 (process_task /
 *                find_middle / set_children, as a recursive top-down split),
 *                :262-311 (build_leaf_bbox / build_node_bbox).
 *   Trace        src/kernel/trace-bvh.cl:191-417, 465-481 (trace_single).
 *   Shadow       src/kernel/shadow-trace-bvh.cl:161-315, 375-418.
 *   Shade        src/kernel/ray-shader.cl:101-333 (untextured, no cubemap).
 *   Secondary    src/kernel/secondary-ray-generator.cl:184-326 (reflection).
 *   Primary      src/kernel/primary-ray-generator.cl:27-103.
 *   Framebuffer  src/kernel/framebuffer.cl:30-54 + RGBA8 UNORM conversion.
 *   Renderer     src/rt/renderer.cpp:113-214 (tile loop, bounce loop).
 *   Animation    src/kernel/mangler.cl:12-32 (mangle).
 *
 * Documented restatement choices (identical in the CUDA path):
 *   normalize(v) = v * (1 / sqrt(dot(v, v)))  (zero vector stays zero);
 *   pow(x, 2) = x*x and pow(x, 8) = ((x*x)^2)^2;
 *   point lights (type 2) and several lights are extensions: each light adds
 *   the reference's per-light term in order, with its own shadow ray;
 *   the LBVH sort is stable (std::stable_sort); orc_sort_bitonic restates the
 *   reference's bitonic network exactly, for tie-order comparisons.
 *
 * Parity pin: tests/test_oracle_pin.py checks this file against the
 * reference's own OpenCL kernels compiled for the CPU (oracle/_ref).
 */
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <thread>
#include <vector>

#include "../include/rt_cuda.h"

namespace {

struct v3 {
    float x, y, z;
};
static inline v3 mk(float x, float y, float z) { return v3{x, y, z}; }
static inline v3 ld3(const float* p) { return v3{p[0], p[1], p[2]}; }
static inline v3 add(v3 a, v3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 sub(v3 a, v3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 mul(v3 a, v3 b) { return mk(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline v3 muls(v3 a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
static inline v3 neg(v3 a) { return mk(-a.x, -a.y, -a.z); }
static inline float dot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline v3 cross(v3 a, v3 b) {
    return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline v3 normalize(v3 v) {
    float d = dot(v, v);
    if (d == 0.0f) return v;
    float inv = 1.0f / std::sqrt(d);
    return muls(v, inv);
}
static inline float clamp01(float x) { return std::fmin(std::fmax(x, 0.0f), 1.0f); }
/* OpenCL max/min as specified ("returns y if x < y, otherwise x"), used by
 * shadow-trace-bvh.cl's bbox_hit. */
static inline float cl_max(float x, float y) { return (x < y) ? y : x; }
static inline float cl_min(float x, float y) { return (y < x) ? y : x; }

struct Node {
    float lo[3], hi[3];
    uint32_t a, b;  /* leaf: [a, b) triangle range; interior: left, right */
    uint32_t leaf;
    uint32_t depth;
    uint32_t start, end;
};

unsigned hw_threads() {
    unsigned n = std::thread::hardware_concurrency();
    return n ? n : 1;
}

template <class F>
void parallel_for(int64_t n, int threads, F f) {
    if (threads <= 1 || n < 1024) {
        for (int64_t i = 0; i < n; ++i) f(i);
        return;
    }
    std::atomic<int64_t> next(0);
    const int64_t chunk = 256;
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; ++t) {
        pool.emplace_back([&]() {
            for (;;) {
                int64_t b = next.fetch_add(chunk);
                if (b >= n) break;
                int64_t e = std::min(n, b + chunk);
                for (int64_t i = b; i < e; ++i) f(i);
            }
        });
    }
    for (auto& th : pool) th.join();
}

}  // namespace

struct orc_scene {
    std::vector<float> pos;       /* V*4 */
    std::vector<float> nrm;       /* V*4 */
    uint32_t V = 0;
    std::vector<uint32_t> idx;    /* N*3, permuted into sorted order by a build */
    std::vector<uint32_t> map;    /* N,   permuted likewise                     */
    uint32_t N = 0;
    std::vector<rt_material> mats;
    rt_lights lights;
    /* build products */
    std::vector<uint32_t> keys;        /* per original triangle of this build */
    std::vector<uint32_t> perm;        /* sorted slot -> triangle id before the build */
    std::vector<uint32_t> sorted_keys;
    std::vector<uint32_t> orig_id;     /* sorted slot -> triangle id at upload */
    std::vector<Node> nodes;           /* LBVH: pre-order; SAH: the reference's numbering; root = 0 */
    int depth = 30, min_leaf = 1;
    bool built = false;
    bool sah = false;                  /* built by orc_build_sah (no refit) */
};

/* ----------------------------------------------------------------------- */
/* LBVH                                                                     */
/* ----------------------------------------------------------------------- */

/* bvh-builder.cl:100-130 build_primitive_bbox. */
static void prim_bbox(const orc_scene* s, uint32_t i, float lo[3], float hi[3]) {
    const float* p0 = &s->pos[4 * (size_t)s->idx[3 * (size_t)i + 0]];
    const float* p1 = &s->pos[4 * (size_t)s->idx[3 * (size_t)i + 1]];
    const float* p2 = &s->pos[4 * (size_t)s->idx[3 * (size_t)i + 2]];
    for (int c = 0; c < 3; ++c) {
        float h = p0[c], l = p0[c];
        h = std::fmax(h, p1[c]);
        h = std::fmax(h, p2[c]);
        l = std::fmin(l, p1[c]);
        l = std::fmin(l, p2[c]);
        hi[c] = h;
        lo[c] = l;
    }
}

/* bvh-builder.cl:181-252 morton_encode (one triangle). */
static uint32_t morton_encode(const float lo[3], const float hi[3], const float glo[3],
                              const float ghi[3], int depth) {
    float scale = (float)std::pow(2.0, std::ceil(depth / 3.0));
    uint32_t m[3];
    for (int c = 0; c < 3; ++c) {
        float center = (hi[c] + lo[c]) * 0.5f;
        float inv = 1.0f / (ghi[c] - glo[c]);
        float slice = (center - glo[c]) * inv;
        slice = std::fmax(0.0f, std::fmin(1.0f, slice));
        slice *= scale;
        m[c] = (uint32_t)slice;
    }
    int offset = depth % 3 ? 3 - (depth % 3) : 0;
    int axis = (offset + 1) % 3;
    uint32_t code = 0;
    for (int i = 0; i < depth; ++i) {
        int src_bit = (i + offset) / 3;
        code |= ((m[axis] >> src_bit) & 1u) << i;
        axis = (axis + 1) % 3;
    }
    return code;
}

/* Top-down split of process_task / find_middle / set_children
 * (bvh-builder.cl:484-580), recursively.  The reference emits the same
 * ranges level by level with atomics; node numbering differs, the range tree
 * does not. */
static void emit(orc_scene* s, uint32_t start, uint32_t end, int level, uint32_t depth_in_tree) {
    const uint32_t* codes = s->sorted_keys.data();
    const int max_level = s->depth;
    uint32_t me = (uint32_t)s->nodes.size();
    s->nodes.push_back(Node{});
    Node nd{};
    nd.start = start;
    nd.end = end;
    nd.depth = depth_in_tree;
    nd.leaf = 1;
    nd.a = start;
    nd.b = end;

    uint32_t first = start, last = end - 1;
    int bit = max_level - 1 - level;
    bool leaf = false;
    if ((uint32_t)(last - first - 1) <= (uint32_t)s->min_leaf) leaf = true;  /* unsigned, :501 */
    if (!leaf && bit < 0) leaf = true;
    auto codebit = [&](uint32_t x) { return (codes[x] >> bit) & 1u; };
    if (!leaf) {
        while (codebit(first) != 0 || codebit(last) == 0) {
            level++;
            bit = max_level - 1 - level;
            if (bit < 0) {
                leaf = true;
                break;
            }
        }
    }
    if (leaf) {
        s->nodes[me] = nd;
        return;
    }
    while (first + 1 < last) {
        uint32_t middle = (first + last) / 2;
        if (codebit(middle) == 0)
            first = middle;
        else
            last = middle;
    }
    uint32_t split = last;
    nd.leaf = 0;
    s->nodes[me] = nd;
    uint32_t l = (uint32_t)s->nodes.size();
    emit(s, start, split, level + 1, depth_in_tree + 1);
    uint32_t r = (uint32_t)s->nodes.size();
    emit(s, split, end, level + 1, depth_in_tree + 1);
    s->nodes[me].a = l;
    s->nodes[me].b = r;
}

/* build_leaf_bbox + build_node_bbox (bvh-builder.cl:262-311): leaves merge
 * their triangles' boxes, interior nodes merge their children (post-order). */
static void refit(orc_scene* s) {
    std::vector<float> tlo((size_t)s->N * 3), thi((size_t)s->N * 3);
    for (uint32_t i = 0; i < s->N; ++i) prim_bbox(s, i, &tlo[3 * (size_t)i], &thi[3 * (size_t)i]);
    for (int64_t k = (int64_t)s->nodes.size() - 1; k >= 0; --k) {
        Node& nd = s->nodes[k];
        if (nd.leaf) {
            for (int c = 0; c < 3; ++c) {
                nd.lo[c] = tlo[3 * (size_t)nd.a + c];
                nd.hi[c] = thi[3 * (size_t)nd.a + c];
            }
            for (uint32_t i = nd.a + 1; i < nd.b; ++i)
                for (int c = 0; c < 3; ++c) {
                    nd.lo[c] = std::fmin(nd.lo[c], tlo[3 * (size_t)i + c]);
                    nd.hi[c] = std::fmax(nd.hi[c], thi[3 * (size_t)i + c]);
                }
        } else {
            const Node& l = s->nodes[nd.a];
            const Node& r = s->nodes[nd.b];
            for (int c = 0; c < 3; ++c) {
                nd.lo[c] = std::fmin(l.lo[c], r.lo[c]);
                nd.hi[c] = std::fmax(l.hi[c], r.hi[c]);
            }
        }
    }
}

/* Bitonic network of bvh-builder-sort.cl:26-232 driven by the host loop of
 * bvh-builder.cpp:361-454.  Returns -1 where the reference would exit(1)
 * (a launch with zero work-items for non-power-of-two N < 16). */
static int bitonic_sort(const uint32_t* codes, uint32_t n, uint32_t* tri) {
    for (uint32_t i = 0; i < n; ++i) tri[i] = i;
    int size = (int)n;
    int n2 = 1;
    while (n2 < size) n2 <<= 1;
    int64_t ms2 = size / 2 + (size % 2);
    int64_t ms4 = size / 4 + (size - size % 4);
    int64_t ms8 = size / 8 + (size - size % 8);
    int64_t ms16 = size / 16 + (size - size % 16);
    auto smaller = [&](uint32_t a, uint32_t b) { return codes[a] < codes[b]; };
    for (int len = 1; len < n2; len <<= 1) {
        int dir = len << 1;
        int inv = ((size - 1) & dir) == 0 && dir != n2;
        int last_step = dir == n2;
        for (int inc = len; inc > 0; inc >>= 1) {
            int G;
            int64_t items;
            if (inc > 4) {
                inc >>= 3;
                G = 16;
                items = ms16;
            } else if (inc > 2) {
                inc >>= 2;
                G = 8;
                items = ms8;
            } else if (inc > 1) {
                inc >>= 1;
                G = 4;
                items = ms4;
            } else {
                G = 2;
                items = ms2;
            }
            if (items == 0) return -1;
            int shift = G == 16 ? 4 : G == 8 ? 3 : G == 4 ? 2 : 1;
            for (int64_t gid = 0; gid < items; ++gid) {
                int64_t i = gid;
                int64_t low = i & (inc - 1);
                if (G == 2)
                    i = (i << 1) - low;
                else
                    i = ((i - low) << shift) + low;
                if (i + inc >= size) continue;
                bool order_asc = !(dir & i) && !last_step;
                if (G == 2) {
                    bool inc_is_smaller = smaller(tri[i + inc], tri[i]);
                    bool swap = (inc_is_smaller == order_asc) == (bool)inv;
                    if (swap) std::swap(tri[i], tri[i + inc]);
                    continue;
                }
                uint32_t t[16], val[16];
                auto in_range = [&](int64_t X) { return i + X * inc < size; };
                for (int j = 0; j < G && in_range(j); ++j) {
                    t[j] = j;
                    val[j] = tri[i + (int64_t)j * inc];
                }
                /* ORDERV / B2V..B16V: recursive half-cleaner on slots [a, a+G). */
                auto orderv = [&](int a, int b) {
                    if (in_range(b)) {
                        bool swap = (smaller(val[t[b]], val[t[a]]) == order_asc) == (bool)inv;
                        if (swap) std::swap(t[a], t[b]);
                    }
                };
                struct Rec {
                    static void run(int a, int g, decltype(orderv)& o) {
                        if (g == 2) {
                            o(a, a + 1);
                            return;
                        }
                        for (int k = 0; k < g / 2; ++k) o(a + k, a + k + g / 2);
                        run(a, g / 2, o);
                        run(a + g / 2, g / 2, o);
                    }
                };
                Rec::run(0, G, orderv);
                for (int j = 0; j < G && in_range(j) && in_range(t[j]); ++j)
                    tri[i + (int64_t)j * inc] = val[t[j]];
            }
        }
    }
    return 0;
}

/* ----------------------------------------------------------------------- */
/* Traversal                                                                */
/* ----------------------------------------------------------------------- */
struct Ray {
    v3 ori, dir, inv;
    float tmin, tmax;
};
static inline Ray ray_of(const rt_sample& s) {
    return Ray{ld3(s.ray.ori), ld3(s.ray.dir), ld3(s.ray.inv_dir), s.ray.tmin, s.ray.tmax};
}

/* trace-bvh.cl:247-273 bbox_hit (fmin / fmax). */
static inline bool bbox_hit(const Node& nd, const Ray& r) {
    float tMin = r.tmin, tMax = r.tmax;
    float lt[3], ht[3];
    const float* o = &r.ori.x;
    const float* iv = &r.inv.x;
    for (int c = 0; c < 3; ++c) {
        lt[c] = (nd.lo[c] - o[c]) * iv[c];
        ht[c] = (nd.hi[c] - o[c]) * iv[c];
    }
    for (int c = 0; c < 3; ++c) {
        if (std::fabs(iv[c]) > 1e-6f) {
            tMin = std::fmax(tMin, std::fmin(lt[c], ht[c]));
            tMax = std::fmin(tMax, std::fmax(lt[c], ht[c]));
        }
    }
    return tMin <= tMax;
}

/* shadow-trace-bvh.cl:160-186 bbox_hit (OpenCL max / min). */
static inline bool bbox_hit_shadow(const Node& nd, const Ray& r) {
    float tMin = r.tmin, tMax = r.tmax;
    float lt[3], ht[3];
    const float* o = &r.ori.x;
    const float* iv = &r.inv.x;
    for (int c = 0; c < 3; ++c) {
        lt[c] = (nd.lo[c] - o[c]) * iv[c];
        ht[c] = (nd.hi[c] - o[c]) * iv[c];
    }
    for (int c = 0; c < 3; ++c) {
        if (std::fabs(iv[c]) > 1e-6f) {
            tMin = cl_max(tMin, cl_min(lt[c], ht[c]));
            tMax = cl_min(tMax, cl_max(lt[c], ht[c]));
        }
    }
    return tMin <= tMax;
}

struct Best {
    int32_t id;
    float t, u, v;
};

/* Möller–Trumbore of leaf_hit (trace-bvh.cl:275-328).  Returns 1 on a
 * candidate and fills t/u/v. */
static inline bool mt(const orc_scene* s, uint32_t tri, const Ray& r, float* T, float* U, float* V) {
    v3 v0 = ld3(&s->pos[4 * (size_t)s->idx[3 * (size_t)tri + 0]]);
    v3 v1 = ld3(&s->pos[4 * (size_t)s->idx[3 * (size_t)tri + 1]]);
    v3 v2 = ld3(&s->pos[4 * (size_t)s->idx[3 * (size_t)tri + 2]]);
    v3 e1 = sub(v1, v0), e2 = sub(v2, v0);
    v3 h = cross(r.dir, e2);
    float a = dot(e1, h);
    if (a > -1e-26f && a < 1e-26f) return false;
    float f = 1.0f / a;
    v3 sv = sub(r.ori, v0);
    float u = f * dot(sv, h);
    if (u < 0.0f || u > 1.0f) return false;
    v3 q = cross(sv, e1);
    float v = f * dot(r.dir, q);
    if (v < 0.0f || u + v > 1.0f) return false;
    *T = f * dot(e2, q);
    *U = u;
    *V = v;
    return true;
}

/* trace_ray (trace-bvh.cl:330-417): 32-entry stack, near child first by
 * dot(dir, right.lo - left.lo) > 0, own box tested when a node is visited. */
/* Traversal work of one ray, as the device layout pays for it: interior
 * nodes entered (one 64-byte record each: both children's boxes and
 * references) and triangles tested (48 bytes each). */
struct TravCounts {
    uint64_t nodes = 0, tris = 0;
};

static Best trace_ray(const orc_scene* s, Ray ray, TravCounts* tc = nullptr) {
    Best best{-1, ray.tmax, 0.f, 0.f};
    uint32_t levels[32];
    uint32_t level = 0, curr = 0;
    const Node* nodes = s->nodes.data();
    for (;;) {
        const Node& nd = nodes[curr];
        if (!bbox_hit(nd, ray)) {
            if (level > 0 && level < 32) {
                curr = levels[--level];
                continue;
            }
            return best;
        }
        if (nd.leaf) {
            if (tc) tc->tris += nd.b - nd.a;
            for (uint32_t i = nd.a; i < nd.b; ++i) {
                float t, u, v;
                if (!mt(s, i, ray, &t, &u, &v)) continue;
                if (t <= best.t && t >= ray.tmin) best = Best{(int32_t)i, t, u, v};
            }
            if (best.id >= 0) ray.tmax = best.t;
            if (level > 0 && level < 32) {
                curr = levels[--level];
                continue;
            }
            return best;
        }
        if (tc) ++tc->nodes;
        const Node& l = nodes[nd.a];
        const Node& r = nodes[nd.b];
        v3 dl = sub(ld3(r.lo), ld3(l.lo));
        bool order = dot(ray.dir, dl) > 0.0f;
        uint32_t first = order ? nd.a : nd.b, second = order ? nd.b : nd.a;
        if (level >= 32) return best; /* cannot happen for depth <= 32 */
        levels[level++] = second;
        curr = first;
    }
}

/* trace_shadow_ray (shadow-trace-bvh.cl:237-315). */
static bool trace_shadow(const orc_scene* s, const Ray& ray, TravCounts* tc = nullptr) {
    uint32_t levels[32];
    uint32_t level = 0, curr = 0;
    const Node* nodes = s->nodes.data();
    for (;;) {
        const Node& nd = nodes[curr];
        if (!bbox_hit_shadow(nd, ray)) {
            if (level > 0 && level < 32) {
                curr = levels[--level];
                continue;
            }
            return false;
        }
        if (nd.leaf) {
            if (tc) tc->tris += nd.b - nd.a;
            for (uint32_t i = nd.a; i < nd.b; ++i) {
                float t, u, v;
                if (!mt(s, i, ray, &t, &u, &v)) continue;
                if (t < ray.tmax && t > ray.tmin) return true;
            }
            if (level > 0 && level < 32) {
                curr = levels[--level];
                continue;
            }
            return false;
        }
        if (tc) ++tc->nodes;
        const Node& l = nodes[nd.a];
        const Node& r = nodes[nd.b];
        v3 dl = sub(ld3(r.lo), ld3(l.lo));
        bool order = dot(ray.dir, dl) > 0.0f;
        uint32_t first = order ? nd.a : nd.b, second = order ? nd.b : nd.a;
        if (level >= 32) return false;
        levels[level++] = second;
        curr = first;
    }
}

/* complete_trace_info (trace-bvh.cl:190-245).  Texture coordinates are not
 * part of this data model: uv is written as 0. */
static void complete(const orc_scene* s, const Ray& ray, const Best& b, rt_hit* out) {
    if (b.id < 0) {
        out->hit = 0;
        return;
    }
    rt_hit h;
    std::memset(&h, 0, sizeof(h));
    h.hit = 1;
    h.shadow_hit = out->shadow_hit;
    h.t = b.t;
    h.id = b.id;
    v3 hp = add(ray.ori, muls(ray.dir, b.t));
    const uint32_t* ix = &s->idx[3 * (size_t)b.id];
    v3 n0 = normalize(ld3(&s->nrm[4 * (size_t)ix[0]]));
    v3 n1 = normalize(ld3(&s->nrm[4 * (size_t)ix[1]]));
    v3 n2 = normalize(ld3(&s->nrm[4 * (size_t)ix[2]]));
    float u = b.u, v = b.v;
    float w = 1.0f - (u + v);
    v3 n = normalize(add(add(muls(n0, w), muls(n2, v)), muls(n1, u)));
    if (dot(n, ray.dir) > 0.0f) {
        h.inverse_n = 1;
        n = neg(n);
    } else {
        h.inverse_n = 0;
    }
    h.n[0] = n.x; h.n[1] = n.y; h.n[2] = n.z;
    h.hit_point[0] = hp.x; h.hit_point[1] = hp.y; h.hit_point[2] = hp.z;
    *out = h;
}

/* Per-light shadow ray setup of shadow_trace_single
 * (shadow-trace-bvh.cl:375-418), extended to point lights. */
static bool light_occluded(const orc_scene* s, const rt_light& L, v3 hp,
                           TravCounts* tc = nullptr) {
    Ray r;
    r.ori = hp;
    if (L.type == RT_DIR_L) {
        r.dir = neg(ld3(L.dir));
    } else if (L.type == RT_SPOT_L) {
        r.dir = normalize(sub(ld3(L.pos), hp));
        if (dot(neg(r.dir), ld3(L.dir)) < L.angle) return true;
    } else if (L.type == RT_POINT_L) {
        r.dir = normalize(sub(ld3(L.pos), hp));
    } else {
        return true;
    }
    r.inv = mk(1.0f / r.dir.x, 1.0f / r.dir.y, 1.0f / r.dir.z);
    r.tmin = 0.01f;
    r.tmax = 1e37f;
    return trace_shadow(s, r, tc);
}

/* shade_sample (ray-shader.cl:116-333), untextured, no cubemap. */
static void shade_one(const orc_scene* s, const rt_sample& smp, const rt_hit& info, uint32_t* image) {
    if (!info.hit) return;
    const rt_lights& Ls = s->lights;
    const rt_material& mat = s->mats[s->map[info.id]];
    v3 diffuse = ld3(mat.diffuse);
    v3 valrgb = mul(ld3(Ls.ambient), diffuse);
    v3 hp = ld3(info.hit_point);
    for (int l = 0; l < Ls.count; ++l) {
        const rt_light& L = Ls.light[l];
        v3 Ld;
        float LD;
        v3 dir_rgb;
        if (L.type == RT_DIR_L) {
            Ld = ld3(L.dir);
            dir_rgb = ld3(L.color);
            LD = 1.0f;
        } else if (L.type == RT_SPOT_L) {
            Ld = normalize(sub(hp, ld3(L.pos)));
            dir_rgb = ld3(L.color);
            LD = dot(Ld, ld3(L.dir)) - L.angle;
            LD /= 1.0f - L.angle;
            LD = clamp01(LD);
        } else { /* RT_POINT_L */
            Ld = normalize(sub(hp, ld3(L.pos)));
            dir_rgb = ld3(L.color);
            LD = 1.0f;
        }
        dir_rgb = muls(dir_rgb, LD);
        if (!((info.shadow_hit >> l) & 1u)) {
            v3 d = ld3(smp.ray.dir);
            v3 n = ld3(info.n);
            float dn = dot(d, n);
            v3 r = sub(d, muls(muls(n, 2.0f), dn));
            float cosL = clamp01(dot(n, neg(Ld)));
            cosL = cosL * cosL;
            float spec = clamp01(dot(r, neg(Ld)));
            spec = spec * spec;
            spec = spec * spec;
            spec = spec * spec;
            spec *= cosL * mat.shininess;
            valrgb = add(valrgb, muls(mul(dir_rgb, diffuse), cosL));
            valrgb = add(valrgb, muls(dir_rgb, spec));
        }
    }
    valrgb = muls(valrgb, 1.0f - mat.reflectiveness);
    v3 f = muls(valrgb, smp.contribution);
    f = mk(clamp01(f.x), clamp01(f.y), clamp01(f.z));
    uint32_t* px = image + 3 * (size_t)smp.pixel;
    /* atomic: with refraction a pixel has two rays in one wavefront, shaded
     * by different threads (integer sums, so any order gives the same bits) */
    __atomic_fetch_add(&px[0], (uint32_t)std::floor(f.x * 1e6f), __ATOMIC_RELAXED);
    __atomic_fetch_add(&px[1], (uint32_t)std::floor(f.y * 1e6f), __ATOMIC_RELAXED);
    __atomic_fetch_add(&px[2], (uint32_t)std::floor(f.z * 1e6f), __ATOMIC_RELAXED);
}

/* pow(x, 5) of the Schlick term: the product in double precision, rounded
 * to float once (identical in the CUDA path and the reference shim; within
 * the 16 ulp OpenCL allows pow). */
static float pow5(float x) {
    const double p = (double)x;
    return (float)((((p * p) * p) * p) * p);
}

/* Refraction branch of generate_secondary_rays_disc
 * (secondary-ray-generator.cl:220-256): the Schlick factor R, and the
 * refracted ray when k > 0.  Returns whether a ray was made. */
static bool refract_ray(const rt_sample& in, const rt_hit& info, const rt_material& mat, float* R,
                        rt_sample* out) {
    const v3 d = neg(normalize(ld3(in.ray.dir)));
    const v3 n = normalize(ld3(info.n));
    float etai, etat;
    if (info.inverse_n) {
        etat = 1.0f;
        etai = mat.refractive_index;
    } else {
        etai = 1.0f;
        etat = mat.refractive_index;
    }
    const float cosi = dot(d, n);
    const float rel_eta = etai / etat;
    const float w = rel_eta * cosi;
    float k = 1.0f + (w - rel_eta) * (w + rel_eta);
    if (!(k > 0.0f)) return false;
    float R0 = (etat - 1.0f) / (etat + 1.0f);
    R0 *= R0;
    const float cos5 = pow5(1.0f - cosi);
    *R = R0 + (1.0f - R0) * cos5;
    k = std::sqrt(k);
    const v3 dir = normalize(sub(muls(n, w - k), muls(d, etai)));
    rt_sample o;
    std::memset(&o, 0, sizeof(o));
    o.ray.ori[0] = info.hit_point[0];
    o.ray.ori[1] = info.hit_point[1];
    o.ray.ori[2] = info.hit_point[2];
    o.ray.dir[0] = dir.x; o.ray.dir[1] = dir.y; o.ray.dir[2] = dir.z;
    o.ray.inv_dir[0] = 1.0f / dir.x;
    o.ray.inv_dir[1] = 1.0f / dir.y;
    o.ray.inv_dir[2] = 1.0f / dir.z;
    o.ray.tmin = 0.0001f;
    o.ray.tmax = 1e37f;
    o.pixel = in.pixel;
    o.contribution = in.contribution * mat.reflectiveness * (1.0f - *R);
    *out = o;
    return true;
}

/* Reflection branch of generate_secondary_rays_disc
 * (secondary-ray-generator.cl:258-270): contribution * reflectiveness * R. */
static void reflect_ray(const rt_sample& in, const rt_hit& info, float refl, float R,
                        rt_sample* out) {
    v3 d = neg(normalize(ld3(in.ray.dir)));
    v3 n = normalize(ld3(info.n));
    d = neg(d);
    v3 dir = normalize(sub(d, muls(muls(n, 2.0f), dot(d, n))));
    rt_sample o;
    std::memset(&o, 0, sizeof(o));
    o.ray.ori[0] = info.hit_point[0];
    o.ray.ori[1] = info.hit_point[1];
    o.ray.ori[2] = info.hit_point[2];
    o.ray.dir[0] = dir.x; o.ray.dir[1] = dir.y; o.ray.dir[2] = dir.z;
    o.ray.inv_dir[0] = 1.0f / dir.x;
    o.ray.inv_dir[1] = 1.0f / dir.y;
    o.ray.inv_dir[2] = 1.0f / dir.z;
    o.ray.tmin = 0.0001f;
    o.ray.tmax = 1e37f;
    o.pixel = in.pixel;
    o.contribution = in.contribution * refl * R;
    *out = o;
}

/* ----------------------------------------------------------------------- */
/* C API                                                                    */
/* ----------------------------------------------------------------------- */

/* ----------------------------------------------------------------------- */
/* CPU SAH BVH (BVH::construct / BVHNode::sort, src/rt/bvh.cpp:6-179;       */
/* BBox, src/rt/bbox.cpp)                                                   */
/* ----------------------------------------------------------------------- */
namespace sah {

/* std::max / std::min, which BBox uses: (a < b) ? b : a, (b < a) ? b : a. */
static inline float smax(float a, float b) { return a < b ? b : a; }
static inline float smin(float a, float b) { return b < a ? b : a; }

struct Box {
    float lo[3], hi[3];
};

/* BBox::reset (bbox.cpp:8-16): hi = FLT_MIN (the least positive normal
 * float, not -FLT_MAX), lo = FLT_MAX.  A merge with such a box raises every
 * negative maximum to FLT_MIN. */
static Box empty_box() {
    Box b;
    for (int c = 0; c < 3; ++c) {
        b.hi[c] = std::numeric_limits<float>::min();
        b.lo[c] = std::numeric_limits<float>::max();
    }
    return b;
}

static inline void merge(Box& a, const Box& b) {   /* BBox::merge, bbox.cpp:30-35 */
    for (int c = 0; c < 3; ++c) {
        a.hi[c] = smax(a.hi[c], b.hi[c]);
        a.lo[c] = smin(a.lo[c], b.lo[c]);
    }
}

static inline float centroid(const Box& b, int ax) { return (b.hi[ax] + b.lo[ax]) * 0.5f; }

static inline float area(const Box& b) {           /* BBox::surfaceArea, bbox.cpp:79-86 */
    float d[3];
    for (int c = 0; c < 3; ++c) d[c] = smax(b.hi[c] - b.lo[c], 0.f);
    return (d[0] * (d[1] + d[2]) + d[1] * d[2]) * 2.f;
}

static inline int largest_axis(const Box& b) {     /* BBox::largestAxis, bbox.cpp:49-68 */
    const float dx = b.hi[0] - b.lo[0], dy = b.hi[1] - b.lo[1], dz = b.hi[2] - b.lo[2];
    if (dx > dy && dx > dz) return 0;
    if (dy > dz) return 1;
    return 2;
}

/* uint32_t(32 * ((c - min) / length)) clamped to 31: the position lies in
 * [0, 32], or is NaN on a flat axis, which converts to 0. */
static inline uint32_t bucket_of(float x) {
    if (!(x > 0.f)) return 0;
    if (x >= 31.f) return 31;
    return (uint32_t)x;
}

constexpr uint32_t BUCKETS = 32;        /* BVH::SAH_BUCKETS */
constexpr uint32_t MIN_PRIMS = 2;       /* BVH::MIN_PRIMS_PER_NODE */
constexpr uint32_t MAX_INTERIOR_DEPTH = 31;   /* the traversal's 32-entry stack */

struct Builder {
    const std::vector<Box>& boxes;
    std::vector<uint32_t>& ot;
    std::vector<Node>& nodes;
    bool too_deep = false;

    /* chooseSplitLocationSAH (bvh.cpp:242-313): buckets over the centroid
     * range of the node box on `axis`; cost of the split after bucket i,
     * whose right side starts from the last bucket and then merges buckets
     * i+1..31 again (the last bucket is counted twice); the first least
     * cost wins; split at the first triangle whose centroid reaches the
     * bucket boundary. */
    uint32_t choose(const Box& bb, int axis, uint32_t start, uint32_t end) const {
        const float len = bb.hi[axis] - bb.lo[axis];
        const float mn = bb.lo[axis];
        const float sa = area(bb);
        uint32_t prims[BUCKETS];
        Box bbox[BUCKETS];
        for (uint32_t k = 0; k < BUCKETS; ++k) {
            prims[k] = 0;
            bbox[k] = empty_box();
        }
        for (uint32_t i = start; i < end; ++i) {
            const Box& t = boxes[ot[i]];
            const float c = centroid(t, axis);
            const uint32_t slot = bucket_of((float)BUCKETS * ((c - mn) / len));
            prims[slot]++;
            merge(bbox[slot], t);
        }
        float cost[BUCKETS - 1];
        for (uint32_t i = 0; i < BUCKETS - 1; ++i) {
            Box bl = bbox[0], br = bbox[BUCKETS - 1];
            uint32_t nl = prims[0], nr = prims[BUCKETS - 1];
            for (uint32_t j = 1; j <= i; ++j) {
                merge(bl, bbox[j]);
                nl += prims[j];
            }
            for (uint32_t j = i + 1; j < BUCKETS; ++j) {
                merge(br, bbox[j]);
                nr += prims[j];
            }
            cost[i] = .125f + ((float)nl * area(bl) + (float)nr * area(br)) / sa;
        }
        float best = cost[0];
        uint32_t best_i = 0;
        for (uint32_t i = 1; i < BUCKETS - 1; ++i)
            if (cost[i] < best) {
                best = cost[i];
                best_i = i;
            }
        float split_value = mn;
        split_value += (float)(best_i + 1) * (len / (float)BUCKETS);
        uint32_t i = start;
        for (; i < end; ++i)
            if (centroid(boxes[ot[i]], axis) >= split_value) break;
        return i;
    }

    /* BVHNode::sort (bvh.cpp:6-90): node `me` over ot[start, end). */
    void sort(uint32_t me, uint32_t start, uint32_t end, uint32_t depth) {
        Box bb = boxes[ot[start]];
        for (uint32_t i = start; i < end; ++i) merge(bb, boxes[ot[i]]);
        Node nd;
        std::memset(&nd, 0, sizeof nd);
        for (int c = 0; c < 3; ++c) {
            nd.lo[c] = bb.lo[c];
            nd.hi[c] = bb.hi[c];
        }
        nd.start = start;
        nd.end = end;
        nd.depth = depth;
        nd.leaf = 1;
        nd.a = start;
        nd.b = end;
        if (end - start <= MIN_PRIMS) {
            nodes[me] = nd;
            return;
        }
        int axis = largest_axis(bb);
        uint32_t split = start;
        for (int tries = 0; tries < 2; ++tries) {
            std::sort(ot.begin() + start, ot.begin() + end, [&](uint32_t x, uint32_t y) {
                return centroid(boxes[x], axis) < centroid(boxes[y], axis);
            });
            split = choose(bb, axis, start, end);
            if (split == start || split == end)
                axis = (axis + 1) % 3;
            else
                break;
        }
        if (split == start || split == end) {
            nodes[me] = nd;
            return;
        }
        if (depth > MAX_INTERIOR_DEPTH) too_deep = true;
        nodes.resize(nodes.size() + 2);
        const uint32_t l = (uint32_t)nodes.size() - 2, r = l + 1;
        nd.leaf = 0;
        nd.a = l;
        nd.b = r;
        nodes[me] = nd;
        sort(l, start, split, depth + 1);
        sort(r, split, end, depth + 1);
    }
};

}  // namespace sah

extern "C" {

orc_scene* orc_scene_new(const float* pos4, const float* nrm4, uint32_t V, const uint32_t* idx,
                         uint32_t N, const rt_material* mats, uint32_t M, const uint32_t* map,
                         const rt_lights* lights) {
    orc_scene* s = new orc_scene();
    s->V = V;
    s->N = N;
    s->pos.assign(pos4, pos4 + 4 * (size_t)V);
    s->nrm.assign(nrm4, nrm4 + 4 * (size_t)V);
    s->idx.assign(idx, idx + 3 * (size_t)N);
    s->map.assign(map, map + (size_t)N);
    s->mats.assign(mats, mats + M);
    s->lights = *lights;
    s->orig_id.resize(N);
    for (uint32_t i = 0; i < N; ++i) s->orig_id[i] = i;
    return s;
}

void orc_scene_free(orc_scene* s) { delete s; }

/* mangle (src/kernel/mangler.cl:12-32), the per-frame vertex animation of
 * src/rt/rt-wave.cpp:141-167, on float4 positions / normals (xyz).  The
 * kernel has no fp64 pragma, so its constants are single precision; index
 * is the vertex number as an int, converted to float by the products. */
int orc_mangle(float* pos4, float* nrm4, uint32_t V, float arg, float last_arg, float height) {
    (void)last_arg;   /* an argument of the kernel that its body does not read */
    for (uint32_t i = 0; i < V; ++i) {
        float* p = pos4 + 4 * (size_t)i;
        float* q = nrm4 + 4 * (size_t)i;
        const int index = (int)i;
        p[1] = height * std::sin(0.33f * arg + p[0]) * std::cos(0.57f * arg + p[2]);
        const float xfactor = (0.33f + std::fmod(0.01238431f * (float)index, 0.23467f)) * arg;
        const float zfactor = (0.57f + std::fmod(0.02173f * (float)index, 0.3237247f)) * arg;
        q[0] = std::cos(xfactor + p[0]);
        q[2] = -std::sin(zfactor + p[2]);
    }
    return 0;
}

int orc_set_positions(orc_scene* s, const float* pos4, const float* nrm4) {
    std::memcpy(s->pos.data(), pos4, sizeof(float) * 4 * (size_t)s->V);
    if (nrm4) std::memcpy(s->nrm.data(), nrm4, sizeof(float) * 4 * (size_t)s->V);
    return 0;
}

/* Morton keys of the current triangle order (stages a2-a4). */
int orc_morton_keys(orc_scene* s, int depth, uint32_t* keys, float* glo_out, float* ghi_out) {
    if (depth < 1 || depth > 32 || s->N == 0) return -1;
    const uint32_t N = s->N;
    std::vector<float> lo((size_t)N * 3), hi((size_t)N * 3);
    float glo[3] = {1e37f, 1e37f, 1e37f}, ghi[3] = {-1e37f, -1e37f, -1e37f};
    for (uint32_t i = 0; i < N; ++i) {
        prim_bbox(s, i, &lo[3 * (size_t)i], &hi[3 * (size_t)i]);
        for (int c = 0; c < 3; ++c) {
            glo[c] = std::fmin(glo[c], lo[3 * (size_t)i + c]);
            ghi[c] = std::fmax(ghi[c], hi[3 * (size_t)i + c]);
        }
    }
    for (uint32_t i = 0; i < N; ++i)
        keys[i] = morton_encode(&lo[3 * (size_t)i], &hi[3 * (size_t)i], glo, ghi, depth);
    if (glo_out) for (int c = 0; c < 3; ++c) glo_out[c] = glo[c];
    if (ghi_out) for (int c = 0; c < 3; ++c) ghi_out[c] = ghi[c];
    return 0;
}

int orc_sort_bitonic(const uint32_t* keys, uint32_t n, uint32_t* perm) {
    return bitonic_sort(keys, n, perm);
}

/* Full build: bbox, bounds, Morton, sort (0 = stable, 1 = the reference's
 * bitonic network), permute index buffer and material map in place, emit,
 * refit. */
int orc_build(orc_scene* s, int depth, int min_leaf, int sort_kind) {
    if (depth < 1 || depth > 32 || min_leaf < 1 || min_leaf > 256 || s->N == 0) return -1;
    const uint32_t N = s->N;
    s->depth = depth;
    s->min_leaf = min_leaf;
    s->keys.resize(N);
    if (orc_morton_keys(s, depth, s->keys.data(), nullptr, nullptr)) return -1;
    s->perm.resize(N);
    if (sort_kind == 1) {
        if (bitonic_sort(s->keys.data(), N, s->perm.data())) return -1;
    } else {
        for (uint32_t i = 0; i < N; ++i) s->perm[i] = i;
        std::stable_sort(s->perm.begin(), s->perm.end(),
                         [&](uint32_t a, uint32_t b) { return s->keys[a] < s->keys[b]; });
    }
    s->sorted_keys.resize(N);
    std::vector<uint32_t> idx2((size_t)N * 3), map2(N), orig2(N);
    for (uint32_t i = 0; i < N; ++i) {
        uint32_t o = s->perm[i];
        s->sorted_keys[i] = s->keys[o];
        idx2[3 * (size_t)i + 0] = s->idx[3 * (size_t)o + 0];
        idx2[3 * (size_t)i + 1] = s->idx[3 * (size_t)o + 1];
        idx2[3 * (size_t)i + 2] = s->idx[3 * (size_t)o + 2];
        map2[i] = s->map[o];
        orig2[i] = s->orig_id[o];
    }
    s->idx.swap(idx2);
    s->map.swap(map2);
    s->orig_id.swap(orig2);
    s->nodes.clear();
    s->nodes.reserve(2 * (size_t)N);
    emit(s, 0, N, 0, 0);
    refit(s);
    s->built = true;
    return 0;
}

/* BVH::construct (bvh.cpp:92-141) over the scene's triangles in their
 * current order: boxes by BBox::set (bbox.cpp:24-28), the recursive SAH
 * split, then the triangles (indices, materials, ids) reordered like
 * Mesh::reorderTriangles.  -2 when an interior node lies deeper than the
 * traversal's 32-entry stack reaches. */
int orc_build_sah(orc_scene* s) {
    if (s->N == 0) return -1;
    const uint32_t N = s->N;
    std::vector<sah::Box> boxes(N);
    for (uint32_t i = 0; i < N; ++i) {
        const float* p0 = &s->pos[4 * (size_t)s->idx[3 * (size_t)i + 0]];
        const float* p1 = &s->pos[4 * (size_t)s->idx[3 * (size_t)i + 1]];
        const float* p2 = &s->pos[4 * (size_t)s->idx[3 * (size_t)i + 2]];
        for (int c = 0; c < 3; ++c) {
            boxes[i].hi[c] = sah::smax(p0[c], sah::smax(p1[c], p2[c]));
            boxes[i].lo[c] = sah::smin(p0[c], sah::smin(p1[c], p2[c]));
        }
    }
    std::vector<uint32_t> ot(N);
    for (uint32_t i = 0; i < N; ++i) ot[i] = i;
    std::vector<Node> nodes(1);
    sah::Builder b{boxes, ot, nodes};
    b.sort(0, 0, N, 0);
    if (b.too_deep) return -2;
    std::vector<uint32_t> idx2((size_t)N * 3), map2(N), orig2(N);
    for (uint32_t i = 0; i < N; ++i) {
        const uint32_t o = ot[i];
        for (int k = 0; k < 3; ++k) idx2[3 * (size_t)i + k] = s->idx[3 * (size_t)o + k];
        map2[i] = s->map[o];
        orig2[i] = s->orig_id[o];
    }
    s->idx.swap(idx2);
    s->map.swap(map2);
    s->orig_id.swap(orig2);
    s->perm = ot;
    s->keys.clear();
    s->sorted_keys.clear();
    s->nodes.swap(nodes);
    s->built = true;
    s->sah = true;
    return 0;
}

/* The SAH tree in the reference's numbering: per node lo[3], hi[3], (a, b)
 * = children or the leaf's [start, end), leaf flag; order = slot ->
 * triangle before the build. */
int orc_sah_nodes(const orc_scene* s, float* lo, float* hi, uint32_t* a, uint32_t* b,
                  uint32_t* leaf, uint32_t* order, uint32_t* count) {
    if (!s->built || !s->sah) return -1;
    *count = (uint32_t)s->nodes.size();
    if (!lo) return 0;
    for (size_t k = 0; k < s->nodes.size(); ++k) {
        const Node& nd = s->nodes[k];
        for (int c = 0; c < 3; ++c) {
            lo[3 * k + c] = nd.lo[c];
            hi[3 * k + c] = nd.hi[c];
        }
        a[k] = nd.a;
        b[k] = nd.b;
        leaf[k] = nd.leaf;
    }
    std::memcpy(order, s->perm.data(), 4 * (size_t)s->N);
    return 0;
}

/* The emit rule alone on given sorted keys (ranges only; AABBs zero). */
int orc_emit_keys(const uint32_t* sorted_keys, uint32_t n, int depth, int min_leaf,
                  rt_canon_node* out, uint32_t cap, uint32_t* count) {
    if (n == 0 || depth < 1 || depth > 32) return -1;
    orc_scene s;
    s.N = n;
    s.depth = depth;
    s.min_leaf = min_leaf;
    s.sorted_keys.assign(sorted_keys, sorted_keys + n);
    emit(&s, 0, n, 0, 0);
    *count = (uint32_t)s.nodes.size();
    if (!out) return 0;
    if (cap < s.nodes.size()) return -1;
    for (size_t k = 0; k < s.nodes.size(); ++k) {
        rt_canon_node c;
        std::memset(&c, 0, sizeof(c));
        c.start = s.nodes[k].start;
        c.end = s.nodes[k].end;
        c.leaf = s.nodes[k].leaf;
        c.depth = s.nodes[k].depth;
        out[k] = c;
    }
    return 0;
}

/* refit_lbvh (bvh-builder.cpp:743-850): new AABBs, same topology and order. */
int orc_refit(orc_scene* s) {
    if (!s->built || s->sah) return -1;
    refit(s);
    return 0;
}

int orc_get_sort(const orc_scene* s, uint32_t* keys, uint32_t* perm, uint32_t* sorted,
                 uint32_t* orig_id) {
    if (!s->built) return -1;
    size_t n = s->N;
    if (keys) std::memcpy(keys, s->keys.data(), 4 * n);
    if (perm) std::memcpy(perm, s->perm.data(), 4 * n);
    if (sorted) std::memcpy(sorted, s->sorted_keys.data(), 4 * n);
    if (orig_id) std::memcpy(orig_id, s->orig_id.data(), 4 * n);
    return 0;
}

int orc_get_buffers(const orc_scene* s, uint32_t* idx, uint32_t* map) {
    if (idx) std::memcpy(idx, s->idx.data(), 12 * (size_t)s->N);
    if (map) std::memcpy(map, s->map.data(), 4 * (size_t)s->N);
    return 0;
}

int orc_export(const orc_scene* s, rt_canon_node* out, uint32_t cap, uint32_t* count) {
    if (!s->built) return -1;
    *count = (uint32_t)s->nodes.size();
    if (!out) return 0;
    if (cap < s->nodes.size()) return -1;
    /* pre-order, left child first (the LBVH's array order already is) */
    std::vector<uint32_t> todo{0}, order;
    order.reserve(s->nodes.size());
    while (!todo.empty()) {
        const uint32_t k = todo.back();
        todo.pop_back();
        order.push_back(k);
        if (!s->nodes[k].leaf) {
            todo.push_back(s->nodes[k].b);
            todo.push_back(s->nodes[k].a);
        }
    }
    for (size_t q = 0; q < order.size(); ++q) {
        const size_t k = q;
        const Node& nd = s->nodes[order[q]];
        rt_canon_node c;
        std::memset(&c, 0, sizeof(c));
        c.start = nd.start;
        c.end = nd.end;
        c.leaf = nd.leaf;
        c.depth = nd.depth;
        for (int i = 0; i < 3; ++i) {
            c.lo[i] = nd.lo[i];
            c.hi[i] = nd.hi[i];
        }
        out[k] = c;
    }
    return 0;
}

/* generate_primary_rays (primary-ray-generator.cl:27-103) for global ids
 * [offset, offset + count). */
int orc_gen_primary(const rt_camera* cam, int32_t width, int32_t height, int32_t quad_size,
                    int32_t spp, const rt_pixel_sample* ps, size_t count, size_t offset,
                    rt_sample* out) {
    (void)spp;
    rt_pixel_sample one = {0.f, 0.f, 1.f};
    const int pixels = width * height;
    const int bs = quad_size, ba = quad_size * quad_size;
    const int xb = width / bs, yb = height / bs;
    const int block_rays = xb * yb * ba;
    const int right_rays = (width - xb * bs) * height;
    for (size_t k = 0; k < count; ++k) {
        int gid = (int)(offset + k);
        int i = gid % pixels;
        const rt_pixel_sample p = ps ? ps[gid / pixels] : one;
        int x, y;
        if (i < block_rays) {
            int block = i / ba, yblk = block / xb, xblk = block % xb;
            int bp = i % ba;
            x = xblk * bs + bp % bs;
            y = yblk * bs + bp / bs;
        } else if (i < block_rays + right_rays) {
            int sx = xb * bs, slab = width - sx, ri = i - block_rays;
            x = sx + ri % slab;
            y = ri / slab;
        } else {
            int sy = yb * bs, slab = height - sy, ti = i - (block_rays + right_rays);
            x = ti / slab;
            y = sy + ti % slab;
        }
        float xn = (0.5f + (float)x + p.ox) / (float)width;
        float yn = (0.5f + (float)y + p.oy) / (float)height;
        float a = xn * 2.0f - 1.0f, b = yn * 2.0f - 1.0f;
        v3 d = add(add(ld3(cam->dir), muls(ld3(cam->right), a)), muls(ld3(cam->up), b));
        d = normalize(d);
        rt_sample& o = out[k];
        std::memset(&o, 0, sizeof(o));
        o.ray.ori[0] = cam->pos[0]; o.ray.ori[1] = cam->pos[1]; o.ray.ori[2] = cam->pos[2];
        o.ray.dir[0] = d.x; o.ray.dir[1] = d.y; o.ray.dir[2] = d.z;
        o.ray.inv_dir[0] = 1.0f / d.x;
        o.ray.inv_dir[1] = 1.0f / d.y;
        o.ray.inv_dir[2] = 1.0f / d.z;
        o.ray.tmin = 0.0f;
        o.ray.tmax = 1e36f;
        o.pixel = width * y + x;
        o.contribution = p.contribution;
    }
    return 0;
}

int orc_trace(const orc_scene* s, const rt_sample* smp, int32_t n, rt_hit* hits, int threads) {
    if (!s->built) return -1;
    parallel_for(n, threads, [&](int64_t i) {
        Ray r = ray_of(smp[i]);
        Best b = trace_ray(s, r);
        complete(s, r, b, &hits[i]);
    });
    return 0;
}

/* Whether light L adds nothing to a hit's colour whatever its shadow ray
 * finds: both terms shade_one adds for an unblocked light (the diffuse
 * rgb * diffuse * cosL and the specular rgb * spec) are zero, as for a light
 * behind the surface or a surface without diffuse colour and shininess.  The
 * GPU's fused renders do not trace that shadow ray, and the work counts below
 * follow them.  Counting aid only; the oracle's own shadow and render
 * functions trace every shadow ray. */
static bool light_vanishes(const rt_light& L, const rt_material& mat, v3 hp, v3 n, v3 d) {
    v3 Ld;
    float LD = 1.0f;
    if (L.type == RT_DIR_L) {
        Ld = ld3(L.dir);
    } else if (L.type == RT_SPOT_L) {
        Ld = normalize(sub(hp, ld3(L.pos)));
        LD = clamp01((dot(Ld, ld3(L.dir)) - L.angle) / (1.0f - L.angle));
    } else {
        Ld = normalize(sub(hp, ld3(L.pos)));
    }
    const v3 rgb = muls(ld3(L.color), LD);
    const v3 r = sub(d, muls(muls(n, 2.0f), dot(d, n)));
    float cosL = clamp01(dot(n, neg(Ld)));
    cosL = cosL * cosL;
    float spec = clamp01(dot(r, neg(Ld)));
    spec = spec * spec;
    spec = spec * spec;
    spec = spec * spec;
    spec *= cosL * mat.shininess;
    const v3 dt = muls(mul(rgb, ld3(mat.diffuse)), cosL), st = muls(rgb, spec);
    return dt.x == 0.0f && dt.y == 0.0f && dt.z == 0.0f && st.x == 0.0f && st.y == 0.0f &&
           st.z == 0.0f;
}

/* Per hit, the lights whose shadow ray the fused GPU renders skip
 * (light_vanishes, bit l for light l; 0 for a miss): a test shades with
 * those bits flipped and expects the same image. */
int orc_vanishing_lights(const orc_scene* s, const rt_sample* smp, const rt_hit* hits, int32_t n,
                         uint32_t* masks) {
    for (int32_t i = 0; i < n; ++i) {
        masks[i] = 0;
        if (!hits[i].hit) continue;
        const rt_material& mat = s->mats[s->map[hits[i].id]];
        for (int l = 0; l < s->lights.count; ++l)
            if (light_vanishes(s->lights.light[l], mat, ld3(hits[i].hit_point), ld3(hits[i].n),
                               ld3(smp[i].ray.dir)))
                masks[i] |= 1u << l;
    }
    return 0;
}

/* Traversal work of the closest-hit rays smp[0, n) and of the shadow rays
 * of their hits toward each light: out = {interior nodes entered, triangles
 * tested} of the closest-hit traversals, the same of the shadow ones over
 * the shadow rays the fused GPU renders trace, the number of shadow rays
 * (hits x lights) and the number of them traced. */
int orc_traversal_counts(const orc_scene* s, const rt_sample* smp, int32_t n, int threads,
                         uint64_t out[6]) {
    if (!s->built) return -1;
    std::atomic<uint64_t> acc[6];
    for (auto& a : acc) a = 0;
    parallel_for(n, threads, [&](int64_t i) {
        const Ray r = ray_of(smp[i]);
        TravCounts c, cs;
        const Best b = trace_ray(s, r, &c);
        if (b.id >= 0) {
            rt_hit h;
            std::memset(&h, 0, sizeof h);
            complete(s, r, b, &h);
            const v3 hp = ld3(h.hit_point), hn = ld3(h.n);
            const rt_material& mat = s->mats[s->map[h.id]];
            for (int l = 0; l < s->lights.count; ++l) {
                if (light_vanishes(s->lights.light[l], mat, hp, hn, r.dir)) continue;
                light_occluded(s, s->lights.light[l], hp, &cs);
                acc[5] += 1;
            }
            acc[4] += (uint64_t)s->lights.count;
        }
        acc[0] += c.nodes;
        acc[1] += c.tris;
        acc[2] += cs.nodes;
        acc[3] += cs.tris;
    });
    for (int k = 0; k < 6; ++k) out[k] = acc[k];
    return 0;
}

int orc_shadow(const orc_scene* s, const rt_sample* smp, int32_t n, rt_hit* hits, int threads) {
    if (!s->built) return -1;
    (void)smp;
    parallel_for(n, threads, [&](int64_t i) {
        rt_hit& h = hits[i];
        if (!h.hit) return;
        v3 hp = ld3(h.hit_point);
        uint8_t mask = 0;
        for (int l = 0; l < s->lights.count; ++l)
            if (light_occluded(s, s->lights.light[l], hp)) mask |= (uint8_t)(1u << l);
        h.shadow_hit = mask;
    });
    return 0;
}

int orc_shade(const orc_scene* s, const rt_sample* smp, const rt_hit* hits, int32_t n,
              uint32_t* image, int threads) {
    parallel_for(n, threads, [&](int64_t i) { shade_one(s, smp[i], hits[i], image); });
    return 0;
}

/* mark + exclusive scan + emit of generate_secondary_rays_disc: reflection
 * rays first (in input order), then refraction rays (in input order); a ray
 * whose slot is at or beyond max_out is dropped, and a hit whose refraction
 * slot is beyond it keeps R = 1 for its reflection ray, as in the kernel. */
int orc_gen_secondary(const orc_scene* s, const rt_sample* in, int32_t n, const rt_hit* hits,
                      rt_sample* out, int32_t max_out, int32_t* count) {
    std::vector<uint8_t> refl_flag(n, 0), refr_flag(n, 0);
    int32_t n_refl = 0, n_refr = 0;
    for (int32_t i = 0; i < n; ++i) {
        if (!hits[i].hit) continue;
        const rt_material& mat = s->mats[s->map[hits[i].id]];
        if (mat.refractive_index > 0.0f) {
            float R;
            rt_sample tmp;
            if (refract_ray(in[i], hits[i], mat, &R, &tmp)) refr_flag[i] = 1;
        }
        if (mat.reflectiveness > 0.0f) refl_flag[i] = 1;
        n_refl += refl_flag[i];
        n_refr += refr_flag[i];
    }
    int32_t refl_id = 0, refr_id = n_refl;
    for (int32_t i = 0; i < n; ++i) {
        if (!hits[i].hit) continue;
        const rt_material& mat = s->mats[s->map[hits[i].id]];
        float R = 1.0f;
        if (mat.refractive_index > 0.0f && refr_id < max_out) {
            rt_sample r;
            if (refract_ray(in[i], hits[i], mat, &R, &r)) out[refr_id] = r;
        }
        if (mat.reflectiveness > 0.0f && refl_id < max_out)
            reflect_ray(in[i], hits[i], mat.reflectiveness, R, &out[refl_id]);
        refl_id += refl_flag[i];
        refr_id += refr_flag[i];
    }
    *count = std::min(n_refl + n_refr, max_out);
    return 0;
}

/* copy (framebuffer.cl:30-54) + UNORM8 conversion (round to nearest even,
 * saturate), alpha = 255. */
int orc_fb_copy(const uint32_t* image, uint8_t* rgba, size_t pixels) {
    const float inv = 1.0f / 1e6f;
    for (size_t p = 0; p < pixels; ++p) {
        for (int c = 0; c < 3; ++c) {
            float v = (float)image[3 * p + c] * inv;
            float x = std::nearbyint(clamp01(v) * 255.0f);
            rgba[4 * p + c] = (uint8_t)x;
        }
        rgba[4 * p + 3] = 255;
    }
    return 0;
}

/* Renderer::render_to_framebuffer (renderer.cpp:113-214) restricted to
 * global sample ids [offset, offset + count) in tiles of tile_size.
 * image: 3 uint32 per pixel, accumulated.  stats: accumulated. */
int orc_render(const orc_scene* s, const rt_camera* cam, int32_t width, int32_t height,
               int32_t max_bounces, size_t offset, size_t count, size_t tile_size,
               uint32_t* image, rt_render_stats* stats, int threads) {
    if (!s->built) return -1;
    if (threads <= 0) threads = (int)hw_threads();
    if (tile_size == 0) tile_size = 1u << 18;
    std::vector<rt_sample> a(tile_size), b(tile_size);
    std::vector<rt_hit> h(tile_size);
    for (size_t off = offset; off < offset + count; off += tile_size) {
        size_t cur = std::min(tile_size, offset + count - off);
        rt_sample* rin = a.data();
        rt_sample* rout = b.data();
        orc_gen_primary(cam, width, height, 32, 1, nullptr, cur, off, rin);
        std::memset(h.data(), 0, sizeof(rt_hit) * cur);
        orc_trace(s, rin, (int32_t)cur, h.data(), threads);
        orc_shadow(s, rin, (int32_t)cur, h.data(), threads);
        orc_shade(s, rin, h.data(), (int32_t)cur, image, threads);
        if (stats) {
            stats->primary_rays += cur;
            for (size_t i = 0; i < cur; ++i)
                if (h[i].hit) {
                    stats->hits++;
                    stats->shadow_rays += (uint64_t)s->lights.count;
                }
        }
        int32_t sec = (int32_t)cur;
        for (int bounce = 0; bounce < max_bounces; ++bounce) {
            int32_t nout = 0;
            orc_gen_secondary(s, rin, sec, h.data(), rout, (int32_t)tile_size, &nout);
            std::swap(rin, rout);
            sec = nout;
            if (!sec) break;
            std::memset(h.data(), 0, sizeof(rt_hit) * (size_t)sec);
            orc_trace(s, rin, sec, h.data(), threads);
            orc_shadow(s, rin, sec, h.data(), threads);
            orc_shade(s, rin, h.data(), sec, image, threads);
            if (stats) {
                stats->secondary_rays += (uint64_t)sec;
                for (int32_t i = 0; i < sec; ++i)
                    if (h[i].hit) {
                        stats->hits++;
                        stats->shadow_rays += (uint64_t)s->lights.count;
                    }
            }
        }
    }
    return 0;
}

/* FP64 brute-force closest hit over all triangles (ray subset); returns the
 * triangle id at upload (orig_id) or -1, and t. */
int orc_fp64_closest(const orc_scene* s, const rt_sample* smp, int32_t n, int32_t* id_out,
                     double* t_out, int threads) {
    if (threads <= 0) threads = (int)hw_threads();
    const uint32_t N = s->N;
    parallel_for(n, threads, [&](int64_t k) {
        const rt_sample& sm = smp[k];
        double o[3] = {sm.ray.ori[0], sm.ray.ori[1], sm.ray.ori[2]};
        double d[3] = {sm.ray.dir[0], sm.ray.dir[1], sm.ray.dir[2]};
        double best = (double)sm.ray.tmax;
        int32_t bid = -1;
        for (uint32_t i = 0; i < N; ++i) {
            const uint32_t* ix = &s->idx[3 * (size_t)i];
            double v0[3], e1[3], e2[3];
            for (int c = 0; c < 3; ++c) {
                v0[c] = s->pos[4 * (size_t)ix[0] + c];
                e1[c] = (double)s->pos[4 * (size_t)ix[1] + c] - v0[c];
                e2[c] = (double)s->pos[4 * (size_t)ix[2] + c] - v0[c];
            }
            double h[3] = {d[1] * e2[2] - d[2] * e2[1], d[2] * e2[0] - d[0] * e2[2],
                           d[0] * e2[1] - d[1] * e2[0]};
            double a = e1[0] * h[0] + e1[1] * h[1] + e1[2] * h[2];
            if (a == 0.0) continue;
            double f = 1.0 / a;
            double sv[3] = {o[0] - v0[0], o[1] - v0[1], o[2] - v0[2]};
            double u = f * (sv[0] * h[0] + sv[1] * h[1] + sv[2] * h[2]);
            if (u < 0.0 || u > 1.0) continue;
            double q[3] = {sv[1] * e1[2] - sv[2] * e1[1], sv[2] * e1[0] - sv[0] * e1[2],
                           sv[0] * e1[1] - sv[1] * e1[0]};
            double v = f * (d[0] * q[0] + d[1] * q[1] + d[2] * q[2]);
            if (v < 0.0 || u + v > 1.0) continue;
            double t = f * (e2[0] * q[0] + e2[1] * q[1] + e2[2] * q[2]);
            if (t >= (double)sm.ray.tmin && t <= best) {
                best = t;
                bid = (int32_t)s->orig_id[i];
            }
        }
        id_out[k] = bid;
        t_out[k] = best;
    });
    return 0;
}

/* FP64 t of a given triangle (id at upload) along a ray, or NaN on a miss. */
int orc_fp64_t_of(const orc_scene* s, const rt_sample* smp, int32_t n, const int32_t* tri_orig,
                  double* t_out) {
    std::vector<uint32_t> slot(s->N);
    for (uint32_t i = 0; i < s->N; ++i) slot[s->orig_id[i]] = i;
    for (int32_t k = 0; k < n; ++k) {
        t_out[k] = NAN;
        if (tri_orig[k] < 0) continue;
        const uint32_t* ix = &s->idx[3 * (size_t)slot[tri_orig[k]]];
        const rt_sample& sm = smp[k];
        double o[3] = {sm.ray.ori[0], sm.ray.ori[1], sm.ray.ori[2]};
        double d[3] = {sm.ray.dir[0], sm.ray.dir[1], sm.ray.dir[2]};
        double v0[3], e1[3], e2[3];
        for (int c = 0; c < 3; ++c) {
            v0[c] = s->pos[4 * (size_t)ix[0] + c];
            e1[c] = (double)s->pos[4 * (size_t)ix[1] + c] - v0[c];
            e2[c] = (double)s->pos[4 * (size_t)ix[2] + c] - v0[c];
        }
        double h[3] = {d[1] * e2[2] - d[2] * e2[1], d[2] * e2[0] - d[0] * e2[2],
                       d[0] * e2[1] - d[1] * e2[0]};
        double a = e1[0] * h[0] + e1[1] * h[1] + e1[2] * h[2];
        if (a == 0.0) continue;
        double f = 1.0 / a;
        double sv[3] = {o[0] - v0[0], o[1] - v0[1], o[2] - v0[2]};
        double q[3] = {sv[1] * e1[2] - sv[2] * e1[1], sv[2] * e1[0] - sv[0] * e1[2],
                       sv[0] * e1[1] - sv[1] * e1[0]};
        t_out[k] = f * (e2[0] * q[0] + e2[1] * q[1] + e2[2] * q[2]);
    }
    return 0;
}

}  /* extern "C" */

/* ----------------------------------------------------------------------- */
/* Multi-root traversal: trace_multi (trace-bvh.cl:420-463), its helpers     */
/* multiply_vector / multiply_point / transform_ray / transform_hit_info /   */
/* complete_transformed_hit_info (:84-181), and shadow_trace_multi           */
/* (shadow-trace-bvh.cl:317-373).  Instances reference built scenes and      */
/* carry a row-major 4x4 transform and its inverse (sqmat4); hit ids are     */
/* global over the distinct scenes in first-use order (instances of one      */
/* scene share its triangles, as the reference's roots of one mesh share its */
/* node range).                                                               */
/* ----------------------------------------------------------------------- */
struct orc_multi {
    std::vector<const orc_scene*> scenes;   /* distinct */
    std::vector<uint32_t> tri_off;          /* per distinct scene */
    std::vector<int> inst_scene;            /* per instance */
    std::vector<float> tr, trinv;           /* 16 per instance */
    orc_scene all;                          /* concatenated geometry and materials */
};

/* M x (v, w), then the homogeneous divide when |w'| > 1e-26 (the
 * kernels' dot of float4 is a left-to-right sum of the four products). */
static v3 mat_apply(const float* M, v3 v, float w) {
    float r[4];
    for (int k = 0; k < 4; ++k)
        r[k] = M[4 * k] * v.x + M[4 * k + 1] * v.y + M[4 * k + 2] * v.z + M[4 * k + 3] * w;
    if (std::fabs(r[3]) > 1e-26f) {
        const float d = r[3];
        r[0] = r[0] / d;
        r[1] = r[1] / d;
        r[2] = r[2] / d;
    }
    return mk(r[0], r[1], r[2]);
}

static Ray transform_ray(const Ray& ray, const float* M) {
    Ray t = ray;
    t.dir = mat_apply(M, ray.dir, 0.0f);
    t.ori = mat_apply(M, ray.ori, 1.0f);
    t.inv = mk(1.0f / t.dir.x, 1.0f / t.dir.y, 1.0f / t.dir.z);
    return t;
}

static Best trace_multi_ray(const orc_multi* m, const Ray& ray, int* root) {
    Best best{-1, 0.f, 0.f, 0.f};
    *root = -1;
    for (size_t i = 0; i < m->inst_scene.size(); ++i) {
        const int k = m->inst_scene[i];
        const Ray tr = transform_ray(ray, &m->trinv[16 * i]);
        Best h = trace_ray(m->scenes[k], tr);
        if (h.id >= 0) {
            v3 hp = add(tr.ori, muls(tr.dir, h.t));
            hp = mat_apply(&m->tr[16 * i], hp, 1.0f);
            const v3 dv = sub(hp, ray.ori);
            h.t = std::sqrt(dot(dv, dv));
            h.id += (int32_t)m->tri_off[k];
        }
        if (h.id >= 0 && (best.id < 0 || h.t < best.t)) {
            best = h;
            *root = (int)i;
        }
    }
    return best;
}

static void complete_multi(const orc_multi* m, const Ray& ray, const Best& b, int root, rt_hit* out) {
    if (b.id < 0) {
        out->hit = 0;
        return;
    }
    const orc_scene* s = &m->all;
    rt_hit h;
    std::memset(&h, 0, sizeof(h));
    h.hit = 1;
    h.shadow_hit = out->shadow_hit;
    h.t = b.t;
    h.id = b.id;
    const v3 hp = add(ray.ori, muls(ray.dir, b.t));
    const uint32_t* ix = &s->idx[3 * (size_t)b.id];
    const v3 n0 = normalize(ld3(&s->nrm[4 * (size_t)ix[0]]));
    const v3 n1 = normalize(ld3(&s->nrm[4 * (size_t)ix[1]]));
    const v3 n2 = normalize(ld3(&s->nrm[4 * (size_t)ix[2]]));
    const float u = b.u, v = b.v;
    const float w = 1.0f - (u + v);
    v3 n = normalize(add(add(muls(n0, w), muls(n2, v)), muls(n1, u)));
    n = mat_apply(&m->tr[16 * (size_t)root], n, 0.0f);   /* not renormalised */
    if (dot(n, ray.dir) > 0.0f) {
        h.inverse_n = 1;
        n = muls(n, -1.0f);
    } else {
        h.inverse_n = 0;
    }
    h.n[0] = n.x; h.n[1] = n.y; h.n[2] = n.z;
    h.hit_point[0] = hp.x; h.hit_point[1] = hp.y; h.hit_point[2] = hp.z;
    *out = h;
}

/* shadow_trace_multi per light: the spot cone test leaves the point lit
 * (shadow-trace-bvh.cl:343-347, unlike the single-root kernel), unknown
 * light types light it; point lights (an extension) are spots without a
 * cone.  The shadow ray is traced against every root in object space. */
static bool light_occluded_multi(const orc_multi* m, const rt_light& L, v3 hp) {
    Ray r;
    r.ori = hp;
    if (L.type == RT_DIR_L) {
        r.dir = neg(ld3(L.dir));
    } else if (L.type == RT_SPOT_L) {
        r.dir = normalize(sub(ld3(L.pos), hp));
        if (dot(r.dir, ld3(L.dir)) < L.angle) return false;
    } else if (L.type == RT_POINT_L) {
        r.dir = normalize(sub(ld3(L.pos), hp));
    } else {
        return false;
    }
    r.inv = mk(1.0f / r.dir.x, 1.0f / r.dir.y, 1.0f / r.dir.z);
    r.tmin = 0.01f;
    r.tmax = 1e37f;
    for (size_t i = 0; i < m->inst_scene.size(); ++i) {
        const Ray tr = transform_ray(r, &m->trinv[16 * i]);
        if (trace_shadow(m->scenes[m->inst_scene[i]], tr)) return true;
    }
    return false;
}

extern "C" {

orc_multi* orc_multi_new(orc_scene** scenes, int32_t nscenes, const int32_t* inst_scene,
                         const float* tr, const float* trinv, int32_t ninst,
                         const rt_lights* lights) {
    orc_multi* m = new orc_multi();
    uint32_t vo = 0, to = 0, mo = 0;
    for (int k = 0; k < nscenes; ++k) {
        const orc_scene* s = scenes[k];
        if (!s->built) {
            delete m;
            return nullptr;
        }
        m->scenes.push_back(s);
        m->tri_off.push_back(to);
        m->all.pos.insert(m->all.pos.end(), s->pos.begin(), s->pos.end());
        m->all.nrm.insert(m->all.nrm.end(), s->nrm.begin(), s->nrm.end());
        for (uint32_t x : s->idx) m->all.idx.push_back(x + vo);
        for (uint32_t x : s->map) m->all.map.push_back(x + mo);
        m->all.mats.insert(m->all.mats.end(), s->mats.begin(), s->mats.end());
        vo += s->V;
        to += s->N;
        mo += (uint32_t)s->mats.size();
    }
    m->all.V = vo;
    m->all.N = to;
    m->all.lights = *lights;
    m->all.built = true;
    m->inst_scene.assign(inst_scene, inst_scene + ninst);
    m->tr.assign(tr, tr + 16 * (size_t)ninst);
    m->trinv.assign(trinv, trinv + 16 * (size_t)ninst);
    return m;
}

void orc_multi_free(orc_multi* m) { delete m; }

int orc_multi_trace(const orc_multi* m, const rt_sample* smp, int32_t n, rt_hit* hits, int threads) {
    parallel_for(n, threads, [&](int64_t i) {
        const Ray r = ray_of(smp[i]);
        int root;
        const Best b = trace_multi_ray(m, r, &root);
        complete_multi(m, r, b, root, &hits[i]);
    });
    return 0;
}

int orc_multi_shadow(const orc_multi* m, const rt_sample* smp, int32_t n, rt_hit* hits, int threads) {
    (void)smp;
    parallel_for(n, threads, [&](int64_t i) {
        if (!hits[i].hit) return;
        uint32_t mask = 0;
        const v3 hp = ld3(hits[i].hit_point);
        for (int l = 0; l < m->all.lights.count; ++l)
            if (light_occluded_multi(m, m->all.lights.light[l], hp)) mask |= 1u << l;
        hits[i].shadow_hit = (uint8_t)mask;
    });
    return 0;
}

/* The renderer's tile and bounce loop (renderer.cpp:113-214) with the
 * multi-root tracer. */
int orc_multi_render(const orc_multi* m, const rt_camera* cam, int32_t width, int32_t height,
                     int32_t max_bounces, size_t tile_size, uint32_t* image, rt_render_stats* stats,
                     int threads) {
    if (threads <= 0) threads = (int)hw_threads();
    if (tile_size == 0) tile_size = 1u << 18;
    const orc_scene* s = &m->all;
    const size_t count = (size_t)width * height;
    std::vector<rt_sample> a(tile_size), b(tile_size);
    std::vector<rt_hit> h(tile_size);
    for (size_t off = 0; off < count; off += tile_size) {
        size_t cur = std::min(tile_size, count - off);
        rt_sample* rin = a.data();
        rt_sample* rout = b.data();
        orc_gen_primary(cam, width, height, 32, 1, nullptr, cur, off, rin);
        int32_t sec = (int32_t)cur;
        for (int bounce = 0;; ++bounce) {
            std::memset(h.data(), 0, sizeof(rt_hit) * (size_t)sec);
            orc_multi_trace(m, rin, sec, h.data(), threads);
            orc_multi_shadow(m, rin, sec, h.data(), threads);
            orc_shade(s, rin, h.data(), sec, image, threads);
            if (stats) {
                if (bounce == 0)
                    stats->primary_rays += (uint64_t)sec;
                else
                    stats->secondary_rays += (uint64_t)sec;
                for (int32_t i = 0; i < sec; ++i)
                    if (h[i].hit) {
                        stats->hits++;
                        stats->shadow_rays += (uint64_t)s->lights.count;
                    }
            }
            if (bounce == max_bounces) break;
            int32_t nout = 0;
            orc_gen_secondary(s, rin, sec, h.data(), rout, (int32_t)tile_size, &nout);
            std::swap(rin, rout);
            sec = nout;
            if (!sec) break;
        }
    }
    return 0;
}

}  /* extern "C" */
