/*
 * ref_driver.cpp — ORACLE test infrastructure.
 *
 * Host-side driver for the reference's own kernels compiled for the CPU
 * (ref_*.cpp).  It restates the reference's host loops, which depend on an
 * OpenCL context and cannot be compiled here:
 *   bitonic launch sequence   src/rt/bvh-builder.cpp:361-454
 *   rearrange via aux copies  src/rt/bvh-builder.cpp:470-527
 *   node refit level loop     src/rt/bvh-builder.cpp:660-695
 *   secondary generation      src/rt/secondary-ray-generator.cpp:148-244
 *                             (mark -> exclusive scan -> generate, "disc")
 *   tile / bounce loop        src/rt/renderer.cpp:113-214
 *   level loop, OC readback   src/rt/bvh-builder.cpp:548-625 (ref_emit.cpp)
 * The two work-group kernels, max_local_bbox (bvh-builder.cl:318-391) and
 * process_task (bvh-builder.cl:582-671), run as emulated work-groups in
 * ref_emit.cpp; refd_build_lbvh chains every stage of build_lbvh
 * (bvh-builder.cpp:201-741) over the reference's own kernels.  The older
 * entry points refd_morton (order-free global AABB) and refd_set_tree (a
 * canonical range tree laid out and refitted by the reference's kernels) stay
 * for pins of single stages.
 */
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../../include/rt_cuda.h"

extern "C" {
size_t refk_sizeof_vertex(void);
size_t refk_sizeof_bbox(void);
size_t refk_sizeof_node(void);
size_t refk_sizeof_morton(void);
size_t refk_sizeof_lights(void);
void refk_make_vertices(const float* pos4, const float* nrm4, size_t v, void* out);
void refk_build_primitive_bbox(void* vtx, int* idx, void* bboxes, unsigned* tris, size_t n);
void refk_morton_encode(void* bboxes, const float* glo, const float* ghi, void* codes, int depth,
                        size_t n);
void refk_bbox_get(const void* bboxes, size_t i, float* lo3, float* hi3);
void refk_morton_get(const void* codes, size_t n, unsigned* lo, unsigned* hi);
void refk_rearrange_indices(int* in, unsigned* tris, int* out, size_t n);
void refk_rearrange_map(int* in, unsigned* tris, int* out, size_t n);
void refk_rearrange_morton_codes(void* in, unsigned* tris, void* out, size_t n);
void refk_node_set(void* nodes, size_t i, unsigned a, unsigned b, unsigned parent, int leaf);
void refk_node_get(const void* nodes, size_t i, float* lo3, float* hi3, unsigned* a, unsigned* b,
                   int* leaf);
void refk_build_leaf_bbox(unsigned* tris, void* bboxes, void* nodes, size_t n);
void refk_build_node_bbox(void* nodes, size_t start, size_t count);
void refk_morton_sort(int g, void* codes, unsigned* tris, int inc, int dir, int inv, int last_step,
                      int size, size_t items);
void refk_trace_single(rt_hit* info, rt_sample* samples, void* vtx, int* idx, void* nodes, size_t n,
                       int threads);
int refk_make_lights(const rt_lights* in, void* out);
void refk_offset_nodes(void* nodes, size_t n, unsigned node_off, unsigned tri_off);
size_t refk_sizeof_root(void);
void refk_make_root(void* roots, size_t i, int node, const float* tr, const float* trinv);
void refk_trace_multi(rt_hit* info, rt_sample* samples, void* vtx, int* idx, void* nodes, void* roots,
                      int root_count, size_t n, int threads);
void refk_shadow_trace_multi(rt_hit* info, rt_sample* samples, void* vtx, int* idx, void* nodes,
                             void* lights, void* roots, int root_count, size_t n, int threads);
void refk_shadow_trace_single(rt_hit* info, rt_sample* samples, void* vtx, int* idx, void* nodes,
                              void* lights, size_t n, int threads);
void refk_shade(int primary, uint32_t* image, rt_hit* info, rt_sample* samples, rt_material* mats,
                unsigned* map, void* lights, size_t n, int threads);
void refk_mark_secondary_rays_disc(rt_hit* info, rt_sample* samples, rt_material* mats,
                                   unsigned* map, int* count, int refract_offset, size_t n);
void refk_generate_secondary_rays_disc(rt_hit* info, rt_sample* samples, rt_material* mats,
                                       unsigned* map, rt_sample* out, int* count,
                                       int refract_offset, int max_count, size_t n);
int refe_global_bbox(const void* bboxes, uint32_t n, int group_size, int concurrent, float* lo3,
                     float* hi3);
int64_t refe_process_levels(const uint32_t* sorted, uint32_t n, int depth, int min_leaf,
                            int group_size, int compute_units, void* nodes_out,
                            uint32_t* level_end);
size_t refe_sizeof_node(void);
size_t refe_sizeof_bbox(void);
void refk_generate_primary_rays(rt_sample* samples, const float* pos, const float* dir,
                                const float* right, const float* up, int w, int h, int quad, int spp,
                                const rt_pixel_sample* ps, size_t count, size_t offset);
}

struct refd_scene {
    uint32_t V = 0, N = 0;
    std::vector<uint8_t> vtx;      /* reference Vertex AoS */
    std::vector<int> idx;
    std::vector<unsigned> map;
    std::vector<rt_material> mats;
    std::vector<uint8_t> lights;   /* reference Lights */
    std::vector<uint8_t> nodes;    /* reference BVHNode, level order */
    std::vector<uint32_t> canon_to_ref;
    uint32_t nnodes = 0;
};

extern "C" {

refd_scene* refd_scene_new(const float* pos4, const float* nrm4, uint32_t V, const uint32_t* idx,
                           uint32_t N, const rt_material* mats, uint32_t M, const uint32_t* map,
                           const rt_lights* lights) {
    refd_scene* s = new refd_scene();
    s->V = V;
    s->N = N;
    s->vtx.resize(refk_sizeof_vertex() * V);
    refk_make_vertices(pos4, nrm4, V, s->vtx.data());
    s->idx.assign(idx, idx + 3 * (size_t)N);
    s->map.assign(map, map + N);
    s->mats.assign(mats, mats + M);
    s->lights.resize(refk_sizeof_lights());
    if (refk_make_lights(lights, s->lights.data())) {
        delete s;
        return nullptr;
    }
    return s;
}

void refd_scene_free(refd_scene* s) { delete s; }

/* build_primitive_bbox -> global AABB -> morton_encode (bvh-builder.cpp:232-349). */
int refd_morton(refd_scene* s, int depth, uint32_t* keys, float* glo_out, float* ghi_out) {
    const size_t N = s->N;
    std::vector<uint8_t> bboxes(refk_sizeof_bbox() * N);
    std::vector<unsigned> tris(N);
    refk_build_primitive_bbox(s->vtx.data(), s->idx.data(), bboxes.data(), tris.data(), N);
    float glo[3] = {1e37f, 1e37f, 1e37f}, ghi[3] = {-1e37f, -1e37f, -1e37f};
    for (size_t i = 0; i < N; ++i) {
        float lo[3], hi[3];
        refk_bbox_get(bboxes.data(), i, lo, hi);
        for (int c = 0; c < 3; ++c) {
            glo[c] = std::fmin(glo[c], lo[c]);
            ghi[c] = std::fmax(ghi[c], hi[c]);
        }
    }
    std::vector<uint8_t> codes(refk_sizeof_morton() * N);
    refk_morton_encode(bboxes.data(), glo, ghi, codes.data(), depth, N);
    std::vector<unsigned> hi(N);
    refk_morton_get(codes.data(), N, keys, hi.data());
    for (size_t i = 0; i < N; ++i)
        if (hi[i] != 0) return -1;
    if (glo_out) std::memcpy(glo_out, glo, sizeof(glo));
    if (ghi_out) std::memcpy(ghi_out, ghi, sizeof(ghi));
    return 0;
}

/* The bitonic launch sequence of bvh-builder.cpp:361-454 over the compiled
 * morton_sort_g* kernels.  Returns -1 where the reference calls exit(1). */
int refd_bitonic(const uint32_t* keys, uint32_t n, uint32_t* perm) {
    std::vector<uint8_t> codes(refk_sizeof_morton() * (size_t)n, 0);
    for (uint32_t i = 0; i < n; ++i) std::memcpy(&codes[refk_sizeof_morton() * i], &keys[i], 4);
    for (uint32_t i = 0; i < n; ++i) perm[i] = i;
    int size = (int)n, n2 = 1;
    while (n2 < size) n2 <<= 1;
    size_t ms2 = size / 2 + (size % 2);
    size_t ms4 = size / 4 + (size - size % 4);
    size_t ms8 = size / 8 + (size - size % 8);
    size_t ms16 = size / 16 + (size - size % 16);
    for (int len = 1; len < n2; len <<= 1) {
        int dir = len << 1;
        int inv = ((size - 1) & dir) == 0 && dir != n2;
        int last_step = dir == n2;
        for (int inc = len; inc > 0; inc >>= 1) {
            int g;
            size_t items;
            if (inc > 4) {
                inc >>= 3;
                g = 16;
                items = ms16;
            } else if (inc > 2) {
                inc >>= 2;
                g = 8;
                items = ms8;
            } else if (inc > 1) {
                inc >>= 1;
                g = 4;
                items = ms4;
            } else {
                g = 2;
                items = ms2;
            }
            if (items == 0) return -1;
            refk_morton_sort(g, codes.data(), perm, inc, dir, inv, last_step, size, items);
        }
    }
    return 0;
}

/* rearrange_indices / rearrange_map through aux copies (bvh-builder.cpp:470-512). */
int refd_apply_perm(refd_scene* s, const uint32_t* perm) {
    std::vector<unsigned> tris(perm, perm + s->N);
    std::vector<int> aux(s->idx);
    refk_rearrange_indices(aux.data(), tris.data(), s->idx.data(), s->N);
    std::vector<int> auxm(s->map.begin(), s->map.end());
    refk_rearrange_map(auxm.data(), tris.data(), (int*)s->map.data(), s->N);
    return 0;
}

int refd_get_buffers(const refd_scene* s, uint32_t* idx, uint32_t* map) {
    if (idx) std::memcpy(idx, s->idx.data(), 12 * (size_t)s->N);
    if (map) std::memcpy(map, s->map.data(), 4 * (size_t)s->N);
    return 0;
}

/* Lays the canonical tree out as the reference does (level order, children
 * adjacent, bvh-builder.cpp:548-625) and refits it with build_leaf_bbox and
 * build_node_bbox, deepest level first (bvh-builder.cpp:660-695).  The
 * triangle order is the scene's current (sorted) order: triangles[i] = i. */
int refd_set_tree(refd_scene* s, const rt_canon_node* canon, uint32_t n) {
    /* children in pre-order: left = k+1, right = after the left subtree */
    std::vector<int64_t> left(n, -1), right(n, -1);
    {
        std::vector<uint32_t> stack;
        std::vector<int> nchild(n, 0);
        for (uint32_t k = 0; k < n; ++k) {
            while (!stack.empty() && nchild[stack.back()] == 2) stack.pop_back();
            if (!stack.empty()) {
                uint32_t p = stack.back();
                if (nchild[p] == 0)
                    left[p] = k;
                else
                    right[p] = k;
                nchild[p]++;
            }
            if (!canon[k].leaf) stack.push_back(k);
        }
    }
    /* BFS order */
    std::vector<uint32_t> order;
    order.reserve(n);
    std::vector<uint32_t> ref_of(n, 0), parent_ref(n, 0);
    order.push_back(0);
    ref_of[0] = 0;
    std::vector<uint32_t> level_start;
    std::vector<uint32_t> level_of_ref;
    for (size_t q = 0; q < order.size(); ++q) {
        uint32_t k = order[q];
        if (!canon[k].leaf) {
            uint32_t l = (uint32_t)left[k], r = (uint32_t)right[k];
            ref_of[l] = (uint32_t)order.size();
            order.push_back(l);
            ref_of[r] = (uint32_t)order.size();
            order.push_back(r);
            parent_ref[l] = parent_ref[r] = ref_of[k];
        }
    }
    s->nodes.assign(refk_sizeof_node() * n, 0);
    uint32_t maxdepth = 0;
    for (uint32_t k = 0; k < n; ++k) {
        const rt_canon_node& c = canon[k];
        maxdepth = std::max(maxdepth, c.depth);
        if (c.leaf)
            refk_node_set(s->nodes.data(), ref_of[k], c.start, c.end, parent_ref[k], 1);
        else
            refk_node_set(s->nodes.data(), ref_of[k], ref_of[left[k]], ref_of[right[k]], parent_ref[k], 0);
    }
    s->nnodes = n;
    s->canon_to_ref = ref_of;
    /* refit */
    std::vector<unsigned> tris(s->N);
    std::vector<uint8_t> bboxes(refk_sizeof_bbox() * s->N);
    refk_build_primitive_bbox(s->vtx.data(), s->idx.data(), bboxes.data(), tris.data(), s->N);
    refk_build_leaf_bbox(tris.data(), bboxes.data(), s->nodes.data(), n);
    /* level ranges in BFS order (depth is non-decreasing along `order`) */
    std::vector<uint32_t> start(maxdepth + 2, n);
    for (int64_t q = (int64_t)n - 1; q >= 0; --q) start[canon[order[q]].depth] = (uint32_t)q;
    start[maxdepth + 1] = n;
    for (int64_t d = maxdepth; d >= 0; --d) {
        uint32_t b = start[d], e = start[d + 1];
        if (e > b) refk_build_node_bbox(s->nodes.data(), b, e - b);
    }
    return 0;
}

/* Pre-order walk (left first) of the reference's node array from the root:
 * the canonical range tree.  Interior ranges come from the subtrees, since
 * set_children overwrites an interior node's range with its child indices;
 * any nonzero `leaf` byte is a leaf (nodes of the last launched level keep
 * the level they would have checked next). */
static int canon_walk(refd_scene* s, uint32_t k, uint32_t depth, std::vector<rt_canon_node>& out,
                      std::vector<uint32_t>& ref_of) {
    if (k >= s->nnodes || out.size() >= s->nnodes || depth > 64) return -1;
    const size_t me = out.size();
    out.emplace_back();
    ref_of.push_back(k);
    rt_canon_node c;
    std::memset(&c, 0, sizeof(c));
    unsigned a, b;
    int leaf;
    refk_node_get(s->nodes.data(), k, c.lo, c.hi, &a, &b, &leaf);
    c.depth = depth;
    if (leaf) {
        c.leaf = 1;
        c.start = a;
        c.end = b;
    } else {
        if (canon_walk(s, a, depth + 1, out, ref_of)) return -1;
        const size_t r = out.size();
        if (canon_walk(s, b, depth + 1, out, ref_of)) return -1;
        c.start = out[me + 1].start;
        c.end = out[r].end;
    }
    out[me] = c;
    return 0;
}

/* BVHBuilder::build_lbvh (bvh-builder.cpp:201-741) over the reference's own
 * kernels: build_primitive_bbox, the max_local_bbox reduction, morton_encode,
 * the bitonic network, rearrange_indices / map / morton_codes, process_task
 * level by level, build_leaf_bbox over every node and build_node_bbox level
 * by level from the deepest.  depth and min_leaf are clamped as
 * update_configuration does (bvh-builder.cpp:194-199); depths above 32 are
 * refused (the keys here are one 32-bit word).  group_size and
 * compute_units shape the emulated launches (the device's
 * max_group_size() and CL_DEVICE_MAX_COMPUTE_UNITS).  Outputs: the
 * unsorted keys, the permutation, the global AABB; the tree stays in the
 * scene (reference numbering) for refd_canon, trace and render. */
int refd_build_lbvh(refd_scene* s, int depth, int min_leaf, int group_size, int compute_units,
                    uint32_t* keys_out, uint32_t* perm_out, float* glo_out, float* ghi_out) {
    depth = std::min(std::max(depth, 1), 64);
    min_leaf = std::min(std::max(min_leaf, 1), 256);
    if (depth > 32 || s->N == 0) return -1;
    const size_t N = s->N;
    std::vector<uint8_t> bboxes(refk_sizeof_bbox() * N);
    std::vector<unsigned> tris(N);
    refk_build_primitive_bbox(s->vtx.data(), s->idx.data(), bboxes.data(), tris.data(), N);
    float glo[3], ghi[3];
    if (refe_global_bbox(bboxes.data(), s->N, group_size, 2, glo, ghi)) return -1;
    std::vector<uint8_t> codes(refk_sizeof_morton() * N);
    refk_morton_encode(bboxes.data(), glo, ghi, codes.data(), depth, N);
    std::vector<uint32_t> keys(N), hi(N), perm(N);
    refk_morton_get(codes.data(), N, keys.data(), hi.data());
    for (size_t i = 0; i < N; ++i)
        if (hi[i] != 0) return -1;
    if (refd_bitonic(keys.data(), s->N, perm.data())) return -1;
    refd_apply_perm(s, perm.data());
    std::vector<uint8_t> sorted_codes(codes.size());
    refk_rearrange_morton_codes(codes.data(), perm.data(), sorted_codes.data(), N);
    std::vector<uint32_t> sorted(N);
    refk_morton_get(sorted_codes.data(), N, sorted.data(), nullptr);
    s->nodes.assign(refe_sizeof_node() * 2 * N, 0);
    uint32_t level_end[64];
    const int64_t cnt = refe_process_levels(sorted.data(), s->N, depth, min_leaf, group_size,
                                            compute_units, s->nodes.data(), level_end);
    if (cnt < 1) return -1;
    s->nnodes = (uint32_t)cnt;
    refk_build_leaf_bbox(perm.data(), bboxes.data(), s->nodes.data(), s->nnodes);
    for (int i = depth - 1; i >= 0; --i) {
        const uint32_t start = i ? level_end[i - 1] : 0;
        const uint32_t count = level_end[i] - start;
        if (count) refk_build_node_bbox(s->nodes.data(), start, count);
    }
    std::vector<rt_canon_node> canon;
    std::vector<uint32_t> ref_of;
    if (canon_walk(s, 0, 0, canon, ref_of)) return -1;
    s->canon_to_ref = ref_of;
    if (keys_out) std::memcpy(keys_out, keys.data(), 4 * N);
    if (perm_out) std::memcpy(perm_out, perm.data(), 4 * N);
    if (glo_out) std::memcpy(glo_out, glo, sizeof(glo));
    if (ghi_out) std::memcpy(ghi_out, ghi, sizeof(ghi));
    return 0;
}

/* The canonical range tree of the scene's reference-numbered tree (after
 * refd_build_lbvh): the node count in *count; nodes into out when cap holds
 * them.  The walk visits every node once when the tree is well formed. */
int refd_canon(refd_scene* s, rt_canon_node* out, uint32_t cap, uint32_t* count) {
    std::vector<rt_canon_node> canon;
    std::vector<uint32_t> ref_of;
    if (canon_walk(s, 0, 0, canon, ref_of)) return -1;
    *count = (uint32_t)canon.size();
    if (!out) return 0;
    if (cap < canon.size()) return -1;
    std::memcpy(out, canon.data(), sizeof(rt_canon_node) * canon.size());
    return 0;
}

int refd_get_tree(const refd_scene* s, rt_canon_node* out) {
    for (uint32_t k = 0; k < s->nnodes; ++k) {
        unsigned a, b;
        int leaf;
        refk_node_get(s->nodes.data(), s->canon_to_ref[k], out[k].lo, out[k].hi, &a, &b, &leaf);
    }
    return 0;
}

int refd_gen_primary(const rt_camera* cam, int32_t w, int32_t h, int32_t quad, int32_t spp,
                     const rt_pixel_sample* ps, size_t count, size_t offset, rt_sample* out) {
    std::memset(out, 0, sizeof(rt_sample) * count);
    refk_generate_primary_rays(out, cam->pos, cam->dir, cam->right, cam->up, w, h, quad, spp, ps,
                               count, offset);
    return 0;
}

int refd_trace(refd_scene* s, rt_sample* samples, int32_t n, rt_hit* hits, int threads) {
    refk_trace_single(hits, samples, s->vtx.data(), s->idx.data(), s->nodes.data(), n, threads);
    return 0;
}

int refd_shadow(refd_scene* s, rt_sample* samples, int32_t n, rt_hit* hits, int threads) {
    refk_shadow_trace_single(hits, samples, s->vtx.data(), s->idx.data(), s->nodes.data(),
                             s->lights.data(), n, threads);
    return 0;
}

/* shade_secondary reads one sample past the run it shades; a sentinel with
 * pixel -1 stands in for the buffer slack the reference relies on. */
int refd_shade(refd_scene* s, const rt_sample* samples, rt_hit* hits, int32_t n, uint32_t* image,
               int primary, int threads) {
    std::vector<rt_sample> pad(samples, samples + n);
    rt_sample sentinel;
    std::memset(&sentinel, 0, sizeof(sentinel));
    sentinel.pixel = -1;
    pad.push_back(sentinel);
    std::vector<rt_hit> hpad(hits, hits + n);
    hpad.push_back(rt_hit{});
    /* one thread: the kernel adds to pixels without atomics, and with
     * refraction one pixel has two samples in a wavefront */
    (void)threads;
    refk_shade(primary, image, hpad.data(), pad.data(), s->mats.data(), s->map.data(),
               s->lights.data(), n, 1);
    return 0;
}

/* gen_scan_disc (secondary-ray-generator.cpp:148-244): mark, exclusive scan
 * over 2 * rays_in counters (the reference's gpu_scan_uint), generate. */
int refd_gen_secondary(refd_scene* s, rt_sample* in, int32_t n, rt_hit* hits, rt_sample* out,
                       int32_t max_out, int32_t* count) {
    std::vector<int> cnt(2 * (size_t)n + 1, 0);
    refk_mark_secondary_rays_disc(hits, in, s->mats.data(), s->map.data(), cnt.data(), n, n);
    int acc = 0;
    for (size_t i = 0; i < 2 * (size_t)n; ++i) {
        int v = cnt[i];
        cnt[i] = acc;
        acc += v;
    }
    cnt[2 * (size_t)n] = acc;
    refk_generate_secondary_rays_disc(hits, in, s->mats.data(), s->map.data(), out, cnt.data(), n,
                                      max_out, n);
    *count = std::min(acc, max_out);
    return 0;
}

int refd_render(refd_scene* s, const rt_camera* cam, int32_t w, int32_t h, int32_t max_bounces,
                size_t offset, size_t count, size_t tile, uint32_t* image, rt_render_stats* stats,
                int threads) {
    if (tile == 0) tile = 1u << 18;
    std::vector<rt_sample> a(tile), b(tile);
    std::vector<rt_hit> hits(tile);
    for (size_t off = offset; off < offset + count; off += tile) {
        size_t cur = std::min(tile, offset + count - off);
        rt_sample* rin = a.data();
        rt_sample* rout = b.data();
        refd_gen_primary(cam, w, h, 32, 1, nullptr, cur, off, rin);
        std::memset(hits.data(), 0, sizeof(rt_hit) * cur);
        refd_trace(s, rin, (int32_t)cur, hits.data(), threads);
        refd_shadow(s, rin, (int32_t)cur, hits.data(), threads);
        refd_shade(s, rin, hits.data(), (int32_t)cur, image, 1, threads);
        if (stats) stats->primary_rays += cur;
        int32_t sec = (int32_t)cur;
        for (int bounce = 0; bounce < max_bounces; ++bounce) {
            int32_t nout = 0;
            refd_gen_secondary(s, rin, sec, hits.data(), rout, (int32_t)tile, &nout);
            std::swap(rin, rout);
            sec = nout;
            if (!sec) break;
            std::memset(hits.data(), 0, sizeof(rt_hit) * (size_t)sec);
            refd_trace(s, rin, sec, hits.data(), threads);
            refd_shadow(s, rin, sec, hits.data(), threads);
            refd_shade(s, rin, hits.data(), sec, image, 0, threads);
            if (stats) stats->secondary_rays += (uint64_t)sec;
        }
    }
    return 0;
}

/* Scene::create_bvhs (src/rt/scene.cpp:636-703) over built scenes: the
 * meshes' vertices, indices, materials and trees concatenated (node and
 * triangle references offset), one BVHRoot per instance. */
struct refd_multi {
    refd_scene all;
    std::vector<uint8_t> roots;
    int nroots = 0;
};

refd_multi* refd_multi_new(refd_scene** scenes, int32_t nscenes, const int32_t* inst_scene,
                           const float* tr, const float* trinv, int32_t ninst,
                           const rt_lights* lights) {
    refd_multi* m = new refd_multi();
    std::vector<uint32_t> node_off;
    uint32_t vo = 0, to = 0, no = 0, mo = 0;
    for (int k = 0; k < nscenes; ++k) {
        refd_scene* s = scenes[k];
        node_off.push_back(no);
        m->all.vtx.insert(m->all.vtx.end(), s->vtx.begin(), s->vtx.end());
        for (int x : s->idx) m->all.idx.push_back(x + (int)vo);
        for (unsigned x : s->map) m->all.map.push_back(x + mo);
        m->all.mats.insert(m->all.mats.end(), s->mats.begin(), s->mats.end());
        const size_t at = m->all.nodes.size();
        m->all.nodes.insert(m->all.nodes.end(), s->nodes.begin(), s->nodes.end());
        refk_offset_nodes(m->all.nodes.data() + at, s->nnodes, no, to);
        vo += s->V;
        to += s->N;
        no += s->nnodes;
        mo += (uint32_t)s->mats.size();
    }
    m->all.V = vo;
    m->all.N = to;
    m->all.nnodes = no;
    m->all.lights.resize(refk_sizeof_lights());
    if (refk_make_lights(lights, m->all.lights.data())) {
        delete m;
        return nullptr;
    }
    m->nroots = ninst;
    m->roots.assign(refk_sizeof_root() * (size_t)ninst, 0);
    for (int i = 0; i < ninst; ++i)
        refk_make_root(m->roots.data(), i, (int)node_off[inst_scene[i]], tr + 16 * i, trinv + 16 * i);
    return m;
}

void refd_multi_free(refd_multi* m) { delete m; }

int refd_multi_trace(refd_multi* m, rt_sample* smp, int32_t n, rt_hit* hits, int threads) {
    refk_trace_multi(hits, smp, m->all.vtx.data(), m->all.idx.data(), m->all.nodes.data(),
                     m->roots.data(), m->nroots, n, threads);
    return 0;
}

int refd_multi_shadow(refd_multi* m, rt_sample* smp, int32_t n, rt_hit* hits, int threads) {
    refk_shadow_trace_multi(hits, smp, m->all.vtx.data(), m->all.idx.data(), m->all.nodes.data(),
                            m->all.lights.data(), m->roots.data(), m->nroots, n, threads);
    return 0;
}

int refd_multi_render(refd_multi* m, const rt_camera* cam, int32_t w, int32_t h,
                      int32_t max_bounces, size_t tile, uint32_t* image, rt_render_stats* stats,
                      int threads) {
    if (tile == 0) tile = 1u << 18;
    const size_t count = (size_t)w * h;
    std::vector<rt_sample> a(tile), b(tile);
    std::vector<rt_hit> hits(tile);
    for (size_t off = 0; off < count; off += tile) {
        size_t cur = std::min(tile, count - off);
        rt_sample* rin = a.data();
        rt_sample* rout = b.data();
        refd_gen_primary(cam, w, h, 32, 1, nullptr, cur, off, rin);
        int32_t sec = (int32_t)cur;
        for (int bounce = 0;; ++bounce) {
            std::memset(hits.data(), 0, sizeof(rt_hit) * (size_t)sec);
            refd_multi_trace(m, rin, sec, hits.data(), threads);
            refd_multi_shadow(m, rin, sec, hits.data(), threads);
            refd_shade(&m->all, rin, hits.data(), sec, image, bounce == 0, threads);
            if (stats && bounce > 0) stats->secondary_rays += (uint64_t)sec;
            if (bounce == max_bounces) break;
            int32_t nout = 0;
            refd_gen_secondary(&m->all, rin, sec, hits.data(), rout, (int32_t)tile, &nout);
            std::swap(rin, rout);
            sec = nout;
            if (!sec) break;
        }
    }
    return 0;
}

}  /* extern "C" */
