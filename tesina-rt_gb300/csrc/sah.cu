// sah.cu — the reference's CPU SAH BVH (BVH::construct / BVHNode::sort,
// src/rt/bvh.cpp:6-179; BBox, src/rt/bbox.cpp), built on the host as the
// reference builds it and laid out in the device node format of the LBVH,
// so that every render path traverses it unchanged.
//
// The tree is the reference's: per node the box of its triangles (std::max /
// std::min merges), a leaf at <= 2 triangles, otherwise the largest axis,
// the node's triangles sorted by centroid on it (std::sort), 32 buckets over
// the centroid range, the split after the bucket of least cost (the right
// side counts the last bucket twice, empty buckets carry the FLT_MIN
// maximum of BBox::reset), then the first triangle at or past the bucket
// boundary; if that split is empty, one more try on the next axis, else a
// leaf.  Subtrees below the top levels are built on host threads: each node
// only reorders its own range, so the result does not depend on the order
// in which subtrees are built.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <atomic>
#include <cstring>
#include <limits>
#include <thread>
#include <vector>

#include "sah.cuh"

namespace rt {
namespace {

inline float smax(float a, float b) { return a < b ? b : a; }   // std::max
inline float smin(float a, float b) { return b < a ? b : a; }   // std::min

struct Box {
    float lo[3], hi[3];
};

inline Box empty_box() {   // BBox::reset: hi = FLT_MIN, lo = FLT_MAX
    Box b;
    for (int c = 0; c < 3; ++c) {
        b.hi[c] = std::numeric_limits<float>::min();
        b.lo[c] = std::numeric_limits<float>::max();
    }
    return b;
}

inline void merge(Box& a, const Box& b) {
    for (int c = 0; c < 3; ++c) {
        a.hi[c] = smax(a.hi[c], b.hi[c]);
        a.lo[c] = smin(a.lo[c], b.lo[c]);
    }
}

inline float area(const Box& b) {
    float d[3];
    for (int c = 0; c < 3; ++c) d[c] = smax(b.hi[c] - b.lo[c], 0.f);
    return (d[0] * (d[1] + d[2]) + d[1] * d[2]) * 2.f;
}

inline int largest_axis(const Box& b) {
    const float dx = b.hi[0] - b.lo[0], dy = b.hi[1] - b.lo[1], dz = b.hi[2] - b.lo[2];
    if (dx > dy && dx > dz) return 0;
    if (dy > dz) return 1;
    return 2;
}

// uint32_t(32 * ((c - min) / length)) clamped to 31; the position lies in
// [0, 32], or is NaN on a flat axis, which converts to 0.
inline uint32_t bucket_of(float x) {
    if (!(x > 0.f)) return 0;
    if (x >= 31.f) return 31;
    return (uint32_t)x;
}

constexpr uint32_t kBuckets = 32;
constexpr uint32_t kMinPrims = 2;

struct TNode {
    Box box;
    uint32_t start, end, depth;
    int32_t l, r;       // children in the same tree, or -1
    int32_t task;       // >= 0: the subtree is built as task `task`
    bool leaf;
};

constexpr uint32_t kMaxInteriorDepth = 31;   // the traversal's 32-entry stack

struct Builder {
    const std::vector<Box>& boxes;
    const std::vector<float>& cen;   // centroid per triangle and axis: cen[3 t + axis]
    std::vector<uint32_t>& ot;
    std::atomic<bool>& too_deep;     // an interior node below kMaxInteriorDepth: stop there

    uint32_t choose(const Box& bb, int axis, uint32_t start, uint32_t end) const {
        const float len = bb.hi[axis] - bb.lo[axis];
        const float mn = bb.lo[axis];
        const float sa = area(bb);
        uint32_t prims[kBuckets];
        Box bbox[kBuckets];
        for (uint32_t k = 0; k < kBuckets; ++k) {
            prims[k] = 0;
            bbox[k] = empty_box();
        }
        for (uint32_t i = start; i < end; ++i) {
            const uint32_t t = ot[i];
            const uint32_t slot = bucket_of((float)kBuckets * ((cen[3 * (size_t)t + axis] - mn) / len));
            prims[slot]++;
            merge(bbox[slot], boxes[t]);
        }
        // prefix boxes from the left; from the right the sweep starts at the
        // last bucket and merges buckets i+1..31 again (the last one twice)
        Box left[kBuckets - 1];
        uint32_t nleft[kBuckets - 1];
        Box acc = bbox[0];
        uint32_t n = prims[0];
        for (uint32_t i = 0; i < kBuckets - 1; ++i) {
            if (i > 0) {
                merge(acc, bbox[i]);
                n += prims[i];
            }
            left[i] = acc;
            nleft[i] = n;
        }
        float best = 0.f;
        uint32_t best_i = 0;
        for (uint32_t i = 0; i < kBuckets - 1; ++i) {
            Box br = bbox[kBuckets - 1];
            uint32_t nr = prims[kBuckets - 1];
            for (uint32_t j = i + 1; j < kBuckets; ++j) {
                merge(br, bbox[j]);
                nr += prims[j];
            }
            const float cost =
                .125f + ((float)nleft[i] * area(left[i]) + (float)nr * area(br)) / sa;
            if (i == 0 || cost < best) {
                best = cost;
                best_i = i;
            }
        }
        float split_value = mn;
        split_value += (float)(best_i + 1) * (len / (float)kBuckets);
        uint32_t i = start;
        for (; i < end; ++i)
            if (cen[3 * (size_t)ot[i] + axis] >= split_value) break;
        return i;
    }

    // Box, leaf test and split of one node; returns false for a leaf.
    bool split(uint32_t start, uint32_t end, Box& bb, uint32_t& at) const {
        bb = boxes[ot[start]];
        for (uint32_t i = start; i < end; ++i) merge(bb, boxes[ot[i]]);
        if (end - start <= kMinPrims) return false;
        int axis = largest_axis(bb);
        at = start;
        for (int tries = 0; tries < 2; ++tries) {
            const float* c = cen.data();
            std::sort(ot.begin() + start, ot.begin() + end, [c, axis](uint32_t x, uint32_t y) {
                return c[3 * (size_t)x + axis] < c[3 * (size_t)y + axis];
            });
            at = choose(bb, axis, start, end);
            if (at == start || at == end)
                axis = (axis + 1) % 3;
            else
                break;
        }
        return !(at == start || at == end);
    }

    // Whole subtree into T (root first); `task_depth` > depth hands the
    // nodes reached at task_depth to separate tasks instead.
    int32_t build(std::vector<TNode>& T, uint32_t start, uint32_t end, uint32_t depth,
                  uint32_t task_depth, std::vector<TNode>* tasks) const {
        const int32_t me = (int32_t)T.size();
        T.push_back(TNode{});
        if (tasks && depth == task_depth && end - start > kMinPrims) {
            TNode t{};
            t.start = start;
            t.end = end;
            t.depth = depth;
            t.task = (int32_t)tasks->size();
            tasks->push_back(t);
            T[me] = t;
            return me;
        }
        TNode nd{};
        nd.start = start;
        nd.end = end;
        nd.depth = depth;
        nd.l = nd.r = -1;
        nd.task = -1;
        uint32_t at = start;
        nd.leaf = !split(start, end, nd.box, at);
        if (!nd.leaf && depth > kMaxInteriorDepth) {   // the tree is rejected: go no deeper
            too_deep = true;
            nd.leaf = true;
        }
        T[me] = nd;
        if (!nd.leaf) {
            const int32_t l = build(T, start, at, depth + 1, task_depth, tasks);
            const int32_t r = build(T, at, end, depth + 1, task_depth, tasks);
            T[me].l = l;
            T[me].r = r;
        }
        return me;
    }
};

struct Flat {
    const std::vector<TNode>& top;
    const std::vector<std::vector<TNode>>& sub;
    std::vector<float4>& nodes;
    uint32_t max_interior_depth = 0;

    const TNode& at(int tree, int32_t k) const { return tree < 0 ? top[k] : sub[tree][k]; }

    // The node that stands for (tree, k): a task placeholder is its subtree's root.
    void resolve(int& tree, int32_t& k) const {
        if (tree < 0 && top[k].task >= 0) {
            tree = top[k].task;
            k = 0;
        }
    }

    // A child reference: a leaf's (first triangle, count) or an interior
    // node's index (count 0), assigned in pre-order.
    void ref_of(int tree, int32_t k, int32_t& ref, int32_t& cnt, Box& box) {
        resolve(tree, k);
        const TNode& n = at(tree, k);
        box = n.box;
        if (n.leaf) {
            ref = (int32_t)n.start;
            cnt = (int32_t)(n.end - n.start);
            return;
        }
        ref = (int32_t)(nodes.size() / 4);
        cnt = 0;
        emit(tree, k);
    }

    void emit(int tree, int32_t k) {
        const TNode& n = at(tree, k);
        if (n.depth > max_interior_depth) max_interior_depth = n.depth;
        const size_t me = nodes.size();
        nodes.resize(me + 4);
        int32_t rl, cl, rr, cr;
        Box bl, br;
        ref_of(tree, n.l, rl, cl, bl);
        ref_of(tree, n.r, rr, cr, br);
        nodes[me] = make_float4(bl.lo[0], bl.lo[1], bl.lo[2], bl.hi[0]);
        nodes[me + 1] = make_float4(bl.hi[1], bl.hi[2], br.lo[0], br.lo[1]);
        nodes[me + 2] = make_float4(br.lo[2], br.hi[0], br.hi[1], br.hi[2]);
        int32_t q[4] = {rl, rr, cl, cr};
        std::memcpy(&nodes[me + 3], q, sizeof q);
    }
};

}  // namespace

int sah_build(const float4* pos, uint32_t V, const uint32_t* idx, uint32_t N, int threads,
              SahTree* out) {
    if (N == 0) return -1;
    std::vector<Box> boxes(N);
    std::vector<float> cen(3 * (size_t)N);
    for (uint32_t t = 0; t < N; ++t) {
        const uint32_t a = idx[3 * (size_t)t], b = idx[3 * (size_t)t + 1], c = idx[3 * (size_t)t + 2];
        if (a >= V || b >= V || c >= V) return -1;
        const float pa[3] = {pos[a].x, pos[a].y, pos[a].z};
        const float pb[3] = {pos[b].x, pos[b].y, pos[b].z};
        const float pc[3] = {pos[c].x, pos[c].y, pos[c].z};
        for (int k = 0; k < 3; ++k) {   // BBox::set
            boxes[t].hi[k] = smax(pa[k], smax(pb[k], pc[k]));
            boxes[t].lo[k] = smin(pa[k], smin(pb[k], pc[k]));
            cen[3 * (size_t)t + k] = (boxes[t].hi[k] + boxes[t].lo[k]) * 0.5f;
        }
    }
    out->order.resize(N);
    for (uint32_t i = 0; i < N; ++i) out->order[i] = i;
    std::atomic<bool> too_deep(false);
    Builder B{boxes, cen, out->order, too_deep};
    // the top levels on this thread, the subtrees below them on `threads`
    if (threads < 1) threads = 1;
    uint32_t task_depth = 0;
    while ((1u << task_depth) < 4u * (uint32_t)threads && task_depth < 8) ++task_depth;
    std::vector<TNode> top;
    std::vector<TNode> tasks;
    B.build(top, 0, N, 0, threads > 1 ? task_depth : 0xffffffffu, threads > 1 ? &tasks : nullptr);
    std::vector<std::vector<TNode>> sub(tasks.size());
    if (!tasks.empty()) {
        std::vector<std::thread> pool;
        std::atomic_size_t next(0);
        for (int w = 0; w < threads; ++w)
            pool.emplace_back([&]() {
                for (size_t k; (k = next.fetch_add(1)) < tasks.size();)
                    B.build(sub[k], tasks[k].start, tasks[k].end, tasks[k].depth, 0, nullptr);
            });
        for (auto& th : pool) th.join();
    }
    if (too_deep) return -2;
    // device layout: interior nodes in pre-order, leaves inline in their parents
    out->nodes.clear();
    out->nodes.reserve(4 * (size_t)(N > 1 ? N - 1 : 1));
    Flat F{top, sub, out->nodes};
    int tree = -1;
    int32_t root = 0;
    F.resolve(tree, root);
    const TNode& R = F.at(tree, root);
    std::memset(&out->hdr, 0, sizeof out->hdr);
    out->hdr.n_tris = N;
    out->hdr.root_lo = make_float4(R.box.lo[0], R.box.lo[1], R.box.lo[2], 0.f);
    out->hdr.root_hi = make_float4(R.box.hi[0], R.box.hi[1], R.box.hi[2], 0.f);
    if (R.leaf) {
        out->hdr.root_ref = (int32_t)R.start;
        out->hdr.root_cnt = (int32_t)(R.end - R.start);
    } else {
        out->hdr.root_ref = 0;
        out->hdr.root_cnt = 0;
        F.emit(tree, root);
    }
    out->max_interior_depth = F.max_interior_depth;
    out->interior_nodes = (uint32_t)(out->nodes.size() / 4);
    return 0;
}

}  // namespace rt
