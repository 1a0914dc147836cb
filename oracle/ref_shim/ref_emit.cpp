/*
 * ref_emit.cpp — ORACLE test infrastructure.
 *
 * The two work-group kernels of the reference's LBVH build, compiled
 * unmodified from src/kernel/bvh-builder.cl and run on the CPU as emulated
 * OpenCL work-groups:
 *   max_local_bbox                         bvh-builder.cl:318-391
 *   process_task, find_middle,             bvh-builder.cl:439-671
 *   set_children, prefix_sum
 * together with the host loops that launch them, restated:
 *   global AABB reduction launches         src/rt/bvh-builder.cpp:289-334
 *   level loop, launch sizes, OC readback  src/rt/bvh-builder.cpp:548-625
 *
 * Emulation.  A work-group of W work-items is W host threads.  barrier() is a
 * barrier of those W threads (mutex + condition variable, which also orders
 * their memory accesses).  Each __local kernel argument is one array per
 * running group.  Several groups run at once and share the OC / PC counters
 * through atomic adds, as on the device, so the node numbering depends on
 * thread timing exactly as the reference's does on a GPU; the range tree does
 * not, and it is what parity is defined on.
 *
 * The two __local scalars of process_task.  The kernel declares
 * `local int firstNode;` and `local int localOffset;` in its body.  With
 * `local` expanding to nothing they would be private to each thread, so the
 * two names are macros: the declaration becomes a block-scope declaration of
 * the function `int* wg_firstNode()` (resp. wg_localOffset) and every use
 * goes through it.  Work-item 0 writes both; the others read them.  The
 * kernel has a race here: work-item 0 stores the next firstNode
 * (bvh-builder.cl:666-668) while other work-items may still be inside
 * set_children for the current one (:657-662), with no barrier between.  On a
 * GPU the value read after the loop-head barrier stays in a register for the
 * rest of the iteration; the emulation gives the same behaviour by giving
 * each work-item its own view of the two scalars, which only a barrier
 * refreshes: a store by work-item 0 is published when it arrives at the next
 * barrier, and every work-item leaves that barrier holding the published
 * value.
 */
#include "cl_shim_pre.hpp"

#include <climits>
#include <condition_variable>
#include <memory>
#include <mutex>

namespace rk {
namespace {

/* A work-item's view of process_task's two __local scalars: the values it
 * holds, and the values it left the last barrier with (a difference means
 * this work-item stored one since). */
struct ScalarView {
    int v[2];
    int seen[2];
};
constexpr int kUnset = INT32_MIN;
thread_local ScalarView t_view;

/* The barrier of one emulated work-group, carrying the two __local scalars:
 * stores are published on arrival, and the last arrival snapshots them for
 * every work-item to take on leaving. */
class GroupBarrier {
public:
    explicit GroupBarrier(int n) : n_(n) {}
    void wait() {
        std::unique_lock<std::mutex> lk(m_);
        for (int k = 0; k < 2; ++k)
            if (t_view.v[k] != t_view.seen[k]) pub_[k] = t_view.v[k];
        const unsigned gen = gen_;
        if (++waiting_ == n_) {
            waiting_ = 0;
            snap_[0] = pub_[0];
            snap_[1] = pub_[1];
            ++gen_;
            cv_.notify_all();
        } else {
            cv_.wait(lk, [&] { return gen_ != gen; });
        }
        for (int k = 0; k < 2; ++k) t_view.v[k] = t_view.seen[k] = snap_[k];
    }

private:
    std::mutex m_;
    std::condition_variable cv_;
    int n_;
    int waiting_ = 0;
    unsigned gen_ = 0;
    int pub_[2] = {kUnset, kUnset};
    int snap_[2] = {kUnset, kUnset};
};

/* Everything one running group shares: its barrier and its __local argument
 * arrays. */
struct GroupSlot {
    GroupSlot(int w, size_t local_bytes) : bar(w), local_mem(local_bytes) {}
    GroupBarrier bar;
    std::vector<uint8_t> local_mem;
};

thread_local GroupSlot* t_slot = nullptr;
int* wg_firstNode() { return &t_view.v[0]; }
int* wg_localOffset() { return &t_view.v[1]; }

#define firstNode (*wg_firstNode())
#define localOffset (*wg_localOffset())
#include "cl_shim_body.hpp"
#include "bvh-builder.cl"
#undef firstNode
#undef localOffset

void group_barrier(void) { t_slot->bar.wait(); }

/* Runs kern(slot) as an NDRange of `groups` work-groups of W work-items, at
 * most `concurrent` groups at a time: running slot s takes groups s,
 * s + concurrent, ...  A barrier closes each group before its slot's threads
 * (and __local memory) start the next one. */
template <class K>
void launch(size_t groups, int w, size_t concurrent, size_t local_bytes, K kern) {
    concurrent = std::max<size_t>(1, std::min(concurrent, groups));
    std::vector<std::unique_ptr<GroupSlot>> slots;
    for (size_t s = 0; s < concurrent; ++s) slots.emplace_back(new GroupSlot(w, local_bytes));
    std::vector<std::thread> th;
    for (size_t s = 0; s < concurrent; ++s)
        for (int lid = 0; lid < w; ++lid)
            th.emplace_back([&, s, lid]() {
                t_slot = slots[s].get();
                g_barrier_hook = group_barrier;
                for (size_t g = s; g < groups; g += concurrent) {
                    g_wi.lid = (size_t)lid;
                    g_wi.lsize = (size_t)w;
                    g_wi.grp = g;
                    g_wi.ngrp = groups;
                    g_wi.gid = g * (size_t)w + (size_t)lid;
                    g_wi.gsize = groups * (size_t)w;
                    g_wi.goff = 0;
                    t_view = ScalarView{{kUnset, kUnset}, {kUnset, kUnset}};
                    kern(t_slot);
                    t_slot->bar.wait();
                }
                g_barrier_hook = nullptr;
                t_slot = nullptr;
            });
    for (auto& t : th) t.join();
}

}  // namespace
}  // namespace rk
#include "cl_shim_post.hpp"

extern "C" {

/* The global AABB as the reference computes it: repeated max_local_bbox
 * launches over 2 * group_size boxes per group until one group remains
 * (bvh-builder.cpp:289-334).  bboxes: BBox[n] in the kernels' layout.
 * Returns -1 for a group size that is not a power of two >= 2. */
int refe_global_bbox(const void* bboxes, uint32_t n, int group_size, int concurrent, float* lo3,
                     float* hi3) {
    if (n == 0 || group_size < 2 || (group_size & (group_size - 1))) return -1;
    const size_t gs = (size_t)group_size;
    size_t bbox_count = n;
    size_t out_bbox_count = (size_t)std::ceil(bbox_count / (2. * gs));
    size_t real_size = (size_t)std::ceil(bbox_count / 2.);
    size_t global_size = (size_t)std::ceil(real_size / (double)gs) * gs;
    std::vector<rk::BBox> in((const rk::BBox*)bboxes, (const rk::BBox*)bboxes + n);
    for (;;) {
        std::vector<rk::BBox> out(out_bbox_count);
        const unsigned size = (unsigned)bbox_count;
        rk::launch(global_size / gs, group_size, (size_t)concurrent, 2 * gs * sizeof(rk::BBox),
                   [&](rk::GroupSlot* slot) {
                       rk::max_local_bbox(in.data(), (rk::BBox*)slot->local_mem.data(), size,
                                          out.data());
                   });
        bbox_count = out_bbox_count;
        out_bbox_count = (size_t)std::ceil(bbox_count / (2. * gs));
        in.swap(out);
        if (global_size <= gs) break;
        real_size = (size_t)std::ceil(bbox_count / 2.);
        global_size = (size_t)std::ceil(real_size / (double)gs) * gs;
    }
    lo3[0] = in[0].lo.x; lo3[1] = in[0].lo.y; lo3[2] = in[0].lo.z;
    hi3[0] = in[0].hi.x; hi3[1] = in[0].hi.y; hi3[2] = in[0].hi.z;
    return 0;
}

/* The hierarchy emit of build_lbvh (bvh-builder.cpp:548-625): an empty root
 * over [0, n), then bvh_depth launches of process_task, launch i with
 * global size gsize * k for the least k with gsize * k >= 2^i, capped below
 * gsize * compute_units; then the OC readback.  sorted: the sorted Morton
 * keys (code[0]; code[1] = 0, bvh_depth <= 32).  nodes: BVHNode[2n] in the
 * kernels' layout (the reference's buffer size), zeroed.  level_end[i]
 * receives the reference's processedCounter[i] (one past the last node of
 * level i).  Returns the node count, or -1 on bad arguments. */
int64_t refe_process_levels(const uint32_t* sorted, uint32_t n, int depth, int min_leaf,
                            int group_size, int compute_units, void* nodes_out,
                            uint32_t* level_end) {
    if (n == 0 || depth < 1 || depth > 32 || min_leaf < 1 || group_size < 2 ||
        (group_size & (group_size - 1)) || compute_units < 1)
        return -1;
    std::vector<rk::morton_code_t> codes(n);
    for (uint32_t i = 0; i < n; ++i) {
        codes[i].code[0] = sorted[i];
        codes[i].code[1] = 0;
    }
    rk::BVHNode* nodes = (rk::BVHNode*)nodes_out;
    std::memset(nodes, 0, sizeof(rk::BVHNode) * 2 * (size_t)n);
    nodes[0].parent = 0;
    nodes[0].split_axis = 0;
    nodes[0].start_index = 0;
    nodes[0].end_index = n;
    nodes[0].leaf = 0;
    int OC[64] = {0}, PC[64] = {0};
    const size_t gsize = (size_t)group_size;
    const size_t lbytes = sizeof(int) * (gsize * 2 + 1);
    for (int i = 0; i < depth; ++i) {
        size_t max_size = (size_t)powf(2, (float)i);
        size_t global_size = gsize;
        while (global_size < max_size && global_size < gsize * compute_units - 1)
            global_size += gsize;
        const size_t groups = global_size / gsize;
        rk::launch(groups, group_size, groups, 2 * lbytes, [&](rk::GroupSlot* slot) {
            int* LC = (int*)slot->local_mem.data();
            int* PS = (int*)(slot->local_mem.data() + lbytes);
            rk::process_task(OC, PC, nodes, codes.data(), LC, PS, depth, min_leaf, i);
        });
    }
    uint32_t node_count = 1;
    for (int i = 0; i < depth; ++i) {
        if (level_end) level_end[i] = node_count;
        node_count += (uint32_t)OC[i];
    }
    return node_count;
}

size_t refe_sizeof_node(void) { return sizeof(rk::BVHNode); }
size_t refe_sizeof_bbox(void) { return sizeof(rk::BBox); }
}
