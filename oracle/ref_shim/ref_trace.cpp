/* ref_trace.cpp — ORACLE test infrastructure: the reference's
 * src/kernel/trace-bvh.cl compiled unmodified for the CPU. */
#include "cl_shim_pre.hpp"
namespace rk {
namespace {  /* internal linkage: every kernel file defines its own helpers */
#include "cl_shim_body.hpp"
#include "trace-bvh.cl"
}  // namespace
}  // namespace rk
#include "cl_shim_post.hpp"

static_assert(sizeof(rk::Sample) == sizeof(rt_sample), "Sample layout");
static_assert(sizeof(rk::SampleTraceInfo) == sizeof(rt_hit), "SampleTraceInfo layout");
static_assert(offsetof(rk::SampleTraceInfo, uv) == offsetof(rt_hit, uv), "uv offset");
static_assert(offsetof(rk::SampleTraceInfo, n) == offsetof(rt_hit, n), "n offset");
static_assert(offsetof(rk::SampleTraceInfo, hit_point) == offsetof(rt_hit, hit_point), "hp offset");
static_assert(offsetof(rk::Sample, pixel) == offsetof(rt_sample, pixel), "pixel offset");

extern "C" {
void refk_trace_single(rt_hit* info, rt_sample* samples, void* vtx, int* idx, void* nodes, size_t n,
                       int threads) {
    refk_run(0, n, threads, [&](size_t g) {
        rk::g_wi.gid = g;
        rk::g_wi.goff = 0;
        rk::trace_single((rk::SampleTraceInfo*)info, (rk::Sample*)samples, (rk::Vertex*)vtx, idx,
                         (rk::BVHNode*)nodes);
    });
}
}

extern "C" {
size_t refk_sizeof_root(void) { return sizeof(rk::BVHRoot); }

/* BVHRoot i: its root node and the row-major transform and inverse. */
void refk_make_root(void* roots, size_t i, int node, const float* tr, const float* trinv) {
    rk::BVHRoot& r = ((rk::BVHRoot*)roots)[i];
    std::memset(&r, 0, sizeof(r));
    r.node = node;
    for (int k = 0; k < 4; ++k) {
        r.tr.row[k] = rk::float4(tr[4 * k], tr[4 * k + 1], tr[4 * k + 2], tr[4 * k + 3]);
        r.trInv.row[k] = rk::float4(trinv[4 * k], trinv[4 * k + 1], trinv[4 * k + 2], trinv[4 * k + 3]);
    }
}

void refk_trace_multi(rt_hit* info, rt_sample* samples, void* vtx, int* idx, void* nodes, void* roots,
                      int root_count, size_t n, int threads) {
    refk_run(0, n, threads, [&](size_t g) {
        rk::g_wi.gid = g;
        rk::g_wi.goff = 0;
        rk::trace_multi((rk::SampleTraceInfo*)info, (rk::Sample*)samples, (rk::Vertex*)vtx, idx,
                        (rk::BVHNode*)nodes, (rk::BVHRoot*)roots, root_count);
    });
}
}

