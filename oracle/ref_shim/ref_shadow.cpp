/* ref_shadow.cpp — ORACLE test infrastructure: the reference's
 * src/kernel/shadow-trace-bvh.cl compiled unmodified for the CPU. */
#include "cl_shim_pre.hpp"
namespace rk {
namespace {  /* internal linkage: every kernel file defines its own helpers */
#include "cl_shim_body.hpp"
#include "shadow-trace-bvh.cl"
}  // namespace
}  // namespace rk
#include "cl_shim_post.hpp"

extern "C" {
size_t refk_sizeof_lights(void) { return sizeof(rk::Lights); }

/* The reference's Lights holds one spot or directional light.  A point light
 * (type 2) is expressed exactly as a spot light whose cosine cutoff is -1e30:
 * the cone test never fires and (dot - angle) / (1 - angle) rounds to 1. */
int refk_make_lights(const rt_lights* in, void* out) {
    if (in->count < 1) return -1;
    rk::Lights L;
    std::memset(&L, 0, sizeof(L));
    L.ambient = rk::float3(in->ambient[0], in->ambient[1], in->ambient[2]);
    const rt_light& l = in->light[0];
    if (l.type == RT_DIR_L) {
        L.light.type = rk::DIR_L;
        L.light.directional.dir = rk::float3(l.dir[0], l.dir[1], l.dir[2]);
        L.light.directional.color = rk::float3(l.color[0], l.color[1], l.color[2]);
    } else {
        L.light.type = rk::SPOT_L;
        L.light.spot.pos = rk::float3(l.pos[0], l.pos[1], l.pos[2]);
        L.light.spot.radius = l.radius;
        if (l.type == RT_POINT_L) {
            L.light.spot.angle = -1e30f;
            L.light.spot.dir = rk::float3(0.f, 0.f, 1.f);
        } else {
            L.light.spot.angle = l.angle;
            L.light.spot.dir = rk::float3(l.dir[0], l.dir[1], l.dir[2]);
        }
        L.light.spot.color = rk::float3(l.color[0], l.color[1], l.color[2]);
    }
    std::memcpy(out, &L, sizeof(L));
    return 0;
}

void refk_shadow_trace_single(rt_hit* info, rt_sample* samples, void* vtx, int* idx, void* nodes,
                              void* lights, size_t n, int threads) {
    refk_run(0, n, threads, [&](size_t g) {
        rk::g_wi.gid = g;
        rk::g_wi.goff = 0;
        rk::shadow_trace_single((rk::SampleTraceInfo*)info, (rk::Sample*)samples, (rk::Vertex*)vtx,
                                idx, (rk::BVHNode*)nodes, (rk::Lights*)lights);
    });
}
}

extern "C" {
void refk_shadow_trace_multi(rt_hit* info, rt_sample* samples, void* vtx, int* idx, void* nodes,
                             void* lights, void* roots, int root_count, size_t n, int threads) {
    refk_run(0, n, threads, [&](size_t g) {
        rk::g_wi.gid = g;
        rk::g_wi.goff = 0;
        rk::shadow_trace_multi((rk::SampleTraceInfo*)info, (rk::Sample*)samples, (rk::Vertex*)vtx,
                               idx, (rk::BVHNode*)nodes, (rk::Lights*)lights,
                               (rk::BVHRoot*)roots, root_count);
    });
}
}

