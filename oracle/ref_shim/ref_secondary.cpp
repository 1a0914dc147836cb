/* ref_secondary.cpp — ORACLE test infrastructure: the reference's
 * src/kernel/secondary-ray-generator.cl compiled unmodified for the CPU. */
#include "cl_shim_pre.hpp"
namespace rk {
namespace {  /* internal linkage: every kernel file defines its own helpers */
#include "cl_shim_body.hpp"
#include "secondary-ray-generator.cl"
}  // namespace
}  // namespace rk
#include "cl_shim_post.hpp"

extern "C" {
void refk_mark_secondary_rays_disc(rt_hit* info, rt_sample* samples, rt_material* mats,
                                   unsigned* map, int* count, int refract_offset, size_t n) {
    for (size_t g = 0; g < n; ++g) {
        rk::g_wi.gid = g;
        rk::g_wi.goff = 0;
        rk::mark_secondary_rays_disc((rk::SampleTraceInfo*)info, (rk::Sample*)samples,
                                     (rk::Material*)mats, map, count, refract_offset);
    }
}
void refk_generate_secondary_rays_disc(rt_hit* info, rt_sample* samples, rt_material* mats,
                                       unsigned* map, rt_sample* out, int* count,
                                       int refract_offset, int max_count, size_t n) {
    for (size_t g = 0; g < n; ++g) {
        rk::g_wi.gid = g;
        rk::g_wi.goff = 0;
        rk::generate_secondary_rays_disc((rk::SampleTraceInfo*)info, (rk::Sample*)samples,
                                         (rk::Material*)mats, map, (rk::Sample*)out, count,
                                         refract_offset, max_count);
    }
}
}
