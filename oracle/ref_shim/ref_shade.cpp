/* ref_shade.cpp — ORACLE test infrastructure: the reference's
 * src/kernel/ray-shader.cl compiled unmodified for the CPU (untextured
 * materials, no cubemap: the image arguments are never read). */
#include "cl_shim_pre.hpp"
namespace rk {
namespace {  /* internal linkage: every kernel file defines its own helpers */
#include "cl_shim_body.hpp"
#include "ray-shader.cl"
}  // namespace
}  // namespace rk
#include "cl_shim_post.hpp"

static_assert(sizeof(rk::Material) == sizeof(rt_material), "Material layout");

extern "C" {
void refk_shade(int primary, uint32_t* image, rt_hit* info, rt_sample* samples, rt_material* mats,
                unsigned* map, void* lights, size_t n, int threads) {
    rk::image2d_t im = {0, 0};
    refk_run(0, n, threads, [&](size_t g) {
        rk::g_wi.gid = g;
        rk::g_wi.goff = 0;
        if (primary)
            rk::shade_primary((rk::ColorInt*)image, (rk::SampleTraceInfo*)info, (rk::Sample*)samples,
                              (rk::Material*)mats, map, 
                              im, im, im, im, im, im, im, im, im, im, im, im, im, im, im, im, im, im, im, im, im, im, im, im, im, im, im, im, im, im, im, im,
                              (unsigned)n, 0, (rk::Lights*)lights);
        else
            rk::shade_secondary((rk::ColorInt*)image, (rk::SampleTraceInfo*)info,
                                (rk::Sample*)samples, (rk::Material*)mats, map, 
                              im, im, im, im, im, im, im, im, im, im, im, im, im, im, im, im, im, im, im, im, im, im, im, im, im, im, im, im, im, im, im, im,
                                (unsigned)n, 0, (rk::Lights*)lights);
    });
}
}
