/* ref_primary.cpp — ORACLE test infrastructure: the reference's
 * src/kernel/primary-ray-generator.cl compiled unmodified for the CPU. */
#include "cl_shim_pre.hpp"
namespace rk {
namespace {  /* internal linkage: every kernel file defines its own helpers */
#include "cl_shim_body.hpp"
#include "primary-ray-generator.cl"
}  // namespace
}  // namespace rk
#include "cl_shim_post.hpp"

extern "C" {
void refk_generate_primary_rays(rt_sample* samples, const float* pos, const float* dir,
                                const float* right, const float* up, int w, int h, int quad, int spp,
                                const rt_pixel_sample* ps, size_t count, size_t offset) {
    rt_pixel_sample one = {0.f, 0.f, 1.f};
    const rt_pixel_sample* p = ps ? ps : &one;
    rk::float4 P(pos[0], pos[1], pos[2], 0.f), D(dir[0], dir[1], dir[2], 0.f),
        R(right[0], right[1], right[2], 0.f), U(up[0], up[1], up[2], 0.f);
    /* global offset semantics: sample index = gid - offset */
    for (size_t g = offset; g < offset + count; ++g) {
        rk::g_wi.gid = g;
        rk::g_wi.goff = offset;
        rk::generate_primary_rays((rk::Sample*)samples, P, D, R, U, w, h, quad, spp,
                                  (rk::PixelSample*)p);
    }
}
}
