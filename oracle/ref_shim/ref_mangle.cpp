/* ref_mangle.cpp — ORACLE test infrastructure: the reference's
 * src/kernel/mangler.cl compiled unmodified for the CPU.  The kernel has no
 * cl_khr_fp64 pragma, so its unsuffixed constants are single precision: this
 * unit is compiled with -fsingle-precision-constant to match. */
#include "cl_shim_pre.hpp"
namespace rk {
namespace {  /* internal linkage: every kernel file defines its own helpers */
#include "cl_shim_body.hpp"
#include "mangler.cl"
}  // namespace
}  // namespace rk
#include "cl_shim_post.hpp"

extern "C" {
/* mangle over V vertices given as float4 positions / normals (xyz used). */
void refk_mangle(float* pos4, float* nrm4, uint32_t V, float arg, float last_arg, float height) {
    std::vector<rk::Vertex> vb(V);
    for (uint32_t i = 0; i < V; ++i) {
        std::memset(&vb[i], 0, sizeof(rk::Vertex));
        vb[i].position = rk::float3(pos4[4 * i], pos4[4 * i + 1], pos4[4 * i + 2]);
        vb[i].normal = rk::float3(nrm4[4 * i], nrm4[4 * i + 1], nrm4[4 * i + 2]);
    }
    for (uint32_t i = 0; i < V; ++i) {
        rk::g_wi.gid = i;
        rk::g_wi.goff = 0;
        rk::mangle(vb.data(), arg, last_arg, height);
    }
    for (uint32_t i = 0; i < V; ++i) {
        pos4[4 * i] = vb[i].position.x;
        pos4[4 * i + 1] = vb[i].position.y;
        pos4[4 * i + 2] = vb[i].position.z;
        nrm4[4 * i] = vb[i].normal.x;
        nrm4[4 * i + 1] = vb[i].normal.y;
        nrm4[4 * i + 2] = vb[i].normal.z;
    }
}
}
