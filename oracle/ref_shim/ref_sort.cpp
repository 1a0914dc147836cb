/* ref_sort.cpp — ORACLE test infrastructure: the reference's
 * src/kernel/bvh-builder-sort.cl compiled unmodified for the CPU. */
#include "cl_shim_pre.hpp"
namespace rk {
namespace {  /* internal linkage: every kernel file defines its own helpers */
#include "cl_shim_body.hpp"
#include "bvh-builder-sort.cl"
}  // namespace
}  // namespace rk
#include "cl_shim_post.hpp"

extern "C" {
/* One launch of morton_sort_g{2,4,8,16} over `items` work-items.  Work-items
 * of one launch touch disjoint elements, so running them in order is exact. */
void refk_morton_sort(int g, void* codes, unsigned* tris, int inc, int dir, int inv, int last_step,
                      int size, size_t items) {
    rk::morton_code_t* c = (rk::morton_code_t*)codes;
    for (size_t i = 0; i < items; ++i) {
        rk::g_wi.gid = i;
        rk::g_wi.goff = 0;
        switch (g) {
            case 2: rk::morton_sort_g2(c, tris, inc, dir, inv, last_step, size); break;
            case 4: rk::morton_sort_g4(c, tris, inc, dir, inv, last_step, size); break;
            case 8: rk::morton_sort_g8(c, tris, inc, dir, inv, last_step, size); break;
            default: rk::morton_sort_g16(c, tris, inc, dir, inv, last_step, size); break;
        }
    }
}
}
