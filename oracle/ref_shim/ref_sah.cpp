/* ref_sah.cpp — ORACLE test infrastructure: the reference's CPU SAH BVH
 * (BVH::construct / BVHNode::sort, src/rt/bvh.cpp:6-179, with BBox from
 * src/rt/bbox.cpp) compiled unmodified for the CPU, to pin the oracle's
 * restatement and, through it, the library's rt_bvh_build_sah.
 * include/CL/opencl.h beside this file stands in for the OpenCL host types. */
#include <stdint.h>
#include <string.h>

#include <rt/bvh.hpp>
#include <rt/mesh.hpp>

struct refs_bvh {
    BVH bvh;
};

extern "C" {
/* Builds over V float4 positions and N index triples; node and triangle
 * counts are returned for refs_copy. */
void* refs_build(const float* pos4, uint32_t V, const uint32_t* idx, uint32_t N,
                 uint32_t* node_count) {
    Mesh m;
    m.vertices.resize(V);
    for (uint32_t i = 0; i < V; ++i) {
        memset(&m.vertices[i], 0, sizeof(Vertex));
        for (int k = 0; k < 3; ++k) m.vertices[i].position.s[k] = pos4[4 * (size_t)i + k];
    }
    m.triangles.resize(N);
    for (uint32_t i = 0; i < N; ++i)
        for (int k = 0; k < 3; ++k) m.triangles[i].v[k] = idx[3 * (size_t)i + k];
    refs_bvh* b = new refs_bvh;
    b->bvh.construct(m);
    *node_count = (uint32_t)b->bvh.m_nodes.size();
    return b;
}

/* Per node in the reference's numbering: lo[3], hi[3]; (a, b) = children or
 * the leaf's [start, end); leaf flag.  order: slot -> triangle. */
void refs_copy(void* h, float* lo, float* hi, uint32_t* a, uint32_t* b, uint32_t* leaf,
               uint32_t* order) {
    refs_bvh* r = (refs_bvh*)h;
    for (size_t k = 0; k < r->bvh.m_nodes.size(); ++k) {
        const BVHNode& n = r->bvh.m_nodes[k];
        for (int c = 0; c < 3; ++c) {
            lo[3 * k + c] = n.m_bbox.lo.s[c];
            hi[3 * k + c] = n.m_bbox.hi.s[c];
        }
        a[k] = n.m_l_child;
        b[k] = n.m_r_child;
        leaf[k] = n.m_leaf ? 1u : 0u;
    }
    for (size_t i = 0; i < r->bvh.m_triangle_order.size(); ++i) order[i] = r->bvh.m_triangle_order[i];
}

void refs_free(void* h) { delete (refs_bvh*)h; }
}  /* extern "C" */
