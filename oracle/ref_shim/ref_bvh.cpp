/* ref_bvh.cpp — ORACLE test infrastructure: the reference's
 * src/kernel/bvh-builder.cl compiled unmodified for the CPU. */
#include "cl_shim_pre.hpp"
namespace rk {
namespace {  /* internal linkage: every kernel file defines its own helpers */
#include "cl_shim_body.hpp"
#include "bvh-builder.cl"
}  // namespace
}  // namespace rk
#include "cl_shim_post.hpp"

#define WI(g, off) do { rk::g_wi.gid = (g); rk::g_wi.goff = (off); } while (0)

extern "C" {
size_t refk_sizeof_vertex(void) { return sizeof(rk::Vertex); }
size_t refk_sizeof_bbox(void) { return sizeof(rk::BBox); }
size_t refk_sizeof_node(void) { return sizeof(rk::BVHNode); }
size_t refk_sizeof_morton(void) { return sizeof(rk::morton_code_t); }

/* Vertex AoS from float4 positions / normals. */
void refk_make_vertices(const float* pos4, const float* nrm4, size_t v, void* out) {
    rk::Vertex* vx = (rk::Vertex*)out;
    for (size_t i = 0; i < v; ++i) {
        std::memset(&vx[i], 0, sizeof(rk::Vertex));
        vx[i].position = rk::float3(pos4[4 * i], pos4[4 * i + 1], pos4[4 * i + 2]);
        vx[i].normal = rk::float3(nrm4[4 * i], nrm4[4 * i + 1], nrm4[4 * i + 2]);
    }
}

void refk_build_primitive_bbox(void* vtx, int* idx, void* bboxes, unsigned* tris, size_t n) {
    for (size_t g = 0; g < n; ++g) {
        WI(g, 0);
        rk::build_primitive_bbox((rk::Vertex*)vtx, idx, (rk::BBox*)bboxes, tris);
    }
}

void refk_morton_encode(void* bboxes, const float* glo, const float* ghi, void* codes, int depth,
                        size_t n) {
    rk::BBox gb;
    std::memset(&gb, 0, sizeof(gb));
    gb.lo = rk::float3(glo[0], glo[1], glo[2]);
    gb.hi = rk::float3(ghi[0], ghi[1], ghi[2]);
    for (size_t g = 0; g < n; ++g) {
        WI(g, 0);
        rk::morton_encode((rk::BBox*)bboxes, &gb, (rk::morton_code_t*)codes, depth);
    }
}

void refk_bbox_get(const void* bboxes, size_t i, float* lo3, float* hi3) {
    const rk::BBox& b = ((const rk::BBox*)bboxes)[i];
    lo3[0] = b.lo.x; lo3[1] = b.lo.y; lo3[2] = b.lo.z;
    hi3[0] = b.hi.x; hi3[1] = b.hi.y; hi3[2] = b.hi.z;
}

void refk_morton_get(const void* codes, size_t n, unsigned* lo, unsigned* hi) {
    const rk::morton_code_t* c = (const rk::morton_code_t*)codes;
    for (size_t i = 0; i < n; ++i) {
        lo[i] = c[i].code[0];
        if (hi) hi[i] = c[i].code[1];
    }
}

void refk_rearrange_indices(int* in, unsigned* tris, int* out, size_t n) {
    for (size_t g = 0; g < n; ++g) {
        WI(g, 0);
        rk::rearrange_indices(in, tris, out);
    }
}

void refk_rearrange_map(int* in, unsigned* tris, int* out, size_t n) {
    for (size_t g = 0; g < n; ++g) {
        WI(g, 0);
        rk::rearrange_map(in, tris, out);
    }
}

void refk_rearrange_morton_codes(void* in, unsigned* tris, void* out, size_t n) {
    for (size_t g = 0; g < n; ++g) {
        WI(g, 0);
        rk::rearrange_morton_codes((rk::morton_code_t*)in, tris, (rk::morton_code_t*)out);
    }
}

void refk_node_set(void* nodes, size_t i, unsigned a, unsigned b, unsigned parent, int leaf) {
    rk::BVHNode& nd = ((rk::BVHNode*)nodes)[i];
    std::memset(&nd, 0, sizeof(nd));
    nd.l_child = a;
    nd.r_child = b;
    nd.parent = parent;
    nd.leaf = (char)leaf;
}

void refk_node_get(const void* nodes, size_t i, float* lo3, float* hi3, unsigned* a, unsigned* b,
                   int* leaf) {
    const rk::BVHNode& nd = ((const rk::BVHNode*)nodes)[i];
    lo3[0] = nd.bbox.lo.x; lo3[1] = nd.bbox.lo.y; lo3[2] = nd.bbox.lo.z;
    hi3[0] = nd.bbox.hi.x; hi3[1] = nd.bbox.hi.y; hi3[2] = nd.bbox.hi.z;
    *a = nd.l_child;
    *b = nd.r_child;
    *leaf = nd.leaf;
}

void refk_build_leaf_bbox(unsigned* tris, void* bboxes, void* nodes, size_t n) {
    for (size_t g = 0; g < n; ++g) {
        WI(g, 0);
        rk::build_leaf_bbox(tris, (rk::BBox*)bboxes, (rk::BVHNode*)nodes);
    }
}

void refk_build_node_bbox(void* nodes, size_t start, size_t count) {
    for (size_t g = start; g < start + count; ++g) {
        WI(g, start);
        rk::build_node_bbox((rk::BVHNode*)nodes);
    }
}
}

extern "C" {
/* Offsets node references for a node array placed at node_off among others
 * whose triangles start at tri_off (leaf ranges) -- the layout the
 * reference's Scene::create_bvhs gives several meshes' trees. */
void refk_offset_nodes(void* nodes, size_t n, unsigned node_off, unsigned tri_off) {
    rk::BVHNode* nd = (rk::BVHNode*)nodes;
    for (size_t i = 0; i < n; ++i) {
        const unsigned o = nd[i].leaf ? tri_off : node_off;
        nd[i].l_child += o;
        nd[i].r_child += o;
        nd[i].parent += node_off;
    }
}
}
