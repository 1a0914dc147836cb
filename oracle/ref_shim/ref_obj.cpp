/* ref_obj.cpp — ORACLE test infrastructure: the reference's OBJ import
 * (ModelOBJ::import + get_aggregate_mesh, src/rt/obj-loader.cpp, as
 * Scene::load_obj_file_as_aggregate runs it, src/rt/scene.cpp:441-453)
 * compiled unmodified for the CPU, to pin the library's own OBJ reader.
 * include/CL/opencl.h beside this file stands in for the OpenCL host types. */
#include <stdint.h>
#include <string.h>

#include <rt/mesh.hpp>
#include <rt/obj-loader.hpp>

struct refo_model {
    Mesh mesh;
};

extern "C" {
void* refo_load(const char* path) {
    ModelOBJ obj;
    if (!obj.import(path)) return nullptr;
    refo_model* m = new refo_model;
    obj.get_aggregate_mesh(&m->mesh);
    return m;
}

void refo_sizes(void* h, uint32_t* V, uint32_t* N, uint32_t* G) {
    refo_model* m = (refo_model*)h;
    *V = (uint32_t)m->mesh.vertices.size();
    *N = (uint32_t)m->mesh.triangles.size();
    *G = (uint32_t)m->mesh.original_materials.size();
}

/* positions / normals as float4, indices, and per group: first index (of the
 * index buffer, 3 per triangle), end index, diffuse rgb, shininess */
void refo_copy(void* h, float* pos4, float* nrm4, uint32_t* idx, uint32_t* gstart, uint32_t* gend,
               float* gdiffuse, float* gshininess) {
    refo_model* m = (refo_model*)h;
    for (size_t i = 0; i < m->mesh.vertices.size(); ++i)
        for (int k = 0; k < 4; ++k) {
            pos4[4 * i + k] = k < 3 ? m->mesh.vertices[i].position.s[k] : 0.f;
            nrm4[4 * i + k] = k < 3 ? m->mesh.vertices[i].normal.s[k] : 0.f;
        }
    for (size_t t = 0; t < m->mesh.triangles.size(); ++t)
        for (int k = 0; k < 3; ++k) idx[3 * t + k] = m->mesh.triangles[t].v[k];
    for (size_t g = 0; g < m->mesh.original_materials.size(); ++g) {
        const MeshMaterial& mm = m->mesh.original_materials[g];
        gstart[g] = (uint32_t)mm.start_index;
        gend[g] = (uint32_t)mm.end_index;
        for (int k = 0; k < 3; ++k) gdiffuse[3 * g + k] = mm.material.diffuse.rgb.s[k];
        gshininess[g] = mm.material.shininess;
    }
}

void refo_free(void* h) { delete (refo_model*)h; }
}
