/*
 * rt/scene.hpp — the reference's Scene (include/rt/scene.hpp) reduced to
 * what the hot path reads: the aggregate mesh on the device, its materials,
 * lights and LBVH, the camera and the cubemap.  The reference assembles its
 * aggregate mesh from OBJ files and objects before
 * transfer_aggregate_mesh_to_device() (src/rt/scene.cpp:236-321); here the
 * caller passes the arrays in an rt_scene_desc (the reference's 80-byte
 * Vertex array is accepted as is: stride 80, position at 0, normal at 16).
 * The buffer accessors (scene.hpp:125-133) return views of the library's
 * buffers; a build permutes the index buffer and material map into sorted
 * order, as the reference's builder does.
 */
#pragma once
#ifndef RT_SCENE_HPP
#define RT_SCENE_HPP

#include <stddef.h>
#include <stdint.h>

#include "../gpu/interface.hpp"
#include "camera.hpp"
#include "cubemap.hpp"

class Scene {
public:
    Scene();
    ~Scene();
    Scene(const Scene&) = delete;
    Scene& operator=(const Scene&) = delete;

    int32_t initialize();
    int32_t transfer_aggregate_mesh_to_device(const rt_scene_desc& desc);
    /* Scene::set_dir_light / set_spot_light / set_ambient_light in one call. */
    int32_t set_lights(const rt_lights& lights);
    size_t triangle_count();

    DeviceMemory& index_mem();
    DeviceMemory& material_map_mem();
    DeviceMemory& vertex_mem();     /* float4 positions */
    DeviceMemory& normal_mem();     /* float4 normals   */
    /* The scene's LBVH.  It is held inside the library; this object stands
     * for it (Tracer's bvh_mem overloads accept it and nothing else). */
    DeviceMemory& bvh_nodes_mem();

    rt_scene* rt_handle();

    Camera camera;
    Cubemap cubemap;

private:
    int32_t refresh_views();
    rt_scene* m_scene;
    size_t m_triangles;
    DeviceMemory m_index, m_map, m_vertex, m_normal, m_bvh;
};

#endif /* RT_SCENE_HPP */
