/*
 * scene.cpp — Scene and Camera of the drop-in C++ layer (include/rt/scene.hpp,
 * include/rt/camera.hpp).  Reference: Scene::transfer_aggregate_mesh_to_device
 * (src/rt/scene.cpp:236-321) and the buffer accessors (include/rt/scene.hpp:
 * 125-133); Camera::set (src/rt/camera.cpp:31-59).
 */
#include <cstring>

#include "../../include/rt/camera.hpp"
#include "../../include/rt/scene.hpp"

/* ---- Camera -------------------------------------------------------------- */
Camera::Camera() : right_handed(false), fov(1.0471976f), aspect(1.f) {}

Camera::Camera(const vec3& Position, const vec3& Direction, const vec3& Up, float FOV,
               float Aspect, bool RightHanded)
    : right_handed(false), fov(1.0471976f), aspect(1.f) {
    set(Position, Direction, Up, FOV, Aspect, RightHanded);
}

void Camera::set(const vec3& Position, const vec3& Direction, const vec3& Up, float FOV,
                 float Aspect, bool RightHanded) {
    if (FOV > 0.f) fov = FOV;
    if (Aspect > 0.f) aspect = Aspect;
    right_handed = RightHanded;
    rt_camera c;
    std::memset(&c, 0, sizeof(c));
    pos = Position;
    /* Camera::set takes tan(FOV / 2) of the argument, even when it is 0 and
     * the stored fov is kept; the same argument is passed on.  A zero
     * direction or an up vector along it leaves the basis as it was. */
    if (rt_camera_set(&c, Position.s, Direction.s, Up.s, FOV, aspect, RightHanded ? 1 : 0) != RT_OK)
        return;
    dir = vec3(c.dir[0], c.dir[1], c.dir[2]);
    right = vec3(c.right[0], c.right[1], c.right[2]);
    up = vec3(c.up[0], c.up[1], c.up[2]);
}

rt_camera Camera::to_rt() const {
    rt_camera c;
    std::memset(&c, 0, sizeof(c));
    for (int i = 0; i < 3; ++i) {
        c.pos[i] = pos[i];
        c.dir[i] = dir[i];
        c.right[i] = right[i];
        c.up[i] = up[i];
    }
    return c;
}

/* ---- Scene --------------------------------------------------------------- */
Scene::Scene() : m_scene(nullptr), m_triangles(0) {}

Scene::~Scene() {
    DeviceInterface* dev = DeviceInterface::instance();
    if (m_scene && dev->good()) rt_scene_destroy(dev->context(), m_scene);
}

int32_t Scene::initialize() {
    DeviceInterface* dev = DeviceInterface::instance();
    if (!dev->good()) return -1;
    if (m_scene) return 0;
    return rt_scene_create(dev->context(), &m_scene) == RT_OK ? 0 : -1;
}

int32_t Scene::refresh_views() {
    DeviceInterface* dev = DeviceInterface::instance();
    uint32_t *idx = nullptr, *map = nullptr, n = 0;
    float *pos = nullptr, *nrm = nullptr;
    if (rt_scene_buffers(dev->context(), m_scene, &idx, &map, &pos, &nrm, &n) != RT_OK) return -1;
    m_triangles = n;
    m_index.set_view(idx, 12 * (size_t)n);
    m_map.set_view(map, 4 * (size_t)n);
    m_vertex.set_view(pos, 0);
    m_normal.set_view(nrm, 0);
    return 0;
}

int32_t Scene::transfer_aggregate_mesh_to_device(const rt_scene_desc& desc) {
    DeviceInterface* dev = DeviceInterface::instance();
    if (initialize()) return -1;
    if (rt_scene_upload(dev->context(), m_scene, &desc, nullptr) != RT_OK) return -1;
    if (refresh_views()) return -1;
    m_vertex.set_view(m_vertex.ptr(), 16 * (size_t)desc.vertex_count);
    m_normal.set_view(m_normal.ptr(), 16 * (size_t)desc.vertex_count);
    return 0;
}

int32_t Scene::set_lights(const rt_lights& lights) {
    DeviceInterface* dev = DeviceInterface::instance();
    if (!m_scene) return -1;
    return rt_scene_set_lights(dev->context(), m_scene, &lights) == RT_OK ? 0 : -1;
}

size_t Scene::triangle_count() { return m_triangles; }

DeviceMemory& Scene::index_mem() { return m_index; }
DeviceMemory& Scene::material_map_mem() { return m_map; }
DeviceMemory& Scene::vertex_mem() { return m_vertex; }
DeviceMemory& Scene::normal_mem() { return m_normal; }
DeviceMemory& Scene::bvh_nodes_mem() { return m_bvh; }

rt_scene* Scene::rt_handle() { return m_scene; }
