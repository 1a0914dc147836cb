/*
 * rt/tracer.hpp — the reference's Tracer (include/rt/tracer.hpp:12-34), same
 * public methods, over rt_trace / rt_shadow_trace (closest hit and shadow
 * any-hit on the scene's LBVH).  The bvh_mem overloads take the scene's own
 * bvh_nodes_mem(); any other memory object returns -1.
 */
#pragma once
#ifndef RT_TRACER_HPP
#define RT_TRACER_HPP

#include <stdint.h>

#include "ray.hpp"
#include "renderer-config.hpp"
#include "scene.hpp"

class Tracer {
public:
    Tracer();
    int32_t initialize();

    int32_t trace(Scene& scene, int32_t ray_count, RayBundle& rays, HitBundle& hits,
                  bool secondary = false);
    int32_t trace(Scene& scene, DeviceMemory& bvh_mem, int32_t ray_count, RayBundle& rays,
                  HitBundle& hits, bool secondary = false);
    int32_t shadow_trace(Scene& scene, int32_t ray_count, RayBundle& rays, HitBundle& hits,
                         bool secondary = false);
    int32_t shadow_trace(Scene& scene, DeviceMemory& bvh_mem, int32_t ray_count,
                         RayBundle& rays, HitBundle& hits, bool secondary = false);

    void timing(bool b);
    double get_trace_exec_time();
    double get_shadow_exec_time();
    void update_configuration(const RendererConfig& conf);

private:
    bool m_initialized;
    bool m_timing;
    double m_tracer_time_ms;
    double m_shadow_time_ms;
};

#endif /* RT_TRACER_HPP */
