/*
 * rt/secondary-ray-generator.hpp — the reference's SecondaryRayGenerator
 * (include/rt/secondary-ray-generator.hpp:12-27), same public methods, over
 * rt_gen_secondary: one reflection ray per mirror hit (and a refraction ray
 * per refracting hit), in the stable order of the reference's "disc" scan
 * path.  The other configurations (sec_ray_use_atomics, no disc) produce the
 * same rays in another order in the reference; here every configuration
 * takes the stable order.  At most max(set_max_rays, 0 = no limit) rays and
 * never more than ray_out holds are written; *rays_out is the number
 * written (the count is read back, a synchronisation, as in the reference).
 */
#pragma once
#ifndef RT_SECONDARY_RAY_GENERATOR_HPP
#define RT_SECONDARY_RAY_GENERATOR_HPP

#include <stddef.h>
#include <stdint.h>

#include "ray.hpp"
#include "renderer-config.hpp"
#include "scene.hpp"

class SecondaryRayGenerator {
public:
    SecondaryRayGenerator();
    ~SecondaryRayGenerator();
    int32_t initialize();
    int32_t generate(Scene& scene, RayBundle& ray_in, size_t rays_in, HitBundle& hits,
                     RayBundle& ray_out, size_t* rays_out);
    void set_max_rays(size_t max);
    void timing(bool b);
    double get_exec_time();
    void update_configuration(const RendererConfig& conf);

private:
    int32_t m_max_rays;
    bool m_tasks;
    bool m_disc;
    bool m_initialized;
    bool m_timing;
    double m_time_ms;
    memory_id count_id;
};

#endif /* RT_SECONDARY_RAY_GENERATOR_HPP */
