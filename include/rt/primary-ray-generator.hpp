/*
 * rt/primary-ray-generator.hpp — the reference's PrimaryRayGenerator
 * (include/rt/primary-ray-generator.hpp:12-50), same public methods, over
 * rt_gen_primary: rays for sample ids [offset, offset + ray_count) of a
 * w x h x spp image, pixels in quad_size blocks.  The Z-curve kernel the
 * reference picks for square power-of-two images when prim_ray_use_zcurve is
 * set is not provided: generate() returns -1 in that case.
 */
#pragma once
#ifndef PRIMARY_RAY_GENERATOR_HPP
#define PRIMARY_RAY_GENERATOR_HPP

#include <stddef.h>
#include <stdint.h>

#include "camera.hpp"
#include "ray.hpp"
#include "renderer-config.hpp"

struct pixel_sample_cl {
    float ox;
    float oy;
    float contribution;
};

class PrimaryRayGenerator {
public:
    PrimaryRayGenerator();
    ~PrimaryRayGenerator();
    int32_t initialize();
    int32_t set_spp(size_t spp, pixel_sample_cl const* psamples);
    size_t get_spp() const;
    DeviceMemory& get_pixel_samples();
    int32_t generate(const Camera& cam, RayBundle& bundle, size_t size[2], const size_t ray_count,
                     const size_t offset);
    void timing(bool b);
    double get_exec_time();
    void update_configuration(const RendererConfig& conf);

private:
    memory_id pixel_samples_id;
    bool m_initialized;
    bool m_timing;
    double m_time_ms;
    bool m_use_zcurve;
    int32_t m_quad_size;
    int32_t m_spp;
};

#endif /* PRIMARY_RAY_GENERATOR_HPP */
