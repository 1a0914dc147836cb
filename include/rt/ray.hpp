/*
 * rt/ray.hpp — the reference's RayBundle and HitBundle
 * (include/rt/ray.hpp:63-102): device arrays of the kernels' sample records
 * (rt_sample, 80 B: ray, pixel, contribution) and hit records (rt_hit, 64 B),
 * each held in a DeviceInterface memory object.
 */
#pragma once
#ifndef RT_RAY_HPP
#define RT_RAY_HPP

#include <stddef.h>
#include <stdint.h>

#include "../gpu/interface.hpp"

class RayBundle {
public:
    RayBundle();
    ~RayBundle();
    int32_t initialize(const size_t rays);
    int32_t resize(const size_t rays);
    bool valid();
    int32_t count();
    DeviceMemory& mem();

private:
    memory_id ray_id;
    int32_t m_ray_count;
    bool m_initialized;
};

class HitBundle {
public:
    HitBundle();
    ~HitBundle();
    int32_t initialize(const size_t sz);
    int32_t resize(const size_t rays);
    bool valid();
    int32_t count();
    DeviceMemory& mem();

private:
    memory_id hit_id;
    size_t m_size;
    bool m_initialized;
};

#endif /* RT_RAY_HPP */
