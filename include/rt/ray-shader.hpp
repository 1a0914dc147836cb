/*
 * rt/ray-shader.hpp — the reference's RayShader (include/rt/ray-shader.hpp:
 * 14-33), same public methods, over rt_shade: Whitted local shading of the
 * hits into the framebuffer's fixed-point sums.  The cubemap must be
 * disabled (the non-cubemap branch of ray-shader.cl).
 */
#pragma once
#ifndef RT_RAY_SHADER_HPP
#define RT_RAY_SHADER_HPP

#include <stddef.h>
#include <stdint.h>

#include "cubemap.hpp"
#include "framebuffer.hpp"
#include "ray.hpp"
#include "renderer-config.hpp"
#include "scene.hpp"

class RayShader {
public:
    RayShader();
    int32_t initialize();
    int32_t shade(RayBundle& rays, HitBundle& hb, Scene& scene, Cubemap& cm, FrameBuffer& fb,
                  size_t size, bool primary = false);
    void timing(bool b);
    double get_exec_time();
    void update_configuration(const RendererConfig& conf);

private:
    bool m_timing;
    double m_time_ms;
};

#endif /* RT_RAY_SHADER_HPP */
