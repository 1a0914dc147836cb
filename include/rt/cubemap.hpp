/*
 * rt/cubemap.hpp — stand-in for the reference's Cubemap
 * (include/rt/cubemap.hpp).  The shading path here is the reference's
 * non-cubemap branch (use_cubemap = 0, ray-shader.cl): RayShader::shade
 * accepts a Cubemap and requires it disabled.
 */
#pragma once
#ifndef RT_CUBEMAP_HPP
#define RT_CUBEMAP_HPP

class Cubemap {
public:
    Cubemap() : enabled(false) {}
    bool enabled;
};

#endif /* RT_CUBEMAP_HPP */
