/*
 * rt/framebuffer.hpp — the reference's FrameBuffer (include/rt/framebuffer.hpp:
 * 14-44), same public methods: a w x h image of fixed-point RGB sums
 * (3 uint32 per pixel, x 1e6) that the shader accumulates into; copy()
 * writes RGBA8 (round-to-nearest-even saturate(255 * v * 1e-6), A = 255)
 * into a device memory object of at least 4 w h bytes, where the reference
 * writes a GL texture.
 */
#pragma once
#ifndef RT_FRAMEBUFFER_HPP
#define RT_FRAMEBUFFER_HPP

#include <stddef.h>
#include <stdint.h>

#include "../gpu/interface.hpp"

class FrameBuffer {
public:
    FrameBuffer();
    ~FrameBuffer();
    int32_t initialize(size_t sz[2]);
    int32_t resize(size_t sz[2]);
    bool initialized();
    DeviceMemory& image_mem();
    int32_t clear();
    int32_t copy(DeviceMemory& tex_mem);
    void timing(bool b);
    double get_clear_exec_time();
    double get_copy_exec_time();

private:
    size_t size[2];
    memory_id img_mem_id;
    bool m_initialized;
    bool m_timing;
    double m_clear_time_ms;
    double m_copy_time_ms;
};

#endif /* RT_FRAMEBUFFER_HPP */
