/*
 * rt/bvh-builder.hpp — the reference's BVHBuilder (include/rt/bvh-builder.hpp:
 * 16-28), same public methods, over rt_bvh_build_lbvh / rt_bvh_refit_lbvh.
 * bvh_depth and bvh_min_leaf_size are clamped as update_configuration does
 * (src/rt/bvh-builder.cpp:194-199: [1, 64] and [1, 256]); the keys here are
 * one 32-bit word, so builds with bvh_depth above 32 return -1.
 */
#pragma once
#ifndef BVH_BUILDER_HPP
#define BVH_BUILDER_HPP

#include <stddef.h>
#include <stdint.h>

#include "renderer-config.hpp"
#include "scene.hpp"

class Log;

class BVHBuilder {
public:
    BVHBuilder();
    int32_t initialize();
    int32_t build_lbvh(Scene& scene, size_t cq_i = 0);
    int32_t refit_lbvh(Scene& scene, size_t cq_i = 0);
    void set_log(Log* log);
    void timing(bool b);
    void logging(bool l);
    /* Device time of the last build, milliseconds (timing on). */
    double get_exec_time();
    void update_configuration(const RendererConfig& conf);

    bool bvh_created;

private:
    Log* m_log;
    bool m_logging;
    bool m_timing;
    double m_time_ms;
    int32_t bvh_depth;
    int32_t bvh_min_leaf_size;
};

#endif /* BVH_BUILDER_HPP */
