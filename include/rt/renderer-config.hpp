/*
 * rt/renderer-config.hpp — the reference's RendererConfig
 * (include/rt/renderer-config.hpp:7-33) with its defaults
 * (src/rt/renderer-config.cpp:4-16).  The constructor is public here: there
 * is no Renderer class to hand configurations out.
 */
#pragma once
#ifndef RTCONFIG_HPP
#define RTCONFIG_HPP

class RendererConfig {
public:
    RendererConfig()
        : use_lbvh(1), bvh_refit_only(0), bvh_depth(32), bvh_min_leaf_size(1),
          sec_ray_use_atomics(0), sec_ray_use_disc(1), prim_ray_quad_size(32),
          prim_ray_use_zcurve(0), tile_to_cores_ratio(128) {}

    int use_lbvh;
    int bvh_refit_only;
    int bvh_depth;
    int bvh_min_leaf_size;
    int sec_ray_use_atomics;
    int sec_ray_use_disc;
    int prim_ray_quad_size;
    int prim_ray_use_zcurve;
    double tile_to_cores_ratio;
};

#endif /* RTCONFIG_HPP */
