// trace.cuh — host interface of the traversal / shading kernels (trace.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "rt_internal.cuh"

namespace rt {


struct RenderArgs {
    SceneView scene;
    rt_lights lights;
    rt_camera cam;
    int width, height, max_bounces;
    float inv1e6;                 // 1.0f / 1e6f, the framebuffer's cint_max_inv
    uint8_t* rgba;                // width * height RGBA8
    uint32_t* image_rgb;          // optional fixed-point accumulation (3 per pixel)
    rt_render_stats* stats;       // optional, accumulated
    uint32_t* work_counter;       // zeroed before launch
    uint32_t* status;
    int chunk;                    // pixels per warp work fetch, multiple of 32
    uint32_t* accum;              // pooled variants: fixed-point sums (3 per pixel)
};

// Render kernel variants (block size, minimum blocks per SM) for the autotuner.
int render_variant_count();
int render_variant_info(int v, int* threads, int* min_blocks, const void** fn);
// True for variants that accumulate into RenderArgs::accum (k_render_pool).
bool render_variant_pooled(int v);
// True for the variants that follow refracted rays; the scenes with
// refracting materials render with one of them.
bool render_variant_refracts(int v);
// Whether variant v renders frames of max_bounces bounces (the pooled
// refraction variants hold 32 (b + 2) rays per warp for up to b bounces).
bool render_variant_fits(int v, int max_bounces);
// The refraction variant for frames of max_bounces bounces: the pooled one
// where it fits, else the ray-tree walk.
int render_refract_variant(int max_bounces);
cudaError_t launch_render(const RenderArgs& a, int variant, int grid, cudaStream_t s);
cudaError_t launch_gen_primary(const rt_camera& cam, int w, int h, int q, const rt_pixel_sample* ps,
                               size_t count, size_t offset, rt_sample* out, cudaStream_t s);
cudaError_t launch_trace(const SceneView& S, const rt_sample* smp, int n, rt_hit* hits,
                         uint32_t* status, cudaStream_t s);
cudaError_t launch_shadow(const SceneView& S, const rt_lights& L, int n, rt_hit* hits,
                          uint32_t* status, cudaStream_t s);
cudaError_t launch_shade(const SceneView& S, const rt_lights& L, const rt_sample* smp,
                         const rt_hit* hits, int n, uint32_t* image, cudaStream_t s);
cudaError_t launch_gen_secondary(const SceneView& S, const rt_sample* in, int n, const rt_hit* hits,
                                 rt_sample* out, int max_out, int32_t* d_count,
                                 uint32_t* block_scratch, cudaStream_t s);
cudaError_t launch_fb_copy(const uint32_t* img, uint8_t* rgba, size_t px, float inv1e6,
                           cudaStream_t s);
size_t gen_secondary_scratch_bytes(int n);

}  // namespace rt
