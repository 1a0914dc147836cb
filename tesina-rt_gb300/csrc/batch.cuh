// batch.cuh — host interface of the many-scene build and many-image render.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "rt_internal.cuh"

namespace rt {

constexpr int kMaxBatchViews = 4096;

// One scene of a batched build: its arrays, as a one-scene build would use
// them, plus its slices of the batch scratch.
struct BatchScene {
    uint32_t n;
    int depth, min_leaf, passes;
    const float4* pos;
    const uint32_t* idx_in;
    const uint32_t* map_in;
    const uint32_t* orig_in;
    uint32_t* idx_out;
    uint32_t* map_out;
    uint32_t* orig_out;
    uint32_t* keys_unsorted;
    uint32_t* keys1;
    uint32_t* vals1;
    uint32_t* keys_sorted;
    uint32_t* vals_sorted;
    float4* tris;
    float4* nodes;
    BvhHeader* hdr;
    uint32_t* bounds;     // 8 words
    uint32_t* hist;       // 4 * 256 words
    uint32_t* lookback;   // passes * tiles * 256 words
    uint8_t* emit;        // the scene's emit item buffers (emit_buffers)
};

constexpr int kMaxEmitLevels = 16;

struct BatchBuildArgs {
    const BatchScene* scenes;
    int count;
    int passes;
    const uint32_t* tri_off;    // count + 1 prefix offsets of triangles
    const uint32_t* tile_off;   // count + 1 prefix offsets of sort tiles
    uint32_t* tile_ctr;         // one counter per pass
    uint32_t* status;
    unsigned long long* stage_ns;   // optional: globaltimer after each stage (8 entries)
    // the emit's levels over all scenes: level L has emit_jobs[L] blocks, the
    // blocks of scene s being emit_off[L * (count + 1) + s] ..
    const uint32_t* emit_off;
    int emit_levels;
    uint32_t emit_jobs[kMaxEmitLevels];
};

struct BatchView {
    SceneView scene;
    const rt_lights* lights;
    rt_camera cam;
    int width, height, max_bounces;
    uint32_t rgba_offset;       // first pixel of this image in the output
};

struct BatchRenderArgs {
    const BatchView* views;
    int count;
    const uint32_t* pix_off;    // count + 1 prefix offsets of pixels
    uint8_t* rgba;
    rt_render_stats* stats;
    uint32_t* work_counter;
    uint32_t* status;
    int chunk;
    float inv1e6;
    uint32_t* accum;            // pooled variants: 3 sums per pixel of the launch
    uint32_t total;             // pixels of the launch (pix_off[count])
};

const void* batch_build_kernel();
int batch_build_threads();
int batch_max_scenes();
int sort_tile_size();
cudaError_t launch_batch_build(const BatchBuildArgs& a, int grid, cudaStream_t s);
int batch_render_variant_count();
int batch_render_variant_info(int v, int* threads, const void** fn);
// True for variants that sum into BatchRenderArgs::accum before RGBA8.
bool batch_render_variant_pooled(int v);
// True for the variants that follow refracted rays (scenes with refracting
// materials); batch_refract_variant gives the unpooled one (pooled = false)
// or the pooled one with the smallest ray pool that holds views of
// max_bounces bounces (-1: none does).
bool batch_render_variant_refracts(int v);
int batch_refract_variant(bool pooled, int max_bounces);
cudaError_t launch_batch_render(const BatchRenderArgs& a, int variant, int grid, cudaStream_t s);

}  // namespace rt
