/*
 * rt_cuda.h — C ABI of librt_cuda.so, the GB300 (sm_103a) implementation of the
 * Tesina-RT hot path: LBVH construction (Morton codes over triangle centroids,
 * key/value radix sort, hierarchy emit, bottom-up AABB refit), closest-hit BVH
 * traversal, shadow-ray any-hit, Whitted shading and reflection-ray generation.
 *
 * Conventions (the reference's own: every host method returns int32_t 0 / -1):
 *   - every entry point returns RT_OK (0) or a negative rt_status;
 *   - rt_last_error() returns a message for the last failure on this thread;
 *   - "d_" pointers are device pointers, "h_" pointers are host pointers;
 *   - descriptor structs passed by pointer are caller-owned and copied on entry;
 *   - a NULL stream means the context's default stream.
 *
 * Struct layouts marked "reference layout" are byte-compatible with the device
 * structs of the reference's OpenCL kernels so that buffers can be exchanged
 * with code written against the reference's RayBundle / HitBundle.
 */
#ifndef RT_CUDA_H
#define RT_CUDA_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define RT_API __attribute__((visibility("default")))
#else
#define RT_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------------ */
/* Status codes                                                             */
/* ------------------------------------------------------------------------ */
typedef enum rt_status {
    RT_OK = 0,
    RT_ERR = -1,              /* generic failure (the reference's -1)          */
    RT_ERR_INVALID = -2,      /* bad argument / size / descriptor              */
    RT_ERR_CUDA = -3,         /* CUDA runtime error                            */
    RT_ERR_OOM = -4,          /* device allocation failed or budget exceeded   */
    RT_ERR_TIMEOUT = -5,      /* a device-side bounded wait gave up            */
    RT_ERR_NOT_BUILT = -6,    /* scene has no BVH yet                          */
    RT_ERR_OVERFLOW = -7,     /* traversal stack or queue overflow             */
    RT_ERR_REJECTED = -8      /* serving: request refused by admission control */
} rt_status;

/* Device status bits reported by rt_device_status(). */
#define RT_DEV_TIMEOUT   0x1u  /* a decoupled look-back spin hit its cap      */
#define RT_DEV_OVERFLOW  0x2u  /* a traversal stack overflowed                */
#define RT_DEV_BADINDEX  0x4u  /* an index check failed (checked builds)      */

/* ------------------------------------------------------------------------ */
/* Scene data model (reference: include/rt/{material,light,camera}.hpp)     */
/* ------------------------------------------------------------------------ */
#define RT_MAX_LIGHTS 8

/* Light types: SPOT_L and DIR_L keep the reference's values
 * (include/rt/light.hpp:69-72); POINT_L is an extension (omni light, no cone,
 * shadow ray as for a spot light, LD = 1). */
enum { RT_SPOT_L = 0, RT_DIR_L = 1, RT_POINT_L = 2 };

typedef struct rt_light {        /* 64 B */
    int32_t type;                /* RT_SPOT_L / RT_DIR_L / RT_POINT_L          */
    float   radius;              /* spot: unused by the shading math           */
    float   angle;               /* spot: cosine cutoff                        */
    float   _pad0;
    float   pos[4];              /* spot / point position                      */
    float   dir[4];              /* spot axis or directional light direction   */
    float   color[4];
} rt_light;

/* Ambient colour plus 1..RT_MAX_LIGHTS lights.  With count == 1 this is the
 * reference's lights_cl (include/rt/light.hpp:86-92); more lights are summed in
 * order, each with its own shadow ray. */
typedef struct rt_lights {
    float    ambient[4];
    int32_t  count;
    int32_t  _pad[3];
    rt_light light[RT_MAX_LIGHTS];
} rt_lights;

/* reference layout: material_cl (include/rt/material.hpp:57-73), 32 B */
typedef struct rt_material {
    float   diffuse[4];
    float   shininess;
    float   reflectiveness;
    float   refractive_index;
    int32_t texture;             /* < 0: untextured (only case supported)      */
} rt_material;

/* Pinhole camera basis as passed to generate_primary_rays
 * (src/kernel/primary-ray-generator.cl:27-37): right and up are pre-scaled by
 * tan(fov/2) and aspect (src/rt/camera.cpp:31-59). */
typedef struct rt_camera {
    float pos[4];
    float dir[4];
    float right[4];
    float up[4];
} rt_camera;

/* Mirror of Camera::set (src/rt/camera.cpp:31-59).  fov is the vertical full
 * angle in radians, aspect = width / height. */
RT_API int32_t rt_camera_set(rt_camera* cam, const float pos[3], const float dir[3],
                      const float up[3], float fov, float aspect,
                      int32_t right_handed);

/* Host scene description.  Vertices may be SoA float4 (stride 16) or the
 * reference's 80-byte Vertex AoS (stride 80, position at 0, normal at 16). */
typedef struct rt_scene_desc {
    const void*        h_vertices;       /* positions (and normals if interleaved) */
    uint32_t           vertex_count;
    uint32_t           vertex_stride;    /* bytes between consecutive positions    */
    uint32_t           position_offset;  /* byte offset of position in a vertex    */
    uint32_t           normal_offset;    /* byte offset of normal (if h_normals==0)*/
    const void*        h_normals;        /* optional separate float4 normals       */
    const uint32_t*    h_indices;        /* 3 per triangle                         */
    uint32_t           triangle_count;
    uint32_t           material_count;
    const rt_material* h_materials;
    const uint32_t*    h_material_map;   /* material index per triangle            */
    rt_lights          lights;
} rt_scene_desc;

/* LBVH configuration: the reference's bvh_depth and bvh_min_leaf_size
 * (src/rt/bvh-builder.cpp:194-199; clamps depth to [1,32] here, min_leaf to
 * [1,256]). */
typedef struct rt_bvh_cfg {
    int32_t depth;               /* Morton bits, 1..32 (the workloads use 30)  */
    int32_t min_leaf_size;       /* 1..256                                     */
} rt_bvh_cfg;

/* One node of the canonical range tree, emitted in pre-order (left first).
 * Node numbering of the reference is nondeterministic; the canonical tree is
 * what parity is defined on. */
typedef struct rt_canon_node {
    uint32_t start, end;         /* triangle range [start, end) in sorted order */
    uint32_t leaf;               /* 1 = leaf                                    */
    uint32_t depth;              /* tree depth (root = 0)                       */
    float    lo[4];
    float    hi[4];
} rt_canon_node;

/* ------------------------------------------------------------------------ */
/* Reference-layout ray / sample / hit records (device structs of the .cl)  */
/* ------------------------------------------------------------------------ */
typedef struct rt_ray {          /* Ray: float3 ori, dir, invDir; tMin, tMax   */
    float ori[4];
    float dir[4];
    float inv_dir[4];
    float tmin, tmax;
    float _pad[2];
} rt_ray;                        /* 64 B */

typedef struct rt_sample {       /* Sample: Ray ray; int pixel; float contribution */
    rt_ray  ray;
    int32_t pixel;
    float   contribution;
    int32_t _pad[2];
} rt_sample;                     /* 80 B */

typedef struct rt_hit {          /* SampleTraceInfo (device layout, bool = 1 B) */
    uint8_t hit;
    uint8_t shadow_hit;          /* bit l set: light l occluded (1 light: 0/1) */
    uint8_t inverse_n;
    uint8_t reserved;
    float   t;
    int32_t id;                  /* triangle index in sorted order             */
    float   _pad0;
    float   uv[2];
    float   _pad1[2];
    float   n[4];
    float   hit_point[4];
} rt_hit;                        /* 64 B */

typedef struct rt_pixel_sample { /* PixelSample: ox, oy, contribution */
    float ox, oy, contribution;
} rt_pixel_sample;

/* Per-render counters (reference convention: rays = primary + secondary). */
typedef struct rt_render_stats {
    uint64_t primary_rays;
    uint64_t secondary_rays;
    uint64_t shadow_rays;
    uint64_t hits;
} rt_render_stats;

typedef struct rt_ctx    rt_ctx;
typedef struct rt_scene  rt_scene;
typedef void*            rt_stream;   /* a cudaStream_t */

/* ------------------------------------------------------------------------ */
/* Context, errors, streams, buffers (replaces DeviceInterface/DeviceMemory, */
/* include/gpu/interface.hpp:20-80, include/gpu/memory.hpp)                 */
/* ------------------------------------------------------------------------ */
RT_API const char* rt_last_error(void);
RT_API int32_t rt_init(rt_ctx** ctx, int32_t device);
RT_API int32_t rt_shutdown(rt_ctx* ctx);
/* Reads (and clears) the device status word: RT_DEV_* bits. */
RT_API int32_t rt_device_status(rt_ctx* ctx, uint32_t* bits);
/* Self-test of the device-side timeout (no reference counterpart; the
 * failure-detection form of a bounded wait): launches one radix-pass tile
 * whose predecessor tile is never launched, so its decoupled look-back polls
 * an unpublished word until its limit (1,024 polls here) runs out.  The
 * kernel then sets RT_DEV_TIMEOUT, finishes its tile inside its buffers and
 * returns; the call synchronises and maps the status as rt_render_host does:
 * RT_ERR_TIMEOUT when the timeout path worked (RT_OK would mean it did not).
 * The status stays set for rt_device_status to read and clear; the context
 * stays usable. */
RT_API int32_t rt_selftest_wait_timeout(rt_ctx* ctx, rt_stream s);
RT_API int32_t rt_stream_create(rt_ctx* ctx, rt_stream* stream);
RT_API int32_t rt_stream_destroy(rt_ctx* ctx, rt_stream stream);
RT_API int32_t rt_stream_sync(rt_ctx* ctx, rt_stream stream);
RT_API int32_t rt_buf_alloc(rt_ctx* ctx, size_t bytes, void** d_ptr);
RT_API int32_t rt_buf_free(rt_ctx* ctx, void* d_ptr);
RT_API int32_t rt_buf_write(rt_ctx* ctx, void* d_dst, const void* h_src, size_t bytes, rt_stream s);
RT_API int32_t rt_buf_read(rt_ctx* ctx, void* h_dst, const void* d_src, size_t bytes, rt_stream s);
RT_API int32_t rt_buf_copy(rt_ctx* ctx, void* d_dst, const void* d_src, size_t bytes, rt_stream s);
RT_API int32_t rt_buf_zero(rt_ctx* ctx, void* d_dst, size_t bytes, rt_stream s);

/* ------------------------------------------------------------------------ */
/* Scene (replaces Scene::transfer_aggregate_mesh_to_device,                */
/* src/rt/scene.cpp:236-321, and the buffer accessors scene.hpp:125-133)    */
/* ------------------------------------------------------------------------ */
RT_API int32_t rt_scene_create(rt_ctx* ctx, rt_scene** scene);
RT_API int32_t rt_scene_destroy(rt_ctx* ctx, rt_scene* scene);
RT_API int32_t rt_scene_upload(rt_ctx* ctx, rt_scene* scene, const rt_scene_desc* desc, rt_stream s);
/* Replace vertex positions/normals (float4 each, host memory) keeping topology;
 * analogue of Scene::update_aggregate_mesh_vertices (scene.cpp:967-984). */
RT_API int32_t rt_scene_update_vertices(rt_ctx* ctx, rt_scene* scene, const float* h_pos4,
                                 const float* h_nrm4, uint32_t vertex_count, rt_stream s);
/* Same, from device memory. */
RT_API int32_t rt_scene_update_vertices_device(rt_ctx* ctx, rt_scene* scene, const float* d_pos4,
                                        const float* d_nrm4, uint32_t vertex_count, rt_stream s);
/* Device-side animation: the mangle kernel (src/kernel/mangler.cl:12-32) on the
 * scene's vertices, as the reference's wave demo runs it before each frame
 * (src/rt/rt-wave.cpp:141-167; height 0.2 at :408-413): position.y = height *
 * sin(0.33 arg + x) * cos(0.57 arg + z), normal.x / normal.z from per-vertex
 * phases.  last_arg is accepted and unused, as in the kernel.  Follow with
 * rt_bvh_refit_lbvh (the refit-only mode, renderer.cpp:53-70) or a rebuild. */
RT_API int32_t rt_scene_mangle(rt_ctx* ctx, rt_scene* scene, float arg, float last_arg,
                               float height, rt_stream s);
/* Wavefront OBJ input, host side: the role of Scene::load_obj_file_as_aggregate
 * (src/rt/scene.cpp:441-453) with the import rules of the loader the
 * reference vendors (src/rt/obj-loader.cpp:163-1123): polygons split as fans,
 * corners shared by bytewise-equal vertex records, material groups, normals
 * generated when the file has none.  Group materials come from an mtllib file
 * beside the model (newmtl, Kd, Ns / 1000, d, Tr) or the loader's default. */
typedef struct rt_obj rt_obj;
typedef struct {
    uint32_t first_triangle, triangle_count;
    float diffuse[3];
    float shininess, alpha;
} rt_obj_group;
RT_API int32_t rt_obj_load(const char* path, rt_obj** out);
RT_API int32_t rt_obj_info(const rt_obj* obj, uint32_t* vertex_count, uint32_t* triangle_count,
                           uint32_t* group_count);
/* Positions / normals as float4 (w = 0), uint3 indices, groups (highest alpha first). */
RT_API int32_t rt_obj_copy(const rt_obj* obj, float* pos4, float* nrm4, uint32_t* indices,
                           rt_obj_group* groups);
RT_API int32_t rt_obj_free(rt_obj* obj);
/* Multi-root (instanced) scenes: the reference's objects with their own BVH
 * roots and transforms (Scene::create_bvhs / update_bvh_roots,
 * src/rt/scene.cpp:595-703; trace_multi, src/kernel/trace-bvh.cl:420-463;
 * shadow_trace_multi, src/kernel/shadow-trace-bvh.cl:317-373).  Instance i
 * draws built scene inst_scene[i] under the row-major 4x4 transform tr[16 i]
 * whose inverse is tr_inv[16 i] (both given, as BVHRoot holds both).  Each
 * scene keeps its materials; lights are the instance set's.  With refracting
 * materials a frame renders up to 6 bounces.  The set refers to its scenes: destroy
 * it before them; a scene rebuilt (on any stream) is seen by the next render. */
typedef struct rt_instances rt_instances;
RT_API int32_t rt_instances_create(rt_ctx* ctx, rt_scene* const* scenes, int32_t scene_count,
                                   const int32_t* inst_scene, const float* tr, const float* tr_inv,
                                   int32_t instance_count, const rt_lights* lights,
                                   rt_instances** out);
/* New transforms for every instance (Scene::update_bvh_roots). */
RT_API int32_t rt_instances_set_transforms(rt_ctx* ctx, rt_instances* inst, const float* tr,
                                           const float* tr_inv);
/* The Whitted frame over all instances (reflection, shadows, max_bounces). */
RT_API int32_t rt_instances_render(rt_ctx* ctx, rt_instances* inst, const rt_camera* cam,
                                   int32_t width, int32_t height, int32_t max_bounces,
                                   uint8_t* d_rgba, uint32_t* d_image_rgb,
                                   rt_render_stats* d_stats, rt_stream s);
RT_API int32_t rt_instances_destroy(rt_ctx* ctx, rt_instances* inst);
RT_API int32_t rt_scene_set_lights(rt_ctx* ctx, rt_scene* scene, const rt_lights* lights);
/* Device buffers of the scene (reference: Scene::index_mem(), material_map_mem()).
 * After a build, indices and material map are permuted into sorted order, as
 * the reference permutes them in place (bvh-builder.cpp:470-527). */
RT_API int32_t rt_scene_buffers(rt_ctx* ctx, rt_scene* scene, uint32_t** d_indices,
                         uint32_t** d_material_map, float** d_positions,
                         float** d_normals, uint32_t* triangle_count);
/* Host copies of the per-build arrays used for parity:
 * unsorted Morton keys (per original triangle), the sort permutation
 * (sorted slot -> original triangle) and the sorted keys.  Any may be NULL. */
RT_API int32_t rt_scene_read_sort(rt_ctx* ctx, rt_scene* scene, uint32_t* h_keys,
                           uint32_t* h_perm, uint32_t* h_sorted_keys);
/* Triangle id at upload of each triangle in the current order (maps the
 * sorted-order ids of rt_hit.id back to the caller's triangles). */
RT_API int32_t rt_scene_read_orig(rt_ctx* ctx, rt_scene* scene, uint32_t* h_orig);

/* ------------------------------------------------------------------------ */
/* LBVH (replaces BVHBuilder, include/rt/bvh-builder.hpp:16-28)             */
/* ------------------------------------------------------------------------ */
/* BVHBuilder::build_lbvh (src/rt/bvh-builder.cpp:201-741). */
RT_API int32_t rt_bvh_build_lbvh(rt_ctx* ctx, rt_scene* scene, const rt_bvh_cfg* cfg, rt_stream s);
/* BVHBuilder::refit_lbvh (src/rt/bvh-builder.cpp:743-850): recompute AABBs on
 * the existing topology and triangle order. */
RT_API int32_t rt_bvh_refit_lbvh(rt_ctx* ctx, rt_scene* scene, rt_stream s);
/* The reference's CPU SAH BVH (BVH::construct, src/rt/bvh.cpp:6-179) over the
 * scene's triangles in their current order, built on the host's threads and
 * laid out as the LBVH's device tree (the triangles reordered likewise), so
 * that every render call traverses it; returns when it is on the device.
 * RT_ERR_INVALID when an interior node lies deeper than the traversal's
 * 32-entry stack; such a tree cannot be refit (build it again). */
RT_API int32_t rt_bvh_build_sah(rt_ctx* ctx, rt_scene* scene, rt_stream s);
/* Canonical pre-order tree (synchronous).  *count receives the node count;
 * pass out == NULL to query it. */
RT_API int32_t rt_bvh_export(rt_ctx* ctx, rt_scene* scene, rt_canon_node* out,
                      uint32_t capacity, uint32_t* count);
/* Device time of the last build / refit in milliseconds (CUDA events). */
RT_API int32_t rt_bvh_last_time_ms(rt_ctx* ctx, rt_scene* scene, float* ms);

/* ------------------------------------------------------------------------ */
/* Stage-wise pipeline on reference-layout buffers (drop-in for the         */
/* reference's PrimaryRayGenerator, Tracer, RayShader,                      */
/* SecondaryRayGenerator, FrameBuffer)                                      */
/* ------------------------------------------------------------------------ */
/* PrimaryRayGenerator::generate (src/rt/primary-ray-generator.cpp:57-165,
 * kernel primary-ray-generator.cl:27-103). Rays for global ids
 * [offset, offset+ray_count) of a w*h*spp image, quad_size pixel blocks.
 * d_pixel_samples may be NULL (one sample {0,0,1}). */
RT_API int32_t rt_gen_primary(rt_ctx* ctx, const rt_camera* cam, int32_t width, int32_t height,
                       int32_t quad_size, int32_t spp, const rt_pixel_sample* d_pixel_samples,
                       size_t ray_count, size_t offset, rt_sample* d_samples, rt_stream s);
/* Tracer::trace (src/rt/tracer.cpp:140-269, kernel trace-bvh.cl:465-481). */
RT_API int32_t rt_trace(rt_ctx* ctx, rt_scene* scene, const rt_sample* d_samples, int32_t ray_count,
                 rt_hit* d_hits, int32_t secondary, rt_stream s);
/* Tracer::shadow_trace (src/rt/tracer.cpp:273-352, kernel
 * shadow-trace-bvh.cl:375-418); one shadow ray per light, result bitmask in
 * rt_hit.shadow_hit. */
RT_API int32_t rt_shadow_trace(rt_ctx* ctx, rt_scene* scene, const rt_sample* d_samples,
                        int32_t ray_count, rt_hit* d_hits, int32_t secondary, rt_stream s);
/* RayShader::shade (src/rt/ray-shader.cpp:32-154, kernel ray-shader.cl:116-459).
 * d_image_rgb: 3 uint32 per pixel, fixed point x1e6, accumulated with atomics. */
RT_API int32_t rt_shade(rt_ctx* ctx, rt_scene* scene, const rt_sample* d_samples,
                 const rt_hit* d_hits, int32_t ray_count, uint32_t* d_image_rgb,
                 int32_t primary, rt_stream s);
/* SecondaryRayGenerator::generate (src/rt/secondary-ray-generator.cpp:57-244,
 * kernels secondary-ray-generator.cl:184-326): reflection rays, stable order.
 * *d_count (device int32) receives the number of rays written (clamped to
 * max_out).  If h_count != NULL the call synchronises and stores it there. */
RT_API int32_t rt_gen_secondary(rt_ctx* ctx, rt_scene* scene, const rt_sample* d_in, int32_t rays_in,
                         const rt_hit* d_hits, rt_sample* d_out, int32_t max_out,
                         int32_t* d_count, int32_t* h_count, rt_stream s);
/* FrameBuffer::clear / copy (src/rt/framebuffer.cpp:117-165,
 * framebuffer.cl:20-54): RGBA8 = round-to-nearest-even saturate(255 * v * 1e-6). */
RT_API int32_t rt_fb_clear(rt_ctx* ctx, uint32_t* d_image_rgb, size_t pixels, rt_stream s);
RT_API int32_t rt_fb_copy(rt_ctx* ctx, const uint32_t* d_image_rgb, uint8_t* d_rgba, size_t pixels,
                   rt_stream s);

/* ------------------------------------------------------------------------ */
/* Fused plain path: Renderer::render_to_framebuffer (src/rt/renderer.cpp:  */
/* 113-214) + FrameBuffer::copy in one persistent kernel.                   */
/* ------------------------------------------------------------------------ */
/* d_rgba: w*h RGBA8 (required).  d_image_rgb: optional fixed-point
 * accumulation buffer (3 uint32 per pixel, written, not accumulated).
 * d_stats: optional device rt_render_stats (accumulated; caller zeroes). */
RT_API int32_t rt_render(rt_ctx* ctx, rt_scene* scene, const rt_camera* cam, int32_t width,
                  int32_t height, int32_t max_bounces, uint8_t* d_rgba, uint32_t* d_image_rgb,
                  rt_render_stats* d_stats, rt_stream s);

/* ------------------------------------------------------------------------ */
/* Render kernel configuration and autotuning                               */
/* ------------------------------------------------------------------------ */
/* All variants produce identical images; they differ in block size and in
 * the register budget (minimum resident blocks per SM), the number of
 * resident blocks launched, and the pixels a warp takes per work fetch. */
typedef struct rt_render_config {
    int32_t variant;         /* kernel variant, 0 .. rt_render_variants() - 1           */
    int32_t blocks_per_sm;   /* resident blocks per SM to launch; 0 = occupancy maximum */
    int32_t chunk;           /* pixels per warp work fetch: 32, 64, 128 or 256          */
    int32_t stack_depth;     /* traversal stack entries (fixed: 32, enough for depth <= 31) */
} rt_render_config;

RT_API int32_t rt_render_variants(int32_t* count);
/* threads per block, minimum blocks per SM it was compiled for, and the
 * blocks per SM the occupancy calculator allows on this context's GPU. */
RT_API int32_t rt_render_variant_info(rt_ctx* ctx, int32_t variant, int32_t* threads,
                                      int32_t* min_blocks, int32_t* occupancy_blocks);
/* *pooled = 1 for the variants that pool shadow and reflection rays per warp
 * and sum per pixel before writing RGBA8 (two kernels per render), 0 for the
 * one-path-per-lane variants.  Same image either way. */
RT_API int32_t rt_render_variant_pooled(int32_t variant, int32_t* pooled);
RT_API int32_t rt_set_render_config(rt_ctx* ctx, const rt_render_config* cfg);
RT_API int32_t rt_get_render_config(rt_ctx* ctx, rt_render_config* cfg);
/* Times every variant x resident-block count x chunk on this scene and
 * camera (trials timed launches each, best kept), installs the fastest
 * configuration in the context and returns it.  Results are cached per
 * (image size, triangle count, bounces) class in the context. */
RT_API int32_t rt_autotune_render(rt_ctx* ctx, rt_scene* scene, const rt_camera* cam,
                                  int32_t width, int32_t height, int32_t max_bounces,
                                  int32_t trials, rt_render_config* best, float* best_ms);

/* ------------------------------------------------------------------------ */
/* Batched form: many scenes per build launch, many images per render launch */
/* ------------------------------------------------------------------------ */
typedef struct rt_batch rt_batch;

/* One image of a batch.  Images are packed in view order in one RGBA8
 * buffer: view v starts at pixel rgba_offset = sum of the earlier views'
 * width * height. */
typedef struct rt_batch_view {
    rt_scene* scene;             /* uploaded scene (several views may share one) */
    rt_camera cam;
    int32_t   width, height, max_bounces;
    uint32_t  rgba_offset;
} rt_batch_view;

RT_API int32_t rt_batch_create(rt_ctx* ctx, rt_batch** batch);
RT_API int32_t rt_batch_destroy(rt_ctx* ctx, rt_batch* batch);
/* Declares the views (<= 4096) and their distinct scenes (<= 1024), one LBVH
 * configuration for all of them, and prepares device tables and buffers. */
RT_API int32_t rt_batch_set(rt_ctx* ctx, rt_batch* batch, const rt_batch_view* views,
                            int32_t count, const rt_bvh_cfg* cfg);
/* Builds the LBVH of every distinct scene in ONE persistent cooperative
 * launch; results are the same as rt_bvh_build_lbvh on each scene. */
RT_API int32_t rt_batch_build(rt_ctx* ctx, rt_batch* batch, rt_stream s);
/* Renders every view in ONE persistent launch into d_rgba (total pixels x 4
 * bytes); same pixels as rt_render per view.  d_stats optional, accumulated. */
RT_API int32_t rt_batch_render(rt_ctx* ctx, rt_batch* batch, uint8_t* d_rgba,
                               rt_render_stats* d_stats, rt_stream s);
/* Captures build + render into a CUDA graph (on the context stream).  Each
 * replay rebuilds every scene from the triangle order the capture saw and
 * renders; d_stats (optional) is zeroed by every replay. */
RT_API int32_t rt_batch_capture(rt_ctx* ctx, rt_batch* batch, uint8_t* d_rgba,
                                rt_render_stats* d_stats);
RT_API int32_t rt_batch_replay(rt_ctx* ctx, rt_batch* batch, rt_stream s);
RT_API int32_t rt_batch_info(rt_ctx* ctx, rt_batch* batch, uint32_t* scenes,
                             uint32_t* triangles, uint32_t* pixels);
/* Profiling of the batched build: when enabled, the build kernel records a
 * device timestamp after each of its stages; rt_batch_stage_times returns the
 * durations in ms of: init, scene bounds, Morton + histograms, radix passes,
 * permutation (near 0: the permutation runs inside the emit's first level),
 * emit + refit (synchronous). */
RT_API int32_t rt_batch_profile(rt_ctx* ctx, rt_batch* batch, int32_t enable);
RT_API int32_t rt_batch_stage_times(rt_ctx* ctx, rt_batch* batch, float ms[6]);

/* ------------------------------------------------------------------------ */
/* Served form: resident scenes, admission, continuous batching             */
/* ------------------------------------------------------------------------ */
typedef struct rt_server rt_server;

enum { RT_REQ_RENDER = 0, RT_REQ_UPLOAD = 1 };

typedef struct rt_server_cfg {
    uint64_t hbm_budget_bytes;   /* resident scenes + framebuffer arena            */
    uint64_t fb_arena_bytes;     /* device framebuffers of admitted requests        */
    int32_t  max_batch_views;    /* requests per render launch; 1 = plain path     */
    int32_t  max_inflight;       /* render launches on the GPU at once (streams)   */
    int32_t  max_scenes;         /* resident-scene cap, 0 = none: an upload beyond
                                    it evicts the least recently used scene        */
    int32_t  reserved;           /* 0                                              */
} rt_server_cfg;

typedef struct rt_request {
    int32_t  type;               /* RT_REQ_RENDER / RT_REQ_UPLOAD                   */
    int32_t  max_bounces;
    int32_t  width, height;
    uint64_t scene_id;           /* render: target scene                           */
    rt_camera cam;
    const rt_scene_desc* upload; /* upload: caller-owned until the request is done */
} rt_request;

typedef struct rt_request_info {
    int32_t  status;             /* RT_OK or the failure (RT_ERR_REJECTED, ...)     */
    int32_t  batch_views;        /* requests in the launch that served this one     */
    uint64_t scene_id;           /* upload: id of the new scene                     */
    double   submit_ms, start_ms, done_ms;   /* server clock                        */
    uint64_t rays;               /* primary + secondary rays traced                 */
} rt_request_info;

typedef struct rt_server_stats {
    uint64_t completed, rejected, evicted, batches, rays, resident_scenes;
    uint64_t resident_bytes;
    double   p50_ms, p99_ms, mean_batch_views, first_submit_ms, last_done_ms;
} rt_server_stats;

RT_API int32_t rt_server_create(rt_ctx* ctx, const rt_server_cfg* cfg, rt_server** server);
RT_API int32_t rt_server_destroy(rt_server* server);
/* Synchronous upload + LBVH build of a resident scene (counted in the budget). */
RT_API int32_t rt_server_add_scene(rt_server* server, const rt_scene_desc* desc,
                                   uint64_t* scene_id);
/* Thread-safe, non-blocking.  Renders and uploads are admitted in arrival
 * order as framebuffer space and memory allow; uploads that do not fit even
 * after evicting least-recently-used idle scenes are rejected.  Recency is
 * the order of submission (add_scene, upload and render submits).  With
 * max_scenes set, an upload that would exceed it marks the least recently
 * used scene evicted at submit: renders already submitted for it are still
 * served, later ones fail with RT_ERR_INVALID. */
RT_API int32_t rt_server_submit(rt_server* server, const rt_request* req, uint64_t* ticket);
/* An upload request that returns the new scene's id at once: renders may
 * name it immediately and are served once its LBVH is built (they fail if
 * the upload is rejected).  The descriptor stays caller-owned until the
 * upload's result is taken. */
RT_API int32_t rt_server_upload(rt_server* server, const rt_scene_desc* desc, uint64_t* ticket,
                                uint64_t* scene_id);
/* Blocks until the request is done; copies a render's RGBA8 image to h_rgba
 * (may be NULL) and releases it. */
RT_API int32_t rt_server_result(rt_server* server, uint64_t ticket, uint8_t* h_rgba,
                                rt_request_info* info);
/* Latency percentiles over render requests completed since the last reset. */
RT_API int32_t rt_server_get_stats(rt_server* server, rt_server_stats* stats);
RT_API int32_t rt_server_reset_stats(rt_server* server);

/* End-to-end convenience: host vertices in, host image out, synchronous:
 * optional vertex update -> LBVH build -> render -> RGBA8 to host.  The
 * normals, which only the render reads, are uploaded on a stream of the
 * context's own once the positions are up, beside the build; pinned host
 * buffers make the copies asynchronous.  Equal to rt_render_host_async
 * followed by rt_render_host_wait on the same stream. */
RT_API int32_t rt_render_host(rt_ctx* ctx, rt_scene* scene, const float* h_pos4, const float* h_nrm4,
                       uint32_t vertex_count, const rt_bvh_cfg* cfg, const rt_camera* cam,
                       int32_t width, int32_t height, int32_t max_bounces, uint8_t* h_rgba,
                       rt_render_stats* h_stats, rt_stream s);
/* rt_render_host without the final wait: queues the frame on stream s
 * (uploads, build, render, image and counter read-back) and returns; the
 * host buffers must stay untouched until rt_render_host_wait(ctx, s) returns,
 * which synchronises s, fills h_stats and maps the device status as
 * rt_render_host does.  One frame may be pending per stream: a second call
 * on the same stream before the wait returns RT_ERR_INVALID.  Frames on two
 * streams (each with its own scene, or the same scene: the scene's accesses
 * are ordered across streams) overlap one frame's copies with the other's
 * build and render.  No reference counterpart (the reference renders one
 * frame at a time, src/rt/renderer.cpp:113-214). */
RT_API int32_t rt_render_host_async(rt_ctx* ctx, rt_scene* scene, const float* h_pos4,
                                    const float* h_nrm4, uint32_t vertex_count,
                                    const rt_bvh_cfg* cfg, const rt_camera* cam, int32_t width,
                                    int32_t height, int32_t max_bounces, uint8_t* h_rgba,
                                    rt_render_stats* h_stats, rt_stream s);
RT_API int32_t rt_render_host_wait(rt_ctx* ctx, rt_stream s);

/* ------------------------------------------------------------------------ */
/* Sort without allocation (no counterpart in the reference)                */
/* ------------------------------------------------------------------------ */
/* Largest n accepted by rt_sort_pairs_noalloc. */
#define RT_NOALLOC_MAX_PAIRS (1u << 20)

/* Stable LSD radix sort of n (key, value) uint32 pairs on the low key_bits
 * bits (1..32), the same passes the LBVH builder runs on Morton codes, for
 * callers that cannot allocate device memory when they sort (their HBM is
 * already handed to their own pool, or a cudaMalloc's implicit
 * synchronisation is not acceptable in their loop).  No counterpart in the
 * reference.  Allocates nothing: its scratch is a fixed ~9 MiB array in
 * device memory that every GPU loading this library keeps until exit.
 *   - n > RT_NOALLOC_MAX_PAIRS is rejected with RT_ERR_INVALID;
 *   - inputs are not modified; an output that overlaps an input or the
 *     other output is rejected with RT_ERR_INVALID;
 *   - every call on a device shares the one scratch array, whichever rt_ctx
 *     it comes from: calls that overlap on the GPU race, also across
 *     contexts; order them on one stream, or with events between streams;
 *   - the return code covers the arguments and the launches; a device-side
 *     failure (a look-back wait that gave up) is reported as RT_DEV_TIMEOUT
 *     by rt_device_status, which the caller reads after synchronising;
 *   - the first call on a device looks up the array's device address; make
 *     that call before any stream capture. */
RT_API int32_t rt_sort_pairs_noalloc(rt_ctx* ctx, const uint32_t* d_keys_in,
                                     const uint32_t* d_vals_in, uint32_t* d_keys_out,
                                     uint32_t* d_vals_out, uint32_t n, int32_t key_bits,
                                     rt_stream s);

#ifdef __cplusplus
}
#endif
#endif /* RT_CUDA_H */
