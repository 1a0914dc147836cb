// batch_api.cu — C ABI of the batched form: many scenes built in one
// persistent launch, many images rendered in one persistent launch, the pair
// captured in a CUDA graph and replayed.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <new>
#include <vector>

#include "../../include/rt_cuda.h"
#include "batch.cuh"
#include "ctx_internal.h"
#include "lbvh.cuh"
#include "lbvh_dev.cuh"

#define fail rt::set_error

#define CU(call)                                                                              \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess)                                                                \
            return fail(RT_ERR_CUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_),  \
                        __FILE__, __LINE__);                                                  \
    } while (0)

struct rt_batch {
    std::vector<rt_batch_view> views;
    std::vector<rt_scene*> scenes;          // distinct scenes, in first-use order
    std::vector<int> view_scene;            // view -> index in scenes
    int depth = 30, min_leaf = 1;
    uint32_t total_tris = 0, total_tiles = 0, total_pixels = 0;
    // device tables
    rt::BatchScene* d_scenes = nullptr;
    uint32_t* d_tri_off = nullptr;
    uint32_t* d_tile_off = nullptr;
    uint32_t* d_ctr = nullptr;              // 4 tile counters + 1 render work counter
    uint32_t* d_scratch = nullptr;          // per scene: bounds 8 | hist 1024 | look-back
    size_t scratch_words = 0;
    std::vector<size_t> scratch_at;         // word offset of each scene's scratch
    rt::BatchView* d_views = nullptr;
    uint32_t* d_pix_off = nullptr;
    uint32_t* d_accum = nullptr;            // render sums, 3 per pixel (pooled render)
    rt_lights* d_lights = nullptr;          // one per distinct scene
    int build_grid = 0;
    int render_variant = 0, render_grid = 0, render_chunk = 32;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    unsigned long long* d_stage = nullptr;  // stage timestamps when profiling is on
    bool profile = false;
    // the emit's levels: per level, the scenes' offsets into its blocks
    uint32_t* d_emit_off = nullptr;
    int emit_levels = 0;
    uint32_t emit_jobs[rt::kMaxEmitLevels] = {};
};

namespace {

template <class T>
void dfree(T*& p) {
    if (p) cudaFree(p);
    p = nullptr;
}

void free_tables(rt_batch* b) {
    dfree(b->d_scenes);
    dfree(b->d_tri_off);
    dfree(b->d_tile_off);
    dfree(b->d_ctr);
    dfree(b->d_scratch);
    dfree(b->d_views);
    dfree(b->d_pix_off);
    dfree(b->d_accum);
    dfree(b->d_lights);
    dfree(b->d_stage);
    dfree(b->d_emit_off);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
}

// Per-scene build descriptors for the scenes' current order: read
// d_idx[cur], write d_idx[cur ^ 1].
std::vector<rt::BatchScene> scene_table(rt_batch* b) {
    const int passes = (b->depth + 7) / 8;
    std::vector<rt::BatchScene> t(b->scenes.size());
    for (size_t k = 0; k < b->scenes.size(); ++k) {
        rt_scene* s = b->scenes[k];
        rt::BatchScene& B = t[k];
        B.n = s->N;
        B.depth = b->depth;
        B.min_leaf = b->min_leaf;
        B.passes = passes;
        B.pos = s->d_pos;
        B.idx_in = s->d_idx[s->cur];
        B.map_in = s->d_map[s->cur];
        B.orig_in = s->d_orig[s->cur];
        B.idx_out = s->d_idx[s->cur ^ 1];
        B.map_out = s->d_map[s->cur ^ 1];
        B.orig_out = s->d_orig[s->cur ^ 1];
        B.keys_unsorted = s->d_keys_unsorted;
        B.keys1 = s->d_keys1;
        B.vals1 = s->d_vals1;
        B.keys_sorted = s->d_keys_sorted;
        B.vals_sorted = s->d_vals_sorted;
        B.tris = s->d_tris;
        B.nodes = s->d_nodes;
        B.hdr = s->d_hdr;
        uint32_t* base = b->d_scratch + b->scratch_at[k];
        B.bounds = base;
        B.hist = base + 8;
        B.lookback = base + 8 + 1024;
        B.emit = reinterpret_cast<uint8_t*>(s->d_scratch) + rt::lbvh_emit_offset(s->N);
    }
    return t;
}

// Render descriptors for the scenes' current (sorted) order.
std::vector<rt::BatchView> view_table(rt_batch* b) {
    std::vector<rt::BatchView> t(b->views.size());
    for (size_t v = 0; v < b->views.size(); ++v) {
        const rt_batch_view& bv = b->views[v];
        rt::BatchView& V = t[v];
        V.scene = rt::scene_view(bv.scene);
        V.lights = b->d_lights + b->view_scene[v];
        V.cam = bv.cam;
        V.width = bv.width;
        V.height = bv.height;
        V.max_bounces = bv.max_bounces;
        V.rgba_offset = bv.rgba_offset;
    }
    return t;
}

int32_t upload_tables(rt_ctx* c, rt_batch* b, cudaStream_t cs) {
    std::vector<rt::BatchScene> st = scene_table(b);
    CU(cudaMemcpyAsync(b->d_scenes, st.data(), sizeof(rt::BatchScene) * st.size(),
                       cudaMemcpyHostToDevice, cs));
    std::vector<rt::BatchView> vt = view_table(b);
    CU(cudaMemcpyAsync(b->d_views, vt.data(), sizeof(rt::BatchView) * vt.size(),
                       cudaMemcpyHostToDevice, cs));
    CU(cudaStreamSynchronize(cs));   // host staging vectors go out of scope
    (void)c;
    return RT_OK;
}

rt::BatchBuildArgs build_args(rt_ctx* c, rt_batch* b) {
    rt::BatchBuildArgs a;
    a.scenes = b->d_scenes;
    a.count = (int)b->scenes.size();
    a.passes = (b->depth + 7) / 8;
    a.tri_off = b->d_tri_off;
    a.tile_off = b->d_tile_off;
    a.tile_ctr = b->d_ctr;
    a.status = c->d_status;
    a.stage_ns = b->profile ? b->d_stage : nullptr;
    a.emit_off = b->d_emit_off;
    a.emit_levels = b->emit_levels;
    for (int L = 0; L < rt::kMaxEmitLevels; ++L) a.emit_jobs[L] = b->emit_jobs[L];
    return a;
}

rt::BatchRenderArgs render_args(rt_ctx* c, rt_batch* b, uint8_t* rgba, rt_render_stats* stats) {
    rt::BatchRenderArgs a;
    a.views = b->d_views;
    a.count = (int)b->views.size();
    a.pix_off = b->d_pix_off;
    a.rgba = rgba;
    a.stats = stats;
    a.work_counter = b->d_ctr + 4;
    a.status = c->d_status;
    a.chunk = b->render_chunk;
    a.inv1e6 = c->inv1e6;
    a.accum = b->d_accum;
    a.total = b->total_pixels;
    return a;
}

}  // namespace

extern "C" {

int32_t rt_batch_create(rt_ctx* c, rt_batch** out) {
    if (!c || !out) return fail(RT_ERR_INVALID, "rt_batch_create: null argument");
    rt_batch* b = new (std::nothrow) rt_batch();
    if (!b) return fail(RT_ERR_OOM, "rt_batch_create: host allocation failed");
    *out = b;
    return RT_OK;
}

int32_t rt_batch_destroy(rt_ctx* c, rt_batch* b) {
    if (!b) return RT_OK;
    if (c) cudaStreamSynchronize(c->stream);
    free_tables(b);
    delete b;
    return RT_OK;
}

int32_t rt_batch_set(rt_ctx* c, rt_batch* b, const rt_batch_view* views, int32_t count,
                     const rt_bvh_cfg* cfg) {
    if (!c || !b || !views) return fail(RT_ERR_INVALID, "rt_batch_set: null argument");
    if (count < 1 || count > rt::kMaxBatchViews)
        return fail(RT_ERR_INVALID, "rt_batch_set: %d views outside [1, %d]", count,
                    rt::kMaxBatchViews);
    int depth = cfg ? cfg->depth : 30, min_leaf = cfg ? cfg->min_leaf_size : 1;
    if (depth < 1 || depth > 32) return fail(RT_ERR_INVALID, "rt_batch_set: bad depth %d", depth);
    min_leaf = std::min(std::max(min_leaf, 1), 256);
    free_tables(b);
    b->views.assign(views, views + count);
    b->scenes.clear();
    b->view_scene.clear();
    b->depth = depth;
    b->min_leaf = min_leaf;
    uint64_t pixels = 0;
    for (int v = 0; v < count; ++v) {
        const rt_batch_view& bv = views[v];
        if (!bv.scene || bv.scene->N == 0)
            return fail(RT_ERR_INVALID, "rt_batch_set: view %d has no uploaded scene", v);
        if (bv.width <= 0 || bv.height <= 0 || bv.max_bounces < 0 || bv.max_bounces > 64)
            return fail(RT_ERR_INVALID, "rt_batch_set: view %d has a bad size or depth", v);
        if (bv.rgba_offset != pixels)
            return fail(RT_ERR_INVALID, "rt_batch_set: view %d rgba_offset %u, expected %llu "
                        "(images are packed in view order)", v, bv.rgba_offset,
                        (unsigned long long)pixels);
        pixels += (uint64_t)bv.width * bv.height;
        auto it = std::find(b->scenes.begin(), b->scenes.end(), bv.scene);
        if (it == b->scenes.end()) {
            b->view_scene.push_back((int)b->scenes.size());
            b->scenes.push_back(bv.scene);
        } else {
            b->view_scene.push_back((int)(it - b->scenes.begin()));
        }
    }
    if (pixels >= (1ull << 32)) return fail(RT_ERR_INVALID, "rt_batch_set: too many pixels");
    if ((int)b->scenes.size() > rt::batch_max_scenes())
        return fail(RT_ERR_INVALID, "rt_batch_set: more than %d scenes", rt::batch_max_scenes());
    const int passes = (depth + 7) / 8;
    const uint32_t tile = (uint32_t)rt::sort_tile_size();
    std::vector<uint32_t> toff(1, 0), tloff(1, 0);
    b->scratch_at.clear();
    size_t words = 0;
    uint64_t tris = 0, tiles = 0;
    for (rt_scene* s : b->scenes) {
        int32_t r = rt::scene_ensure_build(s);
        if (r) return r;
        const uint32_t nt = (s->N + tile - 1) / tile;
        tris += s->N;
        tiles += nt;
        toff.push_back((uint32_t)tris);
        tloff.push_back((uint32_t)tiles);
        b->scratch_at.push_back(words);
        words += 8 + 1024 + (size_t)passes * nt * 256;
    }
    if (tris >= (1ull << 31)) return fail(RT_ERR_INVALID, "rt_batch_set: too many triangles");
    b->total_tris = (uint32_t)tris;
    b->total_tiles = (uint32_t)tiles;
    b->total_pixels = (uint32_t)pixels;
    b->scratch_words = words;
    // the emit's blocks per scene and level, as the one-scene build runs them
    const size_t ns_ = b->scenes.size();
    std::vector<uint32_t> eoff;
    std::vector<uint32_t> below(ns_, 0);   // blocks of the level below (0: done)
    b->emit_levels = 0;
    for (int L = 0; L < rt::kMaxEmitLevels; ++L) {
        uint32_t acc = 0;
        bool any = false;
        for (size_t k = 0; k < ns_; ++k) {
            eoff.push_back(acc);
            uint32_t nb;
            if (L == 0)
                nb = rt::emit_blocks0(b->scenes[k]->N);
            else
                nb = below[k] > 1 ? rt::emit_next_level(below[k]) : 0u;
            below[k] = nb;
            acc += nb;
            any = any || nb > 0;
        }
        eoff.push_back(acc);
        if (!any) {
            eoff.resize(eoff.size() - (ns_ + 1));
            break;
        }
        b->emit_jobs[L] = acc;
        b->emit_levels = L + 1;
    }
    std::vector<uint32_t> poff(1, 0);
    for (const rt_batch_view& bv : b->views) poff.push_back(poff.back() + bv.width * bv.height);
    std::vector<rt_lights> lights;
    for (rt_scene* s : b->scenes) lights.push_back(s->lights);
    const size_t ns = b->scenes.size();
    if (cudaMalloc(&b->d_scenes, sizeof(rt::BatchScene) * ns) ||
        cudaMalloc(&b->d_tri_off, 4 * (ns + 1)) || cudaMalloc(&b->d_tile_off, 4 * (ns + 1)) ||
        cudaMalloc(&b->d_ctr, 4 * 8) || cudaMalloc(&b->d_scratch, 4 * words) ||
        cudaMalloc(&b->d_views, sizeof(rt::BatchView) * count) ||
        cudaMalloc(&b->d_pix_off, 4 * (count + 1)) ||
        cudaMalloc(&b->d_accum, 3 * sizeof(uint32_t) * std::max<size_t>(1, poff.back())) ||
        cudaMalloc(&b->d_lights, sizeof(rt_lights) * ns) ||
        cudaMalloc(&b->d_stage, sizeof(unsigned long long) * 8) ||
        cudaMalloc(&b->d_emit_off, 4 * std::max<size_t>(1, eoff.size()))) {
        cudaGetLastError();
        free_tables(b);
        return fail(RT_ERR_OOM, "rt_batch_set: device allocation failed");
    }
    cudaStream_t cs = c->stream;
    CU(cudaMemcpyAsync(b->d_tri_off, toff.data(), 4 * toff.size(), cudaMemcpyHostToDevice, cs));
    CU(cudaMemcpyAsync(b->d_tile_off, tloff.data(), 4 * tloff.size(), cudaMemcpyHostToDevice, cs));
    CU(cudaMemcpyAsync(b->d_pix_off, poff.data(), 4 * poff.size(), cudaMemcpyHostToDevice, cs));
    CU(cudaMemcpyAsync(b->d_emit_off, eoff.data(), 4 * eoff.size(), cudaMemcpyHostToDevice, cs));
    CU(cudaMemcpyAsync(b->d_lights, lights.data(), sizeof(rt_lights) * ns, cudaMemcpyHostToDevice,
                       cs));
    int32_t r = upload_tables(c, b, cs);
    if (r) return r;
    // one resident wave of the cooperative build kernel
    int bps = 0;
    CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, rt::batch_build_kernel(),
                                                     rt::batch_build_threads(), 0));
    if (bps < 1) return fail(RT_ERR_CUDA, "rt_batch_set: build kernel cannot be resident");
    b->build_grid = bps * c->num_sms;
    // render: the pooled many-view kernel (one large launch keeps its lanes
    // busy by pooling reflection rays across views)
    int threads = 0;
    const void* fn = nullptr;
    b->render_variant = 0;
    bool refracts = false;
    int deepest = 0;
    for (int v = 0; v < count; ++v) {
        refracts = refracts || views[v].scene->refracts;
        deepest = std::max(deepest, (int)views[v].max_bounces);
    }
    if (refracts) {
        // both rays of a glass hit: the pooled kernel whose pool holds the
        // deepest view, else each pixel's ray tree
        b->render_variant = rt::batch_refract_variant(true, deepest);
        if (b->render_variant < 0) b->render_variant = rt::batch_refract_variant(false, deepest);
    } else {
        for (int v = 0; v < rt::batch_render_variant_count(); ++v)
            if (rt::batch_render_variant_pooled(v) && !rt::batch_render_variant_refracts(v)) {
                b->render_variant = v;
                break;
            }
    }
    rt::batch_render_variant_info(b->render_variant, &threads, &fn);
    int rbps = 0;
    CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&rbps, fn, threads, 0));
    b->render_grid = std::max(1, rbps) * c->num_sms;
    b->render_chunk = 32;
    return RT_OK;
}

int32_t rt_batch_build(rt_ctx* c, rt_batch* b, rt_stream stream) {
    if (!c || !b || b->scenes.empty()) return fail(RT_ERR_INVALID, "rt_batch_build: empty batch");
    cudaStream_t cs = stream ? (cudaStream_t)stream : c->stream;
    int32_t r = upload_tables(c, b, cs);
    if (r) return r;
    CU(rt::launch_batch_build(build_args(c, b), b->build_grid, cs));
    for (rt_scene* s : b->scenes) {
        s->cur ^= 1;
        s->built = true;
        s->depth = b->depth;
        s->min_leaf = b->min_leaf;
    }
    return upload_tables(c, b, cs);   // the render reads the sorted order
}

int32_t rt_batch_render(rt_ctx* c, rt_batch* b, uint8_t* d_rgba, rt_render_stats* d_stats,
                        rt_stream stream) {
    if (!c || !b || !d_rgba || b->views.empty())
        return fail(RT_ERR_INVALID, "rt_batch_render: null argument or empty batch");
    for (rt_scene* s : b->scenes)
        if (!s->built) return fail(RT_ERR_NOT_BUILT, "rt_batch_render: a scene has no BVH");
    cudaStream_t cs = stream ? (cudaStream_t)stream : c->stream;
    CU(cudaMemsetAsync(b->d_ctr + 4, 0, sizeof(uint32_t), cs));
    CU(rt::launch_batch_render(render_args(c, b, d_rgba, d_stats), b->render_variant,
                               b->render_grid, cs));
    return RT_OK;
}

int32_t rt_batch_capture(rt_ctx* c, rt_batch* b, uint8_t* d_rgba, rt_render_stats* d_stats) {
    if (!c || !b || !d_rgba || b->scenes.empty())
        return fail(RT_ERR_INVALID, "rt_batch_capture: null argument or empty batch");
    cudaStream_t cs = c->stream;
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
    // the graph reads each scene's current order and writes the other buffer;
    // every replay rebuilds from the order the capture saw
    int32_t r = upload_tables(c, b, cs);
    if (r) return r;
    for (rt_scene* s : b->scenes) s->cur ^= 1;
    std::vector<rt::BatchView> vt = view_table(b);   // views of the sorted order
    CU(cudaMemcpyAsync(b->d_views, vt.data(), sizeof(rt::BatchView) * vt.size(),
                       cudaMemcpyHostToDevice, cs));
    CU(cudaStreamSynchronize(cs));
    CU(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = rt::launch_batch_build(build_args(c, b), b->build_grid, cs);
    if (e == cudaSuccess && d_stats) e = cudaMemsetAsync(d_stats, 0, sizeof(rt_render_stats), cs);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->d_ctr + 4, 0, sizeof(uint32_t), cs);
    if (e == cudaSuccess)
        e = rt::launch_batch_render(render_args(c, b, d_rgba, d_stats), b->render_variant,
                                    b->render_grid, cs);
    cudaGraph_t g = nullptr;
    cudaError_t e2 = cudaStreamEndCapture(cs, &g);
    if (e != cudaSuccess || e2 != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        for (rt_scene* s : b->scenes) s->cur ^= 1;
        return fail(RT_ERR_CUDA, "rt_batch_capture: %s",
                    cudaGetErrorString(e != cudaSuccess ? e : e2));
    }
    b->graph = g;
    CU(cudaGraphInstantiate(&b->exec, g, 0));
    for (rt_scene* s : b->scenes) {
        s->built = true;
        s->depth = b->depth;
        s->min_leaf = b->min_leaf;
    }
    return RT_OK;
}

int32_t rt_batch_replay(rt_ctx* c, rt_batch* b, rt_stream stream) {
    if (!c || !b || !b->exec) return fail(RT_ERR_INVALID, "rt_batch_replay: nothing captured");
    CU(cudaGraphLaunch(b->exec, stream ? (cudaStream_t)stream : c->stream));
    return RT_OK;
}

int32_t rt_batch_profile(rt_ctx* c, rt_batch* b, int32_t enable) {
    if (!c || !b) return fail(RT_ERR_INVALID, "rt_batch_profile: null argument");
    b->profile = enable != 0;
    return RT_OK;
}

int32_t rt_batch_stage_times(rt_ctx* c, rt_batch* b, float* ms) {
    if (!c || !b || !ms || !b->d_stage)
        return fail(RT_ERR_INVALID, "rt_batch_stage_times: null argument or batch not set");
    unsigned long long t[8];
    CU(cudaStreamSynchronize(c->stream));
    CU(cudaMemcpy(t, b->d_stage, sizeof(t), cudaMemcpyDeviceToHost));
    for (int k = 0; k < 6; ++k) ms[k] = (float)((double)(t[k + 1] - t[k]) * 1e-6);
    return RT_OK;
}

int32_t rt_batch_info(rt_ctx* c, rt_batch* b, uint32_t* scenes, uint32_t* triangles,
                      uint32_t* pixels) {
    if (!c || !b) return fail(RT_ERR_INVALID, "rt_batch_info: null argument");
    if (scenes) *scenes = (uint32_t)b->scenes.size();
    if (triangles) *triangles = b->total_tris;
    if (pixels) *pixels = b->total_pixels;
    return RT_OK;
}

}  // extern "C"
