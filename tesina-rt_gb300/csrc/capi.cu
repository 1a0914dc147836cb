// capi.cu — the extern "C" boundary of librt_cuda.so (include/rt_cuda.h).
//
// Replaces the reference's DeviceInterface / DeviceMemory handle tables
// (include/gpu/interface.hpp:20-80, src/gpu/memory.cpp) with plain device
// pointers owned by a context, and its Scene / BVHBuilder / Tracer /
// RayShader / SecondaryRayGenerator / FrameBuffer methods with the entry
// points below.  Every entry point returns 0 or a negative rt_status and never
// throws; rt_last_error() holds the message of the last failure on the
// calling thread.  There is no CPU fallback: without a CUDA device every
// compute entry point fails with RT_ERR_CUDA.
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <new>
#include <thread>
#include <vector>

#include "../../include/rt_cuda.h"
#include "lbvh.cuh"
#include "sah.cuh"
#include "rt_internal.cuh"
#include "trace.cuh"
#include "ctx_internal.h"

namespace {
thread_local char g_err[512] = "";
}  // namespace

namespace rt {
int32_t set_error(int32_t code, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return code;
}
}  // namespace rt

namespace {

#define fail rt::set_error

#define CU(call)                                                                              \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess)                                                                \
            return fail(RT_ERR_CUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_),  \
                        __FILE__, __LINE__);                                                  \
    } while (0)

template <class T>
void dfree(T*& p) {
    if (p) cudaFree(p);
    p = nullptr;
}

// Scene buffers: cudaMalloc/cudaFree, or, for a scene given a memory pool,
// stream-ordered allocation from the pool on the scene's pool stream (a
// free returns memory to the pool without synchronising the device).
template <class T>
cudaError_t salloc(rt_scene* s, T** p, size_t bytes) {
    if (bytes == 0) bytes = 1;
    if (s->pool)
        return cudaMallocFromPoolAsync(reinterpret_cast<void**>(p), bytes, s->pool, s->pool_stream);
    return cudaMalloc(reinterpret_cast<void**>(p), bytes);
}

template <class T>
cudaError_t salloc_n(rt_scene* s, T** p, size_t count) {
    return salloc(s, p, sizeof(T) * (count ? count : 1));
}

template <class T>
void sfree(rt_scene* s, T*& p) {
    if (p) {
        if (s->pool)
            cudaFreeAsync(p, s->pool_stream);
        else
            cudaFree(p);
    }
    p = nullptr;
}

}  // namespace


namespace {

void free_build(rt_scene* s) {
    sfree(s, s->d_keys_unsorted);
    sfree(s, s->d_vals0);
    sfree(s, s->d_keys1);
    sfree(s, s->d_vals1);
    sfree(s, s->d_keys_sorted);
    sfree(s, s->d_vals_sorted);
    sfree(s, s->d_tris);
    sfree(s, s->d_leafbox);
    sfree(s, s->d_nodes);
    sfree(s, s->d_hdr);
    sfree(s, s->d_scratch);
    s->buildN = 0;
    s->scratch_bytes = 0;
}

void free_geometry(rt_scene* s) {
    sfree(s, s->d_pos);
    sfree(s, s->d_nrm);
    for (int i = 0; i < 2; ++i) {
        sfree(s, s->d_idx[i]);
        sfree(s, s->d_map[i]);
        sfree(s, s->d_orig[i]);
    }
    sfree(s, s->d_mats);
    s->capV = s->capN = s->capM = 0;
}

int32_t check_lights(const rt_lights* L) {
    if (L->count < 1 || L->count > RT_MAX_LIGHTS)
        return fail(RT_ERR_INVALID, "light count %d outside [1, %d]", L->count, RT_MAX_LIGHTS);
    for (int i = 0; i < L->count; ++i) {
        const int t = L->light[i].type;
        if (t != RT_SPOT_L && t != RT_DIR_L && t != RT_POINT_L)
            return fail(RT_ERR_INVALID, "light %d has unknown type %d", i, t);
    }
    return RT_OK;
}

cudaStream_t st(rt_ctx* c, rt_stream s) { return s ? (cudaStream_t)s : c->stream; }

}  // namespace

namespace rt {

// Calls on one scene behave as on one in-order queue, whatever streams they
// name (the reference runs every call on one command queue): a call that
// writes the scene (upload, vertex update, build, refit) waits on the device
// for every earlier call on other streams, a call that reads it (trace,
// shade, render, ...) for the last writing call, and host reads of the scene
// for its last writing call.  Reading calls on several streams may overlap.
static cudaError_t order_event(cudaEvent_t* e) {
    return *e ? cudaSuccess : cudaEventCreateWithFlags(e, cudaEventDisableTiming);
}

cudaError_t scene_write_begin(rt_scene* s, cudaStream_t cs) {
    if (s->write_recorded && s->write_stream != cs) {
        const cudaError_t e = cudaStreamWaitEvent(cs, s->ev_write, 0);
        if (e != cudaSuccess) return e;
    }
    for (int i = 0; i < s->n_readers; ++i)
        if (s->readers[i].stream != cs) {
            const cudaError_t e = cudaStreamWaitEvent(cs, s->readers[i].ev, 0);
            if (e != cudaSuccess) return e;
        }
    s->n_readers = 0;
    return cudaSuccess;
}

cudaError_t scene_write_end(rt_scene* s, cudaStream_t cs) {
    cudaError_t e = order_event(&s->ev_write);
    if (e == cudaSuccess) e = cudaEventRecord(s->ev_write, cs);
    if (e != cudaSuccess) return e;
    s->write_stream = cs;
    s->write_recorded = true;
    return cudaSuccess;
}

cudaError_t scene_read_begin(rt_scene* s, cudaStream_t cs) {
    if (s->write_recorded && s->write_stream != cs) return cudaStreamWaitEvent(cs, s->ev_write, 0);
    return cudaSuccess;
}

cudaError_t scene_read_end(rt_scene* s, cudaStream_t cs) {
    int k = 0;
    while (k < s->n_readers && s->readers[k].stream != cs) ++k;
    if (k == s->n_readers) {
        if (k < 4) {
            s->readers[k].stream = cs;
            s->n_readers = k + 1;
        } else {   // the last slot: cs takes over the work it covered
            k = 3;
            const cudaError_t e = cudaStreamWaitEvent(cs, s->readers[k].ev, 0);
            if (e != cudaSuccess) return e;
            s->readers[k].stream = cs;
        }
    }
    const cudaError_t e = order_event(&s->readers[k].ev);
    return e == cudaSuccess ? cudaEventRecord(s->readers[k].ev, cs) : e;
}

// Host side: waits for every call on the scene (reads too, when `all`).
cudaError_t scene_host_wait(rt_scene* s, bool all) {
    if (s->write_recorded) {
        const cudaError_t e = cudaEventSynchronize(s->ev_write);
        if (e != cudaSuccess) return e;
    }
    for (int i = 0; all && i < s->n_readers; ++i) {
        const cudaError_t e = cudaEventSynchronize(s->readers[i].ev);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

}  // namespace rt

using rt::scene_write_begin;
using rt::scene_write_end;
using rt::scene_read_begin;
using rt::scene_read_end;
using rt::scene_host_wait;

namespace {

static void destroy_order_events(rt_scene* s) {
    if (s->ev_write) cudaEventDestroy(s->ev_write);
    for (auto& r : s->readers)
        if (r.ev) cudaEventDestroy(r.ev);
}

}  // namespace

namespace rt {
int32_t scene_ensure_build(rt_scene* s) {
    const uint32_t n = s->N;
    const size_t need_scratch = rt::lbvh_scratch_bytes(n, 4);
    if (s->buildN >= n && s->scratch_bytes >= need_scratch && s->d_hdr) return RT_OK;
    free_build(s);
    const size_t nn = n > 1 ? n - 1 : 1;
    if (salloc_n(s, &s->d_keys_unsorted, n) || salloc_n(s, &s->d_vals0, n) ||
        salloc_n(s, &s->d_keys1, n) || salloc_n(s, &s->d_vals1, n) ||
        salloc_n(s, &s->d_keys_sorted, n) || salloc_n(s, &s->d_vals_sorted, n) ||
        salloc_n(s, &s->d_tris, 3 * (size_t)n) || salloc_n(s, &s->d_leafbox, 2 * (size_t)n) ||
        salloc_n(s, &s->d_nodes, 4 * nn) || salloc_n(s, &s->d_hdr, 1) || salloc(s, &s->d_scratch, need_scratch)) {
        cudaGetLastError();
        free_build(s);
        return fail(RT_ERR_OOM, "device allocation of LBVH buffers for %u triangles failed", n);
    }
    s->buildN = n;
    s->scratch_bytes = need_scratch;
    return RT_OK;
}

SceneView scene_view(const rt_scene* s) {
    rt::SceneView v;
    v.nodes = s->d_nodes;
    v.tris = s->d_tris;
    v.idx = s->d_idx[s->cur];
    v.nrm = s->d_nrm;
    v.map = s->d_map[s->cur];
    v.mats = s->d_mats;
    v.hdr = s->d_hdr;
    return v;
}

void scene_use_pool(rt_scene* s, cudaMemPool_t pool, cudaStream_t stream) {
    s->pool = pool;
    s->pool_stream = stream;
}

uint32_t* work_counter(rt_ctx* c, cudaStream_t s) {
    if (!s || s == c->stream) return c->d_work;
    std::lock_guard<std::mutex> lk(c->work_mu);
    auto it = c->work_by_stream.find(s);
    if (it != c->work_by_stream.end()) return it->second;
    uint32_t* p = nullptr;
    if (cudaMalloc(&p, 64 * sizeof(uint32_t)) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    c->work_by_stream[s] = p;
    return p;
}

// Frees the rt_render_host state of one stream (its side stream finished).
static void free_host_render(rt_ctx::HostRender& R) {
    if (R.side) {
        cudaStreamSynchronize(R.side);
        cudaStreamDestroy(R.side);
    }
    if (R.fork) cudaEventDestroy(R.fork);
    if (R.join) cudaEventDestroy(R.join);
    if (R.d_out) cudaFree(R.d_out);
    if (R.d_stats) cudaFree(R.d_stats);
    if (R.h_stage) cudaFreeHost(R.h_stage);
    R = rt_ctx::HostRender{};
}

void release_work_counter(rt_ctx* c, cudaStream_t s) {
    std::lock_guard<std::mutex> lk(c->work_mu);
    auto it = c->work_by_stream.find(s);
    if (it != c->work_by_stream.end()) {
        cudaFree(it->second);
        c->work_by_stream.erase(it);
    }
    auto ih = c->host_by_stream.find(s);
    if (ih != c->host_by_stream.end()) {
        cudaStreamSynchronize(s);
        free_host_render(ih->second);
        c->host_by_stream.erase(ih);
    }
    for (auto* m : {&c->accum_by_stream, &c->sec_by_stream}) {
        auto ia = m->find(s);
        if (ia != m->end()) {
            if (ia->second.first) cudaFreeAsync(ia->second.first, s);
            m->erase(ia);
        }
    }
}

// The buffer of stream s in `m`, at least `size` units of `unit` bytes.
static uint32_t* stream_buffer(rt_ctx* c, std::map<cudaStream_t, std::pair<uint32_t*, size_t>>& m,
                               cudaStream_t s, size_t size, size_t unit) {
    std::lock_guard<std::mutex> lk(c->work_mu);
    auto& e = m[s];
    if (e.first && e.second >= size) return e.first;
    if (e.first) cudaFreeAsync(e.first, s);
    e = {nullptr, 0};
    uint32_t* p = nullptr;
    if (cudaMallocAsync(reinterpret_cast<void**>(&p), unit * (size ? size : 1), s) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    e = {p, size};
    return p;
}

uint32_t* accum_buffer(rt_ctx* c, cudaStream_t s, size_t pixels) {
    return stream_buffer(c, c->accum_by_stream, s, pixels, 3 * sizeof(uint32_t));
}

uint32_t* sec_scratch(rt_ctx* c, cudaStream_t s, size_t bytes) {
    return stream_buffer(c, c->sec_by_stream, s, bytes, 1);
}

}  // namespace rt

static inline rt::SceneView view_of(const rt_scene* s) { return rt::scene_view(s); }

extern "C" {

const char* rt_last_error(void) { return g_err; }

int32_t rt_camera_set(rt_camera* cam, const float pos[3], const float dir[3], const float up[3],
                      float fov, float aspect, int32_t right_handed) {
    if (!cam || !pos || !dir || !up) return fail(RT_ERR_INVALID, "rt_camera_set: null argument");
    float dn = std::sqrt(dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2]);
    if (!(dn > 0.f)) return fail(RT_ERR_INVALID, "rt_camera_set: zero direction");
    float d[3] = {dir[0] / dn, dir[1] / dn, dir[2] / dn};
    auto cross = [](const float* a, const float* b, float* o) {
        o[0] = a[1] * b[2] - a[2] * b[1];
        o[1] = a[2] * b[0] - a[0] * b[2];
        o[2] = a[0] * b[1] - a[1] * b[0];
    };
    float r[3], u[3];
    if (right_handed) {
        cross(d, up, r);
        cross(r, d, u);
    } else {
        cross(up, d, r);
        cross(d, r, u);
    }
    const float ph = std::tan(fov * 0.5f);
    const float rn = std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
    const float un = std::sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
    if (!(rn > 0.f) || !(un > 0.f)) return fail(RT_ERR_INVALID, "rt_camera_set: up parallel to dir");
    memset(cam, 0, sizeof(*cam));
    for (int i = 0; i < 3; ++i) {
        cam->pos[i] = pos[i];
        cam->dir[i] = d[i];
        cam->right[i] = r[i] * ((ph * aspect) / rn);
        cam->up[i] = u[i] * (ph / un);
    }
    return RT_OK;
}

int32_t rt_init(rt_ctx** out, int32_t device) {
    if (!out) return fail(RT_ERR_INVALID, "rt_init: null output");
    *out = nullptr;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) {
        cudaGetLastError();
        return fail(RT_ERR_CUDA, "rt_init: no CUDA device (%s)", cudaGetErrorString(e));
    }
    if (device < 0 || device >= count) return fail(RT_ERR_INVALID, "rt_init: bad device %d", device);
    CU(cudaSetDevice(device));
    rt_ctx* c = new (std::nothrow) rt_ctx();
    if (!c) return fail(RT_ERR_OOM, "rt_init: host allocation failed");
    c->device = device;
    cudaDeviceProp prop;
    CU(cudaGetDeviceProperties(&prop, device));
    c->num_sms = prop.multiProcessorCount;
    c->smem_per_sm = (int)prop.sharedMemPerMultiprocessor;
    CU(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    CU(cudaMalloc(&c->d_status, sizeof(uint32_t)));
    CU(cudaMemset(c->d_status, 0, sizeof(uint32_t)));
    CU(cudaMalloc(&c->d_work, 64 * sizeof(uint32_t)));
    for (int v = 0; v < rt::kMaxRenderVariants; ++v) c->variant_carveout[v] = -1;
    for (int v = 0; v < rt::render_variant_count(); ++v) {
        int threads = 0, minb = 0, bps = 0;
        const void* fn = nullptr;
        rt::render_variant_info(v, &threads, &minb, &fn);
        CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, fn, threads, 0));
        c->variant_occupancy[v] = bps > 0 ? bps : 1;
    }
    volatile float one = 1.0f, m = 1e6f;
    c->inv1e6 = one / m;
    *out = c;
    return RT_OK;
}

int32_t rt_shutdown(rt_ctx* c) {
    if (!c) return RT_OK;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    dfree(c->d_status);
    dfree(c->d_work);
    for (auto& kv : c->work_by_stream) dfree(kv.second);
    for (auto* m : {&c->accum_by_stream, &c->sec_by_stream})
        for (auto& kv : *m)
            if (kv.second.first) cudaFree(kv.second.first);
    for (auto& kv : c->host_by_stream) {
        cudaStreamSynchronize(kv.first);
        rt::free_host_render(kv.second);
    }
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return RT_OK;
}

int32_t rt_device_status(rt_ctx* c, uint32_t* bits) {
    if (!c || !bits) return fail(RT_ERR_INVALID, "rt_device_status: null argument");
    CU(cudaStreamSynchronize(c->stream));
    CU(cudaMemcpy(bits, c->d_status, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    CU(cudaMemset(c->d_status, 0, sizeof(uint32_t)));
    return RT_OK;
}

int32_t rt_selftest_wait_timeout(rt_ctx* c, rt_stream stream) {
    if (!c) return fail(RT_ERR_INVALID, "rt_selftest_wait_timeout: null context");
    cudaStream_t cs = stream ? (cudaStream_t)stream : c->stream;
    uint32_t* buf = nullptr;
    CU(cudaMalloc(&buf, sizeof(uint32_t) * rt::wait_probe_words()));
    const cudaError_t e = rt::wait_probe(buf, c->d_status, cs);
    const cudaError_t e2 = cudaStreamSynchronize(cs);
    cudaFree(buf);
    CU(e);
    CU(e2);
    uint32_t bits = 0;
    CU(cudaMemcpy(&bits, c->d_status, sizeof(bits), cudaMemcpyDeviceToHost));
    if (bits & RT_DEV_TIMEOUT)
        return fail(RT_ERR_TIMEOUT, "rt_selftest_wait_timeout: device wait timed out");
    return RT_OK;
}

int32_t rt_stream_create(rt_ctx* c, rt_stream* s) {
    if (!c || !s) return fail(RT_ERR_INVALID, "rt_stream_create: null argument");
    cudaStream_t x;
    CU(cudaStreamCreateWithFlags(&x, cudaStreamNonBlocking));
    *s = (rt_stream)x;
    return RT_OK;
}

int32_t rt_stream_destroy(rt_ctx* c, rt_stream s) {
    if (c && s) rt::release_work_counter(c, (cudaStream_t)s);
    if (s) CU(cudaStreamDestroy((cudaStream_t)s));
    return RT_OK;
}

int32_t rt_stream_sync(rt_ctx* c, rt_stream s) {
    if (!c) return fail(RT_ERR_INVALID, "rt_stream_sync: null context");
    CU(cudaStreamSynchronize(st(c, s)));
    return RT_OK;
}

int32_t rt_buf_alloc(rt_ctx* c, size_t bytes, void** p) {
    if (!c || !p) return fail(RT_ERR_INVALID, "rt_buf_alloc: null argument");
    cudaError_t e = cudaMalloc(p, bytes ? bytes : 1);
    if (e != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        return fail(RT_ERR_OOM, "rt_buf_alloc(%zu): %s", bytes, cudaGetErrorString(e));
    }
    return RT_OK;
}

int32_t rt_buf_free(rt_ctx* c, void* p) {
    (void)c;
    if (p) CU(cudaFree(p));
    return RT_OK;
}

int32_t rt_buf_write(rt_ctx* c, void* d, const void* h, size_t bytes, rt_stream s) {
    if (!c) return fail(RT_ERR_INVALID, "rt_buf_write: null context");
    CU(cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, st(c, s)));
    return RT_OK;
}

int32_t rt_buf_read(rt_ctx* c, void* h, const void* d, size_t bytes, rt_stream s) {
    if (!c) return fail(RT_ERR_INVALID, "rt_buf_read: null context");
    CU(cudaMemcpyAsync(h, d, bytes, cudaMemcpyDeviceToHost, st(c, s)));
    CU(cudaStreamSynchronize(st(c, s)));
    return RT_OK;
}

int32_t rt_buf_copy(rt_ctx* c, void* d, const void* src, size_t bytes, rt_stream s) {
    if (!c) return fail(RT_ERR_INVALID, "rt_buf_copy: null context");
    CU(cudaMemcpyAsync(d, src, bytes, cudaMemcpyDeviceToDevice, st(c, s)));
    return RT_OK;
}

int32_t rt_buf_zero(rt_ctx* c, void* d, size_t bytes, rt_stream s) {
    if (!c) return fail(RT_ERR_INVALID, "rt_buf_zero: null context");
    CU(cudaMemsetAsync(d, 0, bytes, st(c, s)));
    return RT_OK;
}

// ---------------------------------------------------------------------------
// scene
// ---------------------------------------------------------------------------
int32_t rt_scene_create(rt_ctx* c, rt_scene** out) {
    if (!c || !out) return fail(RT_ERR_INVALID, "rt_scene_create: null argument");
    rt_scene* s = new (std::nothrow) rt_scene();
    if (!s) return fail(RT_ERR_OOM, "rt_scene_create: host allocation failed");
    memset(&s->lights, 0, sizeof(s->lights));
    CU(cudaEventCreate(&s->ev0));
    CU(cudaEventCreate(&s->ev1));
    *out = s;
    return RT_OK;
}

int32_t rt_scene_destroy(rt_ctx* c, rt_scene* s) {
    if (!s) return RT_OK;
    // pool-allocated buffers are freed in order on the pool stream instead
    if (c && !s->pool) {
        scene_host_wait(s, true);
        cudaStreamSynchronize(c->stream);
    }
    free_build(s);
    free_geometry(s);
    destroy_order_events(s);
    if (s->ev0) cudaEventDestroy(s->ev0);
    if (s->ev1) cudaEventDestroy(s->ev1);
    delete s;
    return RT_OK;
}

int32_t rt_scene_upload(rt_ctx* c, rt_scene* s, const rt_scene_desc* d, rt_stream stream) {
    if (!c || !s || !d) return fail(RT_ERR_INVALID, "rt_scene_upload: null argument");
    if (!d->h_vertices || !d->h_indices || !d->h_materials || !d->h_material_map)
        return fail(RT_ERR_INVALID, "rt_scene_upload: missing vertex, index or material data");
    if (d->triangle_count == 0 || d->vertex_count == 0 || d->material_count == 0)
        return fail(RT_ERR_INVALID, "rt_scene_upload: empty scene (%u tris, %u verts, %u mats)",
                    d->triangle_count, d->vertex_count, d->material_count);
    if (d->triangle_count >= (1u << 30))
        return fail(RT_ERR_INVALID, "rt_scene_upload: %u triangles exceed 2^30", d->triangle_count);
    if (d->vertex_stride < 12 || (!d->h_normals && d->vertex_stride < d->normal_offset + 12))
        return fail(RT_ERR_INVALID, "rt_scene_upload: bad vertex stride %u", d->vertex_stride);
    int32_t r = check_lights(&d->lights);
    if (r) return r;
    const uint32_t V = d->vertex_count, N = d->triangle_count, M = d->material_count;
    for (size_t i = 0; i < 3 * (size_t)N; ++i)
        if (d->h_indices[i] >= V)
            return fail(RT_ERR_INVALID, "rt_scene_upload: index %u of triangle %zu >= %u vertices",
                        d->h_indices[i], i / 3, V);
    for (uint32_t i = 0; i < N; ++i)
        if (d->h_material_map[i] >= M)
            return fail(RT_ERR_INVALID, "rt_scene_upload: material %u of triangle %u >= %u",
                        d->h_material_map[i], i, M);
    for (uint32_t i = 0; i < M; ++i) {
        if (d->h_materials[i].texture >= 0)
            return fail(RT_ERR_INVALID, "rt_scene_upload: material %u is textured (unsupported)", i);
    }
    CU(cudaSetDevice(c->device));
    cudaStream_t cs = st(c, stream);
    CU(scene_write_begin(s, cs));
    CU(cudaStreamSynchronize(cs));
    if (s->capV < V || s->capN < N || s->capM < M) {
        free_geometry(s);
        if (salloc_n(s, &s->d_pos, V) || salloc_n(s, &s->d_nrm, V) ||
            salloc_n(s, &s->d_idx[0], 3 * (size_t)N) || salloc_n(s, &s->d_idx[1], 3 * (size_t)N) ||
            salloc_n(s, &s->d_map[0], N) || salloc_n(s, &s->d_map[1], N) ||
            salloc_n(s, &s->d_orig[0], N) || salloc_n(s, &s->d_orig[1], N) ||
            salloc_n(s, &s->d_mats, M)) {
            cudaGetLastError();
            free_geometry(s);
            return fail(RT_ERR_OOM, "rt_scene_upload: device allocation failed");
        }
        s->capV = V;
        s->capN = N;
        s->capM = M;
    }
    s->V = V;
    s->N = N;
    s->M = M;
    s->cur = 0;
    const char* vb = (const char*)d->h_vertices;
    if (d->vertex_stride == 16 && d->position_offset == 0) {
        CU(cudaMemcpyAsync(s->d_pos, vb, 16 * (size_t)V, cudaMemcpyHostToDevice, cs));
    } else {
        std::vector<float> tmp(4 * (size_t)V, 0.f);
        for (size_t i = 0; i < V; ++i)
            memcpy(&tmp[4 * i], vb + i * d->vertex_stride + d->position_offset, 12);
        CU(cudaMemcpyAsync(s->d_pos, tmp.data(), 16 * (size_t)V, cudaMemcpyHostToDevice, cs));
        CU(cudaStreamSynchronize(cs));
    }
    if (d->h_normals) {
        CU(cudaMemcpyAsync(s->d_nrm, d->h_normals, 16 * (size_t)V, cudaMemcpyHostToDevice, cs));
    } else {
        std::vector<float> tmp(4 * (size_t)V, 0.f);
        for (size_t i = 0; i < V; ++i)
            memcpy(&tmp[4 * i], vb + i * d->vertex_stride + d->normal_offset, 12);
        CU(cudaMemcpyAsync(s->d_nrm, tmp.data(), 16 * (size_t)V, cudaMemcpyHostToDevice, cs));
        CU(cudaStreamSynchronize(cs));
    }
    CU(cudaMemcpyAsync(s->d_idx[0], d->h_indices, 12 * (size_t)N, cudaMemcpyHostToDevice, cs));
    CU(cudaMemcpyAsync(s->d_map[0], d->h_material_map, 4 * (size_t)N, cudaMemcpyHostToDevice, cs));
    CU(cudaMemcpyAsync(s->d_mats, d->h_materials, sizeof(rt_material) * M, cudaMemcpyHostToDevice,
                       cs));
    {
        std::vector<uint32_t> iota(N);
        for (uint32_t i = 0; i < N; ++i) iota[i] = i;
        CU(cudaMemcpyAsync(s->d_orig[0], iota.data(), 4 * (size_t)N, cudaMemcpyHostToDevice, cs));
        CU(cudaStreamSynchronize(cs));
    }
    s->lights = d->lights;
    s->built = false;
    s->refracts = false;
    for (uint32_t i = 0; i < M; ++i) s->refracts = s->refracts || d->h_materials[i].refractive_index > 0.f;
    CU(scene_write_end(s, cs));
    return RT_OK;
}

int32_t rt_scene_update_vertices(rt_ctx* c, rt_scene* s, const float* pos4, const float* nrm4,
                                 uint32_t V, rt_stream stream) {
    if (!c || !s || !pos4) return fail(RT_ERR_INVALID, "rt_scene_update_vertices: null argument");
    if (V != s->V) return fail(RT_ERR_INVALID, "vertex count %u != scene's %u", V, s->V);
    cudaStream_t cs = st(c, stream);
    CU(scene_write_begin(s, cs));
    CU(cudaMemcpyAsync(s->d_pos, pos4, 16 * (size_t)V, cudaMemcpyHostToDevice, cs));
    if (nrm4) CU(cudaMemcpyAsync(s->d_nrm, nrm4, 16 * (size_t)V, cudaMemcpyHostToDevice, cs));
    CU(scene_write_end(s, cs));
    return RT_OK;
}

int32_t rt_scene_update_vertices_device(rt_ctx* c, rt_scene* s, const float* pos4,
                                        const float* nrm4, uint32_t V, rt_stream stream) {
    if (!c || !s || !pos4) return fail(RT_ERR_INVALID, "rt_scene_update_vertices: null argument");
    if (V != s->V) return fail(RT_ERR_INVALID, "vertex count %u != scene's %u", V, s->V);
    cudaStream_t cs = st(c, stream);
    CU(scene_write_begin(s, cs));
    CU(cudaMemcpyAsync(s->d_pos, pos4, 16 * (size_t)V, cudaMemcpyDeviceToDevice, cs));
    if (nrm4) CU(cudaMemcpyAsync(s->d_nrm, nrm4, 16 * (size_t)V, cudaMemcpyDeviceToDevice, cs));
    CU(scene_write_end(s, cs));
    return RT_OK;
}

int32_t rt_scene_mangle(rt_ctx* c, rt_scene* s, float arg, float last_arg, float height,
                        rt_stream stream) {
    (void)last_arg;
    if (!c || !s) return fail(RT_ERR_INVALID, "rt_scene_mangle: null argument");
    if (s->V == 0) return fail(RT_ERR_INVALID, "rt_scene_mangle: scene has no vertices");
    cudaStream_t cs = st(c, stream);
    CU(scene_write_begin(s, cs));
    CU(rt::launch_mangle(s->d_pos, s->d_nrm, s->V, arg, height, cs));
    CU(scene_write_end(s, cs));
    return RT_OK;
}

int32_t rt_scene_set_lights(rt_ctx* c, rt_scene* s, const rt_lights* L) {
    if (!c || !s || !L) return fail(RT_ERR_INVALID, "rt_scene_set_lights: null argument");
    int32_t r = check_lights(L);
    if (r) return r;
    s->lights = *L;
    return RT_OK;
}

int32_t rt_scene_buffers(rt_ctx* c, rt_scene* s, uint32_t** idx, uint32_t** map, float** pos,
                         float** nrm, uint32_t* n) {
    if (!c || !s) return fail(RT_ERR_INVALID, "rt_scene_buffers: null argument");
    if (idx) *idx = s->d_idx[s->cur];
    if (map) *map = s->d_map[s->cur];
    if (pos) *pos = reinterpret_cast<float*>(s->d_pos);
    if (nrm) *nrm = reinterpret_cast<float*>(s->d_nrm);
    if (n) *n = s->N;
    return RT_OK;
}

int32_t rt_scene_read_sort(rt_ctx* c, rt_scene* s, uint32_t* keys, uint32_t* perm,
                           uint32_t* sorted) {
    if (!c || !s) return fail(RT_ERR_INVALID, "rt_scene_read_sort: null argument");
    if (!s->built) return fail(RT_ERR_NOT_BUILT, "rt_scene_read_sort: no BVH built");
    CU(scene_host_wait(s, false));
    CU(cudaStreamSynchronize(c->stream));
    const size_t b = 4 * (size_t)s->N;
    if (keys) CU(cudaMemcpy(keys, s->d_keys_unsorted, b, cudaMemcpyDeviceToHost));
    if (perm) CU(cudaMemcpy(perm, s->d_vals_sorted, b, cudaMemcpyDeviceToHost));
    if (sorted) CU(cudaMemcpy(sorted, s->d_keys_sorted, b, cudaMemcpyDeviceToHost));
    return RT_OK;
}

int32_t rt_scene_read_orig(rt_ctx* c, rt_scene* s, uint32_t* orig) {
    if (!c || !s || !orig) return fail(RT_ERR_INVALID, "rt_scene_read_orig: null argument");
    CU(scene_host_wait(s, false));
    CU(cudaStreamSynchronize(c->stream));
    CU(cudaMemcpy(orig, s->d_orig[s->cur], 4 * (size_t)s->N, cudaMemcpyDeviceToHost));
    return RT_OK;
}

// ---------------------------------------------------------------------------
// LBVH
// ---------------------------------------------------------------------------
static rt::LbvhArgs lbvh_args(rt_ctx* c, rt_scene* s) {
    rt::LbvhArgs a;
    a.n = s->N;
    a.depth = s->depth;
    a.min_leaf = s->min_leaf;
    a.num_sms = c->num_sms;
    a.pos = s->d_pos;
    a.idx_in = s->d_idx[s->cur];
    a.map_in = s->d_map[s->cur];
    a.orig_in = s->d_orig[s->cur];
    a.idx_out = s->d_idx[s->cur ^ 1];
    a.map_out = s->d_map[s->cur ^ 1];
    a.orig_out = s->d_orig[s->cur ^ 1];
    a.keys_unsorted = s->d_keys_unsorted;
    a.vals0 = s->d_vals0;
    a.keys1 = s->d_keys1;
    a.vals1 = s->d_vals1;
    a.keys_sorted = s->d_keys_sorted;
    a.vals_sorted = s->d_vals_sorted;
    a.tris = s->d_tris;
    a.leafbox = s->d_leafbox;
    a.nodes = s->d_nodes;
    a.hdr = s->d_hdr;
    a.scratch = s->d_scratch;
    a.status = c->d_status;
    return a;
}

int32_t rt_bvh_build_lbvh(rt_ctx* c, rt_scene* s, const rt_bvh_cfg* cfg, rt_stream stream) {
    if (!c || !s) return fail(RT_ERR_INVALID, "rt_bvh_build_lbvh: null argument");
    if (s->N == 0) return fail(RT_ERR_INVALID, "rt_bvh_build_lbvh: scene has no triangles");
    int depth = cfg ? cfg->depth : 30, min_leaf = cfg ? cfg->min_leaf_size : 1;
    if (depth > 32) return fail(RT_ERR_INVALID, "bvh depth %d > 32 is not supported", depth);
    if (depth < 1) depth = 1;
    if (min_leaf < 1) min_leaf = 1;
    if (min_leaf > 256) min_leaf = 256;
    s->depth = depth;
    s->min_leaf = min_leaf;
    int32_t r = rt::scene_ensure_build(s);
    if (r) return r;
    cudaStream_t cs = st(c, stream);
    CU(scene_write_begin(s, cs));
    CU(cudaEventRecord(s->ev0, cs));
    rt::LbvhArgs a = lbvh_args(c, s);
    CU(rt::lbvh_build(a, cs));
    CU(cudaEventRecord(s->ev1, cs));
    CU(scene_write_end(s, cs));
    s->cur ^= 1;   // the sorted index buffer / material map are now current
    s->built = true;
    s->sah = false;
    return RT_OK;
}

int32_t rt_bvh_build_sah(rt_ctx* c, rt_scene* s, rt_stream stream) {
    if (!c || !s) return fail(RT_ERR_INVALID, "rt_bvh_build_sah: null argument");
    if (s->N == 0) return fail(RT_ERR_INVALID, "rt_bvh_build_sah: scene has no triangles");
    int32_t r = rt::scene_ensure_build(s);
    if (r) return r;
    cudaStream_t cs = st(c, stream);
    CU(scene_write_begin(s, cs));
    CU(cudaEventRecord(s->ev0, cs));
    // the reference builds this tree on the host from its own copy of the mesh
    std::vector<float4> pos(s->V);
    std::vector<uint32_t> idx(3 * (size_t)s->N);
    CU(cudaMemcpyAsync(pos.data(), s->d_pos, sizeof(float4) * s->V, cudaMemcpyDeviceToHost, cs));
    CU(cudaMemcpyAsync(idx.data(), s->d_idx[s->cur], 12 * (size_t)s->N, cudaMemcpyDeviceToHost,
                       cs));
    CU(cudaStreamSynchronize(cs));
    rt::SahTree t;
    const unsigned hw = std::thread::hardware_concurrency();
    const int rc = rt::sah_build(pos.data(), s->V, idx.data(), s->N,
                                 hw ? (int)std::min(hw, 64u) : 1, &t);
    if (rc == -2)
        return fail(RT_ERR_INVALID, "rt_bvh_build_sah: the tree is deeper than the traversal's "
                    "32-entry stack");
    if (rc) return fail(RT_ERR_INVALID, "rt_bvh_build_sah: vertex index out of range");
    rt::LbvhArgs a = lbvh_args(c, s);
    CU(cudaMemcpyAsync(s->d_vals_sorted, t.order.data(), 4 * (size_t)s->N, cudaMemcpyHostToDevice,
                       cs));
    if (!t.nodes.empty())
        CU(cudaMemcpyAsync(s->d_nodes, t.nodes.data(), sizeof(float4) * t.nodes.size(),
                           cudaMemcpyHostToDevice, cs));
    CU(cudaMemcpyAsync(s->d_hdr, &t.hdr, sizeof(t.hdr), cudaMemcpyHostToDevice, cs));
    CU(rt::lbvh_permute(a, s->d_vals_sorted, cs));
    CU(cudaEventRecord(s->ev1, cs));
    CU(cudaStreamSynchronize(cs));   // the host tree lives until its copies are done
    CU(scene_write_end(s, cs));
    s->cur ^= 1;
    s->built = true;
    s->sah = true;
    return RT_OK;
}

int32_t rt_bvh_refit_lbvh(rt_ctx* c, rt_scene* s, rt_stream stream) {
    if (!c || !s) return fail(RT_ERR_INVALID, "rt_bvh_refit_lbvh: null argument");
    if (!s->built) return fail(RT_ERR_NOT_BUILT, "rt_bvh_refit_lbvh: no BVH built");
    if (s->sah)
        return fail(RT_ERR_INVALID, "rt_bvh_refit_lbvh: the tree came from rt_bvh_build_sah; "
                    "build it again");
    cudaStream_t cs = st(c, stream);
    CU(scene_write_begin(s, cs));
    CU(cudaEventRecord(s->ev0, cs));
    rt::LbvhArgs a = lbvh_args(c, s);
    a.idx_out = s->d_idx[s->cur];   // refit keeps the current (sorted) order
    CU(rt::lbvh_refit(a, cs));
    CU(cudaEventRecord(s->ev1, cs));
    CU(scene_write_end(s, cs));
    return RT_OK;
}

int32_t rt_bvh_last_time_ms(rt_ctx* c, rt_scene* s, float* ms) {
    if (!c || !s || !ms) return fail(RT_ERR_INVALID, "rt_bvh_last_time_ms: null argument");
    CU(cudaEventSynchronize(s->ev1));
    CU(cudaEventElapsedTime(ms, s->ev0, s->ev1));
    return RT_OK;
}

int32_t rt_bvh_export(rt_ctx* c, rt_scene* s, rt_canon_node* out, uint32_t cap, uint32_t* count) {
    if (!c || !s || !count) return fail(RT_ERR_INVALID, "rt_bvh_export: null argument");
    if (!s->built) return fail(RT_ERR_NOT_BUILT, "rt_bvh_export: no BVH built");
    CU(scene_host_wait(s, false));
    CU(cudaStreamSynchronize(c->stream));
    rt::BvhHeader h;
    CU(cudaMemcpy(&h, s->d_hdr, sizeof(h), cudaMemcpyDeviceToHost));
    const size_t nn = s->N > 1 ? s->N - 1 : 0;
    std::vector<float4> nodes(4 * nn + 4);
    if (nn) CU(cudaMemcpy(nodes.data(), s->d_nodes, sizeof(float4) * 4 * nn, cudaMemcpyDeviceToHost));
    std::vector<rt_canon_node> res;
    res.reserve(2 * (size_t)s->N);
    struct Item {
        int32_t ref, cnt;
        uint32_t depth;
        float lo[3], hi[3];
        int64_t slot;
    };
    // iterative pre-order; interior ranges patched after their subtrees
    std::vector<Item> todo;
    std::vector<std::pair<int64_t, int64_t>> pending;   // (slot, right child slot)
    todo.push_back(Item{h.root_ref, h.root_cnt, 0, {h.root_lo.x, h.root_lo.y, h.root_lo.z},
                        {h.root_hi.x, h.root_hi.y, h.root_hi.z}, -1});
    std::vector<int64_t> left_of, right_of;
    while (!todo.empty()) {
        Item it = todo.back();
        todo.pop_back();
        rt_canon_node cn;
        memset(&cn, 0, sizeof(cn));
        cn.depth = it.depth;
        for (int k = 0; k < 3; ++k) {
            cn.lo[k] = it.lo[k];
            cn.hi[k] = it.hi[k];
        }
        const int64_t me = (int64_t)res.size();
        if (it.cnt > 0) {
            cn.leaf = 1;
            cn.start = (uint32_t)it.ref;
            cn.end = (uint32_t)(it.ref + it.cnt);
        } else {
            if (it.ref < 0 || (size_t)it.ref >= nn)
                return fail(RT_ERR, "rt_bvh_export: corrupt node reference %d", it.ref);
            const float4* q = &nodes[4 * (size_t)it.ref];
            const int* qi = reinterpret_cast<const int*>(&q[3]);
            Item L{qi[0], qi[2], it.depth + 1, {q[0].x, q[0].y, q[0].z}, {q[0].w, q[1].x, q[1].y}, me};
            Item R{qi[1], qi[3], it.depth + 1, {q[1].z, q[1].w, q[2].x}, {q[2].y, q[2].z, q[2].w}, me};
            todo.push_back(R);
            todo.push_back(L);
        }
        res.push_back(cn);
        left_of.push_back(-1);
        right_of.push_back(-1);
        if (it.slot >= 0) {
            if (left_of[it.slot] < 0)
                left_of[it.slot] = me;
            else
                right_of[it.slot] = me;
        }
        if (res.size() > 2 * (size_t)s->N) return fail(RT_ERR, "rt_bvh_export: tree has a cycle");
    }
    // ranges of interior nodes from their children (post-order = reverse pre-order)
    for (int64_t k = (int64_t)res.size() - 1; k >= 0; --k)
        if (!res[k].leaf) {
            res[k].start = res[left_of[k]].start;
            res[k].end = res[right_of[k]].end;
        }
    *count = (uint32_t)res.size();
    if (!out) return RT_OK;
    if (cap < res.size()) return fail(RT_ERR_INVALID, "rt_bvh_export: capacity %u < %zu", cap, res.size());
    memcpy(out, res.data(), sizeof(rt_canon_node) * res.size());
    return RT_OK;
}

// ---------------------------------------------------------------------------
// stage-wise pipeline
// ---------------------------------------------------------------------------
int32_t rt_gen_primary(rt_ctx* c, const rt_camera* cam, int32_t w, int32_t h, int32_t quad,
                       int32_t spp, const rt_pixel_sample* ps, size_t count, size_t offset,
                       rt_sample* out, rt_stream s) {
    if (!c || !cam || !out) return fail(RT_ERR_INVALID, "rt_gen_primary: null argument");
    if (w <= 0 || h <= 0 || quad <= 0 || spp <= 0)
        return fail(RT_ERR_INVALID, "rt_gen_primary: bad size %dx%d quad %d spp %d", w, h, quad, spp);
    if (offset + count > (size_t)w * h * spp)
        return fail(RT_ERR_INVALID, "rt_gen_primary: ids beyond w*h*spp");
    CU(rt::launch_gen_primary(*cam, w, h, quad, ps, count, offset, out, st(c, s)));
    return RT_OK;
}

static int32_t need_built(rt_scene* s, const char* who) {
    if (!s) return fail(RT_ERR_INVALID, "%s: null scene", who);
    if (!s->built) return fail(RT_ERR_NOT_BUILT, "%s: no BVH built", who);
    return RT_OK;
}

int32_t rt_trace(rt_ctx* c, rt_scene* s, const rt_sample* smp, int32_t n, rt_hit* hits,
                 int32_t secondary, rt_stream stream) {
    (void)secondary;
    if (!c || !smp || !hits) return fail(RT_ERR_INVALID, "rt_trace: null argument");
    int32_t r = need_built(s, "rt_trace");
    if (r) return r;
    cudaStream_t cs = st(c, stream);
    CU(scene_read_begin(s, cs));
    CU(rt::launch_trace(view_of(s), smp, n, hits, c->d_status, cs));
    CU(scene_read_end(s, cs));
    return RT_OK;
}

int32_t rt_shadow_trace(rt_ctx* c, rt_scene* s, const rt_sample* smp, int32_t n, rt_hit* hits,
                        int32_t secondary, rt_stream stream) {
    (void)secondary;
    (void)smp;
    if (!c || !hits) return fail(RT_ERR_INVALID, "rt_shadow_trace: null argument");
    int32_t r = need_built(s, "rt_shadow_trace");
    if (r) return r;
    cudaStream_t cs = st(c, stream);
    CU(scene_read_begin(s, cs));
    CU(rt::launch_shadow(view_of(s), s->lights, n, hits, c->d_status, cs));
    CU(scene_read_end(s, cs));
    return RT_OK;
}

int32_t rt_shade(rt_ctx* c, rt_scene* s, const rt_sample* smp, const rt_hit* hits, int32_t n,
                 uint32_t* img, int32_t primary, rt_stream stream) {
    (void)primary;
    if (!c || !smp || !hits || !img) return fail(RT_ERR_INVALID, "rt_shade: null argument");
    int32_t r = need_built(s, "rt_shade");
    if (r) return r;
    cudaStream_t cs = st(c, stream);
    CU(scene_read_begin(s, cs));
    CU(rt::launch_shade(view_of(s), s->lights, smp, hits, n, img, cs));
    CU(scene_read_end(s, cs));
    return RT_OK;
}

int32_t rt_gen_secondary(rt_ctx* c, rt_scene* s, const rt_sample* in, int32_t n, const rt_hit* hits,
                         rt_sample* out, int32_t max_out, int32_t* d_count, int32_t* h_count,
                         rt_stream stream) {
    if (!c || !in || !hits || !out || !d_count)
        return fail(RT_ERR_INVALID, "rt_gen_secondary: null argument");
    int32_t r = need_built(s, "rt_gen_secondary");
    if (r) return r;
    cudaStream_t cs = st(c, stream);
    uint32_t* scratch = rt::sec_scratch(c, cs, rt::gen_secondary_scratch_bytes(n));
    if (!scratch) return fail(RT_ERR_OOM, "rt_gen_secondary: scratch allocation failed");
    CU(scene_read_begin(s, cs));
    CU(rt::launch_gen_secondary(view_of(s), in, n, hits, out, max_out, d_count, scratch, cs));
    CU(scene_read_end(s, cs));
    if (h_count) {
        CU(cudaMemcpyAsync(h_count, d_count, sizeof(int32_t), cudaMemcpyDeviceToHost, cs));
        CU(cudaStreamSynchronize(cs));
    }
    return RT_OK;
}

int32_t rt_fb_clear(rt_ctx* c, uint32_t* img, size_t px, rt_stream s) {
    if (!c || !img) return fail(RT_ERR_INVALID, "rt_fb_clear: null argument");
    CU(cudaMemsetAsync(img, 0, 12 * px, st(c, s)));
    return RT_OK;
}

int32_t rt_fb_copy(rt_ctx* c, const uint32_t* img, uint8_t* rgba, size_t px, rt_stream s) {
    if (!c || !img || !rgba) return fail(RT_ERR_INVALID, "rt_fb_copy: null argument");
    CU(rt::launch_fb_copy(img, rgba, px, c->inv1e6, st(c, s)));
    return RT_OK;
}

// ---------------------------------------------------------------------------
// fused path
// ---------------------------------------------------------------------------
static cudaError_t launch_render_cfg(rt_ctx* c, rt::RenderArgs a, const rt_render_config& cfg,
                                     cudaStream_t cs) {
    int threads = 0, minb = 0;
    const void* fn = nullptr;
    rt::render_variant_info(cfg.variant, &threads, &minb, &fn);
    int bps = cfg.blocks_per_sm > 0 ? cfg.blocks_per_sm : c->variant_occupancy[cfg.variant];
    if (bps > c->variant_occupancy[cfg.variant]) bps = c->variant_occupancy[cfg.variant];
    // Shared memory for just the launched blocks per SM: the rest of the
    // SM's 256 KB of L1 / shared memory caches nodes, triangles and the
    // traversal stacks.  Process-wide per kernel: set when it changes.
    if (c->smem_per_sm > 0) {
        cudaFuncAttributes fa;
        if (cudaFuncGetAttributes(&fa, fn) == cudaSuccess) {
            const int64_t need = (int64_t)bps * ((int64_t)fa.sharedSizeBytes + 1024);
            int pct = (int)((need * 100 + c->smem_per_sm - 1) / c->smem_per_sm);
            if (pct > 100) pct = 100;
            if (pct != c->variant_carveout[cfg.variant] &&
                cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, pct) ==
                    cudaSuccess)
                c->variant_carveout[cfg.variant] = pct;
        }
        cudaGetLastError();
    }
    const int64_t pixels = (int64_t)a.width * a.height;
    const int64_t warps_needed = (pixels + cfg.chunk - 1) / cfg.chunk;
    int64_t grid = (int64_t)c->num_sms * bps;
    const int64_t max_useful = (warps_needed + threads / 32 - 1) / (threads / 32);
    if (grid > max_useful) grid = max_useful;
    if (grid < 1) grid = 1;
    a.chunk = cfg.chunk;
    a.accum = nullptr;
    if (rt::render_variant_pooled(cfg.variant)) {
        a.accum = a.image_rgb ? a.image_rgb : rt::accum_buffer(c, cs, (size_t)pixels);
        if (!a.accum) return cudaErrorMemoryAllocation;
    }
    return rt::launch_render(a, cfg.variant, (int)grid, cs);
}

static bool valid_cfg(const rt_render_config& cfg) {
    return cfg.variant >= 0 && cfg.variant < rt::render_variant_count() && cfg.blocks_per_sm >= 0 &&
           (cfg.chunk == 32 || cfg.chunk == 64 || cfg.chunk == 128 || cfg.chunk == 256);
}

int32_t rt_render_variants(int32_t* count) {
    if (!count) return fail(RT_ERR_INVALID, "rt_render_variants: null argument");
    *count = rt::render_variant_count();
    return RT_OK;
}

int32_t rt_render_variant_info(rt_ctx* c, int32_t v, int32_t* threads, int32_t* min_blocks,
                               int32_t* occ) {
    if (!c) return fail(RT_ERR_INVALID, "rt_render_variant_info: null context");
    int t = 0, m = 0;
    if (rt::render_variant_info(v, &t, &m, nullptr))
        return fail(RT_ERR_INVALID, "rt_render_variant_info: no variant %d", v);
    if (threads) *threads = t;
    if (min_blocks) *min_blocks = m;
    if (occ) *occ = c->variant_occupancy[v];
    return RT_OK;
}

int32_t rt_render_variant_pooled(int32_t v, int32_t* pooled) {
    if (!pooled) return fail(RT_ERR_INVALID, "rt_render_variant_pooled: null argument");
    if (v < 0 || v >= rt::render_variant_count())
        return fail(RT_ERR_INVALID, "rt_render_variant_pooled: no variant %d", v);
    *pooled = rt::render_variant_pooled(v) ? 1 : 0;
    return RT_OK;
}

int32_t rt_set_render_config(rt_ctx* c, const rt_render_config* cfg) {
    if (!c || !cfg) return fail(RT_ERR_INVALID, "rt_set_render_config: null argument");
    if (!valid_cfg(*cfg)) return fail(RT_ERR_INVALID, "rt_set_render_config: invalid configuration");
    c->render_cfg = *cfg;
    c->render_cfg.stack_depth = 32;
    return RT_OK;
}

int32_t rt_get_render_config(rt_ctx* c, rt_render_config* cfg) {
    if (!c || !cfg) return fail(RT_ERR_INVALID, "rt_get_render_config: null argument");
    *cfg = c->render_cfg;
    return RT_OK;
}
int32_t rt_render(rt_ctx* c, rt_scene* s, const rt_camera* cam, int32_t w, int32_t h,
                  int32_t max_bounces, uint8_t* rgba, uint32_t* img, rt_render_stats* stats,
                  rt_stream stream) {
    if (!c || !cam || !rgba) return fail(RT_ERR_INVALID, "rt_render: null argument");
    int32_t r = need_built(s, "rt_render");
    if (r) return r;
    if (w <= 0 || h <= 0 || (int64_t)w * h > (1ll << 30))
        return fail(RT_ERR_INVALID, "rt_render: bad size %dx%d", w, h);
    if (max_bounces < 0 || max_bounces > 64)
        return fail(RT_ERR_INVALID, "rt_render: bad max_bounces %d", max_bounces);
    cudaStream_t cs = st(c, stream);
    uint32_t* work = rt::work_counter(c, cs);
    if (!work) return fail(RT_ERR_OOM, "rt_render: work counter");
    CU(cudaMemsetAsync(work, 0, sizeof(uint32_t), cs));
    rt::RenderArgs a;
    a.scene = view_of(s);
    a.lights = s->lights;
    a.cam = *cam;
    a.width = w;
    a.height = h;
    a.max_bounces = max_bounces;
    a.inv1e6 = c->inv1e6;
    a.rgba = rgba;
    a.image_rgb = img;
    a.stats = stats;
    a.work_counter = work;
    a.status = c->d_status;
    rt_render_config cfg = c->render_cfg;
    if ((s->refracts && !rt::render_variant_refracts(cfg.variant)) ||
        !rt::render_variant_fits(cfg.variant, max_bounces)) {
        // refracting materials branch each hit: a variant that follows both rays
        cfg.variant = rt::render_refract_variant(max_bounces);
        cfg.blocks_per_sm = 0;
    }
    CU(scene_read_begin(s, cs));
    CU(launch_render_cfg(c, a, cfg, cs));
    CU(scene_read_end(s, cs));
    return RT_OK;
}

static uint64_t tune_key(int w, int h, uint32_t n, int bounces) {
    auto lg = [](uint64_t x) {
        int k = 0;
        while (x > 1) {
            x >>= 1;
            ++k;
        }
        return (uint64_t)k;
    };
    return (lg((uint64_t)w * h) << 16) | (lg(n) << 8) | (uint64_t)(bounces & 0xff);
}

int32_t rt_autotune_render(rt_ctx* c, rt_scene* s, const rt_camera* cam, int32_t w, int32_t h,
                           int32_t max_bounces, int32_t trials, rt_render_config* best,
                           float* best_ms) {
    if (!c || !cam) return fail(RT_ERR_INVALID, "rt_autotune_render: null argument");
    int32_t r = need_built(s, "rt_autotune_render");
    if (r) return r;
    if (w <= 0 || h <= 0) return fail(RT_ERR_INVALID, "rt_autotune_render: bad size");
    if (trials < 1) trials = 1;
    const uint64_t key = tune_key(w, h, s->N, max_bounces);
    auto it = c->tuned.find(key);
    if (it != c->tuned.end()) {
        c->render_cfg = it->second;
        if (best) *best = it->second;
        if (best_ms) *best_ms = -1.0f;
        return RT_OK;
    }
    cudaStream_t cs = c->stream;
    CU(scene_read_begin(s, cs));
    uint8_t* rgba = nullptr;
    CU(cudaMalloc(&rgba, 4 * (size_t)w * h));
    cudaEvent_t e0, e1;
    CU(cudaEventCreate(&e0));
    CU(cudaEventCreate(&e1));
    rt::RenderArgs a;
    a.scene = view_of(s);
    a.lights = s->lights;
    a.cam = *cam;
    a.width = w;
    a.height = h;
    a.max_bounces = max_bounces;
    a.inv1e6 = c->inv1e6;
    a.rgba = rgba;
    a.image_rgb = nullptr;
    a.stats = nullptr;
    a.work_counter = c->d_work;
    a.status = c->d_status;
    rt_render_config bestc = c->render_cfg;
    float bestt = 1e30f;
    const int chunks[] = {32, 64, 128};
    for (int v = 0; v < rt::render_variant_count(); ++v) {
        if (rt::render_variant_refracts(v) != s->refracts) continue;   // the variants that fit the scene
        if (!rt::render_variant_fits(v, max_bounces)) continue;
        // full residency, one and two blocks fewer (more L1 per block:
        // the carveout follows the launched blocks), and half residency
        const int occ = c->variant_occupancy[v];
        int bps_list[4] = {occ, occ - 1, occ - 2, (occ + 1) / 2};
        for (int bi = 0; bi < 4; ++bi) {
            bool seen = bps_list[bi] < 1;
            for (int bj = 0; bj < bi; ++bj) seen = seen || bps_list[bj] == bps_list[bi];
            if (seen) continue;
            for (int ch : chunks) {
                rt_render_config cfg = {v, bps_list[bi], ch, 32};
                std::vector<float> ts;
                for (int t = 0; t < trials + 1; ++t) {   // the first launch warms caches
                    cudaMemsetAsync(c->d_work, 0, sizeof(uint32_t), cs);
                    cudaEventRecord(e0, cs);
                    cudaError_t e = launch_render_cfg(c, a, cfg, cs);
                    cudaEventRecord(e1, cs);
                    if (e != cudaSuccess) {
                        cudaFree(rgba);
                        return fail(RT_ERR_CUDA, "rt_autotune_render: %s", cudaGetErrorString(e));
                    }
                    cudaEventSynchronize(e1);
                    float ms = 0.f;
                    cudaEventElapsedTime(&ms, e0, e1);
                    if (t > 0) ts.push_back(ms);
                }
                std::sort(ts.begin(), ts.end());
                const float tmin = ts[ts.size() / 2];   // median of the timed launches
                if (tmin < bestt) {
                    bestt = tmin;
                    bestc = cfg;
                }
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(rgba);
    CU(cudaGetLastError());
    CU(scene_read_end(s, cs));
    c->render_cfg = bestc;
    c->tuned[key] = bestc;
    if (best) *best = bestc;
    if (best_ms) *best_ms = bestt;
    return RT_OK;
}

// The work of one rt_render_host frame, queued on cs (see rt_render_host_async).
static int32_t render_host_enqueue(rt_ctx* c, rt_scene* s, rt_ctx::HostRender& R, cudaStream_t cs,
                                   const float* pos4, const float* nrm4, uint32_t V,
                                   const rt_bvh_cfg* cfg, const rt_camera* cam, int32_t w,
                                   int32_t h, int32_t max_bounces, uint8_t* h_rgba,
                                   rt_render_stats* h_stats, rt_stream stream) {
    const bool side_normals = pos4 && nrm4;
    if (pos4) {
        if (V != s->V) return fail(RT_ERR_INVALID, "vertex count %u != scene's %u", V, s->V);
        CU(scene_write_begin(s, cs));
        CU(cudaMemcpyAsync(s->d_pos, pos4, 16 * (size_t)V, cudaMemcpyHostToDevice, cs));
        if (side_normals) {
            // the build reads positions only: the normals go up beside it, on
            // a stream that starts once the positions are up (the two copies
            // would share the link and hold the build back) and that the
            // render waits for
            CU(cudaEventRecord(R.fork, cs));
            CU(cudaStreamWaitEvent(R.side, R.fork, 0));
            CU(cudaMemcpyAsync(s->d_nrm, nrm4, 16 * (size_t)V, cudaMemcpyHostToDevice, R.side));
            CU(cudaEventRecord(R.join, R.side));
        }
        CU(scene_write_end(s, cs));
    }
    int32_t r = rt_bvh_build_lbvh(c, s, cfg, stream);
    if (r) return r;
    if (side_normals) CU(cudaStreamWaitEvent(cs, R.join, 0));
    const size_t bytes = 4 * (size_t)w * h;
    if (R.out_cap < bytes) {
        if (R.d_out) cudaFreeAsync(R.d_out, cs);
        R.d_out = nullptr;
        R.out_cap = 0;
        if (cudaMallocAsync(reinterpret_cast<void**>(&R.d_out), bytes, cs)) {
            cudaGetLastError();
            return fail(RT_ERR_OOM, "rt_render_host: image allocation failed");
        }
        R.out_cap = bytes;
    }
    CU(cudaMemsetAsync(R.d_stats, 0, sizeof(rt_render_stats), cs));
    r = rt_render(c, s, cam, w, h, max_bounces, R.d_out, nullptr, R.d_stats, stream);
    if (r) return r;
    CU(cudaMemcpyAsync(h_rgba, R.d_out, bytes, cudaMemcpyDeviceToHost, cs));
    if (h_stats)
        CU(cudaMemcpyAsync(&R.h_stage->stats, R.d_stats, sizeof(rt_render_stats),
                           cudaMemcpyDeviceToHost, cs));
    CU(cudaMemcpyAsync(&R.h_stage->status, c->d_status, sizeof(uint32_t), cudaMemcpyDeviceToHost,
                       cs));
    return RT_OK;
}

int32_t rt_render_host_async(rt_ctx* c, rt_scene* s, const float* pos4, const float* nrm4,
                             uint32_t V, const rt_bvh_cfg* cfg, const rt_camera* cam, int32_t w,
                             int32_t h, int32_t max_bounces, uint8_t* h_rgba,
                             rt_render_stats* h_stats, rt_stream stream) {
    if (!c || !s || !cam || !h_rgba) return fail(RT_ERR_INVALID, "rt_render_host: null argument");
    cudaStream_t cs = st(c, stream);
    rt_ctx::HostRender* Rp;
    {
        std::lock_guard<std::mutex> lk(c->work_mu);
        Rp = &c->host_by_stream[cs];
    }
    rt_ctx::HostRender& R = *Rp;
    if (R.pending)
        return fail(RT_ERR_INVALID, "rt_render_host_async: the stream's previous frame has not "
                                    "been collected (rt_render_host_wait)");
    if (!R.side) {
        CU(cudaStreamCreateWithFlags(&R.side, cudaStreamNonBlocking));
        CU(cudaEventCreateWithFlags(&R.fork, cudaEventDisableTiming));
        CU(cudaEventCreateWithFlags(&R.join, cudaEventDisableTiming));
        CU(cudaMallocHost(&R.h_stage, sizeof(*R.h_stage)));
        CU(cudaMalloc(&R.d_stats, sizeof(rt_render_stats)));
    }
    const int32_t r = render_host_enqueue(c, s, R, cs, pos4, nrm4, V, cfg, cam, w, h, max_bounces,
                                          h_rgba, h_stats, stream);
    if (r) {
        // what was queued before the failure may still read the caller's
        // buffers: let it finish, so that the buffers are free on return
        cudaStreamSynchronize(R.side);
        cudaStreamSynchronize(cs);
        return r;
    }
    R.user_stats = h_stats;
    R.pending = true;
    return RT_OK;
}

int32_t rt_render_host_wait(rt_ctx* c, rt_stream stream) {
    if (!c) return fail(RT_ERR_INVALID, "rt_render_host_wait: null context");
    cudaStream_t cs = st(c, stream);
    rt_ctx::HostRender* Rp = nullptr;
    {
        std::lock_guard<std::mutex> lk(c->work_mu);
        auto it = c->host_by_stream.find(cs);
        if (it != c->host_by_stream.end()) Rp = &it->second;
    }
    if (!Rp || !Rp->pending)
        return fail(RT_ERR_INVALID, "rt_render_host_wait: no frame pending on this stream");
    rt_ctx::HostRender& R = *Rp;
    R.pending = false;
    CU(cudaStreamSynchronize(cs));
    if (R.user_stats) *R.user_stats = R.h_stage->stats;
    const uint32_t bits = R.h_stage->status;
    if (bits & RT_DEV_TIMEOUT) return fail(RT_ERR_TIMEOUT, "rt_render_host: device wait timed out");
    if (bits & RT_DEV_OVERFLOW) return fail(RT_ERR_OVERFLOW, "rt_render_host: stack overflow");
    return RT_OK;
}

int32_t rt_render_host(rt_ctx* c, rt_scene* s, const float* pos4, const float* nrm4, uint32_t V,
                       const rt_bvh_cfg* cfg, const rt_camera* cam, int32_t w, int32_t h,
                       int32_t max_bounces, uint8_t* h_rgba, rt_render_stats* h_stats,
                       rt_stream stream) {
    const int32_t r = rt_render_host_async(c, s, pos4, nrm4, V, cfg, cam, w, h, max_bounces,
                                           h_rgba, h_stats, stream);
    return r ? r : rt_render_host_wait(c, stream);
}

}  // extern "C"
