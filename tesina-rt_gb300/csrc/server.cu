// server.cu — the served form: a request loop over HBM-resident scenes.
//
// One server thread owns the GPU work.  Each turn it
//   1. retires render launches whose completion event has fired (their
//      images were copied to pinned host staging by the same stream),
//   2. admits uploads in arrival order: a new scene is charged to the HBM
//      budget, least-recently-used idle scenes are evicted to make room, or
//      the upload is rejected; admitted uploads are handed to the upload
//      thread, which copies them and builds their LBVH on a separate,
//      high-priority build stream, and frees evicted scenes, so that
//      pageable copies never hold up render launches.  Scene memory comes
//      from a stream-ordered device pool: an eviction returns it to the pool
//      without the device-wide synchronisation of cudaFree,
//   3. forms a render launch from the queued render requests whose scene is
//      ready and whose framebuffer fits in the device arena, in arrival order,
//      up to max_batch_views, and launches it (one many-image persistent
//      kernel, batch.cu) on a free render stream, followed by the copies of
//      its images to pinned staging and an event.
// Requests that arrive while launches are on the GPU join the next launch
// as soon as a render stream and arena space are free: continuous batching
// at launch granularity, with up to max_inflight launches overlapping.
// With max_batch_views == 1 every request is rendered alone by rt_render's
// kernel: the plain per-request path, for comparison.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <mutex>
#include <new>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/rt_cuda.h"
#include "batch.cuh"
#include "ctx_internal.h"
#include "lbvh.cuh"
#include "trace.cuh"

#define fail rt::set_error

namespace {

double now_ms() {
    using namespace std::chrono;
    return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

// First-fit allocator over [0, size) in 256-byte units.
class Arena {
public:
    void reset(size_t size) {
        free_.clear();
        free_[0] = size;
        size_ = size;
    }
    bool alloc(size_t bytes, size_t* off) {
        bytes = (bytes + 255) & ~(size_t)255;
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second >= bytes) {
                *off = it->first;
                const size_t rest = it->second - bytes, start = it->first + bytes;
                free_.erase(it);
                if (rest) free_[start] = rest;
                return true;
            }
        }
        return false;
    }
    void release(size_t off, size_t bytes) {
        bytes = (bytes + 255) & ~(size_t)255;
        auto it = free_.emplace(off, bytes).first;
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first) {
            it->second += nx->second;
            free_.erase(nx);
        }
        if (it != free_.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                free_.erase(it);
            }
        }
    }
    size_t size() const { return size_; }

private:
    std::map<size_t, size_t> free_;
    size_t size_ = 0;
};

struct ServedScene {
    uint64_t id = 0;
    rt_scene* scene = nullptr;
    rt_lights* d_lights = nullptr;
    uint64_t bytes = 0;
    int refs = 0;               // in-flight renders
    int pending = 0;            // queued renders not yet launched
    uint64_t last_use = 0;      // submission clock of the latest use
    bool ready = false;         // BVH built
    bool admitted = false;      // charged to the budget (an upload waits until then)
    bool doomed = false;        // evicted under the scene cap; freed when idle
    cudaEvent_t built = nullptr;
    uint64_t upload_ticket = 0; // upload request waiting for the build
};

// Work for the upload thread: build a new scene, or free an evicted one.
struct UpJob {
    bool reap = false;
    uint64_t ticket = 0, scene_id = 0;
    const rt_scene_desc* desc = nullptr;
    rt_scene* scene = nullptr;
    rt_lights* lights = nullptr;
    cudaEvent_t built = nullptr;
};

struct Req {
    uint64_t ticket;
    rt_request r;
    double submit_ms = 0, start_ms = 0, done_ms = 0;
    uint64_t stamp = 0;          // submission clock
    int32_t status = 1;          // 1 = pending
    int32_t batch_views = 0;
    uint64_t scene_id = 0;
    size_t fb_off = 0, fb_bytes = 0;
    uint64_t rays = 0;
};

struct Launch {
    int slot;
    cudaEvent_t done;
    std::vector<uint64_t> tickets;
};

}  // namespace

struct rt_server {
    rt_ctx* ctx = nullptr;
    rt_server_cfg cfg;
    std::mutex mu;
    std::condition_variable cv;        // wakes the server thread
    std::condition_variable done_cv;   // wakes result waiters
    std::thread th;
    bool stop = false;
    uint64_t next_ticket = 1, next_scene = 1;
    uint64_t use_clock = 1;            // submission order, for LRU
    // upload thread
    std::thread up_th;
    std::condition_variable up_cv;
    std::deque<UpJob> up_jobs;
    bool up_stop = false;
    std::deque<uint64_t> incoming;     // tickets in arrival order
    std::unordered_map<uint64_t, Req> reqs;
    std::map<uint64_t, ServedScene> scenes;
    uint64_t resident_bytes = 0;
    // device resources
    Arena arena;
    uint8_t* d_fb = nullptr;
    uint8_t* h_fb = nullptr;           // pinned mirror of the arena
    cudaStream_t build_stream = nullptr;
    cudaMemPool_t pool = nullptr;      // scene memory, stream-ordered on build_stream
    std::vector<cudaStream_t> streams;
    std::vector<bool> slot_busy;
    std::vector<rt::BatchView*> d_views;
    std::vector<uint32_t*> d_pix_off;
    std::vector<uint32_t*> d_work;
    std::vector<rt_render_stats*> d_stats;
    std::vector<rt::BatchView*> h_views;   // pinned staging of the tables
    std::vector<uint32_t*> h_pix_off;
    std::vector<rt_render_stats*> h_stats;
    std::deque<Launch> inflight;
    int render_grid = 0, render_threads = 128, render_bps = 1;
    // statistics
    std::vector<double> latencies;
    uint64_t completed = 0, rejected = 0, evicted = 0, batches = 0, rays = 0, views_sum = 0;
    double first_submit = -1, last_done = 0;
};

namespace {

uint64_t scene_bytes(const rt_scene_desc* d) {
    const uint64_t V = d->vertex_count, N = d->triangle_count, M = d->material_count;
    return 32 * V + 40 * N + 32 * M                     // geometry, both orders
           + N * (24 + 48 + 32 + 64)                     // sort, triangles, leaves, nodes
           + rt::lbvh_scratch_bytes((uint32_t)N, 4)      // radix and emit scratch
           + 4096;
}

// Scene memory: a device pool that keeps what is freed for later uploads.
cudaError_t pool_create(int device, cudaMemPool_t* pool) {
    cudaMemPoolProps props;
    memset(&props, 0, sizeof(props));
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = device;
    cudaError_t e = cudaMemPoolCreate(pool, &props);
    if (e != cudaSuccess) return e;
    uint64_t keep = UINT64_MAX;
    return cudaMemPoolSetAttribute(*pool, cudaMemPoolAttrReleaseThreshold, &keep);
}

// Builds run on the highest-priority stream: their blocks are scheduled
// first as render blocks retire, so an upload is not held behind a burst.
cudaError_t build_stream_create(cudaStream_t* s) {
    int lo = 0, hi = 0;
    cudaError_t e = cudaDeviceGetStreamPriorityRange(&lo, &hi);
    if (e != cudaSuccess) return e;
    return cudaStreamCreateWithPriority(s, cudaStreamNonBlocking, hi);
}

void finish(rt_server* S, Req& q, int32_t status, double t) {
    q.status = status;
    q.done_ms = t;
    if (status == RT_OK) {
        S->completed++;
        if (q.r.type == RT_REQ_RENDER) S->latencies.push_back(q.done_ms - q.submit_ms);
        S->last_done = std::max(S->last_done, t);
    } else {
        S->rejected++;
    }
}

// Takes an idle scene out of the table and hands its memory to the upload
// thread.  Called with the lock held.
void evict(rt_server* S, uint64_t id) {
    auto it = S->scenes.find(id);
    UpJob j;
    j.reap = true;
    j.scene = it->second.scene;
    j.lights = it->second.d_lights;
    j.built = it->second.built;
    S->resident_bytes -= it->second.bytes;
    S->evicted++;
    S->scenes.erase(it);
    S->up_jobs.push_back(j);
    S->up_cv.notify_all();
}

// Evicts least-recently-used idle scenes until `need` more bytes fit; evicts
// nothing when even all idle scenes together would not make enough room.
bool make_room(rt_server* S, uint64_t need) {
    if (S->resident_bytes + need <= S->cfg.hbm_budget_bytes) return true;
    uint64_t idle = 0;
    for (auto& kv : S->scenes) {
        const ServedScene& sc = kv.second;
        if (sc.ready && sc.refs == 0 && sc.pending == 0) idle += sc.bytes;
    }
    if (S->resident_bytes - idle + need > S->cfg.hbm_budget_bytes) return false;
    while (S->resident_bytes + need > S->cfg.hbm_budget_bytes) {
        ServedScene* victim = nullptr;
        for (auto& kv : S->scenes) {
            ServedScene& sc = kv.second;
            if (!sc.ready || sc.refs > 0 || sc.pending > 0) continue;
            if (!victim || sc.last_use < victim->last_use) victim = &sc;
        }
        if (!victim) return false;
        evict(S, victim->id);
    }
    return true;
}

int32_t create_scene(rt_server* S, const rt_scene_desc* d, cudaStream_t stream, ServedScene* out) {
    rt_scene* sc = nullptr;
    int32_t r = rt_scene_create(S->ctx, &sc);
    if (r) return r;
    rt::scene_use_pool(sc, S->pool, stream);
    r = rt_scene_upload(S->ctx, sc, d, stream);
    if (r) {
        rt_scene_destroy(S->ctx, sc);
        return r;
    }
    rt_bvh_cfg cfg = {30, 1};
    r = rt_bvh_build_lbvh(S->ctx, sc, &cfg, stream);
    if (r) {
        rt_scene_destroy(S->ctx, sc);
        return r;
    }
    if (cudaMallocFromPoolAsync(reinterpret_cast<void**>(&out->d_lights), sizeof(rt_lights),
                                S->pool, stream) ||
        cudaMemcpyAsync(out->d_lights, &d->lights, sizeof(rt_lights), cudaMemcpyHostToDevice,
                        stream) ||
        cudaEventCreateWithFlags(&out->built, cudaEventDisableTiming) ||
        cudaEventRecord(out->built, stream)) {
        cudaGetLastError();
        if (out->d_lights) cudaFreeAsync(out->d_lights, stream);
        out->d_lights = nullptr;
        rt_scene_destroy(S->ctx, sc);
        return fail(RT_ERR_CUDA, "rt_server: scene resources");
    }
    out->scene = sc;
    return RT_OK;
}

// Retires finished launches.  Called with the lock held.
void retire(rt_server* S) {
    while (!S->inflight.empty()) {
        Launch& L = S->inflight.front();
        if (cudaEventQuery(L.done) != cudaSuccess) break;
        const double t = now_ms();
        const rt_render_stats st = *S->h_stats[L.slot];
        uint64_t px = 0;
        for (uint64_t tk : L.tickets) {
            Req& q = S->reqs[tk];
            px += (uint64_t)q.r.width * q.r.height;
        }
        // rays are counted per launch; shared out by pixel count for reports
        const uint64_t launch_rays = st.primary_rays + st.secondary_rays;
        S->rays += launch_rays;
        for (uint64_t tk : L.tickets) {
            Req& q = S->reqs[tk];
            q.rays = px ? launch_rays * ((uint64_t)q.r.width * q.r.height) / px : 0;
            auto it = S->scenes.find(q.r.scene_id);
            if (it != S->scenes.end()) it->second.refs--;
            finish(S, q, RT_OK, t);
        }
        S->slot_busy[L.slot] = false;
        cudaEventDestroy(L.done);
        S->inflight.pop_front();
        S->done_cv.notify_all();
    }
    // uploads whose build completed
    for (auto& kv : S->scenes) {
        ServedScene& sc = kv.second;
        if (sc.ready || !sc.built) continue;
        if (cudaEventQuery(sc.built) != cudaSuccess) continue;
        sc.ready = true;
        if (sc.upload_ticket) {
            Req& q = S->reqs[sc.upload_ticket];
            q.scene_id = sc.id;
            finish(S, q, RT_OK, now_ms());
            sc.upload_ticket = 0;
            S->done_cv.notify_all();
        }
    }
    // scenes evicted under the scene cap, once their renders are done
    std::vector<uint64_t> idle;
    for (auto& kv : S->scenes) {
        const ServedScene& sc = kv.second;
        if (sc.doomed && sc.ready && sc.refs == 0 && sc.pending == 0) idle.push_back(kv.first);
    }
    for (uint64_t id : idle) evict(S, id);
}

// One render launch from the queued renders.  Called with the lock held.
bool launch_renders(rt_server* S) {
    int slot = -1;
    for (size_t k = 0; k < S->slot_busy.size(); ++k)
        if (!S->slot_busy[k]) {
            slot = (int)k;
            break;
        }
    if (slot < 0) return false;
    std::vector<uint64_t> take;
    std::deque<uint64_t> keep;
    const double t = now_ms();
    while (!S->incoming.empty()) {
        const uint64_t tk = S->incoming.front();
        S->incoming.pop_front();
        Req& q = S->reqs[tk];
        if (q.r.type != RT_REQ_RENDER || (int)take.size() >= S->cfg.max_batch_views) {
            keep.push_back(tk);
            continue;
        }
        auto it = S->scenes.find(q.r.scene_id);
        if (it == S->scenes.end()) {   // unknown or evicted scene
            finish(S, q, RT_ERR_INVALID, t);
            S->done_cv.notify_all();
            continue;
        }
        if (!it->second.ready) {
            keep.push_back(tk);
            continue;
        }
        q.fb_bytes = 4 * (size_t)q.r.width * q.r.height;
        if (!S->arena.alloc(q.fb_bytes, &q.fb_off)) {
            if (q.fb_bytes > S->arena.size()) {
                finish(S, q, RT_ERR_REJECTED, t);
                S->done_cv.notify_all();
            } else {
                keep.push_back(tk);
            }
            continue;
        }
        it->second.refs++;
        it->second.pending--;
        q.start_ms = t;
        take.push_back(tk);
    }
    // requests kept keep their arrival order ahead of later arrivals
    S->incoming.insert(S->incoming.begin(), keep.begin(), keep.end());
    if (take.empty()) return false;
    cudaStream_t cs = S->streams[slot];
    rt_render_stats* dstats = S->d_stats[slot];
    uint64_t launch_px = 0;
    cudaMemsetAsync(dstats, 0, sizeof(rt_render_stats), cs);
    if (S->cfg.max_batch_views == 1 || take.size() == 1) {
        // one request: the one-scene render kernel (pooled, tuned), which
        // renders a lone image faster than the many-view kernel
        Req& q = S->reqs[take[0]];
        ServedScene& sc = S->scenes[q.r.scene_id];
        rt_render(S->ctx, sc.scene, &q.r.cam, q.r.width, q.r.height, q.r.max_bounces,
                  S->d_fb + q.fb_off, nullptr, dstats, (rt_stream)cs);
        q.batch_views = 1;
    } else {
        rt::BatchView* hv = S->h_views[slot];
        uint32_t* hp = S->h_pix_off[slot];
        hp[0] = 0;
        bool refracts = false;
        for (size_t v = 0; v < take.size(); ++v) {
            Req& q = S->reqs[take[v]];
            ServedScene& sc = S->scenes[q.r.scene_id];
            refracts = refracts || sc.scene->refracts;
            rt::BatchView& V = hv[v];
            V.scene = rt::scene_view(sc.scene);
            V.lights = sc.d_lights;
            V.cam = q.r.cam;
            V.width = q.r.width;
            V.height = q.r.height;
            V.max_bounces = q.r.max_bounces;
            V.rgba_offset = (uint32_t)(q.fb_off / 4);
            hp[v + 1] = hp[v] + (uint32_t)(q.r.width * q.r.height);
            q.batch_views = (int32_t)take.size();
        }
        launch_px = hp[take.size()];
        cudaMemcpyAsync(S->d_views[slot], hv, sizeof(rt::BatchView) * take.size(),
                        cudaMemcpyHostToDevice, cs);
        cudaMemcpyAsync(S->d_pix_off[slot], hp, 4 * (take.size() + 1), cudaMemcpyHostToDevice, cs);
        cudaMemsetAsync(S->d_work[slot], 0, 4, cs);
        rt::BatchRenderArgs a;
        a.views = S->d_views[slot];
        a.count = (int)take.size();
        a.pix_off = S->d_pix_off[slot];
        a.rgba = S->d_fb;
        a.stats = dstats;
        a.work_counter = S->d_work[slot];
        a.status = S->ctx->d_status;
        a.chunk = 32;
        a.inv1e6 = S->ctx->inv1e6;
        // a small launch takes only the blocks its pixels need, so that
        // launches on other streams run beside it
        const uint64_t need = (launch_px + S->render_threads - 1) / S->render_threads;
        // while an upload builds, two block slots per SM stay free for its
        // kernels: a persistent launch would otherwise hold every SM until
        // it ends and each of the build's kernels would wait for a gap
        bool building = false;
        for (auto& kv : S->scenes) building |= kv.second.admitted && !kv.second.ready;
        const int cap = building && S->render_bps > 2
                            ? (S->render_bps - 2) * S->ctx->num_sms : S->render_grid;
        const int grid = (int)std::min<uint64_t>(cap, std::max<uint64_t>(1, need));
        // a launch with a refracting scene walks each pixel's ray tree
        rt::launch_batch_render(a, refracts ? rt::batch_refract_variant(false, 0) : 0, grid, cs);
    }
    for (uint64_t tk : take) {
        Req& q = S->reqs[tk];
        cudaMemcpyAsync(S->h_fb + q.fb_off, S->d_fb + q.fb_off, q.fb_bytes, cudaMemcpyDeviceToHost,
                        cs);
    }
    cudaMemcpyAsync(S->h_stats[slot], dstats, sizeof(rt_render_stats), cudaMemcpyDeviceToHost, cs);
    Launch L;
    L.slot = slot;
    L.tickets = take;
    cudaEventCreateWithFlags(&L.done, cudaEventDisableTiming);
    cudaEventRecord(L.done, cs);
    S->slot_busy[slot] = true;
    S->inflight.push_back(L);
    S->batches++;
    S->views_sum += take.size();
    return true;
}

// Admits queued uploads in arrival order.  Called with the lock held.
void admit_uploads(rt_server* S) {
    std::deque<uint64_t> keep;
    while (!S->incoming.empty()) {
        const uint64_t tk = S->incoming.front();
        S->incoming.pop_front();
        Req& q = S->reqs[tk];
        if (q.r.type != RT_REQ_UPLOAD) {
            keep.push_back(tk);
            continue;
        }
        const uint64_t need = scene_bytes(q.r.upload);
        if (!make_room(S, need)) {
            if (S->inflight.empty()) {   // nothing will free memory: reject
                S->scenes.erase(q.scene_id);   // its queued renders fail
                finish(S, q, RT_ERR_REJECTED, now_ms());
                S->done_cv.notify_all();
            } else {
                keep.push_back(tk);      // retry when renders release scenes
            }
            continue;
        }
        ServedScene& sc = S->scenes[q.scene_id];
        sc.bytes = need;
        sc.admitted = true;
        q.start_ms = now_ms();
        S->resident_bytes += need;
        UpJob j;
        j.ticket = tk;
        j.scene_id = q.scene_id;
        j.desc = q.r.upload;
        S->up_jobs.push_back(j);
        S->up_cv.notify_all();
    }
    S->incoming.insert(S->incoming.begin(), keep.begin(), keep.end());
}

// The upload thread: copies and builds admitted uploads on the build stream,
// frees evicted scenes.  The lock is released while it works.
void upload_loop(rt_server* S) {
    cudaSetDevice(S->ctx->device);
    std::unique_lock<std::mutex> lk(S->mu);
    for (;;) {
        S->up_cv.wait(lk, [&] { return S->up_stop || !S->up_jobs.empty(); });
        if (S->up_jobs.empty()) break;   // stopping, nothing left
        const UpJob j = S->up_jobs.front();
        S->up_jobs.pop_front();
        lk.unlock();
        if (j.reap) {   // pool frees: no device synchronisation
            rt_scene_destroy(S->ctx, j.scene);
            cudaFreeAsync(j.lights, S->build_stream);
            if (j.built) cudaEventDestroy(j.built);
            lk.lock();
            continue;
        }
        ServedScene made;
        const int32_t r = create_scene(S, j.desc, S->build_stream, &made);
        lk.lock();
        auto it = S->scenes.find(j.scene_id);
        if (r == RT_OK && it != S->scenes.end()) {
            it->second.scene = made.scene;
            it->second.d_lights = made.d_lights;
            it->second.built = made.built;   // retire() marks it ready
        } else {
            if (r == RT_OK) {   // not reachable: unbuilt scenes are never evicted
                rt_scene_destroy(S->ctx, made.scene);
                cudaFreeAsync(made.d_lights, S->build_stream);
                cudaEventDestroy(made.built);
            }
            if (it != S->scenes.end()) {
                S->resident_bytes -= it->second.bytes;
                S->scenes.erase(it);
            }
            finish(S, S->reqs[j.ticket], r ? r : RT_ERR, now_ms());
            S->done_cv.notify_all();
        }
        S->cv.notify_all();
    }
}

void server_loop(rt_server* S) {
    cudaSetDevice(S->ctx->device);
    std::unique_lock<std::mutex> lk(S->mu);
    while (!S->stop) {
        retire(S);
        admit_uploads(S);
        bool launched = false;
        while (launch_renders(S)) launched = true;
        if (!launched) {
            // wait for new requests, or poll the GPU every 20 us while work is out
            if (S->inflight.empty() && S->incoming.empty()) {
                bool building = false;
                for (auto& kv : S->scenes) building |= !kv.second.ready;
                if (!building) {
                    S->cv.wait(lk);
                    continue;
                }
            }
            S->cv.wait_for(lk, std::chrono::microseconds(20));
        }
    }
}

}  // namespace

extern "C" {

int32_t rt_server_create(rt_ctx* c, const rt_server_cfg* cfg, rt_server** out) {
    if (!c || !cfg || !out) return fail(RT_ERR_INVALID, "rt_server_create: null argument");
    if (cfg->max_batch_views < 1 || cfg->max_batch_views > rt::kMaxBatchViews ||
        cfg->max_inflight < 1 || cfg->max_inflight > 8 || cfg->fb_arena_bytes < 4096 ||
        cfg->fb_arena_bytes >= (1ull << 34) || cfg->fb_arena_bytes > cfg->hbm_budget_bytes ||
        cfg->max_scenes < 0 || cfg->reserved != 0)
        return fail(RT_ERR_INVALID, "rt_server_create: bad configuration");
    rt_server* S = new (std::nothrow) rt_server();
    if (!S) return fail(RT_ERR_OOM, "rt_server_create: host allocation failed");
    S->ctx = c;
    S->cfg = *cfg;
    // the plain per-request path renders with rt_render, whose work counter
    // belongs to the context: one launch at a time
    if (S->cfg.max_batch_views == 1) S->cfg.max_inflight = 1;
    S->arena.reset(cfg->fb_arena_bytes);
    S->resident_bytes = cfg->fb_arena_bytes;
    const int nslot = S->cfg.max_inflight, nv = S->cfg.max_batch_views;
    bool ok = cudaMalloc(&S->d_fb, cfg->fb_arena_bytes) == cudaSuccess &&
              cudaMallocHost(&S->h_fb, cfg->fb_arena_bytes) == cudaSuccess &&
              build_stream_create(&S->build_stream) == cudaSuccess &&
              pool_create(c->device, &S->pool) == cudaSuccess;
    for (int k = 0; ok && k < nslot; ++k) {
        cudaStream_t st;
        rt::BatchView *dv, *hv;
        uint32_t *dp, *hp, *dw;
        rt_render_stats *ds, *hs;
        ok = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) == cudaSuccess &&
             cudaMalloc(&dv, sizeof(rt::BatchView) * nv) == cudaSuccess &&
             cudaMallocHost(&hv, sizeof(rt::BatchView) * nv) == cudaSuccess &&
             cudaMalloc(&dp, 4 * (nv + 1)) == cudaSuccess &&
             cudaMallocHost(&hp, 4 * (nv + 1)) == cudaSuccess &&
             cudaMalloc(&dw, 64) == cudaSuccess &&
             cudaMalloc(&ds, sizeof(rt_render_stats)) == cudaSuccess &&
             cudaMallocHost(&hs, sizeof(rt_render_stats)) == cudaSuccess;
        // the plain path renders with rt_render, whose work counter for
        // this stream is made here rather than in the first request
        if (ok && nv == 1) ok = rt::work_counter(c, st) != nullptr;
        if (!ok) break;
        S->streams.push_back(st);
        S->slot_busy.push_back(false);
        S->d_views.push_back(dv);
        S->h_views.push_back(hv);
        S->d_pix_off.push_back(dp);
        S->h_pix_off.push_back(hp);
        S->d_work.push_back(dw);
        S->d_stats.push_back(ds);
        S->h_stats.push_back(hs);
    }
    int threads = 0, bps = 0;
    const void* fn = nullptr;
    if (ok) {
        rt::batch_render_variant_info(0, &threads, &fn);
        ok = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, fn, threads, 0) == cudaSuccess;
    }
    if (!ok) {
        cudaGetLastError();
        S->stop = true;
        rt_server_destroy(S);
        return fail(RT_ERR_OOM, "rt_server_create: device resources");
    }
    // a launch may fill the machine; launches on other streams fill in as
    // its blocks run out of work
    S->render_grid = std::max(1, bps * c->num_sms);
    S->render_threads = threads;
    S->render_bps = bps;
    S->up_th = std::thread(upload_loop, S);
    S->th = std::thread(server_loop, S);
    *out = S;
    return RT_OK;
}

int32_t rt_server_destroy(rt_server* S) {
    if (!S) return RT_OK;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->stop = true;
    }
    S->cv.notify_all();
    if (S->th.joinable()) S->th.join();
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->up_stop = true;
    }
    S->up_cv.notify_all();
    if (S->up_th.joinable()) S->up_th.join();   // drains its queue first
    cudaSetDevice(S->ctx->device);
    cudaDeviceSynchronize();
    for (auto& kv : S->scenes) {
        if (kv.second.scene) rt_scene_destroy(S->ctx, kv.second.scene);
        if (kv.second.d_lights) cudaFreeAsync(kv.second.d_lights, S->build_stream);
        if (kv.second.built) cudaEventDestroy(kv.second.built);
    }
    if (S->build_stream) cudaStreamSynchronize(S->build_stream);
    if (S->pool) cudaMemPoolDestroy(S->pool);
    for (auto& L : S->inflight) cudaEventDestroy(L.done);
    for (size_t k = 0; k < S->streams.size(); ++k) {
        rt::release_work_counter(S->ctx, S->streams[k]);
        cudaStreamDestroy(S->streams[k]);
        cudaFree(S->d_views[k]);
        cudaFreeHost(S->h_views[k]);
        cudaFree(S->d_pix_off[k]);
        cudaFreeHost(S->h_pix_off[k]);
        cudaFree(S->d_work[k]);
        cudaFree(S->d_stats[k]);
        cudaFreeHost(S->h_stats[k]);
    }
    if (S->build_stream) cudaStreamDestroy(S->build_stream);
    if (S->d_fb) cudaFree(S->d_fb);
    if (S->h_fb) cudaFreeHost(S->h_fb);
    delete S;
    return RT_OK;
}

int32_t rt_server_add_scene(rt_server* S, const rt_scene_desc* d, uint64_t* id) {
    if (!S || !d || !id) return fail(RT_ERR_INVALID, "rt_server_add_scene: null argument");
    const uint64_t need = scene_bytes(d);
    std::unique_lock<std::mutex> lk(S->mu);
    if (!make_room(S, need))
        return fail(RT_ERR_REJECTED, "rt_server_add_scene: %llu bytes exceed the budget",
                    (unsigned long long)need);
    S->resident_bytes += need;   // reserved while the scene is built unlocked
    lk.unlock();
    ServedScene sc;
    int32_t r = create_scene(S, d, S->build_stream, &sc);
    if (r == RT_OK && cudaEventSynchronize(sc.built) != cudaSuccess) {
        rt_scene_destroy(S->ctx, sc.scene);
        cudaFreeAsync(sc.d_lights, S->build_stream);
        cudaEventDestroy(sc.built);
        r = fail(RT_ERR_CUDA, "rt_server_add_scene: build failed");
    }
    lk.lock();
    if (r) {
        S->resident_bytes -= need;
        return r;
    }
    sc.id = S->next_scene++;
    sc.ready = true;
    sc.admitted = true;
    sc.bytes = need;
    sc.last_use = S->use_clock++;
    S->scenes[sc.id] = sc;
    *id = sc.id;
    return RT_OK;
}

static int32_t submit(rt_server* S, const rt_request* r, uint64_t* ticket, uint64_t* scene_id) {
    if (!S || !r || !ticket) return fail(RT_ERR_INVALID, "rt_server_submit: null argument");
    if (r->type == RT_REQ_RENDER) {
        if (r->width <= 0 || r->height <= 0 || r->max_bounces < 0 || r->max_bounces > 64)
            return fail(RT_ERR_INVALID, "rt_server_submit: bad render request");
    } else if (r->type == RT_REQ_UPLOAD) {
        if (!r->upload) return fail(RT_ERR_INVALID, "rt_server_submit: upload without a scene");
    } else {
        return fail(RT_ERR_INVALID, "rt_server_submit: unknown request type %d", r->type);
    }
    {
        std::lock_guard<std::mutex> lk(S->mu);
        Req q;
        q.ticket = S->next_ticket++;
        q.r = *r;
        q.stamp = S->use_clock++;
        q.submit_ms = now_ms();
        if (S->first_submit < 0) S->first_submit = q.submit_ms;
        *ticket = q.ticket;
        if (r->type == RT_REQ_RENDER) {
            auto it = S->scenes.find(r->scene_id);
            if (it != S->scenes.end() && it->second.doomed) {
                S->reqs[q.ticket] = q;   // evicted: fails without queueing
                finish(S, S->reqs[q.ticket], RT_ERR_INVALID, q.submit_ms);
                return RT_OK;
            }
            if (it != S->scenes.end()) {
                it->second.pending++;
                it->second.last_use = q.stamp;
            }
        } else if (S->cfg.max_scenes > 0) {
            // the scene cap: this upload displaces the least recently used
            // scene now, so that eviction follows submission order
            int live = 0;
            for (auto& kv : S->scenes) live += !kv.second.doomed;
            while (live >= S->cfg.max_scenes) {
                ServedScene* victim = nullptr;
                for (auto& kv : S->scenes) {
                    ServedScene& sc = kv.second;
                    if (!sc.doomed && (!victim || sc.last_use < victim->last_use)) victim = &sc;
                }
                if (!victim) break;
                victim->doomed = true;
                live--;
            }
        }
        if (r->type == RT_REQ_UPLOAD) {
            // the scene exists from now on: renders may name it at once and
            // wait for its build
            ServedScene sc;
            sc.id = S->next_scene++;
            sc.upload_ticket = q.ticket;
            sc.last_use = q.stamp;
            S->scenes[sc.id] = sc;
            q.scene_id = sc.id;
            if (scene_id) *scene_id = sc.id;
        }
        S->reqs[q.ticket] = q;
        S->incoming.push_back(q.ticket);
    }
    S->cv.notify_all();
    return RT_OK;
}

int32_t rt_server_submit(rt_server* S, const rt_request* r, uint64_t* ticket) {
    return submit(S, r, ticket, nullptr);
}

int32_t rt_server_upload(rt_server* S, const rt_scene_desc* desc, uint64_t* ticket,
                         uint64_t* scene_id) {
    if (!desc || !scene_id) return fail(RT_ERR_INVALID, "rt_server_upload: null argument");
    rt_request r;
    memset(&r, 0, sizeof(r));
    r.type = RT_REQ_UPLOAD;
    r.upload = desc;
    return submit(S, &r, ticket, scene_id);
}

int32_t rt_server_result(rt_server* S, uint64_t ticket, uint8_t* h_rgba, rt_request_info* info) {
    if (!S) return fail(RT_ERR_INVALID, "rt_server_result: null server");
    std::unique_lock<std::mutex> lk(S->mu);
    auto it = S->reqs.find(ticket);
    if (it == S->reqs.end()) return fail(RT_ERR_INVALID, "rt_server_result: unknown ticket");
    S->done_cv.wait(lk, [&] { return S->reqs[ticket].status != 1; });
    Req q = S->reqs[ticket];
    if (q.status == RT_OK && q.r.type == RT_REQ_RENDER) {
        if (h_rgba) memcpy(h_rgba, S->h_fb + q.fb_off, q.fb_bytes);
        S->arena.release(q.fb_off, q.fb_bytes);
        S->cv.notify_all();   // arena space for queued renders
    }
    if (info) {
        info->status = q.status;
        info->batch_views = q.batch_views;
        info->scene_id = q.scene_id;
        info->submit_ms = q.submit_ms;
        info->start_ms = q.start_ms;
        info->done_ms = q.done_ms;
        info->rays = q.rays;
    }
    S->reqs.erase(ticket);
    return q.status == RT_OK ? RT_OK : fail(q.status, "rt_server_result: request failed (%d)",
                                             q.status);
}

int32_t rt_server_get_stats(rt_server* S, rt_server_stats* st) {
    if (!S || !st) return fail(RT_ERR_INVALID, "rt_server_get_stats: null argument");
    std::lock_guard<std::mutex> lk(S->mu);
    memset(st, 0, sizeof(*st));
    st->completed = S->completed;
    st->rejected = S->rejected;
    st->evicted = S->evicted;
    st->batches = S->batches;
    st->rays = S->rays;
    st->resident_scenes = S->scenes.size();
    st->resident_bytes = S->resident_bytes;
    st->mean_batch_views = S->batches ? (double)S->views_sum / S->batches : 0.0;
    st->first_submit_ms = S->first_submit;
    st->last_done_ms = S->last_done;
    std::vector<double> l = S->latencies;
    if (!l.empty()) {
        std::sort(l.begin(), l.end());
        st->p50_ms = l[(l.size() - 1) / 2];
        st->p99_ms = l[std::min(l.size() - 1, (size_t)((l.size() - 1) * 0.99 + 0.5))];
    }
    return RT_OK;
}

int32_t rt_server_reset_stats(rt_server* S) {
    if (!S) return fail(RT_ERR_INVALID, "rt_server_reset_stats: null server");
    std::lock_guard<std::mutex> lk(S->mu);
    S->latencies.clear();
    S->completed = S->rejected = S->evicted = S->batches = S->rays = S->views_sum = 0;
    S->first_submit = -1;
    S->last_done = 0;
    return RT_OK;
}

}  // extern "C"
