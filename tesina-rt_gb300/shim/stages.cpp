/*
 * stages.cpp — the hot-path classes of the drop-in C++ layer, each method a
 * call into the C ABI of librt_cuda.so on the queue's stream:
 *   BVHBuilder             src/rt/bvh-builder.cpp:117-199, 201-741, 743-850
 *   Tracer                 src/rt/tracer.cpp:140-352, 487-489
 *   RayShader              src/rt/ray-shader.cpp:32-171
 *   SecondaryRayGenerator  src/rt/secondary-ray-generator.cpp:10-445
 *   PrimaryRayGenerator    src/rt/primary-ray-generator.cpp:30-217
 *   FrameBuffer            src/rt/framebuffer.cpp:20-210
 * Timing works as in the reference: with timing on, a call waits for its
 * queue and reports host milliseconds (the builder reports the device time
 * of its build, rt_bvh_last_time_ms).
 */
#include <algorithm>
#include <chrono>

#include "../../include/rt/bvh-builder.hpp"
#include "../../include/rt/framebuffer.hpp"
#include "../../include/rt/primary-ray-generator.hpp"
#include "../../include/rt/ray-shader.hpp"
#include "../../include/rt/secondary-ray-generator.hpp"
#include "../../include/rt/tracer.hpp"

namespace {

using clock_type = std::chrono::steady_clock;

rt_ctx* ctx() { return DeviceInterface::instance()->context(); }

bool ok(int32_t rc) { return rc == RT_OK; }

/* Host milliseconds since t0 after the queue has drained. */
double ms_since(clock_type::time_point t0, size_t cq_i) {
    DeviceInterface::instance()->finish_commands(cq_i);
    return std::chrono::duration<double, std::milli>(clock_type::now() - t0).count();
}

}  // namespace

/* ---- BVHBuilder ---------------------------------------------------------- */
BVHBuilder::BVHBuilder()
    : bvh_created(false), m_log(nullptr), m_logging(false), m_timing(true), m_time_ms(0.0),
      bvh_depth(32), bvh_min_leaf_size(1) {}

int32_t BVHBuilder::initialize() {
    bvh_depth = 32;
    bvh_min_leaf_size = 1;
    bvh_created = false;
    m_timing = true;
    m_logging = false;
    m_log = nullptr;
    return DeviceInterface::instance()->good() ? 0 : -1;
}

int32_t BVHBuilder::build_lbvh(Scene& scene, size_t cq_i) {
    if (!scene.rt_handle() || bvh_depth > 32) return -1;
    const rt_bvh_cfg cfg = {bvh_depth, bvh_min_leaf_size};
    if (!ok(rt_bvh_build_lbvh(ctx(), scene.rt_handle(), &cfg,
                              DeviceInterface::instance()->stream(cq_i))))
        return -1;
    if (m_timing) {
        float ms = 0.f;
        if (!ok(rt_bvh_last_time_ms(ctx(), scene.rt_handle(), &ms))) return -1;
        m_time_ms = ms;
    }
    bvh_created = true;
    return 0;
}

int32_t BVHBuilder::refit_lbvh(Scene& scene, size_t cq_i) {
    if (!scene.rt_handle() || !bvh_created) return -1;
    const auto t0 = clock_type::now();
    if (!ok(rt_bvh_refit_lbvh(ctx(), scene.rt_handle(), DeviceInterface::instance()->stream(cq_i))))
        return -1;
    if (m_timing) m_time_ms = ms_since(t0, cq_i);
    return 0;
}

void BVHBuilder::set_log(Log* log) { m_log = log; }
void BVHBuilder::timing(bool b) { m_timing = b; }
void BVHBuilder::logging(bool l) { m_logging = l; }
double BVHBuilder::get_exec_time() { return m_time_ms; }

void BVHBuilder::update_configuration(const RendererConfig& conf) {
    bvh_depth = std::min(std::max(conf.bvh_depth, 1), 64);
    bvh_min_leaf_size = std::min(std::max(conf.bvh_min_leaf_size, 1), 256);
}

/* ---- Tracer -------------------------------------------------------------- */
Tracer::Tracer() : m_initialized(false), m_timing(false), m_tracer_time_ms(0.0),
                   m_shadow_time_ms(0.0) {}

int32_t Tracer::initialize() {
    m_timing = false;
    m_initialized = DeviceInterface::instance()->good();
    return m_initialized ? 0 : -1;
}

int32_t Tracer::trace(Scene& scene, int32_t ray_count, RayBundle& rays, HitBundle& hits,
                      bool secondary) {
    if (!m_initialized || ray_count < 0 || ray_count > rays.count() || ray_count > hits.count())
        return -1;
    const auto t0 = clock_type::now();
    if (!ok(rt_trace(ctx(), scene.rt_handle(), (const rt_sample*)rays.mem().ptr(), ray_count,
                     (rt_hit*)hits.mem().ptr(), secondary ? 1 : 0, nullptr)))
        return -1;
    if (m_timing) m_tracer_time_ms = ms_since(t0, 0);
    return 0;
}

int32_t Tracer::trace(Scene& scene, DeviceMemory& bvh_mem, int32_t ray_count, RayBundle& rays,
                      HitBundle& hits, bool secondary) {
    if (&bvh_mem != &scene.bvh_nodes_mem()) return -1;
    return trace(scene, ray_count, rays, hits, secondary);
}

int32_t Tracer::shadow_trace(Scene& scene, int32_t ray_count, RayBundle& rays, HitBundle& hits,
                             bool secondary) {
    if (!m_initialized || ray_count < 0 || ray_count > rays.count() || ray_count > hits.count())
        return -1;
    const auto t0 = clock_type::now();
    if (!ok(rt_shadow_trace(ctx(), scene.rt_handle(), (const rt_sample*)rays.mem().ptr(),
                            ray_count, (rt_hit*)hits.mem().ptr(), secondary ? 1 : 0, nullptr)))
        return -1;
    if (m_timing) m_shadow_time_ms = ms_since(t0, 0);
    return 0;
}

int32_t Tracer::shadow_trace(Scene& scene, DeviceMemory& bvh_mem, int32_t ray_count,
                             RayBundle& rays, HitBundle& hits, bool secondary) {
    if (&bvh_mem != &scene.bvh_nodes_mem()) return -1;
    return shadow_trace(scene, ray_count, rays, hits, secondary);
}

void Tracer::timing(bool b) { m_timing = b; }
double Tracer::get_trace_exec_time() { return m_tracer_time_ms; }
double Tracer::get_shadow_exec_time() { return m_shadow_time_ms; }
void Tracer::update_configuration(const RendererConfig&) {}

/* ---- RayShader ----------------------------------------------------------- */
RayShader::RayShader() : m_timing(false), m_time_ms(0.0) {}

int32_t RayShader::initialize() {
    m_timing = false;
    return DeviceInterface::instance()->good() ? 0 : -1;
}

int32_t RayShader::shade(RayBundle& rays, HitBundle& hb, Scene& scene, Cubemap& cm,
                         FrameBuffer& fb, size_t size, bool primary) {
    if (cm.enabled || !fb.initialized() || size > (size_t)rays.count() ||
        size > (size_t)hb.count())
        return -1;
    const auto t0 = clock_type::now();
    if (!ok(rt_shade(ctx(), scene.rt_handle(), (const rt_sample*)rays.mem().ptr(),
                     (const rt_hit*)hb.mem().ptr(), (int32_t)size,
                     (uint32_t*)fb.image_mem().ptr(), primary ? 1 : 0, nullptr)))
        return -1;
    if (m_timing) m_time_ms = ms_since(t0, 0);
    return 0;
}

void RayShader::timing(bool b) { m_timing = b; }
double RayShader::get_exec_time() { return m_time_ms; }
void RayShader::update_configuration(const RendererConfig&) {}

/* ---- SecondaryRayGenerator ----------------------------------------------- */
SecondaryRayGenerator::SecondaryRayGenerator()
    : m_max_rays(0), m_tasks(false), m_disc(true), m_initialized(false), m_timing(false),
      m_time_ms(0.0), count_id(0) {}

SecondaryRayGenerator::~SecondaryRayGenerator() {
    if (m_initialized && DeviceInterface::instance()->good())
        DeviceInterface::instance()->delete_memory(count_id);
}

int32_t SecondaryRayGenerator::initialize() {
    DeviceInterface* dev = DeviceInterface::instance();
    m_max_rays = 0;
    if (!dev->good()) return -1;
    if (m_initialized) return 0;
    count_id = dev->new_memory();
    if (dev->memory(count_id).initialize(sizeof(int32_t))) return -1;
    m_initialized = true;
    return 0;
}

int32_t SecondaryRayGenerator::generate(Scene& scene, RayBundle& ray_in, size_t rays_in,
                                        HitBundle& hits, RayBundle& ray_out, size_t* rays_out) {
    if (!m_initialized || !rays_out || rays_in > (size_t)ray_in.count() ||
        rays_in > (size_t)hits.count())
        return -1;
    const auto t0 = clock_type::now();
    int32_t max_out = ray_out.count();
    if (m_max_rays > 0) max_out = std::min(max_out, m_max_rays);
    int32_t n = 0;
    if (!ok(rt_gen_secondary(ctx(), scene.rt_handle(), (const rt_sample*)ray_in.mem().ptr(),
                             (int32_t)rays_in, (const rt_hit*)hits.mem().ptr(),
                             (rt_sample*)ray_out.mem().ptr(), max_out,
                             (int32_t*)DeviceInterface::instance()->memory(count_id).ptr(), &n,
                             nullptr)))
        return -1;
    *rays_out = (size_t)n;
    if (m_timing) m_time_ms = ms_since(t0, 0);
    return 0;
}

void SecondaryRayGenerator::set_max_rays(size_t max) {
    m_max_rays = (int32_t)std::min<size_t>(max, (size_t)INT32_MAX);
}
void SecondaryRayGenerator::timing(bool b) { m_timing = b; }
double SecondaryRayGenerator::get_exec_time() { return m_time_ms; }

void SecondaryRayGenerator::update_configuration(const RendererConfig& conf) {
    m_tasks = conf.sec_ray_use_atomics != 0;
    m_disc = conf.sec_ray_use_disc != 0;
}

/* ---- PrimaryRayGenerator ------------------------------------------------- */
PrimaryRayGenerator::PrimaryRayGenerator()
    : pixel_samples_id(0), m_initialized(false), m_timing(false), m_time_ms(0.0),
      m_use_zcurve(false), m_quad_size(32), m_spp(1) {}

PrimaryRayGenerator::~PrimaryRayGenerator() {
    if (m_initialized && DeviceInterface::instance()->good())
        DeviceInterface::instance()->delete_memory(pixel_samples_id);
}

int32_t PrimaryRayGenerator::initialize() {
    DeviceInterface* dev = DeviceInterface::instance();
    if (!dev->good()) return -1;
    m_timing = false;
    m_use_zcurve = false;
    m_quad_size = 32;
    m_spp = 1;
    if (m_initialized) dev->delete_memory(pixel_samples_id);
    pixel_samples_id = dev->new_memory();
    const pixel_sample_cl single = {0.f, 0.f, 1.f};
    if (dev->memory(pixel_samples_id).initialize(sizeof(single), &single, READ_ONLY_MEMORY))
        return -1;
    m_initialized = true;
    return 0;
}

int32_t PrimaryRayGenerator::set_spp(size_t spp, pixel_sample_cl const* psamples) {
    if (!m_initialized || spp == 0 || spp > (size_t)INT32_MAX || !psamples) return -1;
    DeviceMemory& m = get_pixel_samples();
    if (m.resize(spp * sizeof(pixel_sample_cl)) || m.write(spp * sizeof(pixel_sample_cl), psamples))
        return -1;
    m_spp = (int32_t)spp;
    return 0;
}

size_t PrimaryRayGenerator::get_spp() const { return (size_t)m_spp; }

DeviceMemory& PrimaryRayGenerator::get_pixel_samples() {
    return DeviceInterface::instance()->memory(pixel_samples_id);
}

int32_t PrimaryRayGenerator::generate(const Camera& cam, RayBundle& bundle, size_t size[2],
                                      const size_t ray_count, const size_t offset) {
    if (!m_initialized || ray_count > (size_t)bundle.count()) return -1;
    if (m_use_zcurve && size[0] == size[1] && (size[0] & (size[0] - 1)) == 0) return -1;
    const auto t0 = clock_type::now();
    const rt_camera c = cam.to_rt();
    if (!ok(rt_gen_primary(ctx(), &c, (int32_t)size[0], (int32_t)size[1], m_quad_size, m_spp,
                           (const rt_pixel_sample*)get_pixel_samples().ptr(), ray_count, offset,
                           (rt_sample*)bundle.mem().ptr(), nullptr)))
        return -1;
    if (m_timing) m_time_ms = ms_since(t0, 0);
    return 0;
}

void PrimaryRayGenerator::timing(bool b) { m_timing = b; }
double PrimaryRayGenerator::get_exec_time() { return m_time_ms; }

void PrimaryRayGenerator::update_configuration(const RendererConfig& conf) {
    m_use_zcurve = conf.prim_ray_use_zcurve != 0;
    m_quad_size = conf.prim_ray_quad_size;
}

/* ---- FrameBuffer --------------------------------------------------------- */
FrameBuffer::FrameBuffer()
    : size{0, 0}, img_mem_id(0), m_initialized(false), m_timing(false), m_clear_time_ms(0.0),
      m_copy_time_ms(0.0) {}

FrameBuffer::~FrameBuffer() {
    if (m_initialized && DeviceInterface::instance()->good())
        DeviceInterface::instance()->delete_memory(img_mem_id);
}

int32_t FrameBuffer::initialize(size_t sz[2]) {
    DeviceInterface* dev = DeviceInterface::instance();
    if (!dev->good() || m_initialized || !sz[0] || !sz[1]) return -1;
    img_mem_id = dev->new_memory();
    if (dev->memory(img_mem_id).initialize(12 * sz[0] * sz[1])) return -1;
    size[0] = sz[0];
    size[1] = sz[1];
    m_initialized = true;
    return clear();
}

int32_t FrameBuffer::resize(size_t sz[2]) {
    if (!m_initialized) return initialize(sz);
    if (!sz[0] || !sz[1] || image_mem().resize(12 * sz[0] * sz[1])) return -1;
    size[0] = sz[0];
    size[1] = sz[1];
    return clear();
}

bool FrameBuffer::initialized() { return m_initialized; }

DeviceMemory& FrameBuffer::image_mem() { return DeviceInterface::instance()->memory(img_mem_id); }

int32_t FrameBuffer::clear() {
    if (!m_initialized) return -1;
    const auto t0 = clock_type::now();
    if (!ok(rt_fb_clear(ctx(), (uint32_t*)image_mem().ptr(), size[0] * size[1], nullptr)))
        return -1;
    if (m_timing) m_clear_time_ms = ms_since(t0, 0);
    return 0;
}

int32_t FrameBuffer::copy(DeviceMemory& tex_mem) {
    const size_t px = size[0] * size[1];
    if (!m_initialized || !tex_mem.valid() || tex_mem.size() < 4 * px) return -1;
    const auto t0 = clock_type::now();
    if (!ok(rt_fb_copy(ctx(), (const uint32_t*)image_mem().ptr(), (uint8_t*)tex_mem.ptr(), px,
                       nullptr)))
        return -1;
    if (m_timing) m_copy_time_ms = ms_since(t0, 0);
    return 0;
}

void FrameBuffer::timing(bool b) { m_timing = b; }
double FrameBuffer::get_clear_exec_time() { return m_clear_time_ms; }
double FrameBuffer::get_copy_exec_time() { return m_copy_time_ms; }
