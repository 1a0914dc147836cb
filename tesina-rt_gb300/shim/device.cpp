/*
 * device.cpp — DeviceInterface, DeviceMemory, RayBundle and HitBundle of the
 * drop-in C++ layer (include/gpu/interface.hpp, include/rt/ray.hpp) over
 * librt_cuda.so.  Reference: src/gpu/interface.cpp:40-103 (memory ids),
 * src/gpu/memory.cpp (blocking reads and writes, resize discards contents),
 * src/rt/ray.cpp (bundles of sample and hit records).
 */
#include <cstdlib>
#include <cstring>

#include "../../include/gpu/interface.hpp"
#include "../../include/rt/ray.hpp"

/* ---- DeviceMemory -------------------------------------------------------- */
DeviceMemory::DeviceMemory() : m_ptr(nullptr), m_size(0), m_initialized(false), m_owned(false) {}

DeviceMemory::~DeviceMemory() { release(); }

bool DeviceMemory::valid() const { return m_initialized; }

int32_t DeviceMemory::initialize(size_t size, DeviceMemoryMode) {
    DeviceInterface* dev = DeviceInterface::instance();
    if (!dev->good() || m_initialized) return -1;
    void* p = nullptr;
    if (size && rt_buf_alloc(dev->context(), size, &p) != RT_OK) return -1;
    m_ptr = p;
    m_size = size;
    m_owned = true;
    m_initialized = true;
    return 0;
}

int32_t DeviceMemory::initialize(size_t size, const void* values, DeviceMemoryMode mode) {
    if (initialize(size, mode)) return -1;
    return values && size ? (int32_t)write(size, values) : 0;
}

size_t DeviceMemory::write(size_t nbytes, const void* values, size_t offset,
                           size_t command_queue_i) {
    DeviceInterface* dev = DeviceInterface::instance();
    if (!valid() || offset + nbytes > m_size) return (size_t)-1;
    if (!nbytes) return 0;
    rt_stream s = dev->stream(command_queue_i);
    if (rt_buf_write(dev->context(), (char*)m_ptr + offset, values, nbytes, s) != RT_OK ||
        rt_stream_sync(dev->context(), s) != RT_OK)
        return (size_t)-1;
    return 0;
}

size_t DeviceMemory::read(size_t nbytes, void* buffer, size_t offset, size_t command_queue_i) {
    DeviceInterface* dev = DeviceInterface::instance();
    if (!valid() || offset + nbytes > m_size) return (size_t)-1;
    if (!nbytes) return 0;
    rt_stream s = dev->stream(command_queue_i);
    if (rt_buf_read(dev->context(), buffer, (const char*)m_ptr + offset, nbytes, s) != RT_OK ||
        rt_stream_sync(dev->context(), s) != RT_OK)
        return (size_t)-1;
    return 0;
}

int32_t DeviceMemory::resize(size_t new_size) {
    if (!m_owned && m_initialized) return -1;     /* a view cannot be resized */
    if (release()) return -1;
    return initialize(new_size);
}

int32_t DeviceMemory::copy_to(DeviceMemory& dst, size_t bytes, size_t offset, size_t dst_offset,
                              size_t command_queue_i) {
    DeviceInterface* dev = DeviceInterface::instance();
    if (!valid() || !dst.valid()) return -1;
    if (!bytes) bytes = m_size - offset;
    if (offset + bytes > m_size || dst_offset + bytes > dst.m_size) return -1;
    if (!bytes) return 0;
    return rt_buf_copy(dev->context(), (char*)dst.m_ptr + dst_offset, (const char*)m_ptr + offset,
                       bytes, dev->stream(command_queue_i)) == RT_OK ? 0 : -1;
}

int32_t DeviceMemory::copy_all_to(DeviceMemory& dst, size_t command_queue_i) {
    if (!valid() || !dst.valid() || dst.m_size < m_size) return -1;
    return copy_to(dst, m_size, 0, 0, command_queue_i);
}

int32_t DeviceMemory::release() {
    if (!m_initialized) return 0;
    int32_t rc = 0;
    if (m_owned && m_ptr) {
        DeviceInterface* dev = DeviceInterface::instance();
        rc = dev->good() && rt_buf_free(dev->context(), m_ptr) == RT_OK ? 0 : -1;
    }
    m_ptr = nullptr;
    m_size = 0;
    m_owned = false;
    m_initialized = false;
    return rc;
}

size_t DeviceMemory::size() const { return m_size; }

void* DeviceMemory::ptr() { return m_ptr; }

int32_t DeviceMemory::set_view(void* d_ptr, size_t size) {
    if (m_owned && m_initialized) return -1;
    m_ptr = d_ptr;
    m_size = size;
    m_owned = false;
    m_initialized = d_ptr != nullptr;
    return 0;
}

/* ---- DeviceInterface ----------------------------------------------------- */
DeviceInterface::DeviceInterface() : m_ctx(nullptr) {}

DeviceInterface* DeviceInterface::instance() {
    static DeviceInterface* s_instance = new DeviceInterface;
    return s_instance;
}

bool DeviceInterface::good() { return m_ctx != nullptr; }

int32_t DeviceInterface::initialize() {
    const char* d = std::getenv("RT_DEVICE");
    return initialize(d ? std::atoi(d) : 0);
}

int32_t DeviceInterface::initialize(int32_t device) {
    if (m_ctx) return 0;
    if (rt_init(&m_ctx, device) != RT_OK) {
        m_ctx = nullptr;
        return -1;
    }
    m_streams.assign(1, nullptr);
    return 0;
}

memory_id DeviceInterface::new_memory() {
    m_memory.emplace_back(new DeviceMemory());
    return m_memory.size() - 1;
}

bool DeviceInterface::valid_memory_id(memory_id id) {
    return id < m_memory.size() && m_memory[id] != nullptr;
}

DeviceMemory& DeviceInterface::memory(memory_id id) {
    return valid_memory_id(id) ? *m_memory[id] : m_invalid;
}

int32_t DeviceInterface::delete_memory(memory_id id) {
    if (!valid_memory_id(id)) return -1;
    const int32_t rc = m_memory[id]->release();
    m_memory[id].reset();
    return rc;
}

int32_t DeviceInterface::enqueue_barrier(size_t command_queue_i) {
    return good() && command_queue_i < 64 ? 0 : -1;
}

int32_t DeviceInterface::finish_commands(size_t command_queue_i) {
    if (!good()) return -1;
    return rt_stream_sync(m_ctx, stream(command_queue_i)) == RT_OK ? 0 : -1;
}

int32_t DeviceInterface::copy_memory(memory_id from, memory_id to, size_t bytes,
                                     size_t from_offset, size_t to_offset,
                                     size_t command_queue_i) {
    if (!valid_memory_id(from) || !valid_memory_id(to)) return -1;
    return memory(from).copy_to(memory(to), bytes, from_offset, to_offset, command_queue_i);
}

rt_ctx* DeviceInterface::context() { return m_ctx; }

rt_stream DeviceInterface::stream(size_t command_queue_i) {
    if (!m_ctx || command_queue_i == 0) return nullptr;
    if (command_queue_i >= m_streams.size()) m_streams.resize(command_queue_i + 1, nullptr);
    if (!m_streams[command_queue_i]) rt_stream_create(m_ctx, &m_streams[command_queue_i]);
    return m_streams[command_queue_i];
}

int32_t DeviceInterface::shutdown() {
    if (!m_ctx) return 0;
    int32_t rc = 0;
    for (auto& m : m_memory)
        if (m) rc |= m->release();
    m_memory.clear();
    for (size_t i = 1; i < m_streams.size(); ++i)
        if (m_streams[i]) rc |= rt_stream_destroy(m_ctx, m_streams[i]) == RT_OK ? 0 : -1;
    m_streams.clear();
    rc |= rt_shutdown(m_ctx) == RT_OK ? 0 : -1;
    m_ctx = nullptr;
    return rc ? -1 : 0;
}

/* ---- RayBundle / HitBundle ----------------------------------------------- */
RayBundle::RayBundle() : ray_id(0), m_ray_count(0), m_initialized(false) {}

RayBundle::~RayBundle() {
    if (m_initialized && DeviceInterface::instance()->good())
        DeviceInterface::instance()->delete_memory(ray_id);
}

int32_t RayBundle::initialize(const size_t rays) {
    DeviceInterface* dev = DeviceInterface::instance();
    if (!dev->good() || m_initialized || rays > (size_t)INT32_MAX) return -1;
    ray_id = dev->new_memory();
    if (dev->memory(ray_id).initialize(rays * sizeof(rt_sample))) return -1;
    m_ray_count = (int32_t)rays;
    m_initialized = true;
    return 0;
}

int32_t RayBundle::resize(const size_t rays) {
    if (!m_initialized) return initialize(rays);
    if (rays > (size_t)INT32_MAX || mem().resize(rays * sizeof(rt_sample))) return -1;
    m_ray_count = (int32_t)rays;
    return 0;
}

bool RayBundle::valid() { return m_initialized; }

int32_t RayBundle::count() { return m_ray_count; }

DeviceMemory& RayBundle::mem() { return DeviceInterface::instance()->memory(ray_id); }

HitBundle::HitBundle() : hit_id(0), m_size(0), m_initialized(false) {}

HitBundle::~HitBundle() {
    if (m_initialized && DeviceInterface::instance()->good())
        DeviceInterface::instance()->delete_memory(hit_id);
}

int32_t HitBundle::initialize(const size_t sz) {
    DeviceInterface* dev = DeviceInterface::instance();
    if (!dev->good() || m_initialized || sz > (size_t)INT32_MAX) return -1;
    hit_id = dev->new_memory();
    if (dev->memory(hit_id).initialize(sz * sizeof(rt_hit))) return -1;
    m_size = sz;
    m_initialized = true;
    return 0;
}

int32_t HitBundle::resize(const size_t rays) {
    if (!m_initialized) return initialize(rays);
    if (rays > (size_t)INT32_MAX || mem().resize(rays * sizeof(rt_hit))) return -1;
    m_size = rays;
    return 0;
}

bool HitBundle::valid() { return m_initialized; }

int32_t HitBundle::count() { return (int32_t)m_size; }

DeviceMemory& HitBundle::mem() { return DeviceInterface::instance()->memory(hit_id); }
