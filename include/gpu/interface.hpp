/*
 * gpu/interface.hpp — drop-in for the reference's DeviceInterface and
 * DeviceMemory (include/gpu/interface.hpp:20-80, include/gpu/memory.hpp:19-52)
 * over librt_cuda.so.  One rt_ctx per process; command queue i is a CUDA
 * stream (queue 0: the context's own stream, queues >= 1 created on first
 * use); a memory object is a device allocation addressed by a memory_id, as
 * in the reference.  Methods return 0 on success and -1 on failure, like the
 * reference's; rt_last_error() holds the library's message.  Kernel objects
 * (DeviceFunction, build_functions) have no counterpart: the stages are
 * compiled into the library.
 */
#pragma once
#ifndef GPU_INTERFACE_HPP
#define GPU_INTERFACE_HPP

#include <stddef.h>
#include <stdint.h>

#include <memory>
#include <vector>

#include "../rt_cuda.h"

typedef size_t memory_id;

enum DeviceMemoryMode { READ_ONLY_MEMORY, WRITE_ONLY_MEMORY, READ_WRITE_MEMORY };

class DeviceMemory {
public:
    DeviceMemory();
    ~DeviceMemory();
    DeviceMemory(const DeviceMemory&) = delete;
    DeviceMemory& operator=(const DeviceMemory&) = delete;

    bool valid() const;
    int32_t initialize(size_t size, DeviceMemoryMode mode = READ_WRITE_MEMORY);
    int32_t initialize(size_t size, const void* values, DeviceMemoryMode mode = READ_WRITE_MEMORY);
    /* Blocking copies, as the reference's (memory.cpp:111-175): 0 = ok. */
    size_t write(size_t nbytes, const void* values, size_t offset = 0, size_t command_queue_i = 0);
    size_t read(size_t nbytes, void* buffer, size_t offset = 0, size_t command_queue_i = 0);
    /* New size; the contents are discarded (memory.cpp:176-215). */
    int32_t resize(size_t new_size);
    int32_t copy_to(DeviceMemory& dst, size_t bytes = 0, size_t offset = 0, size_t dst_offset = 0,
                    size_t command_queue_i = 0);
    int32_t copy_all_to(DeviceMemory& dst, size_t command_queue_i);
    int32_t release();
    size_t size() const;
    /* The device address (the reference returns its cl_mem handle). */
    void* ptr();
    /* Makes this object a view of device memory owned elsewhere (a scene's
     * buffers); release() then forgets it without freeing. */
    int32_t set_view(void* d_ptr, size_t size);

private:
    void* m_ptr;
    size_t m_size;
    bool m_initialized;
    bool m_owned;
};

class DeviceInterface {
public:
    static DeviceInterface* instance();

    bool good();
    /* rt_init on device 0, or on the device RT_DEVICE names. */
    int32_t initialize();
    int32_t initialize(int32_t device);

    memory_id new_memory();
    DeviceMemory& memory(memory_id id);
    int32_t delete_memory(memory_id id);
    bool valid_memory_id(memory_id id);

    /* Commands on one queue run in order: a barrier has nothing to do. */
    int32_t enqueue_barrier(size_t command_queue_i = 0);
    int32_t finish_commands(size_t command_queue_i = 0);
    int32_t copy_memory(memory_id from, memory_id to, size_t bytes = 0, size_t from_offset = 0,
                        size_t to_offset = 0, size_t command_queue_i = 0);

    /* The library handles behind the reference's CLInfo. */
    rt_ctx* context();
    rt_stream stream(size_t command_queue_i);
    /* Frees every memory object and stream and the context (the reference
     * releases them at exit). */
    int32_t shutdown();

private:
    DeviceInterface();
    rt_ctx* m_ctx;
    std::vector<rt_stream> m_streams;
    std::vector<std::unique_ptr<DeviceMemory>> m_memory;
    DeviceMemory m_invalid;
};

#endif /* GPU_INTERFACE_HPP */
