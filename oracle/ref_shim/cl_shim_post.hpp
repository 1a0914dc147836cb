/* cl_shim_post.hpp — ORACLE test infrastructure: removes the OpenCL qualifier
 * macros once a kernel source has been compiled. */
#undef kernel
#undef __kernel
#undef global
#undef __global
#undef local
#undef __local
#undef constant
#undef __constant
#undef private
#undef __private
#undef read_only
#undef write_only
#undef __read_only
#undef __write_only

/* Runs f(gid) for gid in [offset, offset + n) on `threads` host threads.
 * f must set the work-item id of the thread it runs on. */
template <class F>
static void refk_run(size_t offset, size_t n, int threads, F f) {
    if (threads <= 1 || n < 4096) {
        for (size_t g = offset; g < offset + n; ++g) f(g);
        return;
    }
    std::atomic<size_t> next(offset);
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; ++t)
        pool.emplace_back([&]() {
            for (;;) {
                size_t b = next.fetch_add(1024);
                if (b >= offset + n) break;
                size_t e = std::min(offset + n, b + 1024);
                for (size_t g = b; g < e; ++g) f(g);
            }
        });
    for (auto& th : pool) th.join();
}
