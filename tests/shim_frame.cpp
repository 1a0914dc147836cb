/*
 * shim_frame.cpp — a C++ caller of the drop-in classes (the headers in include/rt and
 * include/gpu), as the reference's renderer calls its own: the
 * per-frame loop of Renderer::render_to_framebuffer (src/rt/renderer.cpp:
 * 113-214) — tiles of primary samples; per tile primary generation, trace,
 * shadow trace and shade; then bounces of secondary generation, trace,
 * shadow trace and shade — after BVHBuilder::build_lbvh and
 * FrameBuffer::clear, and FrameBuffer::copy at the end
 * (Renderer::copy_framebuffer, renderer.cpp:216-227).  Bundles are sized as
 * Renderer::update_configuration sizes them (3 x tile, renderer.cpp:83-102).
 *
 * Test program.  Usage: shim_frame DIR.  DIR holds the scene as raw arrays
 * (pos4.bin, nrm4.bin float4 per vertex; idx.bin uint32 x 3 per triangle;
 * mats.bin rt_material; map.bin uint32 per triangle; lights.bin rt_lights;
 * camera.bin rt_camera; params.bin int32 width, height, max_bounces, tile,
 * bvh_depth, bvh_min_leaf_size); it writes image.bin (3 uint32 per pixel),
 * rgba.bin and stats.bin (uint64 total rays, secondary rays).
 */
#include <cstdio>
#include <cstring>
#include <string>
#include <utility>
#include <vector>

#include "gpu/interface.hpp"
#include "rt/bvh-builder.hpp"
#include "rt/framebuffer.hpp"
#include "rt/primary-ray-generator.hpp"
#include "rt/ray-shader.hpp"
#include "rt/secondary-ray-generator.hpp"
#include "rt/tracer.hpp"

static std::vector<char> slurp(const std::string& path) {
    std::vector<char> out;
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) return out;
    char buf[1 << 16];
    size_t k;
    while ((k = std::fread(buf, 1, sizeof(buf), f)) > 0) out.insert(out.end(), buf, buf + k);
    std::fclose(f);
    return out;
}

static bool spill(const std::string& path, const void* p, size_t n) {
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) return false;
    const bool good = std::fwrite(p, 1, n, f) == n;
    return std::fclose(f) == 0 && good;
}

#define CHECK(x)                                                                    \
    do {                                                                            \
        if (x) {                                                                    \
            std::fprintf(stderr, "failed: %s (%s)\n", #x, rt_last_error());         \
            return 1;                                                               \
        }                                                                           \
    } while (0)

int main(int argc, char** argv) {
    if (argc < 2) return 2;
    const std::string dir = argv[1];
    std::vector<char> pos = slurp(dir + "/pos4.bin"), nrm = slurp(dir + "/nrm4.bin"),
                      idx = slurp(dir + "/idx.bin"), mats = slurp(dir + "/mats.bin"),
                      map = slurp(dir + "/map.bin"), lights = slurp(dir + "/lights.bin"),
                      cam = slurp(dir + "/camera.bin"), prm = slurp(dir + "/params.bin");
    if (lights.size() != sizeof(rt_lights) || cam.size() != sizeof(rt_camera) ||
        prm.size() != 6 * sizeof(int32_t) || pos.size() != nrm.size() || pos.empty())
        return 2;
    int32_t p[6];
    std::memcpy(p, prm.data(), sizeof(p));
    const size_t fb_w = (size_t)p[0], fb_h = (size_t)p[1];
    const uint32_t max_bounces = (uint32_t)p[2];

    DeviceInterface& device = *DeviceInterface::instance();
    CHECK(device.initialize());
    {
        Scene scene;
        rt_scene_desc desc;
        std::memset(&desc, 0, sizeof(desc));
        desc.h_vertices = pos.data();
        desc.vertex_count = (uint32_t)(pos.size() / 16);
        desc.vertex_stride = 16;
        desc.h_normals = nrm.data();
        desc.h_indices = (const uint32_t*)idx.data();
        desc.triangle_count = (uint32_t)(idx.size() / 12);
        desc.material_count = (uint32_t)(mats.size() / sizeof(rt_material));
        desc.h_materials = (const rt_material*)mats.data();
        desc.h_material_map = (const uint32_t*)map.data();
        std::memcpy(&desc.lights, lights.data(), sizeof(rt_lights));
        CHECK(scene.transfer_aggregate_mesh_to_device(desc));
        rt_camera c;
        std::memcpy(&c, cam.data(), sizeof(c));
        scene.camera.pos = vec3(c.pos[0], c.pos[1], c.pos[2]);
        scene.camera.dir = vec3(c.dir[0], c.dir[1], c.dir[2]);
        scene.camera.right = vec3(c.right[0], c.right[1], c.right[2]);
        scene.camera.up = vec3(c.up[0], c.up[1], c.up[2]);

        RendererConfig config;
        config.bvh_depth = p[4];
        config.bvh_min_leaf_size = p[5];
        BVHBuilder bvh_builder;
        PrimaryRayGenerator prim_ray_gen;
        SecondaryRayGenerator sec_ray_gen;
        Tracer tracer;
        RayShader ray_shader;
        FrameBuffer framebuffer;
        RayBundle ray_bundle_1, ray_bundle_2;
        HitBundle hit_bundle;
        size_t fb_size[] = {fb_w, fb_h};
        CHECK(bvh_builder.initialize() || prim_ray_gen.initialize() ||
              sec_ray_gen.initialize() || tracer.initialize() || ray_shader.initialize());
        CHECK(framebuffer.initialize(fb_size));
        const size_t pixel_count = fb_w * fb_h;
        const size_t tile_size = std::min(pixel_count, (size_t)p[3]);
        CHECK(ray_bundle_1.initialize(tile_size * 3) || ray_bundle_2.initialize(tile_size * 3) ||
              hit_bundle.initialize(tile_size * 3));
        sec_ray_gen.set_max_rays(ray_bundle_1.count());
        bvh_builder.update_configuration(config);
        prim_ray_gen.update_configuration(config);
        sec_ray_gen.update_configuration(config);
        tracer.update_configuration(config);
        ray_shader.update_configuration(config);

        /* Renderer::set_up_frame: the accelerator, then a clear framebuffer */
        CHECK(bvh_builder.build_lbvh(scene));
        CHECK(framebuffer.clear());

        uint64_t total_ray_count = 0, total_sec_ray_count = 0;
        const size_t sample_count = pixel_count * prim_ray_gen.get_spp();
        for (size_t offset = 0; offset < sample_count; offset += tile_size) {
            RayBundle* ray_in = &ray_bundle_1;
            RayBundle* ray_out = &ray_bundle_2;
            size_t current_tile_size = tile_size;
            if (sample_count - offset < tile_size) current_tile_size = sample_count - offset;
            CHECK(prim_ray_gen.generate(scene.camera, *ray_in, fb_size, current_tile_size, offset));
            total_ray_count += current_tile_size;
            CHECK(tracer.trace(scene, (int32_t)current_tile_size, *ray_in, hit_bundle));
            CHECK(tracer.shadow_trace(scene, (int32_t)current_tile_size, *ray_in, hit_bundle));
            CHECK(ray_shader.shade(*ray_in, hit_bundle, scene, scene.cubemap, framebuffer,
                                   current_tile_size, true));
            size_t sec_ray_count = current_tile_size;
            for (uint32_t bounce = 0; bounce < max_bounces; ++bounce) {
                const size_t sec_ray_in = sec_ray_count;
                CHECK(sec_ray_gen.generate(scene, *ray_in, sec_ray_in, hit_bundle, *ray_out,
                                           &sec_ray_count));
                std::swap(ray_in, ray_out);
                if (!sec_ray_count) break;
                total_ray_count += sec_ray_count;
                total_sec_ray_count += sec_ray_count;
                CHECK(tracer.trace(scene, (int32_t)sec_ray_count, *ray_in, hit_bundle, true));
                CHECK(tracer.shadow_trace(scene, (int32_t)sec_ray_count, *ray_in, hit_bundle,
                                          true));
                CHECK(ray_shader.shade(*ray_in, hit_bundle, scene, scene.cubemap, framebuffer,
                                       sec_ray_count));
            }
        }

        /* Renderer::copy_framebuffer into a device "texture" */
        const memory_id tex_id = device.new_memory();
        DeviceMemory& tex = device.memory(tex_id);
        CHECK(tex.initialize(4 * pixel_count));
        CHECK(framebuffer.copy(tex));
        std::vector<uint32_t> image(3 * pixel_count);
        std::vector<uint8_t> rgba(4 * pixel_count);
        CHECK(framebuffer.image_mem().read(image.size() * 4, image.data()) != 0);
        CHECK(tex.read(rgba.size(), rgba.data()) != 0);
        uint32_t status = 0;
        CHECK(rt_device_status(device.context(), &status) != RT_OK || status != 0);
        const uint64_t stats[2] = {total_ray_count, total_sec_ray_count};
        CHECK(!spill(dir + "/image.bin", image.data(), image.size() * 4) ||
              !spill(dir + "/rgba.bin", rgba.data(), rgba.size()) ||
              !spill(dir + "/stats.bin", stats, sizeof(stats)));
        CHECK(device.delete_memory(tex_id));
    }
    CHECK(device.shutdown());
    return 0;
}
