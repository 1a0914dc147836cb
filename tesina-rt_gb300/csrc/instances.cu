// instances.cu — multi-root (instanced) scenes: the reference's trace_multi /
// shadow_trace_multi (src/kernel/trace-bvh.cl:420-463, :84-181;
// src/kernel/shadow-trace-bvh.cl:317-373) with its BVHRoot records
// (src/rt/scene.cpp:595-703), rendered by one persistent kernel.
//
// An instance is a built scene (its LBVH, triangles, materials) under a
// row-major 4x4 transform and its inverse, given by the caller as the
// reference's objects give them.  Per ray and instance: the ray goes into the
// object's space through the inverse (with the homogeneous divide of
// multiply_point / multiply_vector), is traversed with the scene's own
// closest_hit, and the hit's distance is measured again in world space
// (distance from the origin to the hit point taken back through the
// transform); the nearest wins, the first instance on a tie.  The hit
// normal is the object-space normal through the transform, not renormalised.
// Shadow rays test every instance; a spot light's cone test leaves the point
// lit, as in shadow_trace_multi (the single-root kernel treats it as shadow).
// Refracting scenes are not taken (rt_render renders those).
#include <cuda_runtime.h>
#include <stdint.h>

#include <new>
#include <vector>

#include "../../include/rt_cuda.h"
#include "ctx_internal.h"
#include "rt_internal.cuh"
#include "trace.cuh"
#include "trace_dev.cuh"

namespace rt {

struct InstanceRoot {
    SceneView scene;
    float tr[16], trinv[16];
};

struct InstanceArgs {
    const InstanceRoot* roots;
    int count;
    rt_lights lights;
    rt_camera cam;
    int width, height, max_bounces, chunk;
    uint8_t* rgba;
    uint32_t* image_rgb;
    rt_render_stats* stats;
    uint32_t* work_counter;
    uint32_t* status;
    float inv1e6;
};

// M (v, w): four products summed left to right per row, then divided by the
// fourth row's value when |w'| > 1e-26.
__device__ __forceinline__ f3 mat_apply(const float* M, f3 v, float w) {
    float r[4];
#pragma unroll
    for (int k = 0; k < 4; ++k)
        r[k] = M[4 * k] * v.x + M[4 * k + 1] * v.y + M[4 * k + 2] * v.z + M[4 * k + 3] * w;
    if (fabsf(r[3]) > 1e-26f) {
        const float d = r[3];
        r[0] = r[0] / d;
        r[1] = r[1] / d;
        r[2] = r[2] / d;
    }
    return mk3(r[0], r[1], r[2]);
}

struct MultiHit {
    Hit h;        // id local to the instance's scene; t in world space
    int root;
};

__device__ __forceinline__ MultiHit closest_multi(const InstanceArgs& A, f3 o, f3 d, float tmin,
                                                  float tmax) {
    MultiHit best{{-1, 0.f, 0.f, 0.f}, -1};
    for (int i = 0; i < A.count; ++i) {
        const InstanceRoot& R = A.roots[i];
        const f3 td = mat_apply(R.trinv, d, 0.0f);
        const f3 to = mat_apply(R.trinv, o, 1.0f);
        const TRay tr = make_tray(to, td, mk3(1.0f / td.x, 1.0f / td.y, 1.0f / td.z), tmin);
        const BvhHeader H = *R.scene.hdr;
        Hit h = closest_hit(R.scene, H, tr, tmax, A.status);
        if (h.id >= 0) {
            const f3 hp = mat_apply(R.tr, add(to, muls(td, h.t)), 1.0f);
            const f3 dv = sub(hp, o);
            h.t = sqrtf(dot(dv, dv));
        }
        if (h.id >= 0 && (best.h.id < 0 || h.t < best.h.t)) {
            best.h = h;
            best.root = i;
        }
    }
    return best;
}

__device__ __forceinline__ bool occluded_multi(const InstanceArgs& A, const rt_light& L, f3 hp) {
    f3 dir;
    if (L.type == RT_DIR_L) {
        dir = neg(mk3(L.dir[0], L.dir[1], L.dir[2]));
    } else if (L.type == RT_SPOT_L) {
        dir = normalize(sub(mk3(L.pos[0], L.pos[1], L.pos[2]), hp));
        if (dot(dir, mk3(L.dir[0], L.dir[1], L.dir[2])) < L.angle) return false;
    } else if (L.type == RT_POINT_L) {
        dir = normalize(sub(mk3(L.pos[0], L.pos[1], L.pos[2]), hp));
    } else {
        return false;
    }
    for (int i = 0; i < A.count; ++i) {
        const InstanceRoot& R = A.roots[i];
        const f3 td = mat_apply(R.trinv, dir, 0.0f);
        const f3 to = mat_apply(R.trinv, hp, 1.0f);
        const TRay tr = make_tray(to, td, mk3(1.0f / td.x, 1.0f / td.y, 1.0f / td.z), 0.01f);
        const BvhHeader H = *R.scene.hdr;
        if (any_hit(R.scene, H, tr, 1e37f, A.status)) return true;
    }
    return false;
}

// One pixel's Whitted path over the instances (reflection only).
__device__ __forceinline__ PixelResult render_pixel_multi(const InstanceArgs& A, int x, int y) {
    PixelResult res = {0, 0, 0, 0, 0, 0};
    f3 o = mk3(A.cam.pos[0], A.cam.pos[1], A.cam.pos[2]);
    f3 d = primary_dir(A.cam, x, y, A.width, A.height, 0.0f, 0.0f);
    float tmin = 0.0f, tmax = 1e36f, contribution = 1.0f;
    for (int bounce = 0;; ++bounce) {
        const MultiHit mh = closest_multi(A, o, d, tmin, tmax);
        if (mh.h.id < 0) break;
        ++res.hits;
        const InstanceRoot& R = A.roots[mh.root];
        const SceneView& S = R.scene;
        const f3 hp = add(o, muls(d, mh.h.t));
        const uint32_t* ix = S.idx + 3 * (size_t)mh.h.id;
        const f3 n0 = normalize(ld3(__ldg(&S.nrm[__ldg(ix)])));
        const f3 n1 = normalize(ld3(__ldg(&S.nrm[__ldg(ix + 1)])));
        const f3 n2 = normalize(ld3(__ldg(&S.nrm[__ldg(ix + 2)])));
        const float w = 1.0f - (mh.h.u + mh.h.v);
        f3 n = normalize(add(add(muls(n0, w), muls(n2, mh.h.v)), muls(n1, mh.h.u)));
        n = mat_apply(R.tr, n, 0.0f);
        if (dot(n, d) > 0.0f) n = muls(n, -1.0f);
        const rt_material mat = S.mats[__ldg(&S.map[mh.h.id])];
        uint32_t mask = 0;
        for (int l = 0; l < A.lights.count; ++l)
            if (occluded_multi(A, A.lights.light[l], hp)) mask |= 1u << l;
        res.shadow += (uint32_t)A.lights.count;
        const uint3 c = shade_hit(A.lights, mat, hp, n, d, contribution, mask);
        res.r += c.x;
        res.g += c.y;
        res.b += c.z;
        if (bounce == A.max_bounces) break;
        if (!(mat.reflectiveness > 0.0f)) break;
        f3 nd;
        reflect_ray(d, n, nd);
        contribution = contribution * mat.reflectiveness * 1.0f;
        o = hp;
        d = nd;
        tmin = 0.0001f;
        tmax = 1e37f;
        ++res.secondary;
    }
    return res;
}

__global__ void __launch_bounds__(128, 6) k_render_instances(InstanceArgs A) {
    __shared__ InstanceArgs sA;
    if (threadIdx.x == 0) sA = A;
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int pixels = sA.width * sA.height;
    uint64_t n_sec = 0, n_shadow = 0, n_hits = 0, n_prim = 0;
    for (;;) {
        int base0 = 0;
        if (lane == 0) base0 = (int)atomicAdd(sA.work_counter, (unsigned)sA.chunk);
        base0 = __shfl_sync(0xffffffffu, base0, 0);
        if (base0 >= pixels) break;
        for (int base = base0; base < base0 + sA.chunk && base < pixels; base += 32) {
            const int gid = base + lane;
            if (gid >= pixels) continue;
            int x, y;
            pixel_of(warp_tile_order(gid, sA.width, sA.height), sA.width, sA.height, 32, x, y);
            const PixelResult pr = render_pixel_multi(sA, x, y);
            ++n_prim;
            n_sec += pr.secondary;
            n_shadow += pr.shadow;
            n_hits += pr.hits;
            const int pix = sA.width * y + x;
            if (sA.image_rgb) {
                sA.image_rgb[3 * (size_t)pix] = pr.r;
                sA.image_rgb[3 * (size_t)pix + 1] = pr.g;
                sA.image_rgb[3 * (size_t)pix + 2] = pr.b;
            }
            uchar4 px;
            px.x = to_unorm8(pr.r, sA.inv1e6);
            px.y = to_unorm8(pr.g, sA.inv1e6);
            px.z = to_unorm8(pr.b, sA.inv1e6);
            px.w = 255;
            reinterpret_cast<uchar4*>(sA.rgba)[pix] = px;
        }
    }
    if (sA.stats) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            n_prim += __shfl_down_sync(0xffffffffu, n_prim, o);
            n_sec += __shfl_down_sync(0xffffffffu, n_sec, o);
            n_shadow += __shfl_down_sync(0xffffffffu, n_shadow, o);
            n_hits += __shfl_down_sync(0xffffffffu, n_hits, o);
        }
        if (lane == 0 && n_prim) {
            atomicAdd((unsigned long long*)&sA.stats->primary_rays, (unsigned long long)n_prim);
            atomicAdd((unsigned long long*)&sA.stats->secondary_rays, (unsigned long long)n_sec);
            atomicAdd((unsigned long long*)&sA.stats->shadow_rays, (unsigned long long)n_shadow);
            atomicAdd((unsigned long long*)&sA.stats->hits, (unsigned long long)n_hits);
        }
    }
}

}  // namespace rt

struct rt_instances {
    std::vector<rt_scene*> scenes;
    std::vector<int32_t> inst_scene;
    std::vector<float> tr, trinv;
    rt_lights lights;
    rt::InstanceRoot* d_roots = nullptr;
};

namespace {

#define fail rt::set_error

#define CU(call)                                                                              \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess)                                                                \
            return fail(RT_ERR_CUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_),  \
                        __FILE__, __LINE__);                                                  \
    } while (0)

int32_t upload_roots(rt_instances* I, cudaStream_t s) {
    std::vector<rt::InstanceRoot> roots(I->inst_scene.size());
    for (size_t i = 0; i < roots.size(); ++i) {
        roots[i].scene = rt::scene_view(I->scenes[I->inst_scene[i]]);
        for (int k = 0; k < 16; ++k) {
            roots[i].tr[k] = I->tr[16 * i + k];
            roots[i].trinv[k] = I->trinv[16 * i + k];
        }
    }
    CU(cudaMemcpyAsync(I->d_roots, roots.data(), sizeof(rt::InstanceRoot) * roots.size(),
                       cudaMemcpyHostToDevice, s));
    CU(cudaStreamSynchronize(s));
    return RT_OK;
}

}  // namespace

extern "C" {

int32_t rt_instances_create(rt_ctx* c, rt_scene* const* scenes, int32_t scene_count,
                            const int32_t* inst_scene, const float* tr, const float* tr_inv,
                            int32_t count, const rt_lights* lights, rt_instances** out) {
    if (!c || !scenes || !inst_scene || !tr || !tr_inv || !lights || !out)
        return fail(RT_ERR_INVALID, "rt_instances_create: null argument");
    if (scene_count < 1 || count < 1 || count > 65536)
        return fail(RT_ERR_INVALID, "rt_instances_create: %d scenes, %d instances", scene_count,
                    count);
    if (lights->count < 1 || lights->count > RT_MAX_LIGHTS)
        return fail(RT_ERR_INVALID, "rt_instances_create: light count %d", lights->count);
    for (int k = 0; k < scene_count; ++k) {
        if (!scenes[k] || !scenes[k]->built)
            return fail(RT_ERR_NOT_BUILT, "rt_instances_create: scene %d has no BVH", k);
        if (scenes[k]->refracts)
            return fail(RT_ERR_INVALID, "rt_instances_create: scene %d refracts (rt_render "
                        "renders refraction)", k);
    }
    for (int i = 0; i < count; ++i)
        if (inst_scene[i] < 0 || inst_scene[i] >= scene_count)
            return fail(RT_ERR_INVALID, "rt_instances_create: instance %d names scene %d", i,
                        inst_scene[i]);
    rt_instances* I = new (std::nothrow) rt_instances();
    if (!I) return fail(RT_ERR_OOM, "rt_instances_create: host allocation failed");
    I->scenes.assign(scenes, scenes + scene_count);
    I->inst_scene.assign(inst_scene, inst_scene + count);
    I->tr.assign(tr, tr + 16 * (size_t)count);
    I->trinv.assign(tr_inv, tr_inv + 16 * (size_t)count);
    I->lights = *lights;
    if (cudaMalloc(&I->d_roots, sizeof(rt::InstanceRoot) * (size_t)count) != cudaSuccess) {
        cudaGetLastError();
        delete I;
        return fail(RT_ERR_OOM, "rt_instances_create: device allocation failed");
    }
    const int32_t r = upload_roots(I, c->stream);
    if (r) {
        cudaFree(I->d_roots);
        delete I;
        return r;
    }
    *out = I;
    return RT_OK;
}

int32_t rt_instances_set_transforms(rt_ctx* c, rt_instances* I, const float* tr,
                                    const float* tr_inv) {
    if (!c || !I || !tr || !tr_inv) return fail(RT_ERR_INVALID, "rt_instances_set_transforms: null");
    I->tr.assign(tr, tr + I->tr.size());
    I->trinv.assign(tr_inv, tr_inv + I->trinv.size());
    return upload_roots(I, c->stream);
}

int32_t rt_instances_render(rt_ctx* c, rt_instances* I, const rt_camera* cam, int32_t w, int32_t h,
                            int32_t max_bounces, uint8_t* rgba, uint32_t* img,
                            rt_render_stats* stats, rt_stream stream) {
    if (!c || !I || !cam || !rgba) return fail(RT_ERR_INVALID, "rt_instances_render: null argument");
    if (w <= 0 || h <= 0 || (int64_t)w * h > (1ll << 30) || max_bounces < 0 || max_bounces > 64)
        return fail(RT_ERR_INVALID, "rt_instances_render: bad size or depth");
    for (rt_scene* s : I->scenes)
        if (!s->built || s->refracts)
            return fail(RT_ERR_INVALID, "rt_instances_render: a scene is not built or refracts");
    cudaStream_t cs = stream ? (cudaStream_t)stream : c->stream;
    uint32_t* work = rt::work_counter(c, cs);
    if (!work) return fail(RT_ERR_OOM, "rt_instances_render: work counter");
    CU(cudaMemsetAsync(work, 0, sizeof(uint32_t), cs));
    rt::InstanceArgs A;
    A.roots = I->d_roots;
    A.count = (int)I->inst_scene.size();
    A.lights = I->lights;
    A.cam = *cam;
    A.width = w;
    A.height = h;
    A.max_bounces = max_bounces;
    A.chunk = 64;
    A.rgba = rgba;
    A.image_rgb = img;
    A.stats = stats;
    A.work_counter = work;
    A.status = c->d_status;
    A.inv1e6 = c->inv1e6;
    static int occ = -1;
    if (occ < 0) {
        int b = 0;
        CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, rt::k_render_instances, 128, 0));
        occ = b > 0 ? b : 1;
    }
    int64_t grid = (int64_t)c->num_sms * occ;
    const int64_t useful = ((int64_t)w * h + 127) / 128;
    if (grid > useful) grid = useful;
    rt::k_render_instances<<<(unsigned)grid, 128, 0, cs>>>(A);
    CU(cudaGetLastError());
    return RT_OK;
}

int32_t rt_instances_destroy(rt_ctx* c, rt_instances* I) {
    if (!I) return RT_OK;
    if (c) cudaStreamSynchronize(c->stream);
    cudaFree(I->d_roots);
    delete I;
    return RT_OK;
}

}  // extern "C"
