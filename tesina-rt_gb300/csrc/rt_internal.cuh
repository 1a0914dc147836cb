// rt_internal.cuh — device-side data layout and exact-arithmetic helpers shared
// by the LBVH builder and the tracer.  Every translation unit is compiled with
// --fmad=false: single-precision arithmetic is evaluated in the reference
// kernels' operation order without contraction, so results are bit-identical
// to the IEEE restatement of the reference math.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/rt_cuda.h"

namespace rt {

// --------------------------------------------------------------------------
// BVH layout in HBM
// --------------------------------------------------------------------------
// Interior nodes are stored as child pairs (64 B = 4 x float4), indexed by
// the split position of the Karras radix tree they come from:
//   n0 = (c0.lo.x, c0.lo.y, c0.lo.z, c0.hi.x)
//   n1 = (c0.hi.y, c0.hi.z, c1.lo.x, c1.lo.y)
//   n2 = (c1.lo.z, c1.hi.x, c1.hi.y, c1.hi.z)
//   n3 = (ref0, ref1, cnt0, cnt1) as int: cnt == 0 -> ref is an interior node
//        index; cnt > 0 -> leaf over sorted triangles [ref, ref + cnt).
// c0 is the left child (lower Morton range), c1 the right child.
struct BvhHeader {
    int32_t root_ref;       // interior node index, or first triangle of a root leaf
    int32_t root_cnt;       // 0: interior root; > 0: the whole tree is one leaf
    uint32_t n_tris;
    uint32_t status;        // RT_DEV_* bits raised while building
    float4 root_lo;
    float4 root_hi;
};

// Triangle records in sorted order, 48 B: v0, e1 = v1 - v0, e2 = v2 - v0
// (the same float subtractions as leaf_hit, trace-bvh.cl:297-298).
struct TriRec {
    float4 v0, e1, e2;
};

// Views passed to kernels.
// Render kernel variants a context keeps per-variant state for.
constexpr int kMaxRenderVariants = 32;

struct SceneView {
    const float4* __restrict__ nodes;
    const float4* __restrict__ tris;      // 3 float4 per triangle
    const uint32_t* __restrict__ idx;     // sorted index buffer (3 per tri)
    const float4* __restrict__ nrm;       // vertex normals
    const uint32_t* __restrict__ map;     // sorted material map
    const rt_material* __restrict__ mats;
    const BvhHeader* __restrict__ hdr;
};

// --------------------------------------------------------------------------
// exact float3 helpers (operation order of the OpenCL built-ins as restated)
// --------------------------------------------------------------------------
struct f3 {
    float x, y, z;
};
__device__ __forceinline__ f3 mk3(float x, float y, float z) { return f3{x, y, z}; }
__device__ __forceinline__ f3 ld3(const float4& v) { return f3{v.x, v.y, v.z}; }
__device__ __forceinline__ f3 add(f3 a, f3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ f3 sub(f3 a, f3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ f3 mul(f3 a, f3 b) { return mk3(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ f3 muls(f3 a, float s) { return mk3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ f3 neg(f3 a) { return mk3(-a.x, -a.y, -a.z); }
__device__ __forceinline__ float dot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ f3 cross(f3 a, f3 b) {
    return mk3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
// normalize(v) = v * (1 / sqrt(dot(v, v))), zero vector unchanged
// (correctly rounded sqrt and division: -prec-sqrt / -prec-div defaults).
__device__ __forceinline__ f3 normalize(f3 v) {
    float d = dot(v, v);
    if (d == 0.0f) return v;
    float inv = 1.0f / sqrtf(d);
    return muls(v, inv);
}
__device__ __forceinline__ float clamp01(float x) { return fminf(fmaxf(x, 0.0f), 1.0f); }
// OpenCL max / min ("y if x < y, else x"), used by the shadow slab test.
__device__ __forceinline__ float cl_max(float x, float y) { return (x < y) ? y : x; }
__device__ __forceinline__ float cl_min(float x, float y) { return (y < x) ? y : x; }

// Ray state during traversal.  Axes whose |1/d| <= 1e-6 are excluded from the
// slab test by the reference (trace-bvh.cl:262-270); storing NaN in those
// lanes gives the same result without branches, because fmin/fmax (and the
// OpenCL max/min as used) return the non-NaN operand.
struct TRay {
    f3 o, d, inv;   // inv: masked inverse direction
    float tmin;
};

__device__ __forceinline__ float mask_inv(float inv) {
    return fabsf(inv) > 1e-6f ? inv : __int_as_float(0x7fc00000);
}

__device__ __forceinline__ TRay make_tray(f3 o, f3 d, f3 inv, float tmin) {
    TRay r;
    r.o = o;
    r.d = d;
    r.inv = mk3(mask_inv(inv.x), mask_inv(inv.y), mask_inv(inv.z));
    r.tmin = tmin;
    return r;
}

// Three-operand min / max (sm_100+): exact selections with the same NaN
// rule as fminf / fmaxf (a NaN operand is dropped), so chaining them gives the
// same value as the reference's two-operand sequence.
__device__ __forceinline__ float max3f(float a, float b, float c) {
    float d;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}
__device__ __forceinline__ float min3f(float a, float b, float c) {
    float d;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}

// Slab test of bbox_hit (trace-bvh.cl:247-273).  Returns the entry distance A
// = max(tMin, per-axis near) and whether A <= min(tMax, per-axis far).  The
// per-axis selections are exact, so their grouping does not change A.
__device__ __forceinline__ bool slab(const TRay& r, float tmax, float lox, float loy, float loz,
                                     float hix, float hiy, float hiz, float& A) {
    float ltx = (lox - r.o.x) * r.inv.x, htx = (hix - r.o.x) * r.inv.x;
    float lty = (loy - r.o.y) * r.inv.y, hty = (hiy - r.o.y) * r.inv.y;
    float ltz = (loz - r.o.z) * r.inv.z, htz = (hiz - r.o.z) * r.inv.z;
    const float tmin = fmaxf(max3f(r.tmin, fminf(ltx, htx), fminf(lty, hty)), fminf(ltz, htz));
    tmax = fminf(min3f(tmax, fmaxf(ltx, htx), fmaxf(lty, hty)), fmaxf(ltz, htz));
    A = tmin;
    return tmin <= tmax;
}

// Slab test of the shadow kernel (shadow-trace-bvh.cl:160-186, OpenCL max/min).
__device__ __forceinline__ bool slab_shadow(const TRay& r, float tmax, float lox, float loy,
                                            float loz, float hix, float hiy, float hiz) {
    float ltx = (lox - r.o.x) * r.inv.x, htx = (hix - r.o.x) * r.inv.x;
    float lty = (loy - r.o.y) * r.inv.y, hty = (hiy - r.o.y) * r.inv.y;
    float ltz = (loz - r.o.z) * r.inv.z, htz = (hiz - r.o.z) * r.inv.z;
    float tmin = r.tmin;
    tmin = cl_max(tmin, cl_min(ltx, htx));
    tmax = cl_min(tmax, cl_max(ltx, htx));
    tmin = cl_max(tmin, cl_min(lty, hty));
    tmax = cl_min(tmax, cl_max(lty, hty));
    tmin = cl_max(tmin, cl_min(ltz, htz));
    tmax = cl_min(tmax, cl_max(ltz, htz));
    return tmin <= tmax;
}

// Möller–Trumbore of leaf_hit (trace-bvh.cl:275-328).
__device__ __forceinline__ bool mt(const float4* __restrict__ tris, uint32_t i, f3 o, f3 d, float& t,
                                   float& u, float& v) {
    const float4 a = __ldg(&tris[3 * (size_t)i + 0]);
    const float4 b = __ldg(&tris[3 * (size_t)i + 1]);
    const float4 c = __ldg(&tris[3 * (size_t)i + 2]);
    f3 v0 = ld3(a), e1 = ld3(b), e2 = ld3(c);
    f3 h = cross(d, e2);
    float aa = dot(e1, h);
    if (aa > -1e-26f && aa < 1e-26f) return false;
    float f = 1.0f / aa;
    f3 s = sub(o, v0);
    u = f * dot(s, h);
    if (u < 0.0f || u > 1.0f) return false;
    f3 q = cross(s, e1);
    v = f * dot(d, q);
    if (v < 0.0f || u + v > 1.0f) return false;
    t = f * dot(e2, q);
    return true;
}

}  // namespace rt
