/*
 * cl_shim_body.hpp — ORACLE test infrastructure.
 *
 * Minimal OpenCL C 1.1 built-in environment so that g++ can compile the
 * reference's kernel sources (src/kernel/*.cl) unmodified, as plain C++
 * functions run one work-item at a time on the CPU.  This header is included
 * *inside* a namespace by each wrapper translation unit, after all standard
 * headers, so that its scalar built-ins hide the C library's overloads.
 *
 * Built-ins follow the OpenCL 1.1 specification; where the specification
 * leaves accuracy to the implementation (normalize, pow) the same choice as
 * the restatement in oracle/rt_cpu_ref.cpp is made: normalize(v) =
 * v * (1 / sqrt(dot(v, v))), pow = the C library's powf.
 *
 * Vector literals "(floatN)(a, b, c)" parse in C++ as a cast of a comma
 * expression, i.e. a broadcast of the last element; every literal in the
 * kernels used here repeats one value, so the result is the same.
 */

typedef unsigned int uint;
typedef unsigned char uchar;
typedef unsigned short ushort;

struct float3;
struct swz3 {
    float x, y, z, w;
    inline operator float3() const;
};

struct alignas(8) float2 {
    union {
        struct { float x, y; };
        struct { float s0, s1; };
    };
    float2() = default;
    float2(float v) : x(v), y(v) {}
    float2(float a, float b) : x(a), y(b) {}
};

struct alignas(16) float3 {
    union {
        struct { float x, y, z, w; };
        struct { float s0, s1, s2, s3; };
        swz3 xyz;
    };
    float3() = default;
    float3(float v) : x(v), y(v), z(v), w(0.f) {}
    float3(float a, float b, float c) : x(a), y(b), z(c), w(0.f) {}
};

struct alignas(16) float4 {
    union {
        struct { float x, y, z, w; };
        struct { float s0, s1, s2, s3; };
        swz3 xyz;
    };
    float4() = default;
    float4(float v) : x(v), y(v), z(v), w(v) {}
    float4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
};

struct int2 {
    int x, y;
    int2() = default;
    int2(int v) : x(v), y(v) {}
};

inline swz3::operator float3() const { return float3(x, y, z); }

/* ---- arithmetic ---------------------------------------------------------- */
#define CLSHIM_V3_BIN(op)                                                                    \
    inline float3 operator op(float3 a, float3 b) { return float3(a.x op b.x, a.y op b.y, a.z op b.z); } \
    inline float3 operator op(float3 a, float s) { return float3(a.x op s, a.y op s, a.z op s); }       \
    inline float3 operator op(float s, float3 a) { return float3(s op a.x, s op a.y, s op a.z); }       \
    inline float3& operator op##=(float3& a, float3 b) { a = a op b; return a; }                      \
    inline float3& operator op##=(float3& a, float s) { a = a op s; return a; }
CLSHIM_V3_BIN(+)
CLSHIM_V3_BIN(-)
CLSHIM_V3_BIN(*)
CLSHIM_V3_BIN(/)
#undef CLSHIM_V3_BIN

#define CLSHIM_V4_BIN(op)                                                                   \
    inline float4 operator op(float4 a, float4 b) {                                          \
        return float4(a.x op b.x, a.y op b.y, a.z op b.z, a.w op b.w);                       \
    }                                                                                        \
    inline float4 operator op(float4 a, float s) { return float4(a.x op s, a.y op s, a.z op s, a.w op s); } \
    inline float4 operator op(float s, float4 a) { return float4(s op a.x, s op a.y, s op a.z, s op a.w); } \
    inline float4& operator op##=(float4& a, float4 b) { a = a op b; return a; }             \
    inline float4& operator op##=(float4& a, float s) { a = a op s; return a; }
CLSHIM_V4_BIN(+)
CLSHIM_V4_BIN(-)
CLSHIM_V4_BIN(*)
CLSHIM_V4_BIN(/)
#undef CLSHIM_V4_BIN

#define CLSHIM_V2_BIN(op)                                                                    \
    inline float2 operator op(float2 a, float2 b) { return float2(a.x op b.x, a.y op b.y); } \
    inline float2 operator op(float2 a, float s) { return float2(a.x op s, a.y op s); }      \
    inline float2 operator op(float s, float2 a) { return float2(s op a.x, s op a.y); }
CLSHIM_V2_BIN(+)
CLSHIM_V2_BIN(-)
CLSHIM_V2_BIN(*)
CLSHIM_V2_BIN(/)
#undef CLSHIM_V2_BIN

/* OpenCL's vector literal (float4)(v, s) with v a float3: in C++ the
 * parenthesised pair is a comma expression, so the comma of (float3, float)
 * builds the pair and the cast turns it into the float4 OpenCL means
 * (multiply_vector / multiply_point, trace-bvh.cl:84-113). */
struct V3S {
    float3 v;
    float s;
    operator float4() const { return float4(v.x, v.y, v.z, s); }
};
inline V3S operator,(float3 a, float b) { return V3S{a, b}; }

inline float3 operator-(float3 a) { return float3(-a.x, -a.y, -a.z); }
inline float4 operator-(float4 a) { return float4(-a.x, -a.y, -a.z, -a.w); }

/* ---- scalar built-ins ---------------------------------------------------- */
inline float fmax(float a, float b) { return std::fmax(a, b); }
inline float fmin(float a, float b) { return std::fmin(a, b); }
inline float fabs(float a) { return std::fabs(a); }
inline float fdim(float a, float b) { return std::fdim(a, b); }
inline float sqrt(float a) { return std::sqrt(a); }
/* pow(x, 5) (the Schlick term of refraction) as the product in double
 * precision rounded once, as the oracle and the CUDA path evaluate it (within
 * the 16 ulp OpenCL allows pow); other exponents through the C library. */
inline float pow(float a, float b) {
    if (b == 5.0f) {
        const double p = (double)a;
        return (float)((((p * p) * p) * p) * p);
    }
    return std::pow(a, b);
}
inline float ceil(float a) { return std::ceil(a); }
inline float floor(float a) { return std::floor(a); }
inline float max(float x, float y) { return (x < y) ? y : x; }
inline float min(float x, float y) { return (y < x) ? y : x; }
inline int max(int x, int y) { return (x < y) ? y : x; }
inline int min(int x, int y) { return (y < x) ? y : x; }
inline float clamp(float x, float lo, float hi) { return fmin(fmax(x, lo), hi); }
inline float sin(float a) { return std::sin(a); }
inline float cos(float a) { return std::cos(a); }
inline float fmod(float a, float b) { return std::fmod(a, b); }

/* ---- vector built-ins ---------------------------------------------------- */
inline float3 fmax(float3 a, float3 b) { return float3(fmax(a.x, b.x), fmax(a.y, b.y), fmax(a.z, b.z)); }
inline float3 fmin(float3 a, float3 b) { return float3(fmin(a.x, b.x), fmin(a.y, b.y), fmin(a.z, b.z)); }
inline float4 fmax(float4 a, float4 b) {
    return float4(fmax(a.x, b.x), fmax(a.y, b.y), fmax(a.z, b.z), fmax(a.w, b.w));
}
inline float4 fmin(float4 a, float4 b) {
    return float4(fmin(a.x, b.x), fmin(a.y, b.y), fmin(a.z, b.z), fmin(a.w, b.w));
}
inline float3 max(float3 a, float3 b) { return float3(max(a.x, b.x), max(a.y, b.y), max(a.z, b.z)); }
inline float3 min(float3 a, float3 b) { return float3(min(a.x, b.x), min(a.y, b.y), min(a.z, b.z)); }
inline float3 fabs(float3 a) { return float3(fabs(a.x), fabs(a.y), fabs(a.z)); }
inline float3 fdim(float3 a, float3 b) { return float3(fdim(a.x, b.x), fdim(a.y, b.y), fdim(a.z, b.z)); }
inline float3 clamp(float3 x, float3 lo, float3 hi) { return fmin(fmax(x, lo), hi); }
inline float3 clamp(float3 x, float lo, float hi) { return fmin(fmax(x, float3(lo)), float3(hi)); }
inline float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float dot(float4 a, float4 b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }
inline float3 cross(float3 a, float3 b) {
    return float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline float length(float3 a) { return sqrt(dot(a, a)); }
inline float distance(float3 a, float3 b) { return length(a - b); }
inline float3 normalize(float3 v) {
    float d = dot(v, v);
    if (d == 0.0f) return v;
    float inv = 1.0f / sqrt(d);
    return v * inv;
}

/* ---- work-item functions ------------------------------------------------- */
struct WorkItem {
    size_t gid, goff, gsize, lid, lsize, grp, ngrp;
};
inline thread_local WorkItem g_wi = {0, 0, 1, 0, 1, 0, 1};
inline size_t get_global_id(int) { return g_wi.gid; }
inline size_t get_global_offset(int) { return g_wi.goff; }
inline size_t get_global_size(int) { return g_wi.gsize; }
inline size_t get_local_id(int) { return g_wi.lid; }
inline size_t get_local_size(int) { return g_wi.lsize; }
inline size_t get_group_id(int) { return g_wi.grp; }
inline size_t get_num_groups(int) { return g_wi.ngrp; }

enum { CLK_LOCAL_MEM_FENCE = 1, CLK_GLOBAL_MEM_FENCE = 2 };
/* A kernel run one work-item at a time has nothing to wait for; a kernel run
 * as an emulated work-group (ref_emit.cpp) sets the hook to its group's
 * barrier on every thread of the group. */
inline thread_local void (*g_barrier_hook)(void) = nullptr;
inline void barrier(int) {
    if (g_barrier_hook) g_barrier_hook();
}
inline int atomic_add(int* p, int v) { return __atomic_fetch_add(p, v, __ATOMIC_SEQ_CST); }
inline unsigned atomic_add(unsigned* p, unsigned v) { return __atomic_fetch_add(p, v, __ATOMIC_SEQ_CST); }

/* ---- images: untextured scenes only; reads return 0 ---------------------- */
struct image2d_t {
    int w, h;
};
typedef int sampler_t;
enum {
    CLK_NORMALIZED_COORDS_TRUE = 1,
    CLK_ADDRESS_REPEAT = 2,
    CLK_ADDRESS_CLAMP_TO_EDGE = 4,
    CLK_FILTER_LINEAR = 8
};
inline float4 read_imagef(image2d_t, sampler_t, float2) { return float4(0.f); }
inline void write_imagef(image2d_t, int2, float4) {}
inline int get_image_width(image2d_t i) { return i.w; }
inline int get_image_height(image2d_t i) { return i.h; }

/* ---- address-space and access qualifiers --------------------------------- */
#define kernel
#define __kernel
#define global
#define __global
#define local
#define __local
#define constant
#define __constant
#define private
#define __private
#define read_only
#define write_only
#define __read_only
#define __write_only
