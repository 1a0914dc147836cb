/* opencl.h — ORACLE test infrastructure: the host-side OpenCL vector and
 * scalar types the reference's host headers name, for compiling its OBJ
 * loader on the CPU (no OpenCL runtime is involved).  Layouts follow the
 * OpenCL 1.1 host API: 3-component vectors occupy four floats. */
#ifndef ORACLE_SHIM_OPENCL_H
#define ORACLE_SHIM_OPENCL_H
#include <stdint.h>
typedef float cl_float;
typedef int32_t cl_int;
typedef uint32_t cl_uint;
typedef int8_t cl_char;
typedef uint8_t cl_uchar;
typedef int16_t cl_short;
typedef uint16_t cl_ushort;
typedef int64_t cl_long;
typedef uint64_t cl_ulong;
typedef union { cl_float s[2]; struct { cl_float x, y; }; } cl_float2;
typedef union { cl_float s[4]; struct { cl_float x, y, z, w; }; } cl_float4;
typedef cl_float4 cl_float3;
typedef union { cl_int s[4]; struct { cl_int x, y, z, w; }; } cl_int4;
typedef cl_int4 cl_int3;
typedef union { cl_int s[2]; struct { cl_int x, y; }; } cl_int2;
typedef union { cl_uint s[4]; struct { cl_uint x, y, z, w; }; } cl_uint4;
typedef cl_uint4 cl_uint3;
typedef union { cl_uint s[2]; struct { cl_uint x, y; }; } cl_uint2;
#endif
