/*
 * Host stand-in for the OpenCL 1.2 types that the reference's fluid.h, cutil_math.h and
 * fluid_system_cuda.cu name (TEST INFRASTRUCTURE ONLY: the pinning harness in
 * oracle/ref_harness.cpp compiles the reference's kernels as host C++ against it).
 *
 * The vector types follow the OpenCL layout: cl_float3 is the same 16-byte type as
 * cl_float4 (components x, y, z, w, also reachable as s[0..3]); cl_int3 likewise.
 * ucl_int3 is the unsigned triple cutil_math.h overloads on (not an OpenCL type).
 */
#ifndef MG_REF_SHIM_CL_H
#define MG_REF_SHIM_CL_H
#include <stdint.h>

typedef float cl_float;
typedef int32_t cl_int;
typedef uint32_t cl_uint;
typedef int64_t cl_long;
typedef uint64_t cl_ulong;
typedef void* cl_mem;

typedef union cl_float4 {
    cl_float s[4];
    struct { cl_float x, y, z, w; };
} cl_float4;
typedef cl_float4 cl_float3;

typedef union cl_int4 {
    cl_int s[4];
    struct { cl_int x, y, z, w; };
} cl_int4;
typedef cl_int4 cl_int3;

typedef struct ucl_int3 {
    cl_uint x, y, z, w;
} ucl_int3;

#endif
