/*
 * ref_host.h - host stand-ins for the CUDA names the reference's kernels use, so that their
 * source compiles as host C++ (TEST INFRASTRUCTURE ONLY: the pinning harness
 * oracle/ref_harness.cpp, built into oracle/_ref/ from the reference's own files).
 *
 * One "thread" runs at a time: the harness loops a kernel body over every particle index,
 * setting blockIdx/blockDim/threadIdx, so atomicAdd is a plain read-modify-write whose
 * returned value is the serial arrival rank, and __syncthreads has nothing to wait for (the
 * pinned kernels use no shared memory).  The CUDA vector types cutil_math.h overloads on
 * (float2, float4, int2, int4) are plain structs with their make_* constructors; the
 * cl_float3 / cl_int3 / ucl_int3 element constructors come with them because cutil_math.h
 * calls the three-component forms before defining the others.
 */
#ifndef MG_REF_HOST_H
#define MG_REF_HOST_H

#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <CL/cl.h>

#define __device__
#define __global__
#define __host__
#define __constant
#define __constant__
#define __forceinline__ inline

struct mg_ref_dim3 {
    unsigned int x, y, z;
};
static mg_ref_dim3 blockIdx, blockDim, threadIdx;

static inline int __mul24(int a, int b) { return a * b; }
static inline void __syncthreads(void) {}
static inline unsigned int atomicAdd(unsigned int* a, unsigned int v) {
    unsigned int old = *a;
    *a = old + v;
    return old;
}
static inline float atomicAdd(float* a, float v) {
    float old = *a;
    *a = old + v;
    return old;
}
static inline int max(int a, int b) { return a > b ? a : b; }
static inline int min(int a, int b) { return a < b ? a : b; }

struct float2 { float x, y; };
struct float4 { float x, y, z, w; };
struct int2 { int x, y; };
struct int4 { int x, y, z, w; };
static inline float2 make_float2(float x, float y) { float2 r = {x, y}; return r; }
static inline float4 make_float4(float x, float y, float z, float w) { float4 r = {x, y, z, w}; return r; }
static inline int2 make_int2(int x, int y) { int2 r = {x, y}; return r; }
static inline int4 make_int4(int x, int y, int z, int w) { int4 r = {x, y, z, w}; return r; }

static inline cl_float3 make_cl_float3(float x, float y, float z) {
    cl_float3 r;
    r.x = x; r.y = y; r.z = z; r.w = 0.f;
    return r;
}
static inline cl_int3 make_cl_int3(int x, int y, int z) {
    cl_int3 r;
    r.x = x; r.y = y; r.z = z; r.w = 0;
    return r;
}
static inline ucl_int3 make_ucl_int3(unsigned int x, unsigned int y, unsigned int z) {
    ucl_int3 r = {x, y, z, 0u};
    return r;
}

#endif
