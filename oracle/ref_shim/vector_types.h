/* Host-side stand-in for CUDA's vector_types.h, written for this project's
 * oracle.  It lets the reference's __device__ helper files compile as plain
 * host C++ (test infrastructure only).  Layouts follow the public CUDA
 * documentation: float3/int3 are three packed 4-byte members, float2 is
 * 8-byte aligned, float4 is 16-byte aligned. */
#ifndef FG_SHIM_VECTOR_TYPES_H
#define FG_SHIM_VECTOR_TYPES_H

#define __device__
#define __host__
#define __global__
#define __constant__
#define __shared__
#define __forceinline__ inline

struct float2 { float x, y; } __attribute__((aligned(8)));
struct float3 { float x, y, z; };
struct alignas(16) float4 { float x, y, z, w; };
struct int2 { int x, y; } __attribute__((aligned(8)));
struct int3 { int x, y, z; };
struct uint2 { unsigned int x, y; } __attribute__((aligned(8)));
struct uint3 { unsigned int x, y, z; };
typedef unsigned int uint;

#endif
