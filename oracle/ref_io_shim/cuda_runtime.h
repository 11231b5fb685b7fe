/*
 * Host stand-in for <cuda_runtime.h>, used only to compile libmat's Houdini
 * geometry writer (src/IO/IO_CUDA/io_utils.cpp) with g++ so that the
 * oracle's writer can be checked against it byte for byte.  The writer only
 * needs CUDA's plain vector structs.  Test infrastructure: nothing in the
 * product includes this file.
 */
#ifndef RPD_REF_IO_SHIM_CUDA_RUNTIME_H
#define RPD_REF_IO_SHIM_CUDA_RUNTIME_H

struct alignas(8) int2 { int x, y; };
struct int3 { int x, y, z; };
struct alignas(16) int4 { int x, y, z, w; };
struct alignas(8) uint2 { unsigned int x, y; };
struct uint3 { unsigned int x, y, z; };
struct alignas(16) uint4 { unsigned int x, y, z, w; };
struct alignas(8) float2 { float x, y; };
struct float3 { float x, y, z; };
struct alignas(16) float4 { float x, y, z, w; };

#endif
