/*
 * Host stand-in for <cuda_runtime.h>, used only to compile libmat's device
 * clipper (src/rpd3d/convex_cell.cu) with g++ as a single-threaded CPU
 * function, so the oracle can be checked against the reference's own code.
 * Test infrastructure: nothing in the product includes this file.
 *
 * Each CPU thread that runs the reference code gets its own copy of the
 * kernel's __shared__ pools (thread_local) and its own thread/block index.
 */
#ifndef RPD_REF_SHIM_CUDA_RUNTIME_H
#define RPD_REF_SHIM_CUDA_RUNTIME_H

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>

#define __host__
#define __device__
#define __global__
#define __forceinline__ inline
#define __shared__ static thread_local
#define __constant__ static
#define __align__(n) alignas(n)

typedef int cudaError_t;
#define cudaSuccess 0

struct uchar3 { unsigned char x, y, z; };
struct alignas(4) uchar4 { unsigned char x, y, z, w; };
struct alignas(8) int2 { int x, y; };
struct float3 { float x, y, z; };
struct alignas(16) float4 { float x, y, z, w; };
struct alignas(16) double4 { double x, y, z, w; };
struct uint3 { unsigned int x, y, z; };

inline uchar3 make_uchar3(unsigned char x, unsigned char y, unsigned char z) {
  uchar3 t = {x, y, z};
  return t;
}
inline uchar4 make_uchar4(unsigned char x, unsigned char y, unsigned char z,
                          unsigned char w) {
  uchar4 t = {x, y, z, w};
  return t;
}
inline int2 make_int2(int x, int y) {
  int2 t = {x, y};
  return t;
}
inline float3 make_float3(float x, float y, float z) {
  float3 t = {x, y, z};
  return t;
}
inline float4 make_float4(float x, float y, float z, float w) {
  float4 t = {x, y, z, w};
  return t;
}
inline double4 make_double4(double x, double y, double z, double w) {
  double4 t = {x, y, z, w};
  return t;
}

static thread_local uint3 threadIdx = {0, 0, 0};
static thread_local uint3 blockIdx = {0, 0, 0};
static thread_local uint3 blockDim = {1, 1, 1};

template <class T>
inline T min(T a, T b) { return b < a ? b : a; }
template <class T>
inline T max(T a, T b) { return a < b ? b : a; }

inline int __float2int_rn(float x) { return (int)std::nearbyint(x); }

inline float atomicAdd(float* addr, float v) {
  /* compare-and-swap on the bit pattern */
  uint32_t* bits = reinterpret_cast<uint32_t*>(addr);
  uint32_t old = __atomic_load_n(bits, __ATOMIC_RELAXED), nv;
  float of, nf;
  do {
    __builtin_memcpy(&of, &old, 4);
    nf = of + v;
    __builtin_memcpy(&nv, &nf, 4);
  } while (!__atomic_compare_exchange_n(bits, &old, nv, false, __ATOMIC_RELAXED,
                                        __ATOMIC_RELAXED));
  return of;
}

#endif
