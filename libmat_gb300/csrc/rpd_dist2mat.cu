// rpd_dist2mat.cu -- distance from sample points to their local medial-axis
// primitives (rpd_dist2mat).
//
// libmat's second CUDA kernel, ClosestDistanceToLocalMat
// (src/dist2mat/dist2mat.cu:195-270, launched by compute_closest_dist2mat,
// :272-310), used by its geometry-error check: every sample point p has a
// list of medial primitives, each an int3 of sphere ids -- (-1, -1, s) a
// sphere, (-1, a, b) a cone (the spheres linearly interpolated between a and
// b), (a, b, c) a slab (barycentric interpolation of three) -- and gets the
// smallest signed distance |p - c| - r over the spheres of its primitives and
// the index of the closest primitive in its list.
//
// The distance formulas restate the reference's (:5-193): the sphere; the
// cone's closest interpolation parameter from the stationary point of
// |p - c(t)| - r(t) (clamped to [0, 1]); the slab's interior stationary point
// by the reference's case analysis on the radius differences, and otherwise
// the nearest of its three edge cones.  The index follows the reference's
// block: lane j scans primitives j, j + 32, ... and keeps the first one with
// its smallest distance; the result is the index held by the last lane whose
// smallest distance is within 1e-10 of the minimum.  Here a warp owns a
// sample (the reference: a 32-thread block per sample), eight samples per
// block, and the minimum is a shuffle reduction.  Compiled with -fmad=false:
// every expression is rounded one operation at a time as written (the
// closed forms cancel badly for some slabs, where contraction into FMA
// changes the float result visibly).

#include <cuda_runtime.h>

#include "rpd_kernels.cuh"

namespace rpd {

namespace {

struct f3 {
  float x, y, z;
};
__device__ __forceinline__ f3 mk3(float x, float y, float z) { return f3{x, y, z}; }
__device__ __forceinline__ f3 sub3(f3 a, f3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float dot3(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float len3(f3 a) { return sqrtf(dot3(a, a)); }
__device__ __forceinline__ f3 ctr(float4 s) { return mk3(s.x, s.y, s.z); }

__device__ __forceinline__ float sphere_distance(f3 p, float4 s) { return len3(sub3(p, ctr(s))) - s.w; }

// the sphere at barycentric (t1, t2, 1 - t1 - t2) of m1, m2, m3
__device__ __forceinline__ float4 bary_sphere(float4 m1, float4 m2, float4 m3, float t1, float t2) {
  const float t3 = 1.f - t1 - t2;
  return make_float4(m1.x * t1 + m2.x * t2 + m3.x * t3, m1.y * t1 + m2.y * t2 + m3.y * t3,
                     m1.z * t1 + m2.z * t2 + m3.z * t3, m1.w * t1 + m2.w * t2 + m3.w * t3);
}

// the reference's powf(x, 2.f): the square, rounded once
__device__ __forceinline__ float sq(float x) { return x * x; }

// roots of A x^2 + B x + C (both = -C / B when A = 0; -1 when none)
__device__ __forceinline__ void quad_roots(float A, float B, float C, float* r) {
  r[0] = r[1] = -1.f;
  if (A == 0.f) {
    if (B != 0.f) r[0] = r[1] = -C / B;
  } else {
    const float delta = B * B - 4.f * A * C;
    if (delta >= 0.f) {
      const float sq = sqrtf(delta);
      r[0] = (-B - sq) / (2.f * A);
      r[1] = (-B + sq) / (2.f * A);
    }
  }
}

// cone between spheres m1, m2 (dist2mat.cu:38-66): the stationary point of
// |p - c(t)| - r(t) along the axis, clamped
__device__ float cone_distance(f3 p, float4 m1, float4 m2) {
  if (m1.w > m2.w) {
    const float4 t = m1;
    m1 = m2;
    m2 = t;
  }
  const f3 c21 = sub3(ctr(m1), ctr(m2)), cq2 = sub3(ctr(m2), p);
  const float A = dot3(c21, c21), D = 2.f * dot3(c21, cq2), F = dot3(cq2, cq2);
  const float R1 = m1.w - m2.w;
  // the reference widens D^2 to double for D^2 - 4AF and the products after
  const float root = sqrtf((float)(((double)(D * D) - 4.0 * A * F) * (R1 * R1 - A) * R1 * R1));
  float t = (-(A * D - R1 * R1 * D) - root) / (2.f * (A * A - A * R1 * R1));
  t = fmaxf(0.f, fminf(t, 1.f));  // clamp to [0, 1] (a NaN becomes 1)
  // t runs from the larger sphere m2 (t = 0) to m1 (t = 1): the reference's
  // lerp(a, b, t) is b + t (a - b) (include/cuda_helper_math.h:911-925)
  const float4 s = make_float4(m2.x + t * (m1.x - m2.x), m2.y + t * (m1.y - m2.y),
                               m2.z + t * (m1.z - m2.z), m2.w + t * (m1.w - m2.w));
  return sphere_distance(p, s);
}

// of two parameter pairs, the one whose sphere is nearer to p
__device__ __forceinline__ void pick(f3 p, float4 m1, float4 m2, float4 m3, float a1, float a2,
                                     float b1, float b2, float& t1, float& t2) {
  t1 = a1;
  t2 = a2;
  if (sphere_distance(p, bary_sphere(m1, m2, m3, b1, b2)) <
      sphere_distance(p, bary_sphere(m1, m2, m3, a1, a2))) {
    t1 = b1;
    t2 = b2;
  }
}

// slab of spheres m1, m2, m3 (dist2mat.cu:68-193)
__device__ float slab_distance(f3 p, float4 m1, float4 m2, float4 m3) {
  const f3 c31 = sub3(ctr(m1), ctr(m3)), c32 = sub3(ctr(m2), ctr(m3)), cm3 = sub3(ctr(m3), p);
  const float R1 = m1.w - m3.w, R2 = m2.w - m3.w;
  const float A = dot3(c31, c31), B = 2.f * dot3(c31, c32), C = dot3(c32, c32);
  const float D = 2.f * dot3(c31, cm3), E = 2.f * dot3(c32, cm3), F = dot3(cm3, cm3);
  float t1 = -1.f, t2 = -1.f, r[2];
  if (R1 == 0.f && R2 == 0.f) {
    // equal radii: the foot of p on the plane of the centres
    const float denom = 4.f * A * C - B * B;
    t1 = (float)(((double)(B * E) - 2.0 * C * D) / denom);
    t2 = (float)(((double)(B * D) - 2.0 * A * E) / denom);
  } else if (R1 != 0.f && R2 == 0.f) {
    const float H2 = -B / (2.f * C), K2 = -E / (2.f * C);
    const float W1 = sq(2.f * A + B * H2) - 4.f * R1 * R1 * (A + B * H2 + C * H2 * H2);
    const float W2 = 2.f * (2.f * A + B * H2) * (B * K2 + D) -
                     4.f * R1 * R1 * (B * K2 + 2.f * C * H2 * K2 + D + E * H2);
    const float W3 = sq(B * K2 + D) - 4.f * R1 * R1 * (C * K2 * K2 + E * K2 + F);
    quad_roots(W1, W2, W3, r);
    pick(p, m1, m2, m3, r[0], H2 * r[0] + K2, r[1], H2 * r[1] + K2, t1, t2);
  } else if (R1 == 0.f && R2 != 0.f) {
    const float H1 = -B / (2.f * A), K1 = -D / (2.f * A);
    const float W1 = sq(2.f * C + B * H1) - 4.f * R2 * R2 * (C + B * H1 + A * H1 * H1);
    const float W2 = 2.f * (2.f * C + B * H1) * (B * K1 + E) -
                     4.f * R2 * R2 * (B * K1 + 2.f * A * H1 * K1 + E + D * H1);
    const float W3 = sq(B * K1 + E) - 4.f * R2 * R2 * (A * K1 * K1 + D * K1 + F);
    quad_roots(W1, W2, W3, r);
    pick(p, m1, m2, m3, H1 * r[0] + K1, r[0], H1 * r[1] + K1, r[1], t1, t2);
  } else {
    const float L1 = 2.f * A * R2 - B * R1, L2 = 2.f * C * R1 - B * R2, L3 = E * R1 - D * R2;
    if (L1 == 0.f && L2 != 0.f) {
      t2 = -L3 / L2;
      const float W1 = 4.f * A * A - 4.f * R1 * R1 * A;
      const float W2 = 4.f * A * (B * t2 + D) - 4.f * R1 * R1 * (B * t2 + D);
      const float W3 = sq(B * t2 + D) - (C * t2 * t2 + E * t2 + F);
      quad_roots(W1, W2, W3, r);
      float u;
      pick(p, m1, m2, m3, r[0], t2, r[1], t2, t1, u);
    } else if (L1 != 0.f && L2 == 0.f) {
      t1 = L3 / L1;
      const float W1 = 4.f * C * C - 4.f * R2 * R2 * C;
      const float W2 = 4.f * C * (B * t1 + E) - 4.f * R2 * R2 * (B * t1 + E);
      const float W3 = sq(B * t1 + E) - (A * t1 * t1 + D * t1 + F);
      quad_roots(W1, W2, W3, r);
      float u;
      pick(p, m1, m2, m3, t1, r[0], t1, r[1], u, t2);
    } else {
      const float H3 = L2 / L1, K3 = L3 / L1;
      const float W1 = sq(2.f * C + B * H3) - 4.f * R2 * R2 * (A * H3 * H3 + B * H3 + C);
      const float W2 = 2.f * (2.f * C + B * H3) * (B * K3 + E) -
                       4.f * R2 * R2 * (2.f * A * H3 * K3 + B * K3 + D * H3 + E);
      const float W3 = sq(B * K3 + E) - 4.f * R2 * R2 * (A * K3 * K3 + D * K3 + F);
      quad_roots(W1, W2, W3, r);
      pick(p, m1, m2, m3, H3 * r[0] + K3, r[0], H3 * r[1] + K3, r[1], t1, t2);
    }
  }
  if (t1 + t2 < 1.f && t1 >= 0.f && t1 <= 1.f && t2 >= 0.f && t2 <= 1.f)
    return sphere_distance(p, bary_sphere(m1, m2, m3, t1, t2));
  return fminf(cone_distance(p, m1, m3), fminf(cone_distance(p, m2, m3), cone_distance(p, m1, m2)));
}

constexpr int kD2mWarps = 8;

__global__ void __launch_bounds__(kD2mWarps * 32)
    dist2mat_kernel(const float3* samples, int n_samples, const float4* spheres,
                    const int3* prims, const uint32_t* offsets, const uint32_t* counts,
                    float* dist, int32_t* closest) {
  const int lane = threadIdx.x & 31;
  const long long s = (long long)blockIdx.x * kD2mWarps + (threadIdx.x >> 5);
  if (s >= n_samples) return;  // whole warps
  const float3 q = samples[s];
  const f3 p = mk3(q.x, q.y, q.z);
  const int n = (int)counts[s];
  const long long base = offsets[s];
  float best = 1e16f;
  int best_id = -1;
  for (int i = lane; i < n; i += 32) {
    const int3 pr = prims[base + i];
    float d = 1e16f;
    if (pr.x == -1 && pr.y == -1) d = sphere_distance(p, spheres[pr.z]);
    else if (pr.x == -1) d = cone_distance(p, spheres[pr.y], spheres[pr.z]);
    else d = slab_distance(p, spheres[pr.x], spheres[pr.y], spheres[pr.z]);
    if (d < best) {
      best = d;
      best_id = i;
    }
  }
  float m = best;
  for (int o = 16; o > 0; o >>= 1) m = fminf(m, __shfl_xor_sync(0xffffffffu, m, o));
  const uint32_t near = __ballot_sync(0xffffffffu, fabsf(best - m) < 1e-10f);
  const int last = 31 - __clz(near);
  const int id = __shfl_sync(0xffffffffu, best_id, last < 0 ? 0 : last);
  if (lane == 0) {
    dist[s] = m;
    closest[s] = near ? id : -1;
  }
}

// every primitive's sphere ids in range and every sample's list inside the
// primitive array; counts the offending samples / primitives in *bad
__global__ void dist2mat_check_kernel(const int3* prims, long long n_prims, int n_spheres,
                                      const uint32_t* offsets, const uint32_t* counts,
                                      int n_samples, unsigned int* bad) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n_prims) {
    const int3 pr = prims[i];
    const bool sphere = pr.x == -1 && pr.y == -1, cone = pr.x == -1 && pr.y != -1;
    bool ok = pr.z >= 0 && pr.z < n_spheres;
    if (!sphere) ok &= pr.y >= 0 && pr.y < n_spheres;
    if (!sphere && !cone) ok &= pr.x >= 0 && pr.x < n_spheres;
    if (!ok) atomicAdd(bad, 1u);
  }
  if (i < n_samples && (unsigned long long)offsets[i] + counts[i] > (unsigned long long)n_prims)
    atomicAdd(bad, 1u);
}

}  // namespace

cudaError_t check_dist2mat(const int3* prims, long long n_prims, int n_spheres,
                           const uint32_t* offsets, const uint32_t* counts, int n_samples,
                           unsigned int* bad, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(bad, 0, sizeof(unsigned int), st);
  if (e != cudaSuccess) return e;
  const long long n = n_prims > n_samples ? n_prims : n_samples;
  if (n <= 0) return cudaSuccess;
  dist2mat_check_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(prims, n_prims, n_spheres,
                                                                     offsets, counts, n_samples, bad);
  note_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_dist2mat(const float3* samples, int n_samples, const float4* spheres,
                            const int3* prims, const uint32_t* offsets, const uint32_t* counts,
                            float* dist, int32_t* closest, cudaStream_t st) {
  if (n_samples <= 0) return cudaSuccess;
  dist2mat_kernel<<<(unsigned)((n_samples + kD2mWarps - 1) / kD2mWarps), kD2mWarps * 32, 0, st>>>(
      samples, n_samples, spheres, prims, offsets, counts, dist, closest);
  note_launches(1);
  return cudaGetLastError();
}

}  // namespace rpd
