/*
 * ref_dist2mat_driver.cu -- runs libmat's own dist2mat distance functions
 * (distance_to_sphere, compute_distance_to_cone, compute_distance_to_slab:
 * src/dist2mat/dist2mat.cu:5-193, __host__ __device__) on the CPU, so that
 * the oracle and the device kernel can be pinned to the reference's code.
 * Test infrastructure: built by oracle/build.py into oracle/_ref/ when the
 * reference sources are present; nvcc compiles the reference file in place
 * (include path, never copied) and the host compiler evaluates the
 * functions one IEEE rounding per operation (-ffp-contract=off), the
 * reference source's semantics.
 *
 * refd2m_eval applies them per sample with the selection rule of the
 * kernel ClosestDistanceToLocalMat (:195-270): lane j of the 32-thread block
 * scans primitives j, j + 32, ... keeping the first strictly smaller
 * distance; the minimum over lanes is the result, and the closest index is
 * that of the last lane whose distance is within 1e-10 of it.
 */
#include <cub/cub.cuh>

// CUDA 13's CUB dropped cub::Min, which the reference's kernel names (its
// block reduction, not run here); a stand-in with the same meaning
namespace cub {
struct Min {
  template <class T>
  __host__ __device__ T operator()(const T& a, const T& b) const {
    return b < a ? b : a;
  }
};
}  // namespace cub

#include "dist2mat.cu"

#include <cmath>
#include <cstdint>

extern "C" void refd2m_eval(int n_samples, const float* samples, const float* spheres,
                            const int32_t* prims, const uint32_t* offsets,
                            const uint32_t* counts, float* dist, int32_t* closest) {
  const float4* sp = reinterpret_cast<const float4*>(spheres);
  for (int s = 0; s < n_samples; ++s) {
    const float3 pos = make_float3(samples[3 * s], samples[3 * s + 1], samples[3 * s + 2]);
    const int num = (int)counts[s];
    const int off = (int)offsets[s];
    float local[kWarpSize];
    int lid[kWarpSize];
    for (int tid = 0; tid < kWarpSize; ++tid) {
      local[tid] = 1e16f;
      lid[tid] = -1;
      for (int i = tid; i < num && tid < num; i += kWarpSize) {
        const int32_t* pr = prims + 3 * (int64_t)(off + i);
        float d = 1e16f;
        if (pr[0] == -1 && pr[1] == -1) {
          d = distance_to_sphere(pos, sp[pr[2]]);
        } else if (pr[0] == -1 && pr[1] != -1) {
          d = compute_distance_to_cone(pos, sp[pr[1]], sp[pr[2]]);
        } else if (pr[0] != -1) {
          d = compute_distance_to_slab(pos, sp[pr[0]], sp[pr[1]], sp[pr[2]]);
        }
        if (d < local[tid]) {
          local[tid] = fminf(local[tid], d);
          lid[tid] = i;
        }
      }
    }
    float red = local[0];
    for (int tid = 1; tid < kWarpSize; ++tid) red = local[tid] < red ? local[tid] : red;
    dist[s] = red;
    int cid = -1;
    for (int tid = 0; tid < kWarpSize; ++tid)
      if (fabsf(local[tid] - red) < 1e-10f) cid = lid[tid];
    closest[s] = cid;
  }
}
