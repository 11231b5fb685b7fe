// rpd_hostfloat.cuh -- the float vertex of libmat's host-side cell code.
//
// ConvexCellHost::compute_vertex_coordinates (src/rpd3d_base/
// voronoi_defs.cxx:33-74) intersects a vertex's three planes by Cramer's
// rule with the host's cdet3x3 (include/common_cxx.h:128-135) and divides by
// the fourth minor.  Its consumers (reload_pc_explicit's NaN test and
// pc_points, get_one_convex_cell_faces_const's points) see these floats, so
// translation units that include this header are compiled with -fmad=false:
// one IEEE rounding per operation, as the source states it.
#pragma once

#include <cuda_runtime.h>

namespace rpd {

__device__ __forceinline__ float cdet2(float a11, float a12, float a21, float a22) {
  return a11 * a22 - a12 * a21;
}
__device__ __forceinline__ float cdet3(float a11, float a12, float a13, float a21, float a22,
                                       float a23, float a31, float a32, float a33) {
  return a11 * cdet2(a22, a23, a32, a33) - a21 * cdet2(a12, a13, a32, a33) +
         a31 * cdet2(a12, a13, a22, a23);
}

// the vertex of planes p1, p2, p3 after the perspective divide
__device__ __forceinline__ float3 host_float_vertex(float4 p1, float4 p2, float4 p3) {
  const float x = -cdet3(p1.w, p1.y, p1.z, p2.w, p2.y, p2.z, p3.w, p3.y, p3.z);
  const float y = -cdet3(p1.x, p1.w, p1.z, p2.x, p2.w, p2.z, p3.x, p3.w, p3.z);
  const float z = -cdet3(p1.x, p1.y, p1.w, p2.x, p2.y, p2.w, p3.x, p3.y, p3.w);
  const float w = cdet3(p1.x, p1.y, p1.z, p2.x, p2.y, p2.z, p3.x, p3.y, p3.z);
  return make_float3(x / w, y / w, z / w);
}

__device__ __forceinline__ bool is_null_vertex(float3 v) {
  return isnan(v.x) || isnan(v.y) || isnan(v.z);
}

}  // namespace rpd
