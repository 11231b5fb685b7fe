// rpd_poly.cu -- polygon soup of the emitted cells (rpd_compute_polygons).
//
// libmat writes its cells out for Houdini (save_convex_cells_houdini,
// src/IO/IO_CUDA/io_cuda.cxx:143-186) through get_one_convex_cell_faces_const
// (:21-141): per cell, in order, the float vertices of
// compute_vertex_coordinates are appended to one point list (a NaN vertex
// stops the cell: the points before it stay, it gets no faces); then every
// active face -- with boundary_only, only bisector faces and tet faces whose
// face id is below max_sf_fid -- becomes one polygon over its vertex cycle
// (point ids offset by the cell's first point), or with triangulate the fan
// (0, p, p + 1); each polygon carries the cell's site and the neighbour site
// across the face (-1 for a tet face).
//
// Here the cycles come from the per-cell topology records (the same walk,
// reload_pc_explicit's), one thread per cell counts its points, polygons and
// indices, 64-bit scans give every cell its output ranges, and a second pass
// writes them.  Compiled with -fmad=false (the float vertex formula).
//
// With a slicing plane, a cell is left out (no points, no faces) when
// save_convex_cells_houdini would skip it (io_cuda.cxx:166-170): its
// barycenter (compute_cell_barycenter, io_cuda.cxx:6-17: the float sum of
// its float vertices divided by (float) nb_v) has dot(bary - pos, normal)
// >= 0 in double (is_slice_by_plane, src/IO/IO_CXX/io.cxx:810-820).
//
// The Houdini file (IO::GeometryWriter::OutputGeometry, io_utils.cpp:106-231)
// is assembled on the device: its points one byte per thread (coalesced),
// its polygons one thread each at 13 + id size x (index offset) bytes from
// the section start; the host adds the fixed header, attribute definition
// and footer.

#include <cuda_runtime.h>

#include <algorithm>

#include "rpd_common.cuh"
#include "rpd_hostfloat.cuh"
#include "rpd_kernels.cuh"
#include "rpd_scan.cuh"

namespace rpd {

namespace {

constexpr int kScan64 = 1024;

__global__ void scan64_reduce_kernel(const int32_t* in, long long n, long long* sums) {
  const long long i = (long long)blockIdx.x * kScan64 + threadIdx.x;
  long long tot;
  block_excl_scan<long long>(i < n ? in[i] : 0, &tot);
  if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

__global__ void scan64_blocksums_kernel(long long* sums, int nb) {
  long long carry = 0;
  for (int base = 0; base < nb; base += kScan64) {
    const int i = base + threadIdx.x;
    long long tot;
    const long long ex = block_excl_scan<long long>(i < nb ? sums[i] : 0, &tot);
    if (i < nb) sums[i] = ex + carry;
    carry += tot;
  }
  if (threadIdx.x == 0) sums[nb] = carry;
}

__global__ void scan64_apply_kernel(const int32_t* in, long long n, const long long* sums, int nb,
                                    long long* out) {
  const long long i = (long long)blockIdx.x * kScan64 + threadIdx.x;
  const long long ex = block_excl_scan<long long>(i < n ? in[i] : 0, nullptr);
  if (i < n) out[i] = ex + sums[blockIdx.x];
  if (blockIdx.x == 0 && threadIdx.x == 0) out[n] = sums[nb];
}

__device__ __forceinline__ bool face_shown(int2 hp, const PolyParams& p) {
  return !p.boundary_only || hp.y != -1 || hp.x < p.max_sf_fid;
}

struct PolyCell {
  int nv, np, ne;
  const float4* pl;
  const int2* id2;
  const uchar4* ver;
  const uint8_t* act;
  const uint8_t* faces;
  bool vnull;
};

__device__ __forceinline__ PolyCell poly_cell(const PolyParams& p, long long q,
                                              rpd_cell_header& hd) {
  hd = p.cells[q];
  PolyCell c;
  c.nv = hd.nb_v;
  c.np = hd.nb_p;
  c.ne = hd.nb_e;
  const PayloadLayout L(c.nv, c.np, c.ne);
  const TopoLayout T(c.nv, c.np, c.ne);
  const uint8_t* rec = p.payload + hd.offset;
  const rpd_topo_header th = p.topo_h[q];
  const uint8_t* tr = p.topo + th.offset;
  c.pl = reinterpret_cast<const float4*>(rec + L.plane);
  c.id2 = reinterpret_cast<const int2*>(rec + L.id2);
  c.ver = reinterpret_cast<const uchar4*>(rec + L.ver);
  c.act = tr + T.active;
  c.faces = tr + T.faces;
  c.vnull = (th.flags & RPD_TOPO_VERTEX_NULL) != 0;
  return c;
}

// (plane ids of a valid record are below nb_p; clamped so that no record can
// make the kernel read past its planes)
__device__ __forceinline__ float3 cell_point(const PolyCell& c, int t) {
  const uchar4 v = c.ver[t];
  const int m = c.np - 1;
  return host_float_vertex(c.pl[min((int)v.x, m)], c.pl[min((int)v.y, m)], c.pl[min((int)v.z, m)]);
}

__device__ bool sliced(const PolyCell& c, const PolyParams& p) {
  float bx = 0.f, by = 0.f, bz = 0.f;
  for (int t = 0; t < c.nv; ++t) {
    const float3 v = cell_point(c, t);
    bx = v.x + bx;
    by = v.y + by;
    bz = v.z + bz;
  }
  const float fn = (float)c.nv;
  bx = bx / fn;
  by = by / fn;
  bz = bz / fn;
  const double dx = (double)bx - p.slice_plane[0], dy = (double)by - p.slice_plane[1],
               dz = (double)bz - p.slice_plane[2];
  return dx * p.slice_plane[3] + dy * p.slice_plane[4] + dz * p.slice_plane[5] >= 0.0;
}

__global__ void poly_count_kernel(PolyParams p) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= p.n) return;
  rpd_cell_header hd;
  const PolyCell c = poly_cell(p, q, hd);
  int pts = c.nv, polys = 0, idx = 0;
  if (p.slice && sliced(c, p)) {
    pts = 0;
  } else if (c.vnull) {
    // the points before the first NaN vertex stay, no faces
    pts = 0;
    while (pts < c.nv && !is_null_vertex(cell_point(c, pts))) ++pts;
  } else {
    for (int f = 0; f < c.np; ++f) {
      const int len = c.act[f];
      if (len == 0 || !face_shown(c.id2[f], p)) continue;
      if (p.triangulate) {
        const int tri = len >= 3 ? len - 2 : 0;
        polys += tri;
        idx += 3 * tri;
      } else {
        polys += 1;
        idx += len;
      }
    }
  }
  p.cnt_points[q] = pts;
  p.cnt_polys[q] = polys;
  p.cnt_indices[q] = idx;
}

__global__ void poly_fill_kernel(PolyParams p) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= p.n) return;
  rpd_cell_header hd;
  const PolyCell c = poly_cell(p, q, hd);
  const long long row = p.off_points[q];
  const int pts = p.cnt_points[q];
  for (int t = 0; t < pts; ++t) {
    const float3 v = cell_point(c, t);
    p.points[3 * (row + t)] = v.x;
    p.points[3 * (row + t) + 1] = v.y;
    p.points[3 * (row + t) + 2] = v.z;
  }
  if (c.vnull || p.cnt_polys[q] == 0) return;
  long long pi = p.off_polys[q], ii = p.off_indices[q];
  int slot = 0;
  for (int f = 0; f < c.np; ++f) {
    const int len = c.act[f];
    if (len == 0) continue;
    const uint8_t* cyc = c.faces + slot;
    slot += len;
    const int2 hp = c.id2[f];
    if (!face_shown(hp, p)) continue;
    const int adj = hp.y != -1 ? (hp.x == hd.site_id ? hp.y : hp.x) : -1;
    if (p.triangulate) {
      for (int k = 1; k < len - 1; ++k) {
        p.poly_offsets[pi] = ii;
        p.indices[ii] = (uint32_t)(row + cyc[0]);
        p.indices[ii + 1] = (uint32_t)(row + cyc[k]);
        p.indices[ii + 2] = (uint32_t)(row + cyc[(k + 1) % len]);
        p.poly_site[pi] = hd.site_id;
        p.poly_adj_site[pi] = adj;
        ++pi;
        ii += 3;
      }
    } else {
      p.poly_offsets[pi] = ii;
      for (int k = 0; k < len; ++k) p.indices[ii + k] = (uint32_t)(row + cyc[k]);
      p.poly_site[pi] = hd.site_id;
      p.poly_adj_site[pi] = adj;
      ++pi;
      ii += len;
    }
  }
}

__device__ __forceinline__ void put_be32(uint8_t* d, uint32_t v) {
  d[0] = (uint8_t)(v >> 24);
  d[1] = (uint8_t)(v >> 16);
  d[2] = (uint8_t)(v >> 8);
  d[3] = (uint8_t)v;
}

// byte j of the points section: point j / 16, word (j / 4) % 4 (x, y, z,
// 1.0f), big-endian
__global__ void bgeo_points_kernel(const float* points, long long n_bytes, uint8_t* out) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x; j < n_bytes; j += stride) {
    const long long pt = j >> 4;
    const int w = (int)((j >> 2) & 3), b = (int)(j & 3);
    const float f = w < 3 ? points[3 * pt + w] : 1.0f;
    out[j] = (uint8_t)(__float_as_uint(f) >> (24 - 8 * b));
  }
}

// polygon i: int 1, int count, '<', the ids (16- or 32-bit), int site
__global__ void bgeo_polys_kernel(const long long* poly_offsets, const uint32_t* indices,
                                  const int32_t* poly_site, long long n_polys, int wide,
                                  uint8_t* out) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n_polys; i += stride) {
    const long long a = poly_offsets[i], e = poly_offsets[i + 1];
    uint8_t* d = out + 13 * i + (wide ? 4 : 2) * a;
    put_be32(d, 1u);
    put_be32(d + 4, (uint32_t)(e - a));
    d[8] = (uint8_t)'<';
    d += 9;
    for (long long k = a; k < e; ++k) {
      const uint32_t v = indices[k];
      if (wide) {
        put_be32(d, v);
        d += 4;
      } else {
        d[0] = (uint8_t)(v >> 8);
        d[1] = (uint8_t)v;
        d += 2;
      }
    }
    put_be32(d, (uint32_t)poly_site[i]);
  }
}

}  // namespace

cudaError_t bgeo_fill(const float* points, long long n_points, const long long* poly_offsets,
                      const uint32_t* indices, const int32_t* poly_site, long long n_polys,
                      int wide, uint8_t* points_out, uint8_t* polys_out, int num_sms,
                      cudaStream_t st) {
  const long long cap = (long long)num_sms * 8;
  if (n_points > 0) {
    const long long nb = 16 * n_points;
    bgeo_points_kernel<<<(unsigned)std::min((nb + 255) / 256, cap), 256, 0, st>>>(points, nb,
                                                                                  points_out);
    note_launches(1);
  }
  if (n_polys > 0) {
    bgeo_polys_kernel<<<(unsigned)std::min((n_polys + 255) / 256, cap), 256, 0, st>>>(
        poly_offsets, indices, poly_site, n_polys, wide, polys_out);
    note_launches(1);
  }
  return cudaGetLastError();
}

size_t scan64_temp(long long n) { return (size_t)((n + kScan64 - 1) / kScan64) + 1; }

cudaError_t scan64_exclusive(const int32_t* in, long long* out, long long n, long long* temp,
                             cudaStream_t st) {
  const int nb = (int)((n + kScan64 - 1) / kScan64);
  if (nb == 0) return cudaMemsetAsync(out, 0, sizeof(long long), st);
  scan64_reduce_kernel<<<nb, kScan64, 0, st>>>(in, n, temp);
  scan64_blocksums_kernel<<<1, kScan64, 0, st>>>(temp, nb);
  scan64_apply_kernel<<<nb, kScan64, 0, st>>>(in, n, temp, nb, out);
  note_launches(3);
  return cudaGetLastError();
}

cudaError_t poly_count(const PolyParams& p, cudaStream_t st) {
  if (p.n <= 0) return cudaSuccess;
  poly_count_kernel<<<(unsigned)((p.n + 255) / 256), 256, 0, st>>>(p);
  note_launches(1);
  return cudaGetLastError();
}

cudaError_t poly_fill(const PolyParams& p, cudaStream_t st) {
  if (p.n <= 0) return cudaSuccess;
  poly_fill_kernel<<<(unsigned)((p.n + 255) / 256), 256, 0, st>>>(p);
  note_launches(1);
  return cudaGetLastError();
}

}  // namespace rpd
