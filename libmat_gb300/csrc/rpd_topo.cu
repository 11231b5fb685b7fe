// rpd_topo.cu -- per-cell topology of the emitted cells (rpd_compute_topology).
//
// libmat's consumers of the RPD (update_power_cells, src/rpd3d_base/
// rpd_update.cxx:568-638; the Euler checks of src/matfun_fix/fix_topo.cxx)
// first rebuild, for every ConvexCellHost on the host, with std::map and
// std::set (src/rpd3d_base/voronoi_defs.cxx):
//   reload_active             :76-106   vertices per plane, active planes,
//                                       active edges (>= 2 common vertices)
//   reload_pc_explicit        :108-188  the vertex cycle of every active face
//                                       (walk: from the face's first vertex,
//                                       the next is the first vertex whose
//                                       plane before this face is the plane
//                                       after it in the current vertex), the
//                                       face -> active face map, NaN vertices
//   cal_cell_euler            :190-222  V/#adj - E/#adj + F/#adj, in double
//   cal_halfplane_facet_euler :224-266  the same restricted to the face of a
//                                       neighbour (first active plane whose
//                                       id pair holds the neighbour id)
// Here one warp owns one cell for the integer topology.  The vertices of
// each plane are a 96-bit mask built by all lanes at once (one shared-memory
// atomic OR per vertex and plane); a face's next vertex is looked up among
// the vertices common to the face and the plane just crossed (the mask
// intersection, about two candidates) instead of scanning the face.  The
// Euler numbers follow in a thread-per-cell kernel: every sum that the
// reference forms in double is formed in the same order, so the results are
// the reference's bit for bit.
//
// Compiled with -fmad=false: the float vertex formula of the NaN test is
// evaluated one IEEE rounding at a time, as the reference's host code.

#include <cuda_runtime.h>

#include "rpd_common.cuh"
#include "rpd_hostfloat.cuh"
#include "rpd_kernels.cuh"

namespace rpd {

namespace {

constexpr int kTopoWarps = 4;

struct __align__(16) TopoCell {
  uint32_t vm[kMaxP][3];  // vertex slots on each plane (bit t of word t / 32)
  uchar4 ver[kMaxT];
  uchar4 edge[kMaxE];
  uint8_t act[kMaxP];     // active_clipping_planes
  uint8_t acte[kMaxE];    // active_edges
};

__device__ __forceinline__ int plane_pos(uchar4 t, int p) {
  return t.x == p ? 0 : (t.y == p ? 1 : 2);
}
__device__ __forceinline__ int tri_at(uchar4 t, int i) { return i == 0 ? t.x : (i == 1 ? t.y : t.z); }

// lowest set bit of a 96-bit mask at or above `from`, or -1
__device__ __forceinline__ int next_bit(uint32_t m0, uint32_t m1, uint32_t m2, int from) {
  for (int w = from >> 5; w < 3; ++w) {
    uint32_t m = w == 0 ? m0 : (w == 1 ? m1 : m2);
    if (w == (from >> 5)) m &= ~0u << (from & 31);
    if (m) return 32 * w + __ffs(m) - 1;
  }
  return -1;
}

__global__ void topo_units_kernel(const rpd_cell_header* cells, long long n, int32_t* units) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const rpd_cell_header h = cells[q];
  units[q] = (int32_t)(TopoLayout(h.nb_v, h.nb_p, h.nb_e).total / 16u);
}

__global__ void __launch_bounds__(kTopoWarps * 32)
    topo_fill_kernel(const rpd_cell_header* cells, long long n, const uint8_t* payload,
                     const int32_t* unit_off, rpd_topo_header* out_h, uint8_t* out) {
  __shared__ TopoCell sc[kTopoWarps];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const unsigned full = 0xffffffffu;
  TopoCell& c = sc[wid];
  const long long n_warps = (long long)gridDim.x * kTopoWarps;
  for (long long q = (long long)blockIdx.x * kTopoWarps + wid; q < n; q += n_warps) {
    const rpd_cell_header hd = cells[q];
    const int nv = hd.nb_v, np = hd.nb_p, ne = hd.nb_e;
    const PayloadLayout L(nv, np, ne);
    const TopoLayout T(nv, np, ne);
    const uint8_t* rec = payload + hd.offset;
    const unsigned long long off = 16ull * (unsigned long long)unit_off[q];
    uint8_t* dst = out + off;
    for (int i = lane; i < nv; i += 32) c.ver[i] = reinterpret_cast<const uchar4*>(rec + L.ver)[i];
    for (int i = lane; i < ne; i += 32) c.edge[i] = reinterpret_cast<const uchar4*>(rec + L.edge)[i];
    for (int i = lane; i < np; i += 32) c.vm[i][0] = c.vm[i][1] = c.vm[i][2] = 0u;
    __syncwarp();
    // plane2v: every vertex marks its three planes; NaN float vertices
    bool null_mine = false;
    const float4* pl = reinterpret_cast<const float4*>(rec + L.plane);
    for (int t = lane; t < nv; t += 32) {
      const uchar4 tr = c.ver[t];
      const uint32_t bit = 1u << (t & 31);
      if (tr.x < np) atomicOr(&c.vm[tr.x][t >> 5], bit);
      if (tr.y < np) atomicOr(&c.vm[tr.y][t >> 5], bit);
      if (tr.z < np) atomicOr(&c.vm[tr.z][t >> 5], bit);
      if (tr.x < np && tr.y < np && tr.z < np)
        null_mine |= is_null_vertex(host_float_vertex(pl[tr.x], pl[tr.y], pl[tr.z]));
    }
    const bool vnull = __any_sync(full, null_mine);
    __syncwarp();
    for (int p = lane; p < np; p += 32)
      c.act[p] = (uint8_t)(__popc(c.vm[p][0]) + __popc(c.vm[p][1]) + __popc(c.vm[p][2]));
    __syncwarp();
    // active edges: both planes active and at least two common vertices
    for (int e = lane; e < ne; e += 32) {
      const uchar4 ed = c.edge[e];
      uint8_t a = 0;
      if (ed.x < np && ed.y < np && c.act[ed.x] > 0 && c.act[ed.y] > 0) {
        const int common = __popc(c.vm[ed.x][0] & c.vm[ed.y][0]) +
                           __popc(c.vm[ed.x][1] & c.vm[ed.y][1]) +
                           __popc(c.vm[ed.x][2] & c.vm[ed.y][2]);
        a = common >= 2 ? 1 : 0;
      }
      c.acte[e] = a;
      dst[T.active_e + e] = a;
    }
    __syncwarp();
    // faces, in plane order, 32 planes at a time
    int n_faces = 0, slots = 0;
    bool open_mine = false;
    for (int p0 = 0; p0 < np; p0 += 32) {
      const int p = p0 + lane;
      const int cnt = p < np ? c.act[p] : 0;
      const uint32_t on = __ballot_sync(full, cnt > 0);
      int incl = cnt;
      for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(full, incl, o);
        if (lane >= o) incl += v;
      }
      if (p < np) {
        const int lf = n_faces + __popc(on & ((1u << lane) - 1u));
        dst[T.active + p] = (uint8_t)cnt;
        dst[T.lf2active + p] = (uint8_t)(int8_t)(cnt > 0 && !vnull ? lf : -1);
        // the vertex cycle of face p (reload_pc_explicit)
        if (cnt > 0 && !vnull) {
          const uint32_t w0 = c.vm[p][0], w1 = c.vm[p][1], w2 = c.vm[p][2];
          uint8_t* fo = dst + T.faces + slots + (incl - cnt);
          // a vertex is written once its successor is found (the last one's
          // successor closes the cycle)
          int ti = next_bit(w0, w1, w2, 0);
          for (int k = 0; k < cnt; ++k) {
            const uchar4 tr = c.ver[ti];
            const int qn = tri_at(tr, (plane_pos(tr, p) + 1) % 3);
            int found = -1;
            if (qn < np) {
              const uint32_t c0 = w0 & c.vm[qn][0], c1 = w1 & c.vm[qn][1], c2 = w2 & c.vm[qn][2];
              for (int t = next_bit(c0, c1, c2, 0); t >= 0; t = next_bit(c0, c1, c2, t + 1)) {
                const uchar4 tt = c.ver[t];
                if (tri_at(tt, (plane_pos(tt, p) + 2) % 3) == qn) {
                  found = t;
                  break;
                }
              }
            }
            if (found < 0) {
              open_mine = true;
              for (int r = k; r < cnt; ++r) fo[r] = kEnd;
              break;
            }
            fo[k] = (uint8_t)ti;
            ti = found;
          }
        }
      }
      n_faces += __popc(on);
      slots += __shfl_sync(full, incl, 31);
    }
    // faces of a cell with a NaN vertex stay empty; zero padding
    const int fend = T.faces + 3 * nv;
    if (vnull)
      for (int i = lane; i < 3 * nv; i += 32) dst[T.faces + i] = kEnd;
    for (int i = fend + lane; i < (int)T.total; i += 32) dst[i] = 0;
    const bool open = __any_sync(full, open_mine);
    if (lane == 0) {
      rpd_topo_header th;
      th.offset = off;
      th.euler = 0.f;  // topo_euler_kernel
      th.n_faces = (uint8_t)(vnull ? 0 : n_faces);
      th.flags = (uint8_t)((vnull ? RPD_TOPO_VERTEX_NULL : 0) | (open ? RPD_TOPO_OPEN_FACE : 0));
      th.pad[0] = th.pad[1] = 0;
      out_h[q] = th;
    }
    __syncwarp();
  }
}

// The Euler numbers: cal_cell_euler and, for every active bisector plane,
// cal_halfplane_facet_euler of its neighbour.  The reference forms each sum
// in double, term after term; to give its bits the sums are formed in the
// same order.  GB300's FP64 pipe is narrow, so one thread owns one cell here
// and every FP64 instruction adds for 32 cells at once (a warp-per-cell
// loop would issue them for one lane).  Reads the cell's record and the
// active planes / edges written by topo_fill_kernel.
constexpr int kEulerThreads = 256;

__global__ void __launch_bounds__(kEulerThreads)
    topo_euler_kernel(const rpd_cell_header* cells, long long n, const uint8_t* payload,
                      const int32_t* unit_off, rpd_topo_header* out_h, uint8_t* out) {
  // 1.f / k widened to double (the vertex terms) and 1. / k (face and edge terms)
  __shared__ double inv_f[256], inv_d[256];
  for (int k = threadIdx.x; k < 256; k += blockDim.x) {
    inv_f[k] = (double)(1.0f / (float)k);
    inv_d[k] = 1.0 / (double)k;
  }
  __syncthreads();
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const rpd_cell_header hd = cells[q];
  const int nv = hd.nb_v, np = hd.nb_p, ne = hd.nb_e;
  const PayloadLayout L(nv, np, ne);
  const TopoLayout T(nv, np, ne);
  const uint8_t* rec = payload + hd.offset;
  uint8_t* dst = out + 16ull * (unsigned long long)unit_off[q];
  const uchar4* ver = reinterpret_cast<const uchar4*>(rec + L.ver);
  const uchar4* edge = reinterpret_cast<const uchar4*>(rec + L.edge);
  const int2* id2 = reinterpret_cast<const int2*>(rec + L.id2);
  const uint8_t* h = rec + L.h;
  const uint8_t* act = dst + T.active;
  const uint8_t* acte = dst + T.active_e;
  float* facet = reinterpret_cast<float*>(dst + T.facet_euler);
  // cal_cell_euler (voronoi_defs.cxx:190-222)
  double sum_v = 0.0, sum_f = 0.0, sum_e = 0.0;
  for (int t = 0; t < nv; ++t) sum_v += inv_f[ver[t].w];
  for (int p = 0; p < np; ++p)
    if (act[p] > 0) sum_f += inv_d[h[p]];
  for (int e = 0; e < ne; ++e)
    if (acte[e] > 0) sum_e += inv_d[edge[e].z];
  out_h[q].euler = (float)(sum_v - sum_e + sum_f);
  // cal_halfplane_facet_euler (:224-266): the face is the first active plane
  // whose id pair holds the neighbour (a tet face whose face id equals the
  // neighbour's site id qualifies too, as in the reference)
  for (int p = 0; p < np; ++p) {
    const int2 id = id2[p];
    float fe = 0.f;
    if (act[p] > 0 && id.y != -1) {
      const int nb = id.x == hd.site_id ? id.y : id.x;
      int clip = p;
      for (int r = 0; r < np; ++r) {
        const int2 ir = id2[r];
        if (act[r] > 0 && (ir.x == nb || ir.y == nb)) {
          clip = r;
          break;
        }
      }
      double sv = 0.0, se = 0.0;
      for (int t = 0; t < nv; ++t) {
        const uchar4 tr = ver[t];
        if (tr.x == clip || tr.y == clip || tr.z == clip) sv += inv_f[tr.w];
      }
      for (int e = 0; e < ne; ++e) {
        const uchar4 ed = edge[e];
        if ((ed.x == clip || ed.y == clip) && acte[e] > 0) se += inv_d[ed.z];
      }
      fe = (float)(sv - se + 1.0);
    }
    facet[p] = fe;
  }
}

}  // namespace

cudaError_t topo_units(const rpd_cell_header* cells, long long n, int32_t* units, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  topo_units_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(cells, n, units);
  note_launches(1);
  return cudaGetLastError();
}

cudaError_t topo_fill(const rpd_cell_header* cells, long long n, const uint8_t* payload,
                      const int32_t* unit_off, rpd_topo_header* out_h, uint8_t* out, int num_sms,
                      cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  long long blocks = (n + kTopoWarps - 1) / kTopoWarps;
  const long long cap = (long long)num_sms * 16;
  if (blocks > cap) blocks = cap;
  topo_fill_kernel<<<(unsigned)blocks, kTopoWarps * 32, 0, st>>>(cells, n, payload, unit_off, out_h,
                                                                 out);
  topo_euler_kernel<<<(unsigned)((n + kEulerThreads - 1) / kEulerThreads), kEulerThreads, 0, st>>>(
      cells, n, payload, unit_off, out_h, out);
  note_launches(2);
  return cudaGetLastError();
}

}  // namespace rpd
