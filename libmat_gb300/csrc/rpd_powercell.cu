// rpd_powercell.cu -- the power cells of the emitted cells
// (rpd_compute_power_cells).
//
// libmat's get_all_voro_info (src/rpd3d_base/rpd_update.cxx:80-340), run
// for every medial sphere by update_power_cells (:568-638), gathers the
// convex cells of each power cell into std::map / std::set structures
// (PowerCell, src/matbase/medial_sphere.h:145-260): per cell its active tet
// faces (cell_to_tfids) and the cells across them (cell_neighbors, from
// tfid_to_cells); per neighbour site the cells clipped by that bisector
// (facet_neigh_to_cells); per pair of neighbour sites the cells with an
// active edge on both bisectors and the edge's end vertices (e_to_cells,
// edge_2endvertices); every vertex with at least two neighbour sites among
// its planes, as the sorted triple of them (-1 for one tet face) with its
// float position and surface face (vertex_2id, vertex_2pos); and for every
// active tet face on the surface the centroid of its vertex cycle
// (cell_to_surfv2fid).  Here one thread per cell writes flat records of
// each kind (count, 64-bit scan, fill), and stable radix sorts put the
// keyed ones into the maps' order: by site, then key, then cell.
//
// With TetMesh::tet_es2fe_map given (sorted unique keys tet << 4 | lf_min
// << 2 | lf_max, rpd_set_feature_edges), the feature-edge records of
// rpd_update.cxx:206-254 too: for every active edge of the cell between two
// faces of its tet that the map lists, {cell, the edge's two vertices, line,
// fe id} for sharp (se_covered_lvids) and concave (ce_covered_lvids) edges,
// and for each of the two vertices with a bisector among its planes the
// first such bisector's site, the line and the vertex position
// (se_line_endpos).  A record depends only on the pair of faces, so a cell
// has at most 6 of each kind and 12 endpoints, sorted and made unique per
// cell by one thread.
//
// Compiled with -fmad=false (the float positions and centroids are the
// reference's host float arithmetic).

#include <cuda_runtime.h>

#include "rpd_common.cuh"
#include "rpd_hostfloat.cuh"
#include "rpd_kernels.cuh"

namespace rpd {

namespace {

struct PcCell {
  int nv, np, ne, site;
  const float4* pl;
  const int2* id2;
  const uchar4* ver;
  const uchar4* edge;
  const uint8_t* act;
  const int8_t* lf2a;
  const uint8_t* acte;
  const uint8_t* faces;
  bool vnull;
};

__device__ __forceinline__ PcCell pc_cell(const PowerCellParams& p, long long q) {
  const rpd_cell_header h = p.cells[q];
  PcCell c;
  c.nv = h.nb_v;
  c.np = h.nb_p;
  c.ne = h.nb_e;
  c.site = h.site_id;
  const PayloadLayout L(c.nv, c.np, c.ne);
  const TopoLayout T(c.nv, c.np, c.ne);
  const uint8_t* rec = p.payload + h.offset;
  const rpd_topo_header th = p.topo_h[q];
  const uint8_t* tr = p.topo + th.offset;
  c.pl = reinterpret_cast<const float4*>(rec + L.plane);
  c.id2 = reinterpret_cast<const int2*>(rec + L.id2);
  c.ver = reinterpret_cast<const uchar4*>(rec + L.ver);
  c.edge = reinterpret_cast<const uchar4*>(rec + L.edge);
  c.act = tr + T.active;
  c.lf2a = reinterpret_cast<const int8_t*>(tr + T.lf2active);
  c.acte = tr + T.active_e;
  c.faces = tr + T.faces;
  c.vnull = (th.flags & RPD_TOPO_VERTEX_NULL) != 0;
  return c;
}

__device__ __forceinline__ int neigh_of(int2 id, int site) { return id.x == site ? id.y : id.x; }
__device__ __forceinline__ bool on_plane(uchar4 v, int p) { return v.x == p || v.y == p || v.z == p; }
__device__ __forceinline__ int plane_at(uchar4 v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : v.z); }

// plane ids of a valid record are below nb_p; clamped so that no record can
// make these kernels read past its planes
__device__ __forceinline__ int pid(const PcCell& c, int p) { return p < c.np ? p : c.np - 1; }
__device__ __forceinline__ float3 vertex_pos(const PcCell& c, int t) {
  const uchar4 v = c.ver[t];
  return host_float_vertex(c.pl[pid(c, v.x)], c.pl[pid(c, v.y)], c.pl[pid(c, v.z)]);
}

// the neighbour sites of vertex t (halfplanes), its surface face (the last
// tet face of its planes with id <= max_sf_fid, or -1), and how many
__device__ __forceinline__ int vertex_neighbours(const PcCell& c, int t, int max_sf_fid, int* nb,
                                                 int& sfid) {
  const uchar4 v = c.ver[t];
  int n = 0;
  sfid = -1;
  for (int i = 0; i < 3; ++i) {
    const int2 hp = c.id2[pid(c, plane_at(v, i))];
    if (hp.y != -1) {
      const int s = neigh_of(hp, c.site);
      bool dup = false;
      for (int k = 0; k < n; ++k) dup |= nb[k] == s;
      if (!dup) nb[n++] = s;
    } else if (hp.x <= max_sf_fid) {
      sfid = hp.x;
    }
  }
  return n;
}

// index of key in the sorted feature-edge keys, or -1
__device__ __forceinline__ long long fe_find(const PowerCellParams& p, unsigned long long key) {
  long long lo = 0, hi = p.n_fe;
  while (lo < hi) {
    const long long mid = (lo + hi) >> 1;
    if (p.fe_keys[mid] < key) lo = mid + 1;
    else hi = mid;
  }
  return lo < p.n_fe && p.fe_keys[lo] == key ? lo : -1;
}

template <int N>
__device__ __forceinline__ bool lex_less(const int (&a)[N], const int (&b)[N]) {
  for (int i = 0; i < N; ++i)
    if (a[i] != b[i]) return a[i] < b[i];
  return false;
}

// sorts rec[0, n) ascending and drops repeats; returns the new count
template <int N, int M>
__device__ int sort_unique(int (&rec)[M][N], int n) {
  for (int a = 1; a < n; ++a)
    for (int b = a; b > 0 && lex_less(rec[b], rec[b - 1]); --b)
      for (int i = 0; i < N; ++i) {
        const int t = rec[b][i];
        rec[b][i] = rec[b - 1][i];
        rec[b - 1][i] = t;
      }
  int m = 0;
  for (int a = 0; a < n; ++a) {
    bool same = m > 0;
    for (int i = 0; i < N && same; ++i) same = rec[m - 1][i] == rec[a][i];
    if (same) continue;
    for (int i = 0; i < N; ++i) rec[m][i] = rec[a][i];
    ++m;
  }
  return m;
}

struct FeCell {
  int nse, nce, nend;
  int se[6][4], ce[6][4];  // lvid1, lvid2, fe_line_id, fe_id
  int end[12][3];          // lvid, neighbour site, fe_line_id
};

// the feature-edge records of cell q (without the cell id), sorted and unique
__device__ void fe_cell(const PowerCellParams& p, const PcCell& c, int tet, FeCell& o) {
  o.nse = o.nce = o.nend = 0;
  if (p.n_fe <= 0) return;
  // pairs of tet faces (both without a neighbour site) joined by an active edge
  uint32_t pairs = 0;
  for (int e = 0; e < c.ne; ++e) {
    if (!c.acte[e]) continue;
    const uchar4 ed = c.edge[e];
    const int a = ed.x < ed.y ? ed.x : ed.y, b = ed.x < ed.y ? ed.y : ed.x;
    if (b >= 4 || a == b || c.id2[a].y != -1 || c.id2[b].y != -1) continue;
    pairs |= 1u << (4 * a + b);
  }
  // face cycle offsets of the tet faces
  int cyc[5];
  cyc[0] = 0;
  for (int f = 0; f < 4; ++f) cyc[f + 1] = cyc[f] + (f < c.np ? c.act[f] : 0);
  while (pairs) {
    const int bit = __ffs(pairs) - 1;
    pairs &= pairs - 1;
    const int a = bit >> 2, b = bit & 3;
    const long long k = fe_find(p, ((unsigned long long)(uint32_t)tet << 4) | (unsigned)(a << 2) | (unsigned)b);
    if (k < 0) continue;
    const int type = p.fe_vals[3 * k], fid = p.fe_vals[3 * k + 1], line = p.fe_vals[3 * k + 2];
    // the two smallest vertices on both faces' cycles
    int lv0 = -1, lv1 = -1;
    for (int i = cyc[a]; i < cyc[a + 1]; ++i) {
      const int x = c.faces[i];
      bool both = false;
      for (int j = cyc[b]; j < cyc[b + 1]; ++j) both |= c.faces[j] == x;
      if (!both || x == lv0 || x == lv1) continue;
      if (lv0 < 0 || x < lv0) {
        lv1 = lv0;
        lv0 = x;
      } else if (lv1 < 0 || x < lv1) {
        lv1 = x;
      }
    }
    if (type == 1 || type == 2) {
      int(&r)[4] = type == 1 ? o.se[o.nse++] : o.ce[o.nce++];
      r[0] = lv0;
      r[1] = lv1;
      r[2] = line;
      r[3] = fid;
    }
    for (int v = 0; v < 2; ++v) {
      const int lv = v == 0 ? lv0 : lv1;
      if (lv < 0 || lv >= c.nv) continue;
      const uchar4 vv = c.ver[lv];
      for (int i = 0; i < 3; ++i) {
        const int2 hp = c.id2[pid(c, plane_at(vv, i))];
        if (hp.y == -1) continue;
        o.end[o.nend][0] = lv;
        o.end[o.nend][1] = neigh_of(hp, c.site);
        o.end[o.nend][2] = line;
        ++o.nend;
        break;
      }
    }
  }
  o.nse = sort_unique(o.se, o.nse);
  o.nce = sort_unique(o.ce, o.nce);
  o.nend = sort_unique(o.end, o.nend);
}

__global__ void pc_fe_kernel(PowerCellParams p, int fill) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= p.n) return;
  const PcCell c = pc_cell(p, q);
  FeCell o;
  fe_cell(p, c, p.cells[q].tet_id, o);
  if (!fill) {
    p.cnt[5 * p.n + q] = o.nse;
    p.cnt[6 * p.n + q] = o.nce;
    p.cnt[7 * p.n + q] = o.nend;
    return;
  }
  const int cell = (int)q;
  long long at = p.off[5 * (p.n + 1) + q];
  for (int i = 0; i < o.nse; ++i, ++at) {
    p.se[5 * at] = cell;
    for (int j = 0; j < 4; ++j) p.se[5 * at + 1 + j] = o.se[i][j];
  }
  at = p.off[6 * (p.n + 1) + q];
  for (int i = 0; i < o.nce; ++i, ++at) {
    p.ce[5 * at] = cell;
    for (int j = 0; j < 4; ++j) p.ce[5 * at + 1 + j] = o.ce[i][j];
  }
  at = p.off[7 * (p.n + 1) + q];
  for (int i = 0; i < o.nend; ++i, ++at) {
    p.se_end[4 * at] = cell;
    for (int j = 0; j < 3; ++j) p.se_end[4 * at + 1 + j] = o.end[i][j];
    const float3 x = vertex_pos(c, o.end[i][0]);
    p.se_end_pos[3 * at] = x.x;
    p.se_end_pos[3 * at + 1] = x.y;
    p.se_end_pos[3 * at + 2] = x.z;
  }
}

__global__ void pc_count_kernel(PowerCellParams p) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= p.n) return;
  const PcCell c = pc_cell(p, q);
  int tf = 0, fa = 0, ed = 0, vx = 0, sf = 0;
  for (int f = 0; f < c.np; ++f) {
    if (c.act[f] == 0) continue;
    const int2 hp = c.id2[f];
    if (hp.y != -1) {
      ++fa;
    } else {
      ++tf;
      if (hp.x <= p.max_sf_fid && !c.vnull) ++sf;
    }
  }
  for (int e = 0; e < c.ne; ++e)
    if (c.acte[e] && c.id2[c.edge[e].x].y != -1 && c.id2[c.edge[e].y].y != -1) ++ed;
  for (int t = 0; t < c.nv; ++t) {
    int nb[3], sfid;
    if (vertex_neighbours(c, t, p.max_sf_fid, nb, sfid) >= 2) ++vx;
  }
  p.cnt[0 * p.n + q] = tf;
  p.cnt[1 * p.n + q] = fa;
  p.cnt[2 * p.n + q] = ed;
  p.cnt[3 * p.n + q] = vx;
  p.cnt[4 * p.n + q] = sf;
}

__global__ void pc_fill_kernel(PowerCellParams p) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= p.n) return;
  const PcCell c = pc_cell(p, q);
  const int cell = (int)q;
  // active tet faces: per cell ascending (cell_to_tfids is a set), and
  // (site, face) keys for tfid_to_cells
  {
    long long o = p.off[0 * (p.n + 1) + q];
    int fids[4], n = 0;
    for (int f = 0; f < c.np; ++f)
      if (c.act[f] && c.id2[f].y == -1 && n < 4) fids[n++] = c.id2[f].x;
    for (int a = 1; a < n; ++a)  // insertion sort of <= 4
      for (int b = a; b > 0 && fids[b - 1] > fids[b]; --b) {
        const int t = fids[b];
        fids[b] = fids[b - 1];
        fids[b - 1] = t;
      }
    for (int a = 0; a < n; ++a) {
      p.tf_fid[o + a] = fids[a];
      p.tf_key[o + a] = ((unsigned long long)(uint32_t)c.site << 32) | (uint32_t)fids[a];
      p.tf_val[o + a] = (uint32_t)cell;
    }
  }
  // facets: (site, neighbour) keys, cell values
  {
    long long o = p.off[1 * (p.n + 1) + q];
    for (int f = 0; f < c.np; ++f) {
      if (c.act[f] == 0 || c.id2[f].y == -1) continue;
      p.fa_key[o] = ((unsigned long long)(uint32_t)c.site << 32) | (uint32_t)neigh_of(c.id2[f], c.site);
      p.fa_val[o] = (uint32_t)cell;
      ++o;
    }
  }
  // edges on two bisectors: neighbour pair, cell, the two vertices on both
  // faces (ascending)
  {
    long long o = p.off[2 * (p.n + 1) + q];
    for (int e = 0; e < c.ne; ++e) {
      const uchar4 ed = c.edge[e];
      if (!c.acte[e] || c.id2[ed.x].y == -1 || c.id2[ed.y].y == -1) continue;
      int n0 = neigh_of(c.id2[ed.x], c.site), n1 = neigh_of(c.id2[ed.y], c.site);
      if (n0 > n1) {
        const int t = n0;
        n0 = n1;
        n1 = t;
      }
      int lv[2] = {-1, -1}, k = 0;
      for (int t = 0; t < c.nv && k < 2; ++t)
        if (on_plane(c.ver[t], ed.x) && on_plane(c.ver[t], ed.y)) lv[k++] = t;
      p.ed_key[o] = ((unsigned long long)(uint32_t)n0 << 32) | (uint32_t)n1;
      p.ed_val[o] = (uint32_t)o;
      p.ed_site[o] = c.site;
      p.ed_n0[o] = n0;
      p.ed_n1[o] = n1;
      p.ed_cell[o] = cell;
      p.ed_lv0[o] = lv[0];
      p.ed_lv1[o] = lv[1];
      ++o;
    }
  }
  // vertices with >= 2 neighbour sites
  {
    long long o = p.off[3 * (p.n + 1) + q];
    for (int t = 0; t < c.nv; ++t) {
      int nb[3], sfid;
      const int n = vertex_neighbours(c, t, p.max_sf_fid, nb, sfid);
      if (n < 2) continue;
      if (n == 2) nb[2] = -1;
      for (int a = 1; a < 3; ++a)
        for (int b = a; b > 0 && nb[b - 1] > nb[b]; --b) {
          const int x = nb[b];
          nb[b] = nb[b - 1];
          nb[b - 1] = x;
        }
      const float3 pos = vertex_pos(c, t);
      p.vx_cell[o] = cell;
      p.vx_lvid[o] = t;
      for (int a = 0; a < 3; ++a) p.vx_ids[3 * o + a] = nb[a];
      p.vx_pos[3 * o] = pos.x;
      p.vx_pos[3 * o + 1] = pos.y;
      p.vx_pos[3 * o + 2] = pos.z;
      p.vx_sfid[o] = sfid;
      ++o;
    }
  }
  // surface faces: centroid of the float vertices of the face's cycle
  if (!c.vnull) {
    long long o = p.off[4 * (p.n + 1) + q];
    int slot = 0;
    for (int f = 0; f < c.np; ++f) {
      const int len = c.act[f];
      if (len == 0) continue;
      const uint8_t* cyc = c.faces + slot;
      slot += len;
      const int2 hp = c.id2[f];
      if (hp.y != -1 || hp.x > p.max_sf_fid) continue;
      float sx = 0.f, sy = 0.f, sz = 0.f;
      for (int k = 0; k < len; ++k) {
        const float3 x = vertex_pos(c, cyc[k] < c.nv ? cyc[k] : 0);
        sx = sx + x.x;
        sy = sy + x.y;
        sz = sz + x.z;
      }
      const float fl = (float)len;
      p.sf_cell[o] = cell;
      p.sf_fid[o] = hp.x;
      p.sf_pos[3 * o] = sx / fl;
      p.sf_pos[3 * o + 1] = sy / fl;
      p.sf_pos[3 * o + 2] = sz / fl;
      ++o;
    }
  }
}

// edge arrays in sorted order (val = original record index)
__global__ void pc_edge_gather_kernel(PowerCellParams p, long long n) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t s = p.ed_val[i];
  p.ed_out[7 * i + 0] = p.ed_site[s];
  p.ed_out[7 * i + 1] = p.ed_n0[s];
  p.ed_out[7 * i + 2] = p.ed_n1[s];
  p.ed_out[7 * i + 3] = p.ed_cell[s];
  p.ed_out[7 * i + 4] = p.ed_lv0[s];
  p.ed_out[7 * i + 5] = p.ed_lv1[s];
  p.ed_out[7 * i + 6] = 0;
}

// edge keys: after the (n0, n1) sort, the site (stable: site, n0, n1, cell)
__global__ void pc_edge_site_keys_kernel(PowerCellParams p, long long n) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p.ed_key[i] = (unsigned long long)(uint32_t)p.ed_site[p.ed_val[i]];
}

// neighbour cells across tet faces: consecutive sorted (site, face) records
// with equal keys are the two cells on the face
__global__ void pc_nbr_count_kernel(PowerCellParams p, long long n_tf) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i + 1 >= n_tf) return;
  if (p.tf_key[i] == p.tf_key[i + 1] && (i + 2 >= n_tf || p.tf_key[i + 2] != p.tf_key[i]) &&
      (i == 0 || p.tf_key[i - 1] != p.tf_key[i])) {
    atomicAdd(&p.nbr_cnt[p.tf_val[i]], 1);
    atomicAdd(&p.nbr_cnt[p.tf_val[i + 1]], 1);
  }
}

__global__ void pc_nbr_fill_kernel(PowerCellParams p, long long n_tf) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i + 1 >= n_tf) return;
  if (p.tf_key[i] == p.tf_key[i + 1] && (i + 2 >= n_tf || p.tf_key[i + 2] != p.tf_key[i]) &&
      (i == 0 || p.tf_key[i - 1] != p.tf_key[i])) {
    const uint32_t a = p.tf_val[i], b = p.tf_val[i + 1];
    p.nbr[p.nbr_off[a] + atomicAdd(&p.nbr_fill[a], 1)] = (int32_t)b;
    p.nbr[p.nbr_off[b] + atomicAdd(&p.nbr_fill[b], 1)] = (int32_t)a;
  }
}

// each cell's neighbours ascending (a set; at most four)
__global__ void pc_nbr_sort_kernel(PowerCellParams p) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= p.n) return;
  int32_t* a = p.nbr + p.nbr_off[q];
  const int n = (int)(p.nbr_off[q + 1] - p.nbr_off[q]);
  for (int i = 1; i < n; ++i)
    for (int j = i; j > 0 && a[j - 1] > a[j]; --j) {
      const int32_t t = a[j];
      a[j] = a[j - 1];
      a[j - 1] = t;
    }
}

__global__ void pc_site_keys_kernel(PowerCellParams p) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= p.n) return;
  p.site_key[q] = (unsigned long long)(uint32_t)p.cells[q].site_id;
  p.site_val[q] = (uint32_t)q;
}

// CSR offsets (n_site + 1) of a key array sorted by site, the site being
// the key's bits from `shift` up
__global__ void pc_site_offsets_kernel(const unsigned long long* keys, long long n, int n_site,
                                       int shift, long long* off) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i > n) return;
  const long long prev = i == 0 ? -1 : (long long)(keys[i - 1] >> shift);
  const long long cur = i == n ? (long long)n_site : (long long)(keys[i] >> shift);
  for (long long s = prev + 1; s <= cur && s <= n_site; ++s) off[s] = i;
}

}  // namespace

cudaError_t pc_count(const PowerCellParams& p, cudaStream_t st) {
  if (p.n <= 0) return cudaSuccess;
  pc_count_kernel<<<(unsigned)((p.n + 255) / 256), 256, 0, st>>>(p);
  note_launches(1);
  return cudaGetLastError();
}

cudaError_t pc_fill(const PowerCellParams& p, cudaStream_t st) {
  if (p.n <= 0) return cudaSuccess;
  pc_fill_kernel<<<(unsigned)((p.n + 255) / 256), 256, 0, st>>>(p);
  pc_site_keys_kernel<<<(unsigned)((p.n + 255) / 256), 256, 0, st>>>(p);
  note_launches(2);
  return cudaGetLastError();
}

cudaError_t pc_feature_edges(const PowerCellParams& p, int fill, cudaStream_t st) {
  if (p.n <= 0) return cudaSuccess;
  pc_fe_kernel<<<(unsigned)((p.n + 127) / 128), 128, 0, st>>>(p, fill);
  note_launches(1);
  return cudaGetLastError();
}

cudaError_t pc_edges_finish(const PowerCellParams& p, long long n_ed, int pass, cudaStream_t st) {
  if (n_ed <= 0) return cudaSuccess;
  const unsigned b = (unsigned)((n_ed + 255) / 256);
  if (pass == 0) pc_edge_site_keys_kernel<<<b, 256, 0, st>>>(p, n_ed);
  else pc_edge_gather_kernel<<<b, 256, 0, st>>>(p, n_ed);
  note_launches(1);
  return cudaGetLastError();
}

cudaError_t pc_neighbours(const PowerCellParams& p, long long n_tf, int pass, cudaStream_t st) {
  const unsigned b = (unsigned)((n_tf + 255) / 256 + 1);
  if (pass == 0) pc_nbr_count_kernel<<<b, 256, 0, st>>>(p, n_tf);
  else if (pass == 1) pc_nbr_fill_kernel<<<b, 256, 0, st>>>(p, n_tf);
  else pc_nbr_sort_kernel<<<(unsigned)((p.n + 255) / 256 + 1), 256, 0, st>>>(p);
  note_launches(1);
  return cudaGetLastError();
}

cudaError_t pc_site_offsets(const unsigned long long* keys, long long n, int n_site, int shift,
                            long long* off, cudaStream_t st) {
  pc_site_offsets_kernel<<<(unsigned)((n + 1 + 255) / 256), 256, 0, st>>>(keys, n, n_site, shift,
                                                                          off);
  note_launches(1);
  return cudaGetLastError();
}

}  // namespace rpd
