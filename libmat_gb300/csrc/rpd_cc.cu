// rpd_cc.cu -- connected components of the power cells (the
// update_pc_cc_info / update_pc_facet_cc_info / update_pc_edge_cc_info steps
// of rpd_compute_power_cells).
//
// After get_all_voro_info, libmat's update_power_cells
// (src/rpd3d_base/rpd_update.cxx:568-638) groups, per sphere, its cells into
// connected components over cell_neighbors (two cells of the sphere sharing
// a tet face): all its cells (cc_cells, :496-503), the cells on each
// neighbour's bisector (facet_cc_cells, :454-470, then sorted by component
// size) and the cells on each pair of bisectors (edge_cc_cells, :508-521).
// get_CC_given_neighbors (include/common_cxx.h:447-488) finds components
// breadth-first from the smallest unvisited id, so they come out ordered by
// their smallest cell; libstdc++'s std::sort of at most 16 groups is an
// insertion sort, so the facet components end up ordered by (size, smallest
// cell).
//
// Here the members of all groups are laid out in one row order u: the
// cells in site order (site_cells), then the facet records, then the edge
// records, each sorted by (group, cell).  Group heads and a scan give every
// row its group and the group's range.  A union-find joins every row with
// the rows of its neighbour cells in its group (binary search in the
// group's cell-sorted range) and with an equal cell's row; hooking always
// puts the larger root under the smaller (atomicCAS), so every parent id is
// below its child's, finds end, and each root is its component's smallest
// row, i.e. its smallest cell.  Root flags and a second scan number the
// roots of each group in row order (a prefix count); facet roots are ranked
// by (size, row) among their group's roots, which the scan also compacts.
// Every row then takes its root's number: the index of its component in the
// reference's vector.

#include <cuda_runtime.h>

#include "rpd_kernels.cuh"

namespace rpd {

namespace {

constexpr int kUniteIters = 1 << 20;

// root of x; halves the path on the way (every write points x at an
// ancestor, so concurrent finds stay valid)
__device__ __forceinline__ int uf_find(volatile int32_t* p, int x) {
  for (;;) {
    const int px = p[x];
    if (px == x) return x;
    const int gx = p[px];
    if (gx != px) p[x] = gx;
    x = px;
  }
}

// joins the sets of a and b; false if the retry limit was reached
__device__ bool uf_unite(int32_t* parent, int a, int b) {
  volatile int32_t* p = parent;
  for (int it = 0; it < kUniteIters; ++it) {
    a = uf_find(p, a);
    b = uf_find(p, b);
    if (a == b) return true;
    if (a < b) {
      const int t = a;
      a = b;
      b = t;
    }
    if (atomicCAS(parent + a, a, b) == a) return true;
  }
  return false;
}

// first index in [lo, hi) whose cell is >= c
template <typename F>
__device__ __forceinline__ long long lower_cell(F cell, long long lo, long long hi, long long c) {
  while (lo < hi) {
    const long long mid = (lo + hi) >> 1;
    if (cell(mid) < c) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

__device__ __forceinline__ bool edge_less(const int32_t* e, long long i, long long j) {
  const int32_t* a = e + 7 * i;
  const int32_t* b = e + 7 * j;
  if (a[0] != b[0]) return a[0] < b[0];
  if (a[1] != b[1]) return a[1] < b[1];
  return a[2] < b[2];
}

// row u's cell (cells are taken in site order) and whether u starts a group
__device__ __forceinline__ int row_cell_id(const CcParams& p, long long u) {
  return u < p.n ? (int)p.site_cells[u] : (int)u;
}

__global__ void cc_heads_kernel(CcParams p) {
  const long long u = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long n_total = p.n + p.n_fa + p.n_ed;
  if (u >= n_total) return;
  p.parent[u] = (int32_t)u;
  bool head;
  if (u < p.n) {
    head = u == 0 || p.site_key[u] != p.site_key[u - 1];
  } else if (u < p.n + p.n_fa) {
    const long long r = u - p.n;
    head = r == 0 || p.facet_keys[r] != p.facet_keys[r - 1];
    p.size[r] = 0;
  } else {
    const long long r = u - p.n - p.n_fa;
    head = r == 0 || edge_less(p.edges, r - 1, r);
  }
  p.flag[u] = head ? 1 : 0;
}

// group of every row; gstart[g] = its first row (gstart[n_groups] = n_total)
__global__ void cc_groups_kernel(CcParams p, long long n_groups) {
  const long long u = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long n_total = p.n + p.n_fa + p.n_ed;
  if (u >= n_total) return;
  const long long g = p.pos[u] + p.flag[u] - 1;
  p.gid[u] = g;
  if (p.flag[u]) p.gstart[g] = u;
  if (u == 0) p.gstart[n_groups] = n_total;
}

__global__ void cc_union_kernel(CcParams p) {
  const long long u = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  bool ok = true;
  if (u < p.n) {  // the cells of one site: their neighbours are all of it
    const int a = (int)u;
    for (long long k = p.nbr_off[a]; k < p.nbr_off[a + 1]; ++k) {
      const int b = p.nbrs[k];
      if (b > a) ok &= uf_unite(p.parent, a, b);
    }
  } else if (u < p.n + p.n_fa + p.n_ed) {  // facet or edge records
    const bool facet = u < p.n + p.n_fa;
    const long long base = facet ? p.n : p.n + p.n_fa;
    const long long g = p.gid[u];
    const long long g0 = p.gstart[g] - base, g1 = p.gstart[g + 1] - base, r = u - base;
    auto cell = [&](long long x) {
      return facet ? (long long)p.facet_cells[x] : (long long)p.edges[7 * x + 3];
    };
    const long long a = cell(r);
    if (r > g0 && cell(r - 1) == a) ok &= uf_unite(p.parent, (int)u - 1, (int)u);
    for (long long k = p.nbr_off[a]; k < p.nbr_off[a + 1]; ++k) {
      const long long b = p.nbrs[k];
      if (b <= a) continue;
      const long long j = lower_cell(cell, g0, g1, b);
      if (j < g1 && cell(j) == b) ok &= uf_unite(p.parent, (int)u, (int)(base + j));
    }
  }
  if (!ok) atomicOr(p.err, 1u);
}

// root of every row, root flags in row order, and the number of distinct
// cells of each facet component (at its root)
__global__ void cc_roots_kernel(CcParams p) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long n_total = p.n + p.n_fa + p.n_ed;
  if (i >= n_total) return;
  const int r = uf_find(p.parent, (int)i);
  p.root[i] = r;
  // flag of row order u = i: is the row's cell id its own root
  const int c = row_cell_id(p, i);
  p.flag[i] = uf_find(p.parent, c) == c ? 1 : 0;
  if (i >= p.n && i < p.n + p.n_fa) {
    const long long x = i - p.n;
    if (!(x > 0 && p.facet_keys[x - 1] == p.facet_keys[x] && p.facet_cells[x - 1] == p.facet_cells[x]))
      atomicAdd(&p.size[r - p.n], 1);
  }
}

// compacted roots: croot[pos[u]] = u
__global__ void cc_compact_kernel(CcParams p) {
  const long long u = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (u < p.n + p.n_fa + p.n_ed && p.flag[u]) p.croot[p.pos[u]] = (int32_t)u;
}

// number of each root within its group: its prefix count among the group's
// roots, or for facets its rank by (size, row) among them
__global__ void cc_rank_kernel(CcParams p) {
  const long long u = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= p.n + p.n_fa + p.n_ed || !p.flag[u]) return;
  const long long g = p.gid[u];
  const long long a = p.pos[p.gstart[g]];
  const int id = row_cell_id(p, u);
  if (u >= p.n && u < p.n + p.n_fa) {
    const long long b = p.pos[p.gstart[g + 1]];
    const int su = p.size[u - p.n];
    int k = 0;
    for (long long x = a; x < b; ++x) {
      const long long v = p.croot[x];
      const int sv = p.size[v - p.n];
      k += (sv < su || (sv == su && v < u)) ? 1 : 0;
    }
    p.rank[id] = k;
  } else {
    p.rank[id] = (int32_t)(p.pos[u] - a);
  }
}

__global__ void cc_label_kernel(CcParams p) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < p.n) p.cell_cc[i] = p.rank[p.root[i]];
  else if (i < p.n + p.n_fa) p.facet_cc[i - p.n] = p.rank[p.root[i]];
  else if (i < p.n + p.n_fa + p.n_ed) p.edge_cc[i - p.n - p.n_fa] = p.rank[p.root[i]];
}

unsigned blocks_for(long long n) { return (unsigned)((n + 255) / 256 > 0 ? (n + 255) / 256 : 1); }

// ---- surface groups (update_sphere_surf_v2fids) ----------------------------

__device__ __forceinline__ long long lower_u64(const unsigned long long* a, long long n,
                                               unsigned long long k) {
  long long lo = 0, hi = n;
  while (lo < hi) {
    const long long mid = (lo + hi) >> 1;
    if (a[mid] < k) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// (site, face) key of every surface record, the record as value
__global__ void sfg_keys_kernel(SurfaceGroupParams p) {
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= p.n_sf) return;
  const int site = p.cells[p.surface_cell[k]].site_id;
  p.keys[k] = ((unsigned long long)(uint32_t)site << 32) | (uint32_t)p.surface_fid[k];
  p.vals[k] = (uint32_t)k;
}

// the last record of each (site, face): the map's last assignment (records
// are in cell order, the sort is stable)
__global__ void sfg_last_kernel(SurfaceGroupParams p) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < p.n_sf) p.flag[i] = (i == p.n_sf - 1 || p.keys[i + 1] != p.keys[i]) ? 1 : 0;
}

__global__ void sfg_compact_kernel(SurfaceGroupParams p) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.n_sf || !p.flag[i]) return;
  const long long e = p.pos[i];
  p.ekey[e] = p.keys[i];
  p.erec[e] = (int32_t)p.vals[i];
  p.parent[e] = (int32_t)e;
}

// joins each (site, face) with the site's entries of the faces across its
// edges, unless the edge is sharp (a no-cross pair)
__global__ void sfg_union_kernel(SurfaceGroupParams p, long long n_e) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n_e) return;
  const unsigned long long key = p.ekey[e];
  const unsigned long long site = key >> 32;
  const long long f = (long long)(uint32_t)key;
  if (f >= p.n_faces) return;
  bool ok = true;
  for (int le = 0; le < 3; ++le) {
    const int nf = p.facet_adj[3 * f + le];
    if (nf < 0) continue;
    const unsigned long long lo = (unsigned long long)(f < nf ? f : nf), hi = (unsigned long long)(f < nf ? nf : f);
    const unsigned long long pk = (lo << 32) | hi;
    const long long c = lower_u64(p.no_cross, p.n_no_cross, pk);
    if (c < p.n_no_cross && p.no_cross[c] == pk) continue;
    const unsigned long long want = (site << 32) | (uint32_t)nf;
    const long long j = lower_u64(p.ekey, n_e, want);
    if (j < n_e && p.ekey[j] == want) ok &= uf_unite(p.parent, (int)e, (int)j);
  }
  if (!ok) atomicOr(p.err, 1u);
}

__global__ void sfg_roots_kernel(SurfaceGroupParams p, long long n_e) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n_e) return;
  const int r = uf_find(p.parent, (int)e);
  p.root[e] = r;
  p.flag[e] = r == e ? 1 : 0;
}

// group number of each root: its prefix count among its site's roots (faces
// ascending, so groups are ordered by smallest face)
__global__ void sfg_rank_kernel(SurfaceGroupParams p, long long n_e) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n_e || !p.flag[e]) return;
  const long long start = lower_u64(p.ekey, n_e, p.ekey[e] & 0xffffffff00000000ull);
  p.rank[e] = (int32_t)(p.pos[e] - p.pos[start]);
}

// (site, group) keys for the output order; faces stay ascending in a group
__global__ void sfg_out_keys_kernel(SurfaceGroupParams p, long long n_e) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n_e) return;
  p.keys[e] = (p.ekey[e] & 0xffffffff00000000ull) | (uint32_t)p.rank[p.root[e]];
  p.vals[e] = (uint32_t)e;
}

__global__ void sfg_gather_kernel(SurfaceGroupParams p, long long n_e) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_e) return;
  const long long e = p.vals[i];
  p.out_group[i] = (int32_t)(uint32_t)p.keys[i];
  p.out_fid[i] = (int32_t)(uint32_t)p.ekey[e];
  p.out_rec[i] = p.erec[e];
}

}  // namespace

cudaError_t surface_groups(const SurfaceGroupParams& p, long long* n_entries, cudaStream_t st) {
  *n_entries = 0;
  if (p.n_sf <= 0)
    return cudaMemsetAsync(p.site_off, 0, sizeof(long long) * (size_t)(p.n_site + 1), st);
  if (p.n_sf > 0x7fffffffll) return cudaErrorInvalidValue;
  const unsigned nb = blocks_for(p.n_sf);
  sfg_keys_kernel<<<nb, 256, 0, st>>>(p);
  note_launches(1);
  cudaError_t e = radix_sort_pairs(p.keys, p.vals, p.n_sf, 32 + p.site_bits, p.keys_tmp, p.vals_tmp,
                                   p.hist, p.hist_tmp, st);
  if (e != cudaSuccess) return e;
  sfg_last_kernel<<<nb, 256, 0, st>>>(p);
  note_launches(1);
  e = scan64_exclusive(p.flag, p.pos, p.n_sf, p.scan_tmp, st);
  long long n_e = 0;
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(&n_e, p.pos + p.n_sf, sizeof(n_e), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return e;
  const unsigned ne = blocks_for(n_e);
  sfg_compact_kernel<<<nb, 256, 0, st>>>(p);
  sfg_union_kernel<<<ne, 256, 0, st>>>(p, n_e);
  sfg_roots_kernel<<<ne, 256, 0, st>>>(p, n_e);
  note_launches(3);
  e = scan64_exclusive(p.flag, p.pos, n_e, p.scan_tmp, st);
  if (e != cudaSuccess) return e;
  sfg_rank_kernel<<<ne, 256, 0, st>>>(p, n_e);
  sfg_out_keys_kernel<<<ne, 256, 0, st>>>(p, n_e);
  note_launches(2);
  e = radix_sort_pairs(p.keys, p.vals, n_e, 32 + p.site_bits, p.keys_tmp, p.vals_tmp, p.hist,
                       p.hist_tmp, st);
  if (e != cudaSuccess) return e;
  sfg_gather_kernel<<<ne, 256, 0, st>>>(p, n_e);
  note_launches(1);
  e = pc_site_offsets(p.keys, n_e, p.n_site, 32, p.site_off, st);
  *n_entries = n_e;
  return e != cudaSuccess ? e : cudaGetLastError();
}

size_t power_cell_components_temp(long long n_total) { return scan64_temp(n_total + 1); }

cudaError_t power_cell_components(const CcParams& p, cudaStream_t st) {
  const long long n_total = p.n + p.n_fa + p.n_ed;
  if (n_total <= 0) return cudaSuccess;
  if (n_total > 0x7fffffffll) return cudaErrorInvalidValue;  // ids are int32
  const unsigned nb = blocks_for(n_total);
  cc_heads_kernel<<<nb, 256, 0, st>>>(p);
  note_launches(1);
  cudaError_t e = scan64_exclusive(p.flag, p.pos, n_total, p.scan_tmp, st);
  if (e != cudaSuccess) return e;
  long long n_groups = 0;
  e = cudaMemcpyAsync(&n_groups, p.pos + n_total, sizeof(n_groups), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return e;
  cc_groups_kernel<<<nb, 256, 0, st>>>(p, n_groups);
  cc_union_kernel<<<nb, 256, 0, st>>>(p);
  cc_roots_kernel<<<nb, 256, 0, st>>>(p);
  note_launches(3);
  e = scan64_exclusive(p.flag, p.pos, n_total, p.scan_tmp, st);
  if (e != cudaSuccess) return e;
  cc_compact_kernel<<<nb, 256, 0, st>>>(p);
  cc_rank_kernel<<<nb, 256, 0, st>>>(p);
  cc_label_kernel<<<nb, 256, 0, st>>>(p);
  note_launches(3);
  return cudaGetLastError();
}

}  // namespace rpd
