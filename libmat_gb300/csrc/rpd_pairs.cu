// rpd_pairs.cu -- everything around the clip kernel: uniform grids, the
// k-nearest-power-neighbour build, candidate (tet, site) pairs, scans and
// compaction.
//
// Reference counterparts:
//   * neighbour lists: libmat takes each site's regular-triangulation
//     neighbours from CGAL on the CPU (src/rpd3d_base/triangulation.cxx:
//     62-144, :442-558); here the lists are the k smallest power-bisector
//     distances, found by a ring search over a uniform grid of sites.
//   * candidate pairs: libmat tests every (tet, site) with the rule of
//     tet_sphere_relations_dev (src/rpd3d/voronoi.cu:154-193) -- tet t is a
//     candidate of flagged site i iff for every listed neighbour m some tet
//     vertex v has pd_m(v) > pd_i(v), power distances computed as in
//     src/rpd3d/kNN-CUDA/knncuda.cu:21-94 + :130-160 -- on dense n_site x
//     n_vert and n_site x n_tet matrices, then gathers them on the host
//     (:265-317).  Here the same rule is applied only to tets whose centroid
//     lies in a per-site box that provably contains every tet passing it
//     (see site_box_kernel), and the pairs are written as a per-tet CSR with
//     sites ascending, the reference's tet_knn order.
// Compiled with -fmad=false: the power distances and bisector keys are the
// reference's / oracle's float expressions evaluated without contraction.

#include <cuda_runtime.h>

#include <cstdint>

#include "rpd_common.cuh"
#include "rpd_kernels.cuh"
#include "rpd_scan.cuh"

namespace rpd {

static thread_local int tl_launches = 0;
void note_launches(int n) { tl_launches += n; }
int take_launches() {
  int n = tl_launches;
  tl_launches = 0;
  return n;
}

// ------------------------------------------------------------------------
// scan
// ------------------------------------------------------------------------
constexpr int kScanBlock = 1024;

size_t scan_temp_ints(long long n) { return (size_t)((n + kScanBlock - 1) / kScanBlock) + 1; }

__global__ void scan_reduce_kernel(const int32_t* in, long long n, int32_t* block_sums) {
  long long i = (long long)blockIdx.x * kScanBlock + threadIdx.x;
  int v = i < n ? in[i] : 0;
  int tot;
  block_excl_scan<int>(v, &tot);
  if (threadIdx.x == 0) block_sums[blockIdx.x] = tot;
}

__global__ void scan_blocksums_kernel(int32_t* sums, int nb) {
  int carry = 0;
  for (int base = 0; base < nb; base += kScanBlock) {
    int i = base + threadIdx.x;
    int v = i < nb ? sums[i] : 0;
    int tot;
    int ex = block_excl_scan<int>(v, &tot);
    if (i < nb) sums[i] = ex + carry;
    carry += tot;
  }
  if (threadIdx.x == 0) sums[nb] = carry;
}

__global__ void scan_apply_kernel(const int32_t* in, long long n, const int32_t* block_sums,
                                  int nb, int32_t* out) {
  long long i = (long long)blockIdx.x * kScanBlock + threadIdx.x;
  int v = i < n ? in[i] : 0;
  int ex = block_excl_scan<int>(v, nullptr);
  if (i < n) out[i] = ex + block_sums[blockIdx.x];
  if (blockIdx.x == 0 && threadIdx.x == 0) out[n] = block_sums[nb];
}

cudaError_t scan_exclusive(const int32_t* in, int32_t* out, long long n, int32_t* temp,
                           cudaStream_t st) {
  int nb = (int)((n + kScanBlock - 1) / kScanBlock);
  if (nb == 0) {
    return cudaMemsetAsync(out, 0, sizeof(int32_t), st);
  }
  scan_reduce_kernel<<<nb, kScanBlock, 0, st>>>(in, n, temp);
  note_launches(1);
  scan_blocksums_kernel<<<1, kScanBlock, 0, st>>>(temp, nb);
  note_launches(1);
  scan_apply_kernel<<<nb, kScanBlock, 0, st>>>(in, n, temp, nb, out);
  note_launches(1);
  return cudaGetLastError();
}

// ------------------------------------------------------------------------
// uniform grids
// ------------------------------------------------------------------------
__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

__device__ __forceinline__ int cell_index(const Grid& g, float x, float y, float z) {
  int ix = clampi((int)floorf((x - g.lo.x) * g.inv_cell), 0, g.nx - 1);
  int iy = clampi((int)floorf((y - g.lo.y) * g.inv_cell), 0, g.ny - 1);
  int iz = clampi((int)floorf((z - g.lo.z) * g.inv_cell), 0, g.nz - 1);
  return ix + g.nx * (iy + g.ny * iz);
}

__global__ void bin_points_kernel(const float4* pts, int n, Grid g, int32_t* cell_of,
                                  int32_t* cell_count, const uint8_t* cls, int want,
                                  float* cell_rmax) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (cls && cls[i] != want) {
    cell_of[i] = -1;
    return;
  }
  float4 p = pts[i];
  int c = cell_index(g, p.x, p.y, p.z);
  cell_of[i] = c;
  atomicAdd(cell_count + c, 1);
  // radii are >= 0: their bit patterns order as the floats do
  if (cell_rmax) atomicMax(reinterpret_cast<unsigned int*>(cell_rmax) + c, __float_as_uint(p.w));
}

__global__ void fill_cells_kernel(int n, const int32_t* cell_of, const int32_t* cell_start,
                                  int32_t* cell_fill, int32_t* cell_items) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int c = cell_of[i];
  if (c < 0) return;
  int slot = atomicAdd(cell_fill + c, 1);
  cell_items[cell_start[c] + slot] = i;
}

// insertion sort of each cell's item list (short lists): deterministic order
__global__ void sort_cells_kernel(int n_cells, const int32_t* cell_start, int32_t* items) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n_cells) return;
  int b = cell_start[c], e = cell_start[c + 1];
  for (int i = b + 1; i < e; ++i) {
    int v = items[i];
    int j = i - 1;
    while (j >= b && items[j] > v) {
      items[j + 1] = items[j];
      --j;
    }
    items[j + 1] = v;
  }
}

static cudaError_t grid_finish(int n, const Grid& g, const int32_t* cell_of, int32_t* cell_count,
                               int32_t* cell_start, int32_t* cell_fill, int32_t* cell_items,
                               int32_t* scan_tmp, cudaStream_t st) {
  long long n_cells = (long long)g.nx * g.ny * g.nz;
  cudaError_t err = scan_exclusive(cell_count, cell_start, n_cells, scan_tmp, st);
  if (err != cudaSuccess) return err;
  cudaMemsetAsync(cell_fill, 0, sizeof(int32_t) * n_cells, st);
  fill_cells_kernel<<<(n + 255) / 256, 256, 0, st>>>(n, cell_of, cell_start, cell_fill, cell_items);
  note_launches(1);
  sort_cells_kernel<<<(int)((n_cells + 255) / 256), 256, 0, st>>>((int)n_cells, cell_start,
                                                                 cell_items);
  note_launches(1);
  return cudaGetLastError();
}

cudaError_t grid_build_sites(const float4* pts, int n, const Grid& g, int32_t* cell_of,
                             int32_t* cell_count, int32_t* cell_start, int32_t* cell_fill,
                             int32_t* cell_items, int32_t* scan_tmp, cudaStream_t st) {
  long long n_cells = (long long)g.nx * g.ny * g.nz;
  cudaMemsetAsync(cell_count, 0, sizeof(int32_t) * n_cells, st);
  if (n > 0) {
    bin_points_kernel<<<(n + 255) / 256, 256, 0, st>>>(pts, n, g, cell_of, cell_count, nullptr, 0,
                                                      nullptr);
    note_launches(1);
  }
  return grid_finish(n, g, cell_of, cell_count, cell_start, cell_fill, cell_items, scan_tmp, st);
}

// centroid and radius (largest vertex distance) of every tet
__global__ void tet_centroid_kernel(const float* v, const int4* tets, int n_tet, float4* out,
                                    float4* xyz, const int32_t* v_adjs, uchar4* vadj) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_tet) return;
  int4 q = tets[t];
  int id[4] = {q.x, q.y, q.z, q.w};
  float cx = 0.f, cy = 0.f, cz = 0.f;
  for (int k = 0; k < 4; ++k) {
    cx += v[3 * id[k]];
    cy += v[3 * id[k] + 1];
    cz += v[3 * id[k] + 2];
  }
  cx *= 0.25f;
  cy *= 0.25f;
  cz *= 0.25f;
  float r2 = 0.f;
  for (int k = 0; k < 4; ++k) {
    float dx = v[3 * id[k]] - cx, dy = v[3 * id[k] + 1] - cy, dz = v[3 * id[k] + 2] - cz;
    r2 = fmaxf(r2, dx * dx + dy * dy + dz * dz);
  }
  out[t] = make_float4(cx, cy, cz, sqrtf(r2));
  if (xyz) {  // the four vertices, packed: (v0, v1.x) (v1.yz, v2.xy) (v2.z, v3)
    float f[12];
    for (int k = 0; k < 4; ++k)
      for (int a = 0; a < 3; ++a) f[3 * k + a] = v[3 * id[k] + a];
    xyz[3ll * t] = make_float4(f[0], f[1], f[2], f[3]);
    xyz[3ll * t + 1] = make_float4(f[4], f[5], f[6], f[7]);
    xyz[3ll * t + 2] = make_float4(f[8], f[9], f[10], f[11]);
  }
  if (vadj)
    vadj[t] = make_uchar4((uint8_t)v_adjs[id[0]], (uint8_t)v_adjs[id[1]], (uint8_t)v_adjs[id[2]],
                          (uint8_t)v_adjs[id[3]]);
}

cudaError_t tet_centroids(const float* vert3f, const int4* tets, int n_tet, float4* centroid,
                          cudaStream_t st, float4* tet_xyz, const int32_t* v_adjs,
                          uchar4* tet_vadj) {
  if (n_tet > 0) {
    tet_centroid_kernel<<<(n_tet + 255) / 256, 256, 0, st>>>(vert3f, tets, n_tet, centroid,
                                                              tet_xyz, v_adjs, tet_vadj);
    note_launches(1);
  }
  return cudaGetLastError();
}

cudaError_t grid_build_tets(const float4* centroid, int n_tet, const uint8_t* cls, int want,
                            const Grid& g, int32_t* cell_of, int32_t* cell_count,
                            int32_t* cell_start, int32_t* cell_fill, int32_t* cell_items,
                            int32_t* scan_tmp, cudaStream_t st, float* cell_rmax) {
  long long n_cells = (long long)g.nx * g.ny * g.nz;
  cudaMemsetAsync(cell_count, 0, sizeof(int32_t) * n_cells, st);
  if (cell_rmax) cudaMemsetAsync(cell_rmax, 0, sizeof(float) * n_cells, st);
  if (n_tet > 0) {
    bin_points_kernel<<<(n_tet + 255) / 256, 256, 0, st>>>(centroid, n_tet, g, cell_of, cell_count,
                                                          cls, want, cell_rmax);
    note_launches(1);
  }
  return grid_finish(n_tet, g, cell_of, cell_count, cell_start, cell_fill, cell_items, scan_tmp,
                     st);
}

// ------------------------------------------------------------------------
// warp helper: iterate the items of a set of grid cells, 32 at a time
// ------------------------------------------------------------------------
// cells are enumerated by `cell_at(idx)` for idx in [0, n_cells_iter), which
// returns a cell id or -1; fn(item, valid) is called warp-uniformly for
// batches of 32 items (valid = false for padding lanes).
template <class CellAt, class Fn>
__device__ void for_items(int n_cells_iter, CellAt cell_at, const int32_t* cell_start,
                          const int32_t* cell_items, int lane, Fn fn) {
  for (int cb = 0; cb < n_cells_iter; cb += 32) {
    int ci = cb + lane;
    int cell = ci < n_cells_iter ? cell_at(ci) : -1;
    int b = 0, cnt = 0;
    if (cell >= 0) {
      b = cell_start[cell];
      cnt = cell_start[cell + 1] - b;
    }
    int incl = warp_incl_scan<int>(cnt, lane);
    int total = __shfl_sync(0xffffffffu, incl, 31);
    int excl = incl - cnt;
    for (int ib = 0; ib < total; ib += 32) {
      int g = ib + lane;
      // owner lane: the last lane whose exclusive prefix is <= g
      int owner = 0;
      for (int o = 16; o > 0; o >>= 1) {
        int cand = owner + o;
        int ex = __shfl_sync(0xffffffffu, excl, cand);
        if (ex <= g) owner = cand;
      }
      int ob = __shfl_sync(0xffffffffu, b, owner);
      int oe = __shfl_sync(0xffffffffu, excl, owner);
      bool valid = g < total;
      int item = valid ? cell_items[ob + (g - oe)] : -1;
      fn(item, valid);
    }
  }
}

// ------------------------------------------------------------------------
// k nearest power neighbours
// ------------------------------------------------------------------------
constexpr int kKnnBuf = 1024;
constexpr int kKnnWarps = 4;
constexpr int kKnnLongBuf = 8192;  // long lists (k > kKnnBuf - 64): 64 KB, one warp per block
// base lists (k <= kKnnSmallBuf - 64): half the buffer, twice the warps in
// the same shared memory (more warps to hide the search's latency; 1M-tet
// workload, k = 128: 2.64 -> 1.82 ms; a quarter of the buffer with four
// times the warps measured the same)
constexpr int kKnnSmallBuf = 512;
constexpr int kKnnSmallWarps = 8;

__device__ __forceinline__ uint32_t order_key(float f) {
  uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float key_value(uint32_t u) {
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

// power-bisector distance of site j from site i (same expression as the
// oracle): ((|cj - ci|^2 - wj) + wi) / (2 |cj - ci|)
__device__ __forceinline__ float bisector_key(float4 si, float4 sj) {
  float dx = sj.x - si.x, dy = sj.y - si.y, dz = sj.z - si.z;
  float d2 = dx * dx + dy * dy + dz * dz;
  if (d2 == 0.0f) return sj.w > si.w ? -INFINITY : INFINITY;
  float num = (d2 - sj.w) + si.w;
  float den = 2.0f * sqrtf(d2);
  return num / den;
}

// bitonic sort of buf[0..n) (n power of two) by one warp, ascending
__device__ void warp_bitonic_sort(unsigned long long* buf, int n, int lane) {
  for (int k = 2; k <= n; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = lane; i < n; i += 32) {
        int l = i ^ j;
        if (l > i) {
          unsigned long long a = buf[i], b = buf[l];
          bool up = (i & k) == 0;
          if ((a > b) == up) {
            buf[i] = b;
            buf[l] = a;
          }
        }
      }
      __syncwarp();
    }
  }
}

__device__ __forceinline__ int next_pow2(int x) {
  int p = 32;
  while (p < x) p <<= 1;
  return p;
}

// One warp per row: the k smallest (key, id) of site i = subset[row] (or
// i = row), optionally only keys <= B (B = R_i * bound_scale + bound_abs,
// R_i the float in radius[i]).  Rings of grid cells around the site are
// searched until every site outside has a key above the k-th kept one (or
// above B): keys of sites at distance >= D are >= (D^2 + w_i - w_max)/(2D).
// Candidates collect in a per-warp buffer of BUF entries (key bits | id,
// 64-bit) that is sorted and cut to k whenever it fills.
template <int BUF, int WARPS>
__global__ void __launch_bounds__(WARPS * 32) knn_kernel(KnnArgs a) {
  extern __shared__ __align__(16) unsigned long long knn_smem[];
  __shared__ int scnt[WARPS];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  unsigned long long* buf = knn_smem + (size_t)wid * BUF;
  const int row = blockIdx.x * WARPS + wid;
  if (row >= a.n_rows) return;
  const int i = a.subset ? a.subset[row] : row;
  const int k = a.k;
  const Grid& g = a.g;
  const float4 si = a.site4f[i];
  const int2 rng = a.site_range ? a.site_range[i] : make_int2(0, 0x7fffffff);
  float B = INFINITY;
  if (a.radius) {
    const float R = __uint_as_float(a.radius[i]);
    B = R * a.bound_scale + a.bound_abs;
    if (!(B < INFINITY)) B = INFINITY;  // inf or nan radius: no bound
  }
  const float4 gp = a.grid_pos ? a.grid_pos[i] : si;
  const int cx = clampi((int)floorf((gp.x - g.lo.x) * g.inv_cell), 0, g.nx - 1);
  const int cy = clampi((int)floorf((gp.y - g.lo.y) * g.inv_cell), 0, g.ny - 1);
  const int cz = clampi((int)floorf((gp.z - g.lo.z) * g.inv_cell), 0, g.nz - 1);
  const int rmax = max(max(max(cx, g.nx - 1 - cx), max(cy, g.ny - 1 - cy)), max(cz, g.nz - 1 - cz));
  if (lane == 0) scnt[wid] = 0;
  __syncwarp();
  unsigned long long kth = ~0ull;  // packed k-th best so far (after a sort)
  int done = 0;
  for (int r = 0; r <= rmax && !done; ++r) {
    const int side = 2 * r + 1;
    const int n_cube = side * side * side;
    auto cell_at = [&](int idx) -> int {
      int dx = idx % side - r, dy = (idx / side) % side - r, dz = idx / (side * side) - r;
      if (max(max(abs(dx), abs(dy)), abs(dz)) != r) return -1;
      int x = cx + dx, y = cy + dy, z = cz + dz;
      if (x < 0 || y < 0 || z < 0 || x >= g.nx || y >= g.ny || z >= g.nz) return -1;
      return x + g.nx * (y + g.ny * z);
    };
    for_items(n_cube, cell_at, a.cell_start, a.cell_items, lane, [&](int j, bool valid) {
      bool take = false;
      unsigned long long packed = 0;
      if (valid && j != i && j >= rng.x && j < rng.y) {
        float key = bisector_key(si, a.site4f[j]);
        packed = ((unsigned long long)order_key(key) << 32) | (uint32_t)j;
        take = packed < kth && key <= B;
      }
      uint32_t m = __ballot_sync(0xffffffffu, take);
      int base = scnt[wid];
      if (take) buf[base + __popc(m & ((1u << lane) - 1u))] = packed;
      __syncwarp();
      int cnt = base + __popc(m);
      if (cnt > BUF - 32) {
        // sort and keep the best k
        for (int q = cnt + lane; q < BUF; q += 32) buf[q] = ~0ull;
        __syncwarp();
        warp_bitonic_sort(buf, BUF, lane);
        cnt = min(cnt, k);
        if (cnt >= k) kth = buf[k - 1];
      }
      if (lane == 0) scnt[wid] = cnt;
      __syncwarp();
    });
    int cnt = scnt[wid];
    int n = next_pow2(max(cnt, 1));
    for (int q = cnt + lane; q < n; q += 32) buf[q] = ~0ull;
    __syncwarp();
    warp_bitonic_sort(buf, n, lane);
    cnt = min(cnt, k);
    if (lane == 0) scnt[wid] = cnt;
    float T = B;  // keys above T are not wanted
    if (cnt >= k) {
      kth = buf[k - 1];
      T = fminf(T, key_value((uint32_t)(kth >> 32)));
    }
    // keys of sites outside the searched block are >= f(D) with
    // D >= r * cell, f(D) = (D^2 + wi - wmax) / (2D) increasing in D
    float D = (float)r * g.cell;
    if (D > 0.f && T < INFINITY) {
      float lb = (D * D + si.w - a.w_max) / (2.f * D);
      if (T < lb - 1e-4f * (fabsf(lb) + D)) done = 1;
    }
    __syncwarp();
  }
  int cnt = scnt[wid];
  if (a.status && lane == 0) a.status[row] = done ? 0 : 1;  // 1: exhausted grid
  if (lane == 0) {
    if (a.len_out) a.len_out[row] = cnt;
    // every site not listed has a key >= this: the k-th key when the list
    // is full, else the bound (or none: all sites were seen)
    if (a.bound_out) a.bound_out[row] = cnt >= k ? key_value((uint32_t)(buf[k - 1] >> 32)) : B;
  }
  const long long rb = (long long)row * k;
  // outputs in distance order
  for (int q = lane; q < k; q += 32) {
    int32_t id = q < cnt ? (int32_t)(uint32_t)buf[q] + a.id_offset : -1;
    if (a.keys) a.keys[rb + q] = q < cnt ? key_value((uint32_t)(buf[q] >> 32)) : INFINITY;
    if (!a.order_by_id) a.nbr[rb + q] = id;
    if (a.nbr_dist) a.nbr_dist[rb + q] = id;
  }
  if (a.order_by_id) {
    __syncwarp();
    int n = next_pow2(max(k, 1));
    // reuse the buffer: ids as 64-bit values, padding at the end
    for (int q = lane; q < n; q += 32) {
      unsigned long long v = ~0ull;
      if (q < cnt) v = (unsigned long long)(uint32_t)buf[q];
      __syncwarp();
      buf[q] = v;
    }
    __syncwarp();
    warp_bitonic_sort(buf, n, lane);
    for (int q = lane; q < k; q += 32)
      a.nbr[rb + q] = q < cnt ? (int32_t)buf[q] + a.id_offset : -1;
  }
}

int knn_max_k() { return kKnnLongBuf - 64; }

cudaError_t launch_knn(const KnnArgs& a, cudaStream_t st) {
  if (a.n_rows <= 0) return cudaSuccess;
  if (a.k < 1 || a.k > knn_max_k()) return cudaErrorInvalidValue;
  if (a.k <= kKnnSmallBuf - 64) {
    const size_t smem = (size_t)kKnnSmallWarps * kKnnSmallBuf * sizeof(unsigned long long);
    int blocks = (a.n_rows + kKnnSmallWarps - 1) / kKnnSmallWarps;
    knn_kernel<kKnnSmallBuf, kKnnSmallWarps><<<blocks, kKnnSmallWarps * 32, smem, st>>>(a);
  } else if (a.k <= kKnnBuf - 64) {
    const size_t smem = (size_t)kKnnWarps * kKnnBuf * sizeof(unsigned long long);
    int blocks = (a.n_rows + kKnnWarps - 1) / kKnnWarps;
    knn_kernel<kKnnBuf, kKnnWarps><<<blocks, kKnnWarps * 32, smem, st>>>(a);
  } else {
    // long lists: one warp per block, kKnnLongBuf entries of shared memory
    const size_t smem = (size_t)kKnnLongBuf * sizeof(unsigned long long);
    // (set on every such launch: the attribute belongs to the current device)
    cudaError_t e = cudaFuncSetAttribute(knn_kernel<kKnnLongBuf, 1>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    knn_kernel<kKnnLongBuf, 1><<<a.n_rows, 32, smem, st>>>(a);
  }
  note_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_knn(const float4* site4f, int n_site, const Grid& g, const int32_t* cell_start,
                       const int32_t* cell_items, int k, float w_max, int order_by_id,
                       int32_t* nbr, float* keys, int32_t* nbr_dist, int32_t* status,
                       cudaStream_t st, int id_offset, float* bound_out) {
  KnnArgs a = {};
  a.site4f = site4f;
  a.n_rows = n_site;
  a.g = g;
  a.cell_start = cell_start;
  a.cell_items = cell_items;
  a.k = k;
  a.w_max = w_max;
  a.order_by_id = order_by_id;
  a.nbr = nbr;
  a.keys = keys;
  a.nbr_dist = nbr_dist;
  a.status = status;
  a.id_offset = id_offset;
  a.bound_out = bound_out;
  return launch_knn(a, st);
}

// ------------------------------------------------------------------------
// candidate pairs
// ------------------------------------------------------------------------
// power distance of a mesh vertex to a site, the reference's float order
__device__ __forceinline__ float pow_dist(float4 s, float3 v) {
  float t0 = s.x - v.x, t1 = s.y - v.y, t2 = s.z - v.z;
  float ssd = t0 * t0;
  ssd = ssd + t1 * t1;
  ssd = ssd + t2 * t2;
  return ssd - s.w;
}

constexpr int kPairWarps = 4;
constexpr int kPairMaxK = 128;  // longest neighbour list (rpd_config.knn_k <= 128)
// a tet goes through three stages, each on full warps: the centroid test
// (one tet per lane); the tets that pass wait in a per-warp queue and try
// the rule's first kRuleFirst neighbours 32 at a time; the tets that survive
// those wait in a second queue and are finished 32 at a time against the
// rest of the list (queues of kRuleQueue entries).  kRuleFirst: 4 to 16 were
// measured on the 1M-tet workload, 8 the fastest; the macro only serves such
// sweeps
#ifndef RPD_RULE_FIRST
#define RPD_RULE_FIRST 8
#endif
constexpr int kRuleFirst = RPD_RULE_FIRST;
// (even: the drain steps two neighbours at a time from kRuleFirst, and its
// acceptance checkpoints sit at multiples of 8)
static_assert(kRuleFirst % 2 == 0, "kRuleFirst even");
constexpr int kRuleQueue = 64;

// cell range of the site's box in the tet grid (empty range for no box)
struct CellRange {
  int x0, y0, z0, sx, sy, sz;
};

__device__ __forceinline__ CellRange site_cells(const PairParams& p, int i) {
  CellRange r = {0, 0, 0, 0, 0, 0};
  if (p.flags[p.site_base + i] != 1u) return r;
  const float4 blo = p.site_box[2 * i], bhi = p.site_box[2 * i + 1];
  if (!(blo.x <= bhi.x && blo.y <= bhi.y && blo.z <= bhi.z)) return r;
  const Grid& g = p.tg;
  r.x0 = clampi((int)floorf((blo.x - g.lo.x) * g.inv_cell), 0, g.nx - 1);
  r.y0 = clampi((int)floorf((blo.y - g.lo.y) * g.inv_cell), 0, g.ny - 1);
  r.z0 = clampi((int)floorf((blo.z - g.lo.z) * g.inv_cell), 0, g.nz - 1);
  int x1 = clampi((int)floorf((bhi.x - g.lo.x) * g.inv_cell), 0, g.nx - 1);
  int y1 = clampi((int)floorf((bhi.y - g.lo.y) * g.inv_cell), 0, g.ny - 1);
  int z1 = clampi((int)floorf((bhi.z - g.lo.z) * g.inv_cell), 0, g.nz - 1);
  r.sx = x1 - r.x0 + 1;
  r.sy = y1 - r.y0 + 1;
  r.sz = z1 - r.z0 + 1;
  return r;
}

constexpr int kPairTaskCells = 512;

// tasks per site: its box's grid cells in chunks of kPairTaskCells
__global__ void pair_tasks_kernel(PairParams p, int32_t* n_tasks) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.n_site) return;
  CellRange r = site_cells(p, i);
  long long n = (long long)r.sx * r.sy * r.sz;
  n_tasks[i] = (int)((n + kPairTaskCells - 1) / kPairTaskCells);
}

// Persistent warps take (site, chunk of its box's cells) tasks from a work
// counter, so a site with a large box is spread over many warps.
__global__ void __launch_bounds__(kPairWarps * 32) pairs_kernel(PairParams p,
                                                                const int32_t* task_off,
                                                                unsigned long long* work) {
  __shared__ float4 spl[kPairWarps][kBoxPlanes];
  __shared__ float spn[kPairWarps][kBoxPlanes];  // |normal| of each plane, rounded down
  __shared__ float4 snb[kPairWarps][kPairMaxK];  // the site's neighbours (rule order)
  // queued tets: vertices (12 floats), power distances to the site (4), id
  __shared__ float sq_v[kPairWarps][16][kRuleQueue];
  __shared__ int sq_t[kPairWarps][kRuleQueue];
  // tets whose centroid passed, waiting for the rule's first part
  __shared__ int sa_t[kPairWarps][kRuleQueue];
  // every 8th neighbour r: its key and the smallest site distance |c_m - c_i|
  // (rounded down) of the neighbours from r on
  __shared__ float schk_key[kPairWarps][kPairMaxK / 8];
  __shared__ float schk_d[kPairWarps][kPairMaxK / 8];
  const int lane = threadIdx.x & 31;
  const int wid = threadIdx.x >> 5;
  const long long n_tasks = task_off[p.n_site];
  unsigned int n_cells_seen = 0, n_keep = 0, n_items = 0, n_in = 0;
  for (;;) {
    long long task = 0;
    if (lane == 0) task = (long long)atomicAdd(work, 1ull);
    task = __shfl_sync(0xffffffffu, task, 0);
    if (task >= n_tasks) break;
    // owning site: last i with task_off[i] <= task
    int lo = 0, hi = p.n_site - 1;
    while (lo < hi) {
      int mid = (lo + hi + 1) >> 1;
      if (task_off[mid] <= task) lo = mid;
      else hi = mid - 1;
    }
    const int i = lo;
    const int chunk = (int)(task - task_off[i]);
    const CellRange cr = site_cells(p, i);
    const int n_all = cr.sx * cr.sy * cr.sz;
    const int c_begin = chunk * kPairTaskCells;
    const int n_iter = min(kPairTaskCells, n_all - c_begin);
    const float4 blo = p.site_box[2 * i], bhi = p.site_box[2 * i + 1];
    // planes of the site's grown cell, each loosened by its own float
    // evaluation error so that the tests below never reject a centroid the
    // exact planes accept
    const int npl = p.site_nplanes[i];
    float4* pl = spl[wid];
    float* pn = spn[wid];
    __syncwarp();
    for (int q = lane; q < npl; q += 32) {
      float4 e = p.site_planes[(long long)i * kBoxPlanes + q];
      float tol = 4e-6f * ((fabsf(e.x) + fabsf(e.y) + fabsf(e.z)) * p.coord_scale + fabsf(e.w));
      pl[q] = make_float4(e.x, e.y, e.z, e.w + tol);
      // bisectors only: the region's box planes (axis-aligned, the mesh box
      // and its margin) were not pushed out (an axis-aligned bisector is
      // left as it is too, which only accepts more)
      const int n_zero = (e.x == 0.f) + (e.y == 0.f) + (e.z == 0.f);
      pn[q] = n_zero >= 2 ? 0.f : sqrtf(e.x * e.x + e.y * e.y + e.z * e.z) * (1.0f - 1e-5f);
    }
    // the tests take the planes two at a time: an odd count gets a plane
    // that every point passes (kBoxPlanes is even, so the slot exists)
    static_assert(kBoxPlanes % 2 == 0, "plane pairs");
    if (lane == 0 && (npl & 1)) {
      pl[npl] = make_float4(0.f, 0.f, 0.f, 1.f);
      pn[npl] = 0.f;
    }
    __syncwarp();
    const float4 si = p.site4f[p.site_base + i];
    const Grid& g = p.tg;
    // the rule is over the whole list; in ascending bisector distance (when
    // the GPU built it) the neighbour that dominates a far tet comes first
    const int32_t* L = (p.rule_nbr ? p.rule_nbr : p.nbr) + (long long)i * p.k;
    float4* nb = snb[wid];
    // a hole (-1) never rejects a tet: weight -inf makes its power distance +inf
    const int k_staged = min(p.k, kPairMaxK);
    for (int r = lane; r < k_staged; r += 32) {
      const int m = __ldg(L + r);
      nb[r] = m < 0 ? make_float4(0.f, 0.f, 0.f, -INFINITY) : __ldg(p.site4f + m);
    }
    __syncwarp();
    // the acceptance checkpoints (distance-ordered lists with keys only)
    const bool acc_ok = p.rule_keys != nullptr && k_staged == p.k;
    if (acc_ok) {
      float carry = INFINITY;
      for (int w = (k_staged - 1) >> 5; w >= 0; --w) {
        const int r = lane + 32 * w;
        float d = INFINITY;  // a hole never rejects
        if (r < k_staged) {
          const float4 m = nb[r];
          if (m.w != -INFINITY) {
            const float dx = m.x - si.x, dy = m.y - si.y, dz = m.z - si.z;
            d = sqrtf(dx * dx + dy * dy + dz * dz) * (1.0f - 1e-6f);
          }
        }
        // suffix minimum: lane l gets the minimum over lanes >= l
        for (int o = 1; o < 32; o <<= 1) {
          const float t = __shfl_down_sync(0xffffffffu, d, o);
          if (lane + o < 32) d = fminf(d, t);
        }
        d = fminf(d, carry);
        carry = __shfl_sync(0xffffffffu, d, 0);
        if (r < k_staged && (r & 7) == 0) {
          schk_d[wid][r >> 3] = d;
          schk_key[wid][r >> 3] = __ldg(p.rule_keys + (long long)i * p.k + r);
        }
      }
      __syncwarp();
    }
    // neighbour r of the rule order (staged, or read for long user lists)
    auto rule_site = [&](int r) -> float4 {
      if (r < k_staged) return nb[r];
      const int m = __ldg(L + r);
      return m < 0 ? make_float4(0.f, 0.f, 0.f, -INFINITY) : __ldg(p.site4f + m);
    };
    n_cells_seen += n_iter;
    // half extent of a grid cell, grown for the rounding of the binning
    const float hc = 0.5f * g.cell * (1.0f + 1e-3f) + 1e-6f * p.coord_scale;
    auto cell_at = [&](int idx) -> int {
      idx += c_begin;
      int x = cr.x0 + idx % cr.sx, y = cr.y0 + (idx / cr.sx) % cr.sy, z = cr.z0 + idx / (cr.sx * cr.sy);
      // reject cells lying entirely outside one plane of the grown cell
      float cxm = g.lo.x + ((float)x + 0.5f) * g.cell;
      float cym = g.lo.y + ((float)y + 0.5f) * g.cell;
      float czm = g.lo.z + ((float)z + 0.5f) * g.cell;
      // (the culling tests use FMA: one rounding per term, well inside the
      // planes' loosening; the rule itself keeps the reference's order)
      auto box_max = [&](float4 e, float off) {
        return __fmaf_rn(e.x, cxm, __fmaf_rn(e.y, cym, __fmaf_rn(e.z, czm,
               __fmaf_rn(hc, fabsf(e.x) + fabsf(e.y) + fabsf(e.z), e.w - off))));
      };
      for (int q = 0; q < npl; q += 2)
        if ((box_max(pl[q], 0.f) < 0.f) | (box_max(pl[q + 1], 0.f) < 0.f)) return -1;
      const int cell = x + g.nx * (y + g.ny * z);
      // again with the cell's largest tet radius in place of the class's
      // (the centroid test below, applied to the best centroid in the cell)
      if (p.tcell_rmax) {
        const float shrink =
            fmaxf(p.offset_r - (__ldg(p.tcell_rmax + cell) * (1.0f + 1e-5f) + 1e-6f * p.coord_scale),
                  0.f);
        if (shrink > 0.f) {
          for (int q = 0; q < npl; q += 2)
            if ((box_max(pl[q], shrink * pn[q]) < 0.f) | (box_max(pl[q + 1], shrink * pn[q + 1]) < 0.f))
              return -1;
        }
      }
      ++n_keep;
      return cell;
    };
    // a tet that passed the rule becomes a pair
    auto emit = [&](bool pass, int t) {
      uint32_t msk = __ballot_sync(0xffffffffu, pass);
      if (msk) {
        unsigned long long base = 0;
        if (lane == 0) base = atomicAdd(p.pair_cursor, (unsigned long long)__popc(msk));
        base = __shfl_sync(0xffffffffu, base, 0);
        if (pass) {
          unsigned long long slot = base + __popc(msk & ((1u << lane) - 1u));
          if ((long long)slot < p.pair_cap)
            p.pair_buf[slot] = make_int2(t + p.tet_base, i + p.site_base);
          atomicAdd(p.tet_count + p.tet_base + t, 1);
        }
      }
    };
    float(*qv)[kRuleQueue] = sq_v[wid];
    int* qt = sq_t[wid];
    int qn = 0;  // queued tets (warp-uniform)
    // the first n queued tets, one per lane, against the rest of the list;
    // the others move to the front
    auto drain = [&](int n) {
      bool pass = false;
      int t = -1;
      if (lane < n) {
        float3 v[4];
        float pdi[4];
        for (int a = 0; a < 4; ++a) {
          v[a] = make_float3(qv[3 * a][lane], qv[3 * a + 1][lane], qv[3 * a + 2][lane]);
          pdi[a] = qv[12 + a][lane];
        }
        t = qt[lane];
        pass = true;
        // distance from the site to the tet's nearest vertex, rounded up
        float m2 = INFINITY;
        for (int a = 0; a < 4; ++a) {
          const float dx = v[a].x - si.x, dy = v[a].y - si.y, dz = v[a].z - si.z;
          m2 = fminf(m2, dx * dx + dy * dy + dz * dz);
        }
        const float d_up = sqrtf(m2) * (1.0f + 1e-6f);
        for (int r = kRuleFirst; r < p.k && pass; r += 2) {
          // pd_m(v) - pd_i(v) = 2 |c_m - c_i| (key_m - (v - c_i).u_m) for the
          // unit direction u_m to m: a vertex within key_m of the site,
          // by more than the float error of the two power distances, has
          // pd_m(v) > pd_i(v) as evaluated; keys ascend along the list
          if (acc_ok && (r & 7) == 0) {
            const float g = schk_key[wid][r >> 3] * (1.0f - 64.0f * 5.9604645e-08f) -
                            p.accept_margin - d_up;
            if (g > 0.f && 2.0f * schk_d[wid][r >> 3] * g > p.accept_err) break;
          }
          // two neighbours per step (independent chains; the rule is an AND,
          // so testing one past a failure changes nothing)
          const float4 sm0 = rule_site(r);
          const float4 sm1 = r + 1 < p.k ? rule_site(r + 1) : sm0;
          bool hit0 = false, hit1 = false;
          for (int a = 0; a < 4; ++a) {
            hit0 |= pow_dist(sm0, v[a]) > pdi[a];
            hit1 |= pow_dist(sm1, v[a]) > pdi[a];
          }
          pass = hit0 & hit1;
        }
      }
      emit(pass, t);
      __syncwarp();
      const int rest = qn - n;  // < 32: sources n.., targets 0.. do not overlap
      if (lane < rest) {
        for (int w = 0; w < 16; ++w) qv[w][lane] = qv[w][n + lane];
        qt[lane] = qt[n + lane];
      }
      __syncwarp();
      qn = rest;
    };
    // the first n tets of the centroid queue, one per lane: their vertices,
    // power distances and the rule's first kRuleFirst neighbours; survivors
    // join the drain's queue (qn <= 31 before, so there is room for 32)
    int* qa_t = sa_t[wid];
    int qa = 0;  // tets in the centroid queue (warp-uniform)
    auto first_part = [&](int n) {
      bool pass = false, survive = false;
      float3 v[4] = {};
      float pdi[4] = {};
      int t = -1;
      if (lane < n) {
        t = qa_t[lane];
        const float4 q0 = __ldg(p.tet_xyz + 3ll * t), q1 = __ldg(p.tet_xyz + 3ll * t + 1),
                     q2 = __ldg(p.tet_xyz + 3ll * t + 2);
        v[0] = make_float3(q0.x, q0.y, q0.z);
        v[1] = make_float3(q0.w, q1.x, q1.y);
        v[2] = make_float3(q1.z, q1.w, q2.x);
        v[3] = make_float3(q2.y, q2.z, q2.w);
        for (int a = 0; a < 4; ++a) pdi[a] = pow_dist(si, v[a]);
        // voronoi.cu:154-193 (holes, -1, never reject: voronoi.cu:171):
        // a candidate iff every neighbour m has a tet vertex where
        // pd_m > pd_i; the order of the neighbours does not matter
        pass = true;
        const int r_end = min(p.k, kRuleFirst);
        for (int r = 0; r < r_end && pass; r += 2) {
          const float4 sm0 = rule_site(r);
          const float4 sm1 = r + 1 < r_end ? rule_site(r + 1) : sm0;
          bool hit0 = false, hit1 = false;
          for (int a = 0; a < 4; ++a) {
            hit0 |= pow_dist(sm0, v[a]) > pdi[a];
            hit1 |= pow_dist(sm1, v[a]) > pdi[a];
          }
          pass = hit0 & hit1;
        }
        if (pass && p.k > kRuleFirst) {
          survive = true;
          pass = false;
        }
      }
      __syncwarp();  // every lane has read its entry
      const int rest = qa - n;  // < 32: sources n.., targets 0.. do not overlap
      if (lane < rest) qa_t[lane] = qa_t[n + lane];
      const uint32_t sv = __ballot_sync(0xffffffffu, survive);
      if (survive) {
        const int pos = qn + __popc(sv & ((1u << lane) - 1u));
        for (int a = 0; a < 4; ++a) {
          qv[3 * a][pos] = v[a].x;
          qv[3 * a + 1][pos] = v[a].y;
          qv[3 * a + 2][pos] = v[a].z;
          qv[12 + a][pos] = pdi[a];
        }
        qt[pos] = t;
      }
      qn += __popc(sv);
      emit(pass, t);
      __syncwarp();
      qa = rest;
      if (qn >= 32) drain(32);
    };
    for_items(n_iter, cell_at, p.tcell_start, p.tcell_items, lane, [&](int t, bool valid) {
      bool in = false;
      if (valid) {
        ++n_items;
        float4 c = p.centroid[t];
        in = c.x >= blo.x && c.x <= bhi.x && c.y >= blo.y && c.y <= bhi.y && c.z >= blo.z &&
             c.z <= bhi.z;
        // A tet passes the rule for neighbour m only if a vertex lies on the
        // site's side of their bisector, so its centroid lies within the
        // tet's own radius of it: the planes were pushed out by the class's
        // largest radius, and each test takes back (R - r_t) |n|, r_t the
        // tet's radius (c.w, a float square root) rounded up and |n| rounded
        // down so that the test only ever accepts more than the exact one
        const float shrink = fmaxf(p.offset_r - (c.w * (1.0f + 1e-5f) + 1e-6f * p.coord_scale), 0.f);
        auto side = [&](int q) {
          const float4 e = pl[q];
          return __fmaf_rn(e.x, c.x, __fmaf_rn(e.y, c.y, __fmaf_rn(e.z, c.z,
                 __fmaf_rn(-shrink, pn[q], e.w))));
        };
        for (int q = 0; q < npl && in; q += 2) in = (side(q) >= 0.f) & (side(q + 1) >= 0.f);
        if (in) ++n_in;
      }
      // (the whole warp from here) the tets that passed join the centroid
      // queue: qa <= 31 before, so there is room for 32 more; the rule's
      // first part then runs on full warps
      const uint32_t ia = __ballot_sync(0xffffffffu, in);
      if (in) qa_t[qa + __popc(ia & ((1u << lane) - 1u))] = t;
      qa += __popc(ia);
      __syncwarp();
      if (qa >= 32) first_part(32);
    });
    if (qa > 0) first_part(qa);
    if (qn > 0) drain(qn);
  }
  if (p.diag) {
    n_keep = __reduce_add_sync(0xffffffffu, n_keep);
    n_items = __reduce_add_sync(0xffffffffu, n_items);
    n_in = __reduce_add_sync(0xffffffffu, n_in);
    if (lane == 0) {
      atomicAdd(p.diag + 0, (unsigned long long)n_cells_seen);
      atomicAdd(p.diag + 1, (unsigned long long)n_keep);
      atomicAdd(p.diag + 2, (unsigned long long)n_items);
      atomicAdd(p.diag + 3, (unsigned long long)n_in);
    }
  }
}

cudaError_t launch_pairs(const PairParams& p, int32_t* n_tasks, int32_t* task_off,
                         int32_t* scan_tmp, unsigned long long* work, int num_sms,
                         cudaStream_t st) {
  if (p.n_site <= 0) return cudaSuccess;
  pair_tasks_kernel<<<(p.n_site + 255) / 256, 256, 0, st>>>(p, n_tasks);
  note_launches(1);
  cudaError_t err = scan_exclusive(n_tasks, task_off, p.n_site, scan_tmp, st);
  if (err != cudaSuccess) return err;
  cudaMemsetAsync(work, 0, sizeof(unsigned long long), st);
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, pairs_kernel, kPairWarps * 32, 0);
  pairs_kernel<<<num_sms * (per_sm > 0 ? per_sm : 1), kPairWarps * 32, 0, st>>>(p, task_off, work);
  note_launches(1);
  return cudaGetLastError();
}

__global__ void scatter_pairs_kernel(const int2* buf, long long n, const int32_t* offs,
                                     int32_t* fill, int32_t* pair_site) {
  long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  int2 pr = buf[q];
  int slot = atomicAdd(fill + pr.x, 1);
  pair_site[offs[pr.x] + slot] = pr.y;
}

__global__ void sort_tet_pairs_kernel(int n_tet, const int32_t* offs, int32_t* pair_site,
                                      int32_t* pair_tet, int32_t* tet_k) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_tet) return;
  int b = offs[t], e = offs[t + 1];
  for (int i = b + 1; i < e; ++i) {
    int v = pair_site[i];
    int j = i - 1;
    while (j >= b && pair_site[j] > v) {
      pair_site[j + 1] = pair_site[j];
      --j;
    }
    pair_site[j + 1] = v;
  }
  for (int i = b; i < e; ++i) pair_tet[i] = t;
  if (e > b) atomicMax(tet_k, e - b);
}

cudaError_t pairs_to_csr(const int2* pair_buf, long long n_pairs, int n_tet,
                         const int32_t* tet_offsets, int32_t* tet_fill, int32_t* pair_site,
                         int32_t* pair_tet, int32_t* tet_k_out, cudaStream_t st) {
  cudaMemsetAsync(tet_fill, 0, sizeof(int32_t) * (size_t)n_tet, st);
  cudaMemsetAsync(tet_k_out, 0, sizeof(int32_t), st);
  if (n_pairs > 0) {
    scatter_pairs_kernel<<<(int)((n_pairs + 255) / 256), 256, 0, st>>>(pair_buf, n_pairs,
                                                                      tet_offsets, tet_fill,
                                                                      pair_site);
    note_launches(1);
  }
  if (n_tet > 0) {
    sort_tet_pairs_kernel<<<(n_tet + 255) / 256, 256, 0, st>>>(n_tet, tet_offsets, pair_site,
                                                              pair_tet, tet_k_out);
    note_launches(1);
  }
  return cudaGetLastError();
}

// ------------------------------------------------------------------------
// compaction
// ------------------------------------------------------------------------
__global__ void flag_cells_kernel(const rpd_cell_header* h, long long n, int32_t* flag,
                                  unsigned long long* hist, unsigned long long* n_uncert) {
  __shared__ unsigned int sh[12];
  if (threadIdx.x < 12) sh[threadIdx.x] = 0;
  __syncthreads();
  long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q < n) {
    const rpd_cell_header hq = h[q];
    const int s = hq.status;
    flag[q] = s == kSuccess ? 1 : 0;
    int b = (s >= 0 && s <= 8) ? s : (s == kPayloadFull ? 10 : 9);
    atomicAdd(sh + b, 1u);
    if (s == kSuccess && (hq.flags & RPD_CELL_UNCERTIFIED)) atomicAdd(sh + 11, 1u);
  }
  __syncthreads();
  if (threadIdx.x < 11 && sh[threadIdx.x]) atomicAdd(hist + threadIdx.x, (unsigned long long)sh[threadIdx.x]);
  if (threadIdx.x == 11 && n_uncert && sh[11]) atomicAdd(n_uncert, (unsigned long long)sh[11]);
}

__global__ void gather_cells_kernel(const rpd_cell_header* h, long long n, const int32_t* pos,
                                    rpd_cell_header* out, long long* n_out) {
  long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q < n && h[q].status == kSuccess) out[pos[q]] = h[q];
  if (q == 0) *n_out = pos[n];
}

cudaError_t compact_cells(const rpd_cell_header* pair_headers, long long n_pairs, int32_t* flag_tmp,
                          int32_t* pos_tmp, int32_t* scan_tmp, rpd_cell_header* out,
                          long long* n_out_dev, unsigned long long* status_hist, cudaStream_t st,
                          unsigned long long* n_uncert) {
  int nb = (int)((n_pairs + 255) / 256);
  if (n_pairs > 0) {
    flag_cells_kernel<<<nb, 256, 0, st>>>(pair_headers, n_pairs, flag_tmp, status_hist, n_uncert);
    note_launches(1);
  }
  cudaError_t err = scan_exclusive(flag_tmp, pos_tmp, n_pairs, scan_tmp, st);
  if (err != cudaSuccess) return err;
  gather_cells_kernel<<<nb > 0 ? nb : 1, 256, 0, st>>>(pair_headers, n_pairs, pos_tmp, out, n_out_dev);
  note_launches(1);
  return cudaGetLastError();
}

__global__ void flag_status_kernel(const rpd_cell_header* h, long long n, int status,
                                   int32_t* flag) {
  long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q < n) flag[q] = h[q].status == status ? 1 : 0;
}

__global__ void scatter_index_kernel(const int32_t* flag, const int32_t* pos, long long n,
                                     int32_t* idx) {
  long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q < n && flag[q]) idx[pos[q]] = (int32_t)q;
}

cudaError_t select_pairs(const rpd_cell_header* h, long long n, int status, int32_t* flag_tmp,
                         int32_t* pos_tmp, int32_t* scan_tmp, int32_t* idx_out,
                         cudaStream_t st) {
  int nb = (int)((n + 255) / 256);
  if (n > 0) {
    flag_status_kernel<<<nb, 256, 0, st>>>(h, n, status, flag_tmp);
    note_launches(1);
  }
  cudaError_t err = scan_exclusive(flag_tmp, pos_tmp, n, scan_tmp, st);
  if (err != cudaSuccess) return err;
  if (n > 0) {
    scatter_index_kernel<<<nb, 256, 0, st>>>(flag_tmp, pos_tmp, n, idx_out);
    note_launches(1);
  }
  return cudaGetLastError();
}

__global__ void flag_uncert_kernel(const rpd_cell_header* h, long long n, int32_t* flag) {
  long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q < n) {
    const rpd_cell_header hq = h[q];
    flag[q] = (hq.status == kSuccess && (hq.flags & RPD_CELL_UNCERTIFIED)) ? 1 : 0;
  }
}

cudaError_t select_uncertified(const rpd_cell_header* h, long long n, int32_t* flag_tmp,
                               int32_t* pos_tmp, int32_t* scan_tmp, int32_t* idx_out,
                               cudaStream_t st) {
  int nb = (int)((n + 255) / 256);
  if (n > 0) {
    flag_uncert_kernel<<<nb, 256, 0, st>>>(h, n, flag_tmp);
    note_launches(1);
  }
  cudaError_t err = scan_exclusive(flag_tmp, pos_tmp, n, scan_tmp, st);
  if (err != cudaSuccess) return err;
  if (n > 0) {
    scatter_index_kernel<<<nb, 256, 0, st>>>(flag_tmp, pos_tmp, n, idx_out);
    note_launches(1);
  }
  return cudaGetLastError();
}

__global__ void flag_need_kernel(const unsigned int* need, int n, int32_t* flag) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) flag[i] = need[i] != 0u ? 1 : 0;
}

cudaError_t select_sites(const unsigned int* site_need, int n, int32_t* flag_tmp,
                         int32_t* pos_tmp, int32_t* scan_tmp, int32_t* idx_out, cudaStream_t st) {
  int nb = (n + 255) / 256;
  if (n > 0) {
    flag_need_kernel<<<nb, 256, 0, st>>>(site_need, n, flag_tmp);
    note_launches(1);
  }
  cudaError_t err = scan_exclusive(flag_tmp, pos_tmp, n, scan_tmp, st);
  if (err != cudaSuccess) return err;
  if (n > 0) {
    scatter_index_kernel<<<nb, 256, 0, st>>>(flag_tmp, pos_tmp, n, idx_out);
    note_launches(1);
  }
  return cudaGetLastError();
}

__global__ void assign_rows_kernel(const int32_t* sites, int n, int row0, long long off0,
                                   int stride, int32_t* site_row, long long* ext_off) {
  int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f < n) {
    site_row[sites[f]] = row0 + f;
    ext_off[row0 + f] = off0 + (long long)f * stride;
  }
}

cudaError_t assign_rows(const int32_t* sites, int n, int row0, long long off0, int stride,
                        int32_t* site_row, long long* ext_off, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  assign_rows_kernel<<<(n + 255) / 256, 256, 0, st>>>(sites, n, row0, off0, stride, site_row,
                                                      ext_off);
  note_launches(1);
  return cudaGetLastError();
}

// complete rows: one shared list of every site (ids 0..n_site-1, the seed
// itself included: its bisector is the zero plane, which clips nothing) at
// ext_nbr[off..off + n_site), and rows row0 + f of the sites sites[f] on it
__global__ void complete_rows_kernel(const int32_t* sites, int n, int row0, long long off,
                                     int n_site, int32_t* site_row, long long* ext_off,
                                     int32_t* ext_len, float* ext_bound, int32_t* ext_nbr,
                                     const int2* site_range) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n_site) ext_nbr[off + i] = i;
  if (i < n) {
    const int s = sites[i];
    const int2 r = site_range ? site_range[s] : make_int2(0, n_site);
    site_row[s] = row0 + i;
    ext_off[row0 + i] = off + r.x;
    ext_len[row0 + i] = r.y - r.x;
    ext_bound[row0 + i] = INFINITY;
  }
}

cudaError_t complete_rows(const int32_t* sites, int n, int row0, long long off, int n_site,
                          int32_t* site_row, long long* ext_off, int32_t* ext_len,
                          float* ext_bound, int32_t* ext_nbr, cudaStream_t st,
                          const int2* site_range) {
  const int m = n > n_site ? n : n_site;
  if (m <= 0) return cudaSuccess;
  complete_rows_kernel<<<(m + 255) / 256, 256, 0, st>>>(sites, n, row0, off, n_site, site_row,
                                                        ext_off, ext_len, ext_bound, ext_nbr,
                                                        site_range);
  note_launches(1);
  return cudaGetLastError();
}

// ------------------------------------------------------------------------
// reference site_knn layout ((k+1) rows x n_site) -> row-major lists
// ------------------------------------------------------------------------
__global__ void ref_lists_kernel(const int32_t* ref, int k, int n_site, int32_t* nbr) {
  long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= (long long)n_site * k) return;
  int i = (int)(q / k), r = (int)(q % k);
  nbr[q] = ref[(long long)r * n_site + i];
}

cudaError_t neighbors_from_reference(const int32_t* ref, int k, int n_site, int32_t* nbr,
                                     cudaStream_t st) {
  long long n = (long long)n_site * k;
  if (n > 0) {
    ref_lists_kernel<<<(int)((n + 255) / 256), 256, 0, st>>>(ref, k, n_site, nbr);
    note_launches(1);
  }
  return cudaGetLastError();
}

// ------------------------------------------------------------------------
// batches of meshes
// ------------------------------------------------------------------------
// first compacted cell of every mesh: cells are in ascending tet id and the
// meshes' tets are consecutive ranges starting at tet_base[m]
__global__ void mesh_cell_ranges_kernel(const rpd_cell_header* cells, const long long* n_cells,
                                        const int32_t* tet_base, int n_mesh, long long* first) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m > n_mesh) return;
  const long long n = *n_cells;
  if (m == n_mesh) {
    first[m] = n;
    return;
  }
  const int key = tet_base[m];
  long long lo = 0, hi = n;
  while (lo < hi) {
    const long long mid = (lo + hi) >> 1;
    if (cells[mid].tet_id < key) lo = mid + 1;
    else hi = mid;
  }
  first[m] = lo;
}

cudaError_t mesh_cell_ranges(const rpd_cell_header* cells, const long long* n_cells,
                             const int32_t* tet_base, int n_mesh, long long* first,
                             cudaStream_t st) {
  mesh_cell_ranges_kernel<<<(n_mesh + 1 + 127) / 128, 128, 0, st>>>(cells, n_cells, tet_base,
                                                                     n_mesh, first);
  note_launches(1);
  return cudaGetLastError();
}

// records of cells [0, n) copied to consecutive offsets new_off[q] of out,
// with mesh-local ids: tet - tet_base, site - site_base in the headers and
// in the site pairs of the bisector planes (planes 4.. of a record)
__global__ void gather_records_kernel(const rpd_cell_header* cells, long long n,
                                      const unsigned long long* new_off, const uint8_t* payload,
                                      int tet_base, int site_base, rpd_cell_header* hout,
                                      uint8_t* out) {
  const int lane = threadIdx.x & 31;
  const long long n_warps = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long q = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; q < n; q += n_warps) {
    rpd_cell_header h = cells[q];
    const PayloadLayout L(h.nb_v, h.nb_p, h.nb_e);
    const uint4* src = reinterpret_cast<const uint4*>(payload + h.offset);
    uint4* dst = reinterpret_cast<uint4*>(out + new_off[q]);
    for (uint32_t i = lane; i < L.total / 16u; i += 32) dst[i] = src[i];
    __syncwarp();
    int2* id2 = reinterpret_cast<int2*>(out + new_off[q] + L.id2);
    for (int i = 4 + lane; i < h.nb_p; i += 32) {
      int2 v = id2[i];
      id2[i] = make_int2(v.x - site_base, v.y - site_base);
    }
    if (lane == 0) {
      h.tet_id -= tet_base;
      h.site_id -= site_base;
      h.offset = new_off[q];
      hout[q] = h;
    }
  }
}

cudaError_t gather_records(const rpd_cell_header* cells, long long n,
                           const unsigned long long* new_off, const uint8_t* payload,
                           int tet_base, int site_base, rpd_cell_header* hout, uint8_t* out,
                           cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  long long blocks = (n + 7) / 8;
  if (blocks > 65535) blocks = 65535;
  gather_records_kernel<<<(unsigned)blocks, 256, 0, st>>>(cells, n, new_off, payload, tet_base,
                                                          site_base, hout, out);
  note_launches(1);
  return cudaGetLastError();
}

// record sizes of cells [0, n) (for the offsets of a gather)
__global__ void record_sizes_kernel(const rpd_cell_header* cells, long long n,
                                    unsigned long long* size) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const rpd_cell_header h = cells[q];
  size[q] = PayloadLayout(h.nb_v, h.nb_p, h.nb_e).total;
}

cudaError_t record_sizes(const rpd_cell_header* cells, long long n, unsigned long long* size,
                         cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  record_sizes_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(cells, n, size);
  note_launches(1);
  return cudaGetLastError();
}

}  // namespace rpd
