// rpd_partial.cu -- merge of a partial recompute into the previous cells
// (rpd_compute_partial).
//
// libmat's incremental update (RPD3D_GPU::calculate_partial,
// src/rpd3d_api/rpd_api.cxx:147-316) recomputes the cells of the changed
// spheres and their neighbours and merges them with the cells it had
// (merge_convex_cells): the cells of the recomputed sites are replaced, all
// others kept.  Here both cell lists are already in (tet, site) order and
// their sites are disjoint (old cells of recomputed sites are dropped), so
// the merged position of every cell is its rank in its own list plus the
// number of cells of the other list with a smaller key -- a binary search,
// no sort.  Record sizes are scanned for the merged payload and each warp
// copies one record.

#include <cuda_runtime.h>

#include "rpd_common.cuh"
#include "rpd_kernels.cuh"

namespace rpd {

namespace {

__device__ __forceinline__ unsigned long long cell_key(const rpd_cell_header& h) {
  return ((unsigned long long)(uint32_t)h.tet_id << 32) | (uint32_t)h.site_id;
}

// first index in cells[0, n) whose key is >= key
__device__ __forceinline__ long long lower_bound(const rpd_cell_header* cells, long long n,
                                                 unsigned long long key) {
  long long lo = 0, hi = n;
  while (lo < hi) {
    const long long mid = (lo + hi) >> 1;
    if (cell_key(cells[mid]) < key) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

__global__ void keep_old_kernel(const rpd_cell_header* old_cells, long long n_old,
                                const uint32_t* recomputed, int32_t* keep) {
  const long long a = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (a < n_old) keep[a] = recomputed[old_cells[a].site_id] ? 0 : 1;
}

// merged slot of every kept old cell and every new cell: src[slot] =
// index + 1 for an old cell, -(index + 1) for a new one; units[slot] = its
// record size in 16-byte units
__global__ void merge_slots_kernel(const rpd_cell_header* old_cells, long long n_old,
                                   const int32_t* keep, const int32_t* keep_pos,
                                   const rpd_cell_header* new_cells, long long n_new,
                                   long long n_out, long long* src, int32_t* units) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n_old) {
    if (!keep[i]) return;
    const rpd_cell_header h = old_cells[i];
    const long long slot = keep_pos[i] + lower_bound(new_cells, n_new, cell_key(h));
    if (slot >= n_out) return;  // (both lists sorted with disjoint keys: never)
    src[slot] = i + 1;
    units[slot] = (int32_t)(PayloadLayout(h.nb_v, h.nb_p, h.nb_e).total / 16u);
  } else if (i < n_old + n_new) {
    const long long b = i - n_old;
    const rpd_cell_header h = new_cells[b];
    const long long slot = b + keep_pos[lower_bound(old_cells, n_old, cell_key(h))];
    if (slot >= n_out) return;
    src[slot] = -(b + 1);
    units[slot] = (int32_t)(PayloadLayout(h.nb_v, h.nb_p, h.nb_e).total / 16u);
  }
}

__global__ void merge_gather_kernel(const long long* src, long long n, const long long* off,
                                    const rpd_cell_header* old_cells, const uint8_t* old_payload,
                                    const rpd_cell_header* new_cells, const uint8_t* new_payload,
                                    rpd_cell_header* out_cells, uint8_t* out_payload) {
  const int lane = threadIdx.x & 31;
  const long long n_warps = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long q = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; q < n; q += n_warps) {
    const long long s = src[q];
    if (s == 0) continue;  // an unfilled slot (never, see merge_slots_kernel)
    rpd_cell_header h = s > 0 ? old_cells[s - 1] : new_cells[-s - 1];
    const uint8_t* from = (s > 0 ? old_payload : new_payload) + h.offset;
    const unsigned long long to = 16ull * (unsigned long long)off[q];
    const uint32_t words = PayloadLayout(h.nb_v, h.nb_p, h.nb_e).total / 16u;
    const uint4* a = reinterpret_cast<const uint4*>(from);
    uint4* b = reinterpret_cast<uint4*>(out_payload + to);
    for (uint32_t w = lane; w < words; w += 32) b[w] = a[w];
    if (lane == 0) {
      h.offset = to;
      out_cells[q] = h;
    }
  }
}

}  // namespace

cudaError_t merge_keep(const rpd_cell_header* old_cells, long long n_old, const uint32_t* recomputed,
                       int32_t* keep, cudaStream_t st) {
  if (n_old <= 0) return cudaSuccess;
  keep_old_kernel<<<(unsigned)((n_old + 255) / 256), 256, 0, st>>>(old_cells, n_old, recomputed,
                                                                   keep);
  note_launches(1);
  return cudaGetLastError();
}

cudaError_t merge_slots(const rpd_cell_header* old_cells, long long n_old, const int32_t* keep,
                        const int32_t* keep_pos, const rpd_cell_header* new_cells, long long n_new,
                        long long n_out, long long* src, int32_t* units, cudaStream_t st) {
  const long long n = n_old + n_new;
  if (n <= 0) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(src, 0, sizeof(long long) * (size_t)(n_out > 0 ? n_out : 1), st);
  if (e == cudaSuccess) e = cudaMemsetAsync(units, 0, sizeof(int32_t) * (size_t)(n_out > 0 ? n_out : 1), st);
  if (e != cudaSuccess) return e;
  merge_slots_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(old_cells, n_old, keep, keep_pos,
                                                                  new_cells, n_new, n_out, src,
                                                                  units);
  note_launches(1);
  return cudaGetLastError();
}

cudaError_t merge_gather(const long long* src, long long n, const long long* off,
                         const rpd_cell_header* old_cells, const uint8_t* old_payload,
                         const rpd_cell_header* new_cells, const uint8_t* new_payload,
                         rpd_cell_header* out_cells, uint8_t* out_payload, int num_sms,
                         cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  long long blocks = (n + 7) / 8;
  if (blocks > (long long)num_sms * 32) blocks = (long long)num_sms * 32;
  merge_gather_kernel<<<(unsigned)blocks, 256, 0, st>>>(src, n, off, old_cells, old_payload,
                                                        new_cells, new_payload, out_cells,
                                                        out_payload);
  note_launches(1);
  return cudaGetLastError();
}

}  // namespace rpd
