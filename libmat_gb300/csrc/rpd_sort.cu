// rpd_sort.cu -- stable radix sort of 64-bit keys with 32-bit values.
//
// Used to group per-cell records (power cells: by site, then by neighbour or
// face).  Least-significant-digit first, 8 bits per pass, each pass stable:
// a block of 256 threads takes 256 consecutive keys (warp w the keys
// 32 w .. 32 w + 31), ranks each key among the equal digits before it --
// within its warp by __match_any_sync, across the block's warps by a scan of
// per-warp digit counts -- and the digit-major exclusive scan of all blocks'
// counts gives the block's base for every digit.

#include <cuda_runtime.h>

#include "rpd_kernels.cuh"

namespace rpd {

namespace {

constexpr int kSortBlock = 256;
constexpr int kSortWarps = kSortBlock / 32;
constexpr int kRadix = 256;

// ranks of this thread's key among the equal digits earlier in the block;
// counts[d] = the block's keys with digit d (valid after the call)
__device__ int block_digit_rank(int digit, bool valid, int* wcount /* [kSortWarps][kRadix] */,
                                int* counts) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int i = threadIdx.x; i < kSortWarps * kRadix; i += kSortBlock) wcount[i] = 0;
  __syncthreads();
  const unsigned peers = __match_any_sync(0xffffffffu, valid ? digit : -1);
  const int leader = __ffs(peers) - 1;
  const int before = __popc(peers & ((1u << lane) - 1u));
  if (valid && lane == leader) wcount[wid * kRadix + digit] = __popc(peers);
  __syncthreads();
  // per digit: exclusive scan over the warps (in place), total to counts
  for (int d = threadIdx.x; d < kRadix; d += kSortBlock) {
    int acc = 0;
    for (int w = 0; w < kSortWarps; ++w) {
      const int c = wcount[w * kRadix + d];
      wcount[w * kRadix + d] = acc;
      acc += c;
    }
    counts[d] = acc;
  }
  __syncthreads();
  return valid ? wcount[wid * kRadix + digit] + before : 0;
}

__global__ void __launch_bounds__(kSortBlock)
    radix_count_kernel(const unsigned long long* keys, long long n, int shift, int n_blocks,
                       int32_t* hist /* [kRadix][n_blocks] */) {
  __shared__ int wcount[kSortWarps * kRadix];
  __shared__ int counts[kRadix];
  const long long i = (long long)blockIdx.x * kSortBlock + threadIdx.x;
  const bool valid = i < n;
  const int digit = valid ? (int)((keys[i] >> shift) & 0xffull) : 0;
  block_digit_rank(digit, valid, wcount, counts);
  for (int d = threadIdx.x; d < kRadix; d += kSortBlock)
    hist[(long long)d * n_blocks + blockIdx.x] = counts[d];
}

__global__ void __launch_bounds__(kSortBlock)
    radix_scatter_kernel(const unsigned long long* keys, const uint32_t* vals, long long n,
                         int shift, int n_blocks, const int32_t* base /* scanned hist */,
                         unsigned long long* keys_out, uint32_t* vals_out) {
  __shared__ int wcount[kSortWarps * kRadix];
  __shared__ int counts[kRadix];
  const long long i = (long long)blockIdx.x * kSortBlock + threadIdx.x;
  const bool valid = i < n;
  const unsigned long long k = valid ? keys[i] : 0ull;
  const int digit = (int)((k >> shift) & 0xffull);
  const int r = block_digit_rank(digit, valid, wcount, counts);
  if (valid) {
    const long long pos = (long long)base[(long long)digit * n_blocks + blockIdx.x] + r;
    keys_out[pos] = k;
    vals_out[pos] = vals[i];
  }
}

}  // namespace

size_t radix_hist_ints(long long n) {
  const long long nb = (n + kSortBlock - 1) / kSortBlock;
  return (size_t)(nb * kRadix + 1);
}

// Sorts (keys, vals) by the low `bits` bits of the keys, stably; the result
// is in keys / vals (the *_tmp buffers are scratch of n entries; hist and
// scan_tmp hold radix_hist_ints(n) and scan_temp_ints(of that) ints).
cudaError_t radix_sort_pairs(unsigned long long* keys, uint32_t* vals, long long n, int bits,
                             unsigned long long* keys_tmp, uint32_t* vals_tmp, int32_t* hist,
                             int32_t* scan_tmp, cudaStream_t st) {
  if (n <= 1 || bits <= 0) return cudaSuccess;
  if (n > 0x7fffffffll) return cudaErrorInvalidValue;  // positions are int32
  const int nb = (int)((n + kSortBlock - 1) / kSortBlock);
  const long long nh = (long long)nb * kRadix;
  unsigned long long *ka = keys, *kb = keys_tmp;
  uint32_t *va = vals, *vb = vals_tmp;
  int passes = 0;
  for (int shift = 0; shift < bits; shift += 8) {
    radix_count_kernel<<<nb, kSortBlock, 0, st>>>(ka, n, shift, nb, hist);
    cudaError_t e = scan_exclusive(hist, hist, nh, scan_tmp, st);
    if (e != cudaSuccess) return e;
    radix_scatter_kernel<<<nb, kSortBlock, 0, st>>>(ka, va, n, shift, nb, hist, kb, vb);
    note_launches(2);
    unsigned long long* tk = ka;
    ka = kb;
    kb = tk;
    uint32_t* tv = va;
    va = vb;
    vb = tv;
    ++passes;
  }
  if (passes & 1) {  // result in the scratch buffers: copy back
    cudaError_t e = cudaMemcpyAsync(keys, ka, sizeof(unsigned long long) * (size_t)n,
                                    cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(vals, va, sizeof(uint32_t) * (size_t)n, cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) return e;
  }
  return cudaGetLastError();
}

}  // namespace rpd
