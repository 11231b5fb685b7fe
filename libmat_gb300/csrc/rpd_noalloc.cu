// rpd_noalloc.cu -- cell compaction that allocates no device memory.
//
// Some callers cannot call cudaMalloc while they run the RPD: code that
// records its GPU work into a stream it does not own, applications that hand
// every byte of device memory to their own pool up front and treat an
// allocation in the middle of an iteration as an error, and code running
// where an allocation would implicitly synchronise the device.  For them,
// rpd_compact_cells_noalloc does the compaction step of rpd_compute --
// keep the emitted (status success) records of a pair-header array, in
// pair order, and count statuses -- with buffers the caller passes in, and
// keeps its one temporary (the per-block counts of emitted cells) in a
// fixed array compiled into the library.
//
// The array is sized for kMaxPairs pair headers (32M pairs, 128 KB of
// counts) and is reserved on every GPU that loads the library until the
// process exits.  Larger inputs are rejected with RPD_ERR_CAPACITY before
// anything is launched.
//
// Set-up: the first call on a device (the device current at the call) looks
// up the array's device address with cudaGetSymbolAddress; make that first
// call before any stream capture.  The address is cached per device
// ordinal: calls must run in the device's primary context (the one the CUDA
// runtime uses), and the cached address is not looked up again after
// cudaDeviceReset, so do not call this entry point after a reset in the
// same process.
//
// Errors: the launches' own configuration errors are returned as
// RPD_ERR_CUDA; an error the caller left pending before the call is neither
// reported nor cleared.
//
// Every call reuses the same array, which keeps the last call's contents; a
// call overwrites every count it reads.  Two calls whose kernels overlap on
// the GPU (different streams, or different host threads on one device) race
// on the array and must be serialised by the caller.

#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "rpd_common.cuh"
#include "rpd_scan.cuh"

namespace {

constexpr int kBlock = 1024;
constexpr long long kMaxPairs = 1ll << 25;
constexpr long long kScratchInts = kMaxPairs / kBlock + 2;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) int32_t g_compact_scratch[kScratchInts];

std::mutex g_setup_mutex;
int32_t* g_scratch_ptr[kMaxDevices] = {};

static_assert(kBlock == 1024, "the block scans below assume 32 full warps per block");

__global__ void na_zero(unsigned long long* hist) {
  if (hist && threadIdx.x < 11) hist[threadIdx.x] = 0ull;
}

__global__ void na_count(const rpd_cell_header* h, long long n, int32_t* counts,
                         unsigned long long* hist) {
  __shared__ unsigned int sh[11];
  if (threadIdx.x < 11) sh[threadIdx.x] = 0u;
  long long q = (long long)blockIdx.x * kBlock + threadIdx.x;
  int f = 0;
  __syncthreads();
  if (q < n) {
    int s = h[q].status;
    f = s == rpd::kSuccess ? 1 : 0;
    int b = (s >= 0 && s <= 8) ? s : (s == rpd::kPayloadFull ? 10 : 9);
    atomicAdd(sh + b, 1u);
  }
  int tot;
  rpd::block_excl_scan<int>(f, &tot);
  if (threadIdx.x == 0) counts[blockIdx.x] = tot;
  if (hist && threadIdx.x < 11 && sh[threadIdx.x])
    atomicAdd(hist + threadIdx.x, (unsigned long long)sh[threadIdx.x]);
}

// exclusive scan of the nb block counts in place, total at counts[nb]
__global__ void na_scan_counts(int32_t* counts, int nb) {
  int carry = 0;
  for (int base = 0; base < nb; base += kBlock) {
    int i = base + threadIdx.x;
    int v = i < nb ? counts[i] : 0;
    int tot;
    int ex = rpd::block_excl_scan<int>(v, &tot);
    if (i < nb) counts[i] = ex + carry;
    carry += tot;
  }
  if (threadIdx.x == 0) counts[nb] = carry;
}

__global__ void na_scatter(const rpd_cell_header* h, long long n, const int32_t* offs, int nb,
                           rpd_cell_header* out, int64_t* n_out) {
  long long q = (long long)blockIdx.x * kBlock + threadIdx.x;
  int f = (q < n && h[q].status == rpd::kSuccess) ? 1 : 0;
  int pos = rpd::block_excl_scan<int>(f, nullptr) + offs[blockIdx.x];
  if (f) out[pos] = h[q];
  if (blockIdx.x == 0 && threadIdx.x == 0) *n_out = offs[nb];
}

}  // namespace

extern "C" rpd_status rpd_compact_cells_noalloc(const rpd_cell_header* pair_headers,
                                                int64_t n_pairs, rpd_cell_header* cells_out,
                                                int64_t* n_cells_out, uint64_t* status_counts,
                                                void* stream) {
  if (n_pairs < 0 || !n_cells_out || (n_pairs > 0 && (!pair_headers || !cells_out)))
    return RPD_ERR_INVALID_ARGUMENT;
  if (n_pairs > kMaxPairs) return RPD_ERR_CAPACITY;  // beyond the fixed scratch array
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    return RPD_ERR_NO_DEVICE;
  }
  int32_t* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_ptr[dev]) {
      void* ptr = nullptr;
      if (cudaGetSymbolAddress(&ptr, g_compact_scratch) != cudaSuccess || !ptr) {
        cudaGetLastError();
        return RPD_ERR_CUDA;
      }
      g_scratch_ptr[dev] = static_cast<int32_t*>(ptr);
    }
    scratch = g_scratch_ptr[dev];
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  unsigned long long* hist = reinterpret_cast<unsigned long long*>(status_counts);
  int nb = (int)((n_pairs + kBlock - 1) / kBlock);
  // each launch's own status (cudaLaunchKernel returns it): a launch that
  // fails is reported without consulting the thread's last-error state
  void* a_zero[] = {&hist};
  if (cudaLaunchKernel((const void*)na_zero, dim3(1), dim3(32), a_zero, 0, st) != cudaSuccess)
    return RPD_ERR_CUDA;
  if (nb > 0) {
    void* a_count[] = {&pair_headers, &n_pairs, &scratch, &hist};
    if (cudaLaunchKernel((const void*)na_count, dim3(nb), dim3(kBlock), a_count, 0, st) !=
        cudaSuccess)
      return RPD_ERR_CUDA;
  }
  void* a_scan[] = {&scratch, &nb};
  if (cudaLaunchKernel((const void*)na_scan_counts, dim3(1), dim3(kBlock), a_scan, 0, st) !=
      cudaSuccess)
    return RPD_ERR_CUDA;
  void* a_scatter[] = {&pair_headers, &n_pairs, &scratch, &nb, &cells_out, &n_cells_out};
  if (cudaLaunchKernel((const void*)na_scatter, dim3(nb > 0 ? nb : 1), dim3(kBlock), a_scatter,
                       0, st) != cudaSuccess)
    return RPD_ERR_CUDA;
  return RPD_OK;
}
