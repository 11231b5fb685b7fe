// rpd_prep.cu -- mesh preparation on the device (rpd_set_mesh).
//
// libmat prepares its tet mesh on the host (copy_tet_data,
// load_num_adjacent_cells_and_ids; src/rpd3d/voronoi.cu:324-415).  Here the
// raw arrays are copied to the device once and everything derived from them
// is computed there: float and double-float vertex copies, the bounding box,
// the validation of every vertex id, the radius of every tet (largest
// vertex distance to its centroid, in FP64), the mesh volume, the split of
// the tets into radius classes (the 99.5th-percentile radius, found by a
// histogram; any split is correct, only each class's largest radius must be
// exact) and the marks of boundary vertices.  The host only reads back a
// handful of numbers.

#include <cuda_runtime.h>

#include <cstdint>

#include "rpd_df64.cuh"
#include "rpd_kernels.cuh"

namespace rpd {

namespace {

// order-preserving map of doubles to unsigned 64-bit keys (for atomic
// min / max): negative values bit-inverted, positive ones with the sign bit set
__device__ __forceinline__ unsigned long long dkey(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

constexpr int kPrepBlock = 256;

// block-wide reduction; the result is valid in warp 0.  `identity` fills the
// slots past the block's warp count (0 for sums, the neutral key for min/max).
template <class T, class Op>
__device__ T block_reduce(T v, Op op, T* sh, T identity) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int o = 16; o > 0; o >>= 1) v = op(v, __shfl_xor_sync(0xffffffffu, v, o));
  __syncthreads();
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  if (wid == 0) {
    v = lane < (int)(blockDim.x >> 5) ? sh[lane] : identity;
    for (int o = 16; o > 0; o >>= 1) v = op(v, __shfl_xor_sync(0xffffffffu, v, o));
  }
  return v;
}

__global__ void __launch_bounds__(kPrepBlock) vert_prep_kernel(const double* xyz, int n_vert,
                                                               float* vert3f, float2* vert2,
                                                               MeshPrepOut* out) {
  __shared__ unsigned long long sh[32];
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  double x[3] = {0.0, 0.0, 0.0};
  bool ok = true;
  if (v < n_vert) {
    for (int a = 0; a < 3; ++a) {
      x[a] = xyz[3ll * v + a];
      ok &= isfinite(x[a]);
      vert3f[3ll * v + a] = (float)x[a];
      const df d = df_from_double(x[a]);
      vert2[3ll * v + a] = make_float2(d.hi, d.lo);
    }
    if (!ok) atomicOr(&out->bad, 1u);
  }
  auto mn = [](unsigned long long p, unsigned long long q) { return p < q ? p : q; };
  auto mx = [](unsigned long long p, unsigned long long q) { return p > q ? p : q; };
  for (int a = 0; a < 3; ++a) {
    const unsigned long long kl = v < n_vert && ok ? dkey(x[a]) : ~0ull;
    const unsigned long long kh = v < n_vert && ok ? dkey(x[a]) : 0ull;
    const unsigned long long rl = block_reduce(kl, mn, sh, ~0ull);
    const unsigned long long rh = block_reduce(kh, mx, sh, 0ull);
    if (threadIdx.x == 0) {
      atomicMin(&out->lo_key[a], rl);
      atomicMax(&out->hi_key[a], rh);
    }
  }
}

// tet radius (FP64), id validation, volume, largest radius, boundary marks
__global__ void __launch_bounds__(kPrepBlock) tet_prep_kernel(const double* xyz, const int4* tets,
                                                              const int32_t* f_adjs, int n_tet,
                                                              int n_vert, double* rad,
                                                              uint8_t* bmark, MeshPrepOut* out) {
  __shared__ double shd[32];
  __shared__ unsigned long long shk[32];
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  double vol = 0.0, r = 0.0;
  if (t < n_tet) {
    const int4 q = tets[t];
    const int id[4] = {q.x, q.y, q.z, q.w};
    bool ok = true;
    for (int k = 0; k < 4; ++k) ok &= id[k] >= 0 && id[k] < n_vert;
    if (!ok) {
      atomicOr(&out->bad, 2u);
      rad[t] = 0.0;
    } else {
      double p[4][3], cen[3] = {0.0, 0.0, 0.0};
      for (int k = 0; k < 4; ++k)
        for (int a = 0; a < 3; ++a) {
          p[k][a] = xyz[3ll * id[k] + a];
          cen[a] += 0.25 * p[k][a];
        }
      for (int k = 0; k < 4; ++k) {
        double d2 = 0.0;
        for (int a = 0; a < 3; ++a) {
          const double d = p[k][a] - cen[a];
          d2 += d * d;
        }
        r = fmax(r, sqrt(d2));
      }
      rad[t] = r;
      double e[3][3];
      for (int k = 1; k < 4; ++k)
        for (int a = 0; a < 3; ++a) e[k - 1][a] = p[k][a] - p[0][a];
      vol = fabs(e[0][0] * (e[1][1] * e[2][2] - e[1][2] * e[2][1]) -
                 e[0][1] * (e[1][0] * e[2][2] - e[1][2] * e[2][0]) +
                 e[0][2] * (e[1][0] * e[2][1] - e[1][1] * e[2][0])) / 6.0;
      // face f is opposite vertex f; a face with one tet is on the boundary
      if (bmark)
        for (int f = 0; f < 4; ++f)
          if (f_adjs[4ll * t + f] == 1)
            for (int k = 0; k < 4; ++k)
              if (k != f) bmark[id[k]] = 1;
    }
  }
  const double vs = block_reduce(vol, [](double a, double b) { return a + b; }, shd, 0.0);
  const unsigned long long rk = block_reduce(
      dkey(r), [](unsigned long long a, unsigned long long b) { return a > b ? a : b; }, shk, 0ull);
  if (threadIdx.x == 0) {
    atomicAdd(&out->volume, vs);
    atomicMax(&out->rmax_key, rk);
  }
}

__global__ void radius_hist_kernel(const double* rad, int n_tet, double rmax, int32_t* hist) {
  __shared__ int32_t sh[kRadiusBins];
  for (int i = threadIdx.x; i < kRadiusBins; i += blockDim.x) sh[i] = 0;
  __syncthreads();
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n_tet) {
    int b = rmax > 0.0 ? (int)(rad[t] / rmax * kRadiusBins) : 0;
    b = b < 0 ? 0 : (b >= kRadiusBins ? kRadiusBins - 1 : b);
    atomicAdd(&sh[b], 1);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < kRadiusBins; i += blockDim.x)
    if (sh[i]) atomicAdd(&hist[i], sh[i]);
}

__global__ void __launch_bounds__(kPrepBlock) classify_kernel(const double* rad, int n_tet,
                                                              double r0, uint8_t* cls,
                                                              MeshPrepOut* out) {
  __shared__ int shc[32];
  __shared__ unsigned long long shk[32];
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  int k = -1;
  unsigned long long key = 0ull;
  if (t < n_tet) {
    k = rad[t] <= r0 ? 0 : 1;
    cls[t] = (uint8_t)k;
    key = dkey(rad[t]);
  }
  // one atomic per block and class (the classes' counters are contended)
  for (int cl = 0; cl < 2; ++cl) {
    const int n = block_reduce(k == cl ? 1 : 0, [](int a, int b) { return a + b; }, shc, 0);
    const unsigned long long mk = block_reduce(
        k == cl ? key : 0ull, [](unsigned long long a, unsigned long long b) { return a > b ? a : b; },
        shk, 0ull);
    if (threadIdx.x == 0 && n > 0) {
      atomicAdd(&out->class_count[cl], n);
      atomicMax(&out->class_rmax_key[cl], mk);
    }
  }
}

// boundary vertices (marked) appended as float4 (x, y, z, 0)
__global__ void boundary_list_kernel(const uint8_t* bmark, const float* vert3f, int n_vert,
                                     float4* bverts, int32_t* n_bv) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= n_vert || !bmark[v]) return;
  const int i = atomicAdd(n_bv, 1);
  bverts[i] = make_float4(vert3f[3ll * v], vert3f[3ll * v + 1], vert3f[3ll * v + 2], 0.f);
}

}  // namespace

double key_to_double(unsigned long long k) {
  const unsigned long long b = (k & 0x8000000000000000ull) ? (k & 0x7fffffffffffffffull) : ~k;
  double x;
  static_assert(sizeof(x) == sizeof(b), "double size");
  __builtin_memcpy(&x, &b, sizeof(x));
  return x;
}

cudaError_t mesh_prep_init(MeshPrepOut* out, cudaStream_t st) {
  MeshPrepOut h;
  h.bad = 0u;
  for (int a = 0; a < 3; ++a) {
    h.lo_key[a] = ~0ull;
    h.hi_key[a] = 0ull;
  }
  h.volume = 0.0;
  h.rmax_key = 0ull;
  for (int k = 0; k < 2; ++k) {
    h.class_count[k] = 0;
    h.class_rmax_key[k] = 0ull;
  }
  return cudaMemcpyAsync(out, &h, sizeof(h), cudaMemcpyHostToDevice, st);
}

cudaError_t mesh_prep_geometry(const double* xyz, int n_vert, const int4* tets,
                               const int32_t* f_adjs, int n_tet, float* vert3f, float2* vert2,
                               double* rad, uint8_t* bmark, MeshPrepOut* out, cudaStream_t st) {
  vert_prep_kernel<<<(n_vert + kPrepBlock - 1) / kPrepBlock, kPrepBlock, 0, st>>>(xyz, n_vert, vert3f,
                                                                                 vert2, out);
  if (bmark) cudaMemsetAsync(bmark, 0, (size_t)n_vert, st);
  tet_prep_kernel<<<(n_tet + kPrepBlock - 1) / kPrepBlock, kPrepBlock, 0, st>>>(
      xyz, tets, f_adjs, n_tet, n_vert, rad, bmark, out);
  note_launches(2);
  return cudaGetLastError();
}

cudaError_t mesh_prep_histogram(const double* rad, int n_tet, double rmax, int32_t* hist,
                                cudaStream_t st) {
  cudaMemsetAsync(hist, 0, sizeof(int32_t) * kRadiusBins, st);
  radius_hist_kernel<<<(n_tet + 255) / 256, 256, 0, st>>>(rad, n_tet, rmax, hist);
  note_launches(1);
  return cudaGetLastError();
}

cudaError_t mesh_prep_classify(const double* rad, int n_tet, double r0, uint8_t* cls,
                               MeshPrepOut* out, cudaStream_t st) {
  classify_kernel<<<(n_tet + kPrepBlock - 1) / kPrepBlock, kPrepBlock, 0, st>>>(rad, n_tet, r0, cls,
                                                                               out);
  note_launches(1);
  return cudaGetLastError();
}

cudaError_t boundary_list(const uint8_t* bmark, const float* vert3f, int n_vert, float4* bverts,
                          int32_t* n_bv, cudaStream_t st) {
  cudaMemsetAsync(n_bv, 0, sizeof(int32_t), st);
  boundary_list_kernel<<<(n_vert + 255) / 256, 256, 0, st>>>(bmark, vert3f, n_vert, bverts, n_bv);
  note_launches(1);
  return cudaGetLastError();
}

__global__ void stage_bytes_kernel(const uint8_t* __restrict__ src, uint8_t* dst, int n) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) dst[i] = src[i];
}

cudaError_t launch_stage_bytes(const void* src, void* dst, size_t n, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  stage_bytes_kernel<<<1, 256, 0, st>>>(static_cast<const uint8_t*>(src),
                                       static_cast<uint8_t*>(dst), (int)n);
  note_launches(1);
  return cudaGetLastError();
}

}  // namespace rpd
