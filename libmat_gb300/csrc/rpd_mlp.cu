// rpd_mlp.cu -- the learned list length: a 12 -> 64 -> 64 -> 1 MLP that
// predicts, for every (tet, site) cell, how many entries of the site's
// distance-ordered neighbour list the certified clipping takes before its
// security-radius certificate holds.  The first clipping pass stops at the
// predicted length and tests the certificate once; cells for which it does
// not hold are clipped again with the whole list (and the certificate tested
// as it goes), which also measures the predictor's miss rate.
//
// Training and inference run on the tensor cores with hand-written
// mma.sync.m16n8k16 bf16 x bf16 -> fp32 kernels, one warp per 16 samples.
// The layer-1 accumulator fragment is, register for register, the layer-2 A
// operand (rows g and g+8, columns 2t and 2t+1 of consecutive 8-column
// tiles), so the forward pass never leaves registers; the weight gradients
// stage the transposed operands through shared memory.  Parameters are fp32
// masters updated by Adam (Kingma and Ba, ICLR 2015), with bf16 copies of
// the two weight matrices as mma operands.  bf16 values cross the C ABI as
// their 16-bit patterns (uint16_t).
//
// Rounding points (the CPU gradient oracle rounds at the same places):
//   X, W1, W2 bf16; z1 = X W1 + b1 (fp32); h1 = bf16(relu(z1));
//   z2 = h1 W2 + b2 (fp32); y = relu(z2) . w3 + b3 (fp32);
//   dz2 = dy w3 [z2 > 0] (fp32; bf16 as an mma operand); dW2 = h1^T bf16(dz2);
//   dh1 = bf16(dz2) W2^T; dz1 = dh1 [z1 > 0]; dW1 = X^T bf16(dz1).
//
// Features of a cell (tet t, site i); lengths are divided by the mean site
// spacing h and clamped to [-16, 16]:
//   0 radius of i (sqrt w)
//   1..4 key (power-bisector distance) of i's 1st / 4th / 8th / 16th neighbour
//   5 log2(1 + sites in i's cell of the kNN grid)
//   6 distance from i to the mesh boundary (nearest boundary vertex)
//   7 / 8 largest / smallest distance from i to a vertex of t
//   9 distance from i to t's centroid
//   10 key of i's 32nd neighbour
//   11 log2(1 + keys of i below feature 7)
//   12..15 zero (padding to the mma's k = 16)
// Features 0-6 describe the site; 7-11 place the tet in the site's list: a
// cell lies inside its tet, so its radius about the seed is at most feature
// 7, and the certificate holds at the first key beyond the cell's radius.

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "rpd_common.cuh"
#include "rpd_kernels.cuh"

namespace rpd {

namespace {

constexpr int kNF = kMlpFeatures;  // 16 (12 used)
constexpr int kH = kMlpHidden;     // 64
constexpr int kMlpWarps = 4;

__device__ __forceinline__ uint16_t bf16_bits(float x) {
  return __bfloat16_as_ushort(__float2bfloat16_rn(x));
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  return (uint32_t)bf16_bits(lo) | ((uint32_t)bf16_bits(hi) << 16);
}

__device__ __forceinline__ void mma16816(float* d, uint32_t a0, uint32_t a1, uint32_t a2,
                                         uint32_t a3, uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
      "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// two consecutive bf16 (4-byte aligned)
__device__ __forceinline__ uint32_t ld_pair(const uint16_t* p) {
  return *reinterpret_cast<const uint32_t*>(p);
}

// two bf16 from separate addresses (low half first)
__device__ __forceinline__ uint32_t ld2(const uint16_t* p0, const uint16_t* p1) {
  return (uint32_t)*p0 | ((uint32_t)*p1 << 16);
}

__device__ __forceinline__ void st_pair(uint16_t* p, uint32_t v) {
  *reinterpret_cast<uint32_t*>(p) = v;
}

// Forward pass of 16 rows whose bf16 features sit in shared memory (kNF per
// row).  On return z1/z2 hold the pre-activations as C fragments ([tile][4]:
// rows g, g, g+8, g+8; columns 8 tile + 2t, +1) and y_lo / y_hi the outputs
// of rows g and g+8 (in every lane of the row's quad).
__device__ __forceinline__ void mlp_forward16(const uint16_t* Xs, const MlpWeights& w, int lane,
                                              float (&z1)[8][4], float (&z2)[8][4], float& y_lo,
                                              float& y_hi) {
  const int g = lane >> 2, t = lane & 3;
  const uint32_t a0 = ld_pair(Xs + g * kNF + 2 * t), a1 = ld_pair(Xs + (g + 8) * kNF + 2 * t);
  const uint32_t a2 = ld_pair(Xs + g * kNF + 2 * t + 8);
  const uint32_t a3 = ld_pair(Xs + (g + 8) * kNF + 2 * t + 8);
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    z1[j][0] = z1[j][1] = z1[j][2] = z1[j][3] = 0.f;
    const uint16_t* b = w.W1T + (8 * j + g) * kNF + 2 * t;  // B[k = feature][n = hidden]
    mma16816(z1[j], a0, a1, a2, a3, ld_pair(b), ld_pair(b + 8));
    const float c0 = w.b1[8 * j + 2 * t], c1 = w.b1[8 * j + 2 * t + 1];
    z1[j][0] += c0;
    z1[j][1] += c1;
    z1[j][2] += c0;
    z1[j][3] += c1;
  }
#pragma unroll
  for (int j = 0; j < 8; ++j) z2[j][0] = z2[j][1] = z2[j][2] = z2[j][3] = 0.f;
#pragma unroll
  for (int kc = 0; kc < 4; ++kc) {  // k-chunk of 16 hidden units = tiles 2kc, 2kc+1
    const float* lo = z1[2 * kc];
    const float* hi = z1[2 * kc + 1];
    const uint32_t h0 = pack_bf16(fmaxf(lo[0], 0.f), fmaxf(lo[1], 0.f));
    const uint32_t h1 = pack_bf16(fmaxf(lo[2], 0.f), fmaxf(lo[3], 0.f));
    const uint32_t h2 = pack_bf16(fmaxf(hi[0], 0.f), fmaxf(hi[1], 0.f));
    const uint32_t h3 = pack_bf16(fmaxf(hi[2], 0.f), fmaxf(hi[3], 0.f));
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const uint16_t* b = w.W2T + (8 * j + g) * kH + 16 * kc + 2 * t;  // B[k = in][n = out]
      mma16816(z2[j], h0, h1, h2, h3, ld_pair(b), ld_pair(b + 8));
    }
  }
  float plo = 0.f, phi = 0.f;
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const int col = 8 * j + 2 * t;
    const float c0 = w.b2[col], c1 = w.b2[col + 1];
    z2[j][0] += c0;
    z2[j][1] += c1;
    z2[j][2] += c0;
    z2[j][3] += c1;
    plo += fmaxf(z2[j][0], 0.f) * w.w3[col] + fmaxf(z2[j][1], 0.f) * w.w3[col + 1];
    phi += fmaxf(z2[j][2], 0.f) * w.w3[col] + fmaxf(z2[j][3], 0.f) * w.w3[col + 1];
  }
  plo += __shfl_xor_sync(0xffffffffu, plo, 1);
  plo += __shfl_xor_sync(0xffffffffu, plo, 2);
  phi += __shfl_xor_sync(0xffffffffu, phi, 1);
  phi += __shfl_xor_sync(0xffffffffu, phi, 2);
  y_lo = plo + w.b3[0];
  y_hi = phi + w.b3[0];
}

// 16 feature rows of a warp into shared memory; rows past n are zero
__device__ __forceinline__ void load_rows(uint16_t* xs, const uint16_t* X, const int32_t* idx,
                                          long long row0, long long n, int lane) {
  for (int e = lane; e < 16 * kNF / 2; e += 32) {  // pairs of features
    const long long r = row0 + (2 * e) / kNF;
    uint32_t v = 0u;
    if (r < n) {
      const long long src = idx ? (long long)__ldg(idx + r) : r;
      v = ld_pair(X + src * kNF + (2 * e) % kNF);
    }
    st_pair(xs + 2 * e, v);
  }
  __syncwarp();
}

}  // namespace

// ---------------------------------------------------------------------------
// features
// ---------------------------------------------------------------------------
// distance from every site to the nearest of n_bv boundary vertices
__global__ void boundary_distance_kernel(const float4* site4f, int n_site, const float4* bverts,
                                         int n_bv, float* dist) {
  __shared__ float4 tile[256];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const float4 s = i < n_site ? site4f[i] : make_float4(0.f, 0.f, 0.f, 0.f);
  float best = INFINITY;
  for (int base = 0; base < n_bv; base += 256) {
    __syncthreads();
    if (base + (int)threadIdx.x < n_bv) tile[threadIdx.x] = bverts[base + threadIdx.x];
    __syncthreads();
    const int m = min(256, n_bv - base);
    for (int q = 0; q < m; ++q) {
      const float4 b = tile[q];
      const float dx = b.x - s.x, dy = b.y - s.y, dz = b.z - s.z;
      best = fminf(best, dx * dx + dy * dy + dz * dz);
    }
  }
  if (i < n_site) dist[i] = n_bv > 0 ? sqrtf(best) : 0.f;
}

__device__ __forceinline__ float clamp16(float x) { return fminf(fmaxf(x, -16.f), 16.f); }

__global__ void pair_features_kernel(FeatureParams p) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= p.n_pairs) return;
  const long long w = p.pair_index ? (long long)p.pair_index[q] : q;
  const int t = p.pair_tet[w], i = p.pair_site[w];
  const float inv_h = p.inv_h;
  const float* keys = p.keys + (long long)i * p.k;
  const float4 s = p.site4f[i];
  const float4 c = p.centroid[t];
  const int4 tv = p.tets[t];
  const int kl = p.k - 1;
  float dmax = 0.f, dmin = INFINITY;
  {
    const int ids[4] = {tv.x, tv.y, tv.z, tv.w};
    for (int q2 = 0; q2 < 4; ++q2) {
      const float* v = p.vert3f + 3 * (long long)ids[q2];
      const float ex = v[0] - s.x, ey = v[1] - s.y, ez = v[2] - s.z;
      const float d = sqrtf(ex * ex + ey * ey + ez * ez);
      dmax = fmaxf(dmax, d);
      dmin = fminf(dmin, d);
    }
  }
  float f[kNF];
  f[0] = clamp16(sqrtf(fmaxf(s.w, 0.f)) * inv_h);
  f[1] = clamp16(keys[0] * inv_h);
  f[2] = clamp16(keys[min(3, kl)] * inv_h);
  f[3] = clamp16(keys[min(7, kl)] * inv_h);
  f[4] = clamp16(keys[min(15, kl)] * inv_h);
  f[5] = log2f(1.0f + (float)p.cell_count[p.cell_of[i]]);
  f[6] = clamp16(p.site_bdist[i] * inv_h);
  f[7] = clamp16(dmax * inv_h);
  f[8] = clamp16(dmin * inv_h);
  const float dx = c.x - s.x, dy = c.y - s.y, dz = c.z - s.z;
  f[9] = clamp16(sqrtf(dx * dx + dy * dy + dz * dz) * inv_h);
  f[10] = clamp16(keys[min(31, kl)] * inv_h);
  int lo = 0, hi = p.k;  // keys below dmax (keys ascend)
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (keys[mid] < dmax) lo = mid + 1;
    else hi = mid;
  }
  f[11] = log2f(1.0f + (float)lo);
  for (int a = 12; a < kNF; ++a) f[a] = 0.f;
  uint16_t* out = p.X + q * kNF;
#pragma unroll
  for (int a = 0; a < kNF; a += 2) st_pair(out + a, pack_bf16(f[a], f[a + 1]));
  if (p.target) p.target[q] = log2f((float)max(p.consumed[w], 1));
}

// ---------------------------------------------------------------------------
// inference
// ---------------------------------------------------------------------------
// y = net(X) for rows idx[0..n) (or 0..n); with klen, the list length
// ceil(2^(y + margin)) clamped to [kmin, kmax]
__global__ void __launch_bounds__(kMlpWarps * 32) mlp_predict_kernel(
    const uint16_t* X, const int32_t* idx, long long n, MlpWeights w, float margin, int kmin,
    int kmax, int32_t* klen, float* y_out) {
  __shared__ __align__(16) uint16_t xs[kMlpWarps][16 * kNF];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const long long row0 = ((long long)blockIdx.x * kMlpWarps + wid) * 16;
  if (row0 >= n) return;  // whole warp
  load_rows(xs[wid], X, idx, row0, n, lane);
  float z1[8][4], z2[8][4], ylo, yhi;
  mlp_forward16(xs[wid], w, lane, z1, z2, ylo, yhi);
  if ((lane & 3) == 0) {
    const int g = lane >> 2;
    for (int h = 0; h < 2; ++h) {
      const long long r = row0 + g + 8 * h;
      if (r >= n) continue;
      const float y = h ? yhi : ylo;
      if (y_out) y_out[r] = y;
      if (klen) {
        const float kk = ceilf(exp2f(fminf(y + margin, 10.0f)));
        const int ki = kk != kk ? kmax : (int)kk;  // NaN -> the whole list
        klen[r] = ki < kmin ? kmin : (ki > kmax ? kmax : ki);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// training: gradient of the mean squared error of a batch
// ---------------------------------------------------------------------------
// grads has the parameter layout (W1 [kNF][kH], b1, W2 [kH][kH] (in x out),
// b2, w3, b3) and accumulates d(sum of squared errors)/dparam * scale;
// loss_sum accumulates the sum of squared errors.
__global__ void __launch_bounds__(kMlpWarps * 32) mlp_grad_kernel(
    const uint16_t* X, const float* target, const int32_t* idx, long long n, float scale,
    MlpWeights w, float* grads, float* loss_sum) {
  __shared__ __align__(16) uint16_t xs[kMlpWarps][16 * kNF];
  __shared__ __align__(16) uint16_t h1s[kMlpWarps][16 * kH];
  __shared__ __align__(16) uint16_t dzs[kMlpWarps][16 * kH];
  __shared__ float gW1[kNF * kH], gb1[kH], gW2[kH * kH], gb2[kH], gw3[kH], gb3;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int g = lane >> 2, t = lane & 3;
  for (int e = threadIdx.x; e < kH * kH; e += blockDim.x) gW2[e] = 0.f;
  for (int e = threadIdx.x; e < kNF * kH; e += blockDim.x) gW1[e] = 0.f;
  for (int e = threadIdx.x; e < kH; e += blockDim.x) {
    gb1[e] = 0.f;
    gb2[e] = 0.f;
    gw3[e] = 0.f;
  }
  if (threadIdx.x == 0) gb3 = 0.f;
  __syncthreads();
  const long long row0 = ((long long)blockIdx.x * kMlpWarps + wid) * 16;
  if (row0 < n) {  // whole warp
    uint16_t* XS = xs[wid];
    uint16_t* H = h1s[wid];
    uint16_t* DZ = dzs[wid];
    load_rows(XS, X, idx, row0, n, lane);
    float z1[8][4], z2[8][4], ylo, yhi;
    mlp_forward16(XS, w, lane, z1, z2, ylo, yhi);
    const long long r_lo = row0 + g, r_hi = row0 + g + 8;
    const float tl = r_lo < n ? target[idx ? idx[r_lo] : r_lo] : 0.f;
    const float th = r_hi < n ? target[idx ? idx[r_hi] : r_hi] : 0.f;
    float dlo = r_lo < n ? (ylo - tl) : 0.f, dhi = r_hi < n ? (yhi - th) : 0.f;
    float l2 = t == 0 ? dlo * dlo + dhi * dhi : 0.f;
    for (int o = 1; o < 32; o <<= 1) l2 += __shfl_xor_sync(0xffffffffu, l2, o);
    if (lane == 0) atomicAdd(loss_sum, l2);
    dlo *= 2.0f * scale;  // d(sum of squares) = 2 (y - target)
    dhi *= 2.0f * scale;
    // output layer: db3, dw3; dz2 = dy w3 [z2 > 0]; h1 and dz2 (bf16) to smem
    float db3p = t == 0 ? dlo + dhi : 0.f;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int col = 8 * j + 2 * t;
      const float w30 = w.w3[col], w31 = w.w3[col + 1];
      float s0 = dlo * fmaxf(z2[j][0], 0.f) + dhi * fmaxf(z2[j][2], 0.f);
      float s1 = dlo * fmaxf(z2[j][1], 0.f) + dhi * fmaxf(z2[j][3], 0.f);
      const float d0 = z2[j][0] > 0.f ? dlo * w30 : 0.f;
      const float d1 = z2[j][1] > 0.f ? dlo * w31 : 0.f;
      const float d2 = z2[j][2] > 0.f ? dhi * w30 : 0.f;
      const float d3 = z2[j][3] > 0.f ? dhi * w31 : 0.f;
      z2[j][0] = d0;
      z2[j][1] = d1;
      z2[j][2] = d2;
      z2[j][3] = d3;
      float c0 = d0 + d2, c1 = d1 + d3;
      for (int o = 4; o < 32; o <<= 1) {  // sum over the 8 row groups
        s0 += __shfl_xor_sync(0xffffffffu, s0, o);
        s1 += __shfl_xor_sync(0xffffffffu, s1, o);
        c0 += __shfl_xor_sync(0xffffffffu, c0, o);
        c1 += __shfl_xor_sync(0xffffffffu, c1, o);
      }
      if (g == 0) {
        atomicAdd(&gw3[col], s0);
        atomicAdd(&gw3[col + 1], s1);
        atomicAdd(&gb2[col], c0);
        atomicAdd(&gb2[col + 1], c1);
      }
      st_pair(DZ + g * kH + col, pack_bf16(d0, d1));
      st_pair(DZ + (g + 8) * kH + col, pack_bf16(d2, d3));
      st_pair(H + g * kH + col, pack_bf16(fmaxf(z1[j][0], 0.f), fmaxf(z1[j][1], 0.f)));
      st_pair(H + (g + 8) * kH + col, pack_bf16(fmaxf(z1[j][2], 0.f), fmaxf(z1[j][3], 0.f)));
    }
    for (int o = 1; o < 32; o <<= 1) db3p += __shfl_xor_sync(0xffffffffu, db3p, o);
    if (lane == 0) atomicAdd(&gb3, db3p);
    __syncwarp();
    // dW2 [in][out] = h1^T dz2: M = in, N = out, K = the 16 samples
#pragma unroll
    for (int mi = 0; mi < 4; ++mi) {
      const int m0 = 16 * mi + g;
      const uint32_t a0 = ld2(H + (2 * t) * kH + m0, H + (2 * t + 1) * kH + m0);
      const uint32_t a1 = ld2(H + (2 * t) * kH + m0 + 8, H + (2 * t + 1) * kH + m0 + 8);
      const uint32_t a2 = ld2(H + (2 * t + 8) * kH + m0, H + (2 * t + 9) * kH + m0);
      const uint32_t a3 = ld2(H + (2 * t + 8) * kH + m0 + 8, H + (2 * t + 9) * kH + m0 + 8);
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const int n0 = 8 * j + g;
        const uint32_t b0 = ld2(DZ + (2 * t) * kH + n0, DZ + (2 * t + 1) * kH + n0);
        const uint32_t b1 = ld2(DZ + (2 * t + 8) * kH + n0, DZ + (2 * t + 9) * kH + n0);
        float acc[4] = {0.f, 0.f, 0.f, 0.f};
        mma16816(acc, a0, a1, a2, a3, b0, b1);
        const int col = 8 * j + 2 * t;
        atomicAdd(&gW2[m0 * kH + col], acc[0]);
        atomicAdd(&gW2[m0 * kH + col + 1], acc[1]);
        atomicAdd(&gW2[(m0 + 8) * kH + col], acc[2]);
        atomicAdd(&gW2[(m0 + 8) * kH + col + 1], acc[3]);
      }
    }
    // dh1 = dz2 W2^T: A = dz2 fragments, B[k = out][n = in] = W2[in][out]
    float dh[8][4];
#pragma unroll
    for (int j = 0; j < 8; ++j) dh[j][0] = dh[j][1] = dh[j][2] = dh[j][3] = 0.f;
#pragma unroll
    for (int kc = 0; kc < 4; ++kc) {
      const float* lo = z2[2 * kc];
      const float* hi = z2[2 * kc + 1];
      const uint32_t q0 = pack_bf16(lo[0], lo[1]), q1 = pack_bf16(lo[2], lo[3]);
      const uint32_t q2 = pack_bf16(hi[0], hi[1]), q3 = pack_bf16(hi[2], hi[3]);
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const uint16_t* b = w.W2 + (8 * j + g) * kH + 16 * kc + 2 * t;
        mma16816(dh[j], q0, q1, q2, q3, ld_pair(b), ld_pair(b + 8));
      }
    }
    __syncwarp();  // every lane has read dz2 from DZ
    // dz1 = dh1 [z1 > 0]; db1; dz1 (bf16) to smem in place of dz2
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int col = 8 * j + 2 * t;
      const float d0 = z1[j][0] > 0.f ? dh[j][0] : 0.f;
      const float d1 = z1[j][1] > 0.f ? dh[j][1] : 0.f;
      const float d2 = z1[j][2] > 0.f ? dh[j][2] : 0.f;
      const float d3 = z1[j][3] > 0.f ? dh[j][3] : 0.f;
      float c0 = d0 + d2, c1 = d1 + d3;
      for (int o = 4; o < 32; o <<= 1) {
        c0 += __shfl_xor_sync(0xffffffffu, c0, o);
        c1 += __shfl_xor_sync(0xffffffffu, c1, o);
      }
      if (g == 0) {
        atomicAdd(&gb1[col], c0);
        atomicAdd(&gb1[col + 1], c1);
      }
      st_pair(DZ + g * kH + col, pack_bf16(d0, d1));
      st_pair(DZ + (g + 8) * kH + col, pack_bf16(d2, d3));
    }
    __syncwarp();
    // dW1 [feature][hidden] = X^T dz1: M = 16 features, N = hidden, K = samples
    const uint32_t a0 = ld2(XS + (2 * t) * kNF + g, XS + (2 * t + 1) * kNF + g);
    const uint32_t a1 = ld2(XS + (2 * t) * kNF + g + 8, XS + (2 * t + 1) * kNF + g + 8);
    const uint32_t a2 = ld2(XS + (2 * t + 8) * kNF + g, XS + (2 * t + 9) * kNF + g);
    const uint32_t a3 = ld2(XS + (2 * t + 8) * kNF + g + 8, XS + (2 * t + 9) * kNF + g + 8);
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int n0 = 8 * j + g;
      const uint32_t b0 = ld2(DZ + (2 * t) * kH + n0, DZ + (2 * t + 1) * kH + n0);
      const uint32_t b1 = ld2(DZ + (2 * t + 8) * kH + n0, DZ + (2 * t + 9) * kH + n0);
      float acc[4] = {0.f, 0.f, 0.f, 0.f};
      mma16816(acc, a0, a1, a2, a3, b0, b1);
      const int col = 8 * j + 2 * t;
      atomicAdd(&gW1[g * kH + col], acc[0]);
      atomicAdd(&gW1[g * kH + col + 1], acc[1]);
      atomicAdd(&gW1[(g + 8) * kH + col], acc[2]);
      atomicAdd(&gW1[(g + 8) * kH + col + 1], acc[3]);
    }
  }
  __syncthreads();
  float* G = grads;
  for (int e = threadIdx.x; e < kNF * kH; e += blockDim.x) atomicAdd(G + e, gW1[e]);
  G += kNF * kH;
  for (int e = threadIdx.x; e < kH; e += blockDim.x) atomicAdd(G + e, gb1[e]);
  G += kH;
  for (int e = threadIdx.x; e < kH * kH; e += blockDim.x) atomicAdd(G + e, gW2[e]);
  G += kH * kH;
  for (int e = threadIdx.x; e < kH; e += blockDim.x) atomicAdd(G + e, gb2[e]);
  G += kH;
  for (int e = threadIdx.x; e < kH; e += blockDim.x) atomicAdd(G + e, gw3[e]);
  G += kH;
  if (threadIdx.x == 0) atomicAdd(G, gb3);
}

// bf16 operand copies of the two weight matrices from the fp32 masters
__device__ __forceinline__ void write_operand(int e, float p, uint16_t* W1T, uint16_t* W2,
                                              uint16_t* W2T) {
  if (e < kNF * kH) {
    const int f = e / kH, h = e % kH;
    W1T[h * kNF + f] = bf16_bits(p);
    return;
  }
  const int o = e - kNF * kH - kH;
  if (o >= 0 && o < kH * kH) {
    const int in = o / kH, out = o % kH;
    W2[in * kH + out] = bf16_bits(p);
    W2T[out * kH + in] = bf16_bits(p);
  }
}

// one Adam step on the fp32 masters; refreshes the operand copies and clears
// the gradient
__global__ void mlp_adam_kernel(float* params, float* grads, float* m, float* v, int n, float lr,
                                float beta1, float beta2, float eps, float bc1, float bc2,
                                uint16_t* W1T, uint16_t* W2, uint16_t* W2T) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  const float gr = grads[e];
  grads[e] = 0.f;
  const float mm = beta1 * m[e] + (1.f - beta1) * gr;
  const float vv = beta2 * v[e] + (1.f - beta2) * gr * gr;
  m[e] = mm;
  v[e] = vv;
  const float p = params[e] - lr * (mm / bc1) / (sqrtf(vv / bc2) + eps);
  params[e] = p;
  write_operand(e, p, W1T, W2, W2T);
}

__global__ void mlp_sync_operands_kernel(const float* params, int n, uint16_t* W1T, uint16_t* W2,
                                         uint16_t* W2T) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e < n) write_operand(e, params[e], W1T, W2, W2T);
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
MlpWeights mlp_weights_view(const float* params, const uint16_t* W1T, const uint16_t* W2,
                            const uint16_t* W2T) {
  MlpWeights w;
  w.W1T = W1T;
  w.W2 = W2;
  w.W2T = W2T;
  w.b1 = params + kNF * kH;
  w.b2 = w.b1 + kH + kH * kH;
  w.w3 = w.b2 + kH;
  w.b3 = w.w3 + kH;
  return w;
}

cudaError_t launch_boundary_distance(const float4* site4f, int n_site, const float4* bverts,
                                     int n_bv, float* dist, cudaStream_t st) {
  if (n_site <= 0) return cudaSuccess;
  boundary_distance_kernel<<<(n_site + 255) / 256, 256, 0, st>>>(site4f, n_site, bverts, n_bv,
                                                                 dist);
  note_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_pair_features(const FeatureParams& p, cudaStream_t st) {
  if (p.n_pairs <= 0) return cudaSuccess;
  pair_features_kernel<<<(unsigned)((p.n_pairs + 255) / 256), 256, 0, st>>>(p);
  note_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_mlp_predict(const uint16_t* X, const int32_t* idx, long long n,
                               const MlpWeights& w, float margin, int kmin, int kmax,
                               int32_t* klen, float* y, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  const long long blocks = (n + 16 * kMlpWarps - 1) / (16 * kMlpWarps);
  mlp_predict_kernel<<<(unsigned)blocks, kMlpWarps * 32, 0, st>>>(X, idx, n, w, margin, kmin,
                                                                  kmax, klen, y);
  note_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_mlp_grad(const uint16_t* X, const float* target, const int32_t* idx,
                            long long n, float scale, const MlpWeights& w, float* grads,
                            float* loss_sum, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  const long long blocks = (n + 16 * kMlpWarps - 1) / (16 * kMlpWarps);
  mlp_grad_kernel<<<(unsigned)blocks, kMlpWarps * 32, 0, st>>>(X, target, idx, n, scale, w,
                                                               grads, loss_sum);
  note_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_mlp_adam(float* params, float* grads, float* m, float* v, int step, float lr,
                            uint16_t* W1T, uint16_t* W2, uint16_t* W2T, cudaStream_t st) {
  const float beta1 = 0.9f, beta2 = 0.999f;
  const float bc1 = 1.f - powf(beta1, (float)step), bc2 = 1.f - powf(beta2, (float)step);
  const int n = kMlpParams;
  mlp_adam_kernel<<<(n + 255) / 256, 256, 0, st>>>(params, grads, m, v, n, lr, beta1, beta2,
                                                   1e-8f, bc1, bc2, W1T, W2, W2T);
  note_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_mlp_sync_operands(const float* params, uint16_t* W1T, uint16_t* W2,
                                     uint16_t* W2T, cudaStream_t st) {
  const int n = kMlpParams;
  mlp_sync_operands_kernel<<<(n + 255) / 256, 256, 0, st>>>(params, n, W1T, W2, W2T);
  note_launches(1);
  return cudaGetLastError();
}

}  // namespace rpd
