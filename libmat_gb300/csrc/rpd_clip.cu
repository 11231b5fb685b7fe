// rpd_clip.cu -- warp-cooperative convex-cell clipping on sm_103a.
//
// One warp owns one cell: the tet (or a box) clipped by the power bisectors
// of one site's neighbour list, in list order.  The cell's planes, dual
// triangles (vertices), edges and boundary links live in shared memory in
// the reference's representation (convex_cell.h:73-115, :117-185), so the
// records it emits are the reference's ConvexCell contents.
//
// Semantics follow src/rpd3d/convex_cell.cu exactly:
//   cell = tet                         :116-214
//   bisector plane (FP32)              :561-592
//   conflict predicate, tie = none     :437-500 (FP64 det4x4 of float planes)
//   conflict partition (swap to tail)  :706-721
//   cavity boundary walk               :618-678
//   new edges / vertices / perturb     :524-554, :604-616, :274-316
//   per-list driver and drop rules     :1166-1337
// What is GB300-specific is the execution: the plane coefficients of 32
// neighbours are built by 32 lanes at once; while the cell has <= 16
// vertices each predicate step tests several consecutive planes against all
// vertices in one ballot and jumps to the first plane that clips anything
// (planes that clip nothing leave the cell unchanged, so skipping them is
// exact); predicate signs come from an FP32 cofactor filter with a proven
// error bound and fall back to the reference's FP64 determinant only when
// undecided; the topology update of a clipping plane runs on lane 0 while
// the vertex cofactors of the new vertices are rebuilt in parallel.
//
// This translation unit is compiled with -fmad=false: every float/double
// expression below that restates a reference formula is evaluated one IEEE
// rounding at a time, as in the reference's source.  FMA is used only where
// written explicitly (the filter).

#include <cuda_runtime.h>

#include "rpd_common.cuh"
#include "rpd_df64.cuh"
#include "rpd_kernels.cuh"

namespace rpd {

// ------------------------------------------------------------------------
// shared-memory cell
// ------------------------------------------------------------------------
struct __align__(16) WarpCell {
  float4 pl[kMaxP];  // plane (a, b, c, d), inside: a x + b y + c z + d >= 0
  union {
    struct {
      float4 K[kMaxT];  // cofactors of each vertex (filter)
      float4 M[kMaxT];  // 3x3 permanents matching each cofactor (filter)
      float rad[kMaxT]; // bound on each vertex's distance to the seed (certificate)
    } f;
    struct {
      df n[kMaxP][3];   // plane normal, seed frame, double-float (geometry)
      df d[kMaxP];      // plane offset, seed frame
      float3 foot[kMaxP];  // foot of the volume origin on each plane
    } g;
  } u;
  int2 id2[kMaxP];
  uchar4 ver[kMaxT];
  uchar4 edge[kMaxE];
  uint8_t h[kMaxP];
  uint8_t bnext[kMaxP];
  uint8_t perm[kMaxT];  // during a clip: the slot each surviving vertex came from
  float4 cand[32];      // the planes of the list chunk being tested, one per lane
};

struct CellState {
  int nb_v, nb_p, nb_e;
  int status;
  int kept;  // vertices that survived the last clip (slots [0, kept))
};

// local faces / edges of a tet (convex_cell.h:25-29, convex_cell.cu:193-211)
__constant__ int8_t cFaceLv[4][3] = {{2, 1, 3}, {0, 2, 3}, {1, 0, 3}, {0, 1, 2}};
__constant__ int8_t cEdgeFaces[6][2] = {{2, 3}, {1, 3}, {1, 2}, {0, 3}, {0, 2}, {0, 1}};
__constant__ int8_t cTetTri[4][3] = {{1, 3, 2}, {0, 2, 3}, {0, 3, 1}, {0, 1, 2}};
// slot of the initial edge between tet faces (lo, hi), lo < hi < 4
__constant__ int8_t cTetEdgeSlot[4][4] = {{-1, 5, 4, 3}, {5, -1, 2, 1}, {4, 2, -1, 0}, {3, 1, 0, -1}};

// ------------------------------------------------------------------------
// reference arithmetic (no contraction in this TU)
// ------------------------------------------------------------------------
__device__ __forceinline__ float4 tri2plane_f(float3 v0, float3 v1, float3 v2) {
  float ax = v1.x - v0.x, ay = v1.y - v0.y, az = v1.z - v0.z;
  float bx = v2.x - v0.x, by = v2.y - v0.y, bz = v2.z - v0.z;
  float nx = ay * bz - az * by;
  float ny = az * bx - ax * bz;
  float nz = ax * by - ay * bx;
  return make_float4(nx, ny, nz, -(v0.x * nx + v0.y * ny + v0.z * nz));
}

__device__ __forceinline__ float4 bisector_f(float4 S, float4 B) {
  float dx = S.x - B.x, dy = S.y - B.y, dz = S.z - B.z;
  float ax = S.x + B.x, ay = S.y + B.y, az = S.z + B.z;
  float dot = (ax * dx + ay * dy + az * dz) + (B.w - S.w);
  return make_float4(dx, dy, dz, -dot / 2.f);
}

__device__ __forceinline__ double det4x4_ref(float4 p1, float4 p2, float4 p3,
                                             float4 e) {
  double a11 = p1.x, a12 = p2.x, a13 = p3.x, a14 = e.x;
  double a21 = p1.y, a22 = p2.y, a23 = p3.y, a24 = e.y;
  double a31 = p1.z, a32 = p2.z, a33 = p3.z, a34 = e.z;
  double a41 = p1.w, a42 = p2.w, a43 = p3.w, a44 = e.w;
  double m12 = a21 * a12 - a11 * a22;
  double m13 = a31 * a12 - a11 * a32;
  double m14 = a41 * a12 - a11 * a42;
  double m23 = a31 * a22 - a21 * a32;
  double m24 = a41 * a22 - a21 * a42;
  double m34 = a41 * a32 - a31 * a42;
  double m123 = m23 * a13 - m13 * a23 + m12 * a33;
  double m124 = m24 * a13 - m14 * a23 + m12 * a43;
  double m134 = m34 * a13 - m14 * a33 + m13 * a43;
  double m234 = m34 * a23 - m24 * a33 + m23 * a43;
  return (m234 * a14 - m134 * a24 + m124 * a34 - m123 * a44);
}

// float det3x3 of the three plane normals (convex_cell.cu:274-316, the w
// of the homogeneous vertex); zero means the vertex needs a perturbation
__device__ __forceinline__ float det3x3_f(float4 a, float4 b, float4 c) {
  float t1 = b.y * c.z - b.z * c.y;
  float t2 = a.y * c.z - a.z * c.y;
  float t3 = a.y * b.z - a.z * b.y;
  return a.x * t1 - b.x * t2 + c.x * t3;
}

// ------------------------------------------------------------------------
// FP32 filter: det4x4(p1,p2,p3,e) = sum_r e_r K_r, K_r the signed 3x3
// minors of the vertex planes.  |fl(K_r) - K_r| <= gamma_5 M_r (M_r the 3x3
// permanent), the FMA dot adds gamma_4 sum|e_r K_r|; the bound also covers
// the reference's FP64 evaluation (gamma_9 in double times the 4x4
// permanent), so a decided sign is the sign of the reference's FP64 det.
// ------------------------------------------------------------------------
__device__ __forceinline__ void minor3(float a1, float b1, float c1, float a2,
                                       float b2, float c2, float a3, float b3,
                                       float c3, float& det, float& perm) {
  float u1 = __fmaf_rn(b2, c3, -(b3 * c2));
  float u2 = __fmaf_rn(a2, c3, -(a3 * c2));
  float u3 = __fmaf_rn(a2, b3, -(a3 * b2));
  det = __fmaf_rn(a1, u1, __fmaf_rn(-b1, u2, c1 * u3));
  float v1 = __fmaf_rn(fabsf(b2), fabsf(c3), fabsf(b3) * fabsf(c2));
  float v2 = __fmaf_rn(fabsf(a2), fabsf(c3), fabsf(a3) * fabsf(c2));
  float v3 = __fmaf_rn(fabsf(a2), fabsf(b3), fabsf(a3) * fabsf(b2));
  perm = __fmaf_rn(fabsf(a1), v1, __fmaf_rn(fabsf(b1), v2, fabsf(c1) * v3));
}

__device__ __forceinline__ void vertex_cofactors(float4 p1, float4 p2, float4 p3,
                                                 float4& K, float4& M) {
  float d;
  minor3(p1.y, p1.z, p1.w, p2.y, p2.z, p2.w, p3.y, p3.z, p3.w, d, M.x);
  K.x = -d;
  minor3(p1.x, p1.z, p1.w, p2.x, p2.z, p2.w, p3.x, p3.z, p3.w, d, M.y);
  K.y = d;
  minor3(p1.x, p1.y, p1.w, p2.x, p2.y, p2.w, p3.x, p3.y, p3.w, d, M.z);
  K.z = -d;
  minor3(p1.x, p1.y, p1.z, p2.x, p2.y, p2.z, p3.x, p3.y, p3.z, d, M.w);
  K.w = d;
}

constexpr float kFiltC1 = 5.0f * 5.9604645e-08f;
constexpr float kFiltC2 = 6.0f * 5.9604645e-08f;
constexpr float kFiltAbs = 1e-30f;

// +1 / -1 decided, 0 undecided.  Bound: c1 sum|e_r K_r| (rounding of the
// dot) + c2 sum|e_r| M_r (rounding of the cofactors, and of the reference's
// own FP64 evaluation, both proportional to the 4x4 permanent
// sum_r |e_r| M_r)
__device__ __forceinline__ int filter_sign(float4 K, float4 M, float4 e) {
  float s = __fmaf_rn(e.w, K.w, __fmaf_rn(e.z, K.z, __fmaf_rn(e.y, K.y, e.x * K.x)));
  float t = __fmaf_rn(fabsf(e.w), fabsf(K.w),
                      __fmaf_rn(fabsf(e.z), fabsf(K.z),
                                __fmaf_rn(fabsf(e.y), fabsf(K.y), fabsf(e.x) * fabsf(K.x))));
  float pm = __fmaf_rn(fabsf(e.w), M.w,
                       __fmaf_rn(fabsf(e.z), M.z, __fmaf_rn(fabsf(e.y), M.y, fabsf(e.x) * M.x)));
  float b = __fmaf_rn(kFiltC1, t, kFiltC2 * pm) + kFiltAbs;
  return s > b ? 1 : (s < -b ? -1 : 0);
}

// ------------------------------------------------------------------------
// FP64 error bound and exact sign of det4x4 (RPD_PRED_EXACT)
// ------------------------------------------------------------------------
// det4x4_ref evaluated with the same operations, plus the same expression
// over absolute values P.  Products of two floats are exact in FP64; every
// other operation rounds once, at most 8 along any path of the expression,
// so |computed - exact| <= gamma_8 P < 10 * 2^-53 * P.
__device__ __forceinline__ double det4x4_with_bound(float4 p1, float4 p2, float4 p3, float4 e,
                                                    double& bound) {
  const double a11 = p1.x, a12 = p2.x, a13 = p3.x, a14 = e.x;
  const double a21 = p1.y, a22 = p2.y, a23 = p3.y, a24 = e.y;
  const double a31 = p1.z, a32 = p2.z, a33 = p3.z, a34 = e.z;
  const double a41 = p1.w, a42 = p2.w, a43 = p3.w, a44 = e.w;
  const double m12 = a21 * a12 - a11 * a22, P12 = fabs(a21 * a12) + fabs(a11 * a22);
  const double m13 = a31 * a12 - a11 * a32, P13 = fabs(a31 * a12) + fabs(a11 * a32);
  const double m14 = a41 * a12 - a11 * a42, P14 = fabs(a41 * a12) + fabs(a11 * a42);
  const double m23 = a31 * a22 - a21 * a32, P23 = fabs(a31 * a22) + fabs(a21 * a32);
  const double m24 = a41 * a22 - a21 * a42, P24 = fabs(a41 * a22) + fabs(a21 * a42);
  const double m34 = a41 * a32 - a31 * a42, P34 = fabs(a41 * a32) + fabs(a31 * a42);
  const double m123 = m23 * a13 - m13 * a23 + m12 * a33;
  const double m124 = m24 * a13 - m14 * a23 + m12 * a43;
  const double m134 = m34 * a13 - m14 * a33 + m13 * a43;
  const double m234 = m34 * a23 - m24 * a33 + m23 * a43;
  const double P123 = P23 * fabs(a13) + P13 * fabs(a23) + P12 * fabs(a33);
  const double P124 = P24 * fabs(a13) + P14 * fabs(a23) + P12 * fabs(a43);
  const double P134 = P34 * fabs(a13) + P14 * fabs(a33) + P13 * fabs(a43);
  const double P234 = P34 * fabs(a23) + P24 * fabs(a33) + P23 * fabs(a43);
  const double P = P234 * fabs(a14) + P134 * fabs(a24) + P124 * fabs(a34) + P123 * fabs(a44);
  bound = 10.0 * 1.1102230246251565e-16 * P + 1e-300;
  return (m234 * a14 - m134 * a24 + m124 * a34 - m123 * a44);
}

// Exact sign by floating-point expansions (Shewchuk, "Adaptive precision
// floating-point arithmetic and fast robust geometric predicates", Discrete
// Comput. Geom. 18, 1997): TwoSum, TwoProduct (with FMA),
// FAST-EXPANSION-SUM and SCALE-EXPANSION, both with zero elimination.
// Expansions are nonoverlapping, in increasing magnitude.
__device__ __forceinline__ void ex_two_sum(double a, double b, double& x, double& y) {
  x = a + b;
  const double bv = x - a;
  const double av = x - bv;
  y = (a - av) + (b - bv);
}
__device__ __forceinline__ void ex_fast_two_sum(double a, double b, double& x, double& y) {
  x = a + b;
  y = b - (x - a);
}
__device__ __forceinline__ void ex_two_prod(double a, double b, double& x, double& y) {
  x = a * b;
  y = fma(a, b, -x);
}

__device__ int ex_sum(int elen, const double* e, int flen, const double* f, double* h) {
  int ei = 0, fi = 0, hi = 0;
  double en = e[0], fn = f[0], Q, Qn, hh;
  if ((fn > en) == (fn > -en)) {
    Q = en;
    en = ++ei < elen ? e[ei] : 0.0;
  } else {
    Q = fn;
    fn = ++fi < flen ? f[fi] : 0.0;
  }
  if (ei < elen && fi < flen) {
    if ((fn > en) == (fn > -en)) {
      ex_fast_two_sum(en, Q, Qn, hh);
      en = ++ei < elen ? e[ei] : 0.0;
    } else {
      ex_fast_two_sum(fn, Q, Qn, hh);
      fn = ++fi < flen ? f[fi] : 0.0;
    }
    Q = Qn;
    if (hh != 0.0) h[hi++] = hh;
    while (ei < elen && fi < flen) {
      if ((fn > en) == (fn > -en)) {
        ex_two_sum(Q, en, Qn, hh);
        en = ++ei < elen ? e[ei] : 0.0;
      } else {
        ex_two_sum(Q, fn, Qn, hh);
        fn = ++fi < flen ? f[fi] : 0.0;
      }
      Q = Qn;
      if (hh != 0.0) h[hi++] = hh;
    }
  }
  while (ei < elen) {
    ex_two_sum(Q, en, Qn, hh);
    en = ++ei < elen ? e[ei] : 0.0;
    Q = Qn;
    if (hh != 0.0) h[hi++] = hh;
  }
  while (fi < flen) {
    ex_two_sum(Q, fn, Qn, hh);
    fn = ++fi < flen ? f[fi] : 0.0;
    Q = Qn;
    if (hh != 0.0) h[hi++] = hh;
  }
  if (Q != 0.0 || hi == 0) h[hi++] = Q;
  return hi;
}

__device__ int ex_scale(int elen, const double* e, double b, double* h) {
  int hi = 0;
  double Q, hh, p1, p0, sum;
  ex_two_prod(e[0], b, Q, hh);
  if (hh != 0.0) h[hi++] = hh;
  for (int i = 1; i < elen; ++i) {
    ex_two_prod(e[i], b, p1, p0);
    ex_two_sum(Q, p0, sum, hh);
    if (hh != 0.0) h[hi++] = hh;
    ex_fast_two_sum(p1, sum, Q, hh);
    if (hh != 0.0) h[hi++] = hh;
  }
  if (Q != 0.0 || hi == 0) h[hi++] = Q;
  return hi;
}

// 2x2 minor a*b - c*d of floats (both products exact in FP64)
__device__ __forceinline__ int ex_minor2(double a, double b, double c, double d, double* h) {
  double x, y;
  ex_two_sum(a * b, -(c * d), x, y);
  int n = 0;
  if (y != 0.0) h[n++] = y;
  if (x != 0.0 || n == 0) h[n++] = x;
  return n;
}

// u*a - v*b + w*c for expansions u, v, w (<= lu, lv, lw terms)
__device__ int ex_combine3(const double* u, int lu, double a, const double* v, int lv, double b,
                           const double* w, int lw, double c, double* h) {
  double t1[24], t2[24], t3[24], t12[48];
  const int n1 = ex_scale(lu, u, a, t1);
  const int n2 = ex_scale(lv, v, -b, t2);
  const int n3 = ex_scale(lw, w, c, t3);
  const int n12 = ex_sum(n1, t1, n2, t2, t12);
  return ex_sum(n12, t12, n3, t3, h);
}

// exact sign of det4x4_ref's determinant (same matrix, no rounding)
__device__ __noinline__ int det4x4_exact_sign(float4 p1, float4 p2, float4 p3, float4 e) {
  const double a11 = p1.x, a12 = p2.x, a13 = p3.x, a14 = e.x;
  const double a21 = p1.y, a22 = p2.y, a23 = p3.y, a24 = e.y;
  const double a31 = p1.z, a32 = p2.z, a33 = p3.z, a34 = e.z;
  const double a41 = p1.w, a42 = p2.w, a43 = p3.w, a44 = e.w;
  double m12[2], m13[2], m14[2], m23[2], m24[2], m34[2];
  const int l12 = ex_minor2(a21, a12, a11, a22, m12);
  const int l13 = ex_minor2(a31, a12, a11, a32, m13);
  const int l14 = ex_minor2(a41, a12, a11, a42, m14);
  const int l23 = ex_minor2(a31, a22, a21, a32, m23);
  const int l24 = ex_minor2(a41, a22, a21, a42, m24);
  const int l34 = ex_minor2(a41, a32, a31, a42, m34);
  double m123[12], m124[12], m134[12], m234[12];
  const int l123 = ex_combine3(m23, l23, a13, m13, l13, a23, m12, l12, a33, m123);
  const int l124 = ex_combine3(m24, l24, a13, m14, l14, a23, m12, l12, a43, m124);
  const int l134 = ex_combine3(m34, l34, a13, m14, l14, a33, m13, l13, a43, m134);
  const int l234 = ex_combine3(m34, l34, a23, m24, l24, a33, m23, l23, a43, m234);
  // m234 a14 - m134 a24 + m124 a34 - m123 a44
  double t1[24], t2[24], t3[24], t4[24], s12[48], s34[48], d[96];
  const int n1 = ex_scale(l234, m234, a14, t1);
  const int n2 = ex_scale(l134, m134, -a24, t2);
  const int n3 = ex_scale(l124, m124, a34, t3);
  const int n4 = ex_scale(l123, m123, -a44, t4);
  const int n12 = ex_sum(n1, t1, n2, t2, s12);
  const int n34 = ex_sum(n3, t3, n4, t4, s34);
  const int n = ex_sum(n12, s12, n34, s34, d);
  const double top = d[n - 1];
  return top > 0.0 ? 1 : (top < 0.0 ? -1 : 0);
}

__device__ __forceinline__ bool plane_eq(float4 a, float4 b) {
  return a.x == b.x && a.y == b.y && a.z == b.z && a.w == b.w;
}

// predicate statistics of a thread: evaluated, escalated to FP64; and where
// the escalations of RPD_PRED_EXACT count their FP64-uncertain / exact-flip
// cases
struct PredCount {
  uint32_t pred, esc;
  unsigned long long* exact;
};

__host__ __device__ constexpr bool uses_filter(int pred) {
  return pred == RPD_PRED_FP32_FILTER || pred == RPD_PRED_EXACT;
}

// RPD_PRED_EXACT: the predicates the filter cannot decide, out of line
// (rare).  counts (optional): [0] FP64 signs not certified by their error
// bound (decided exactly), [1] exact signs different from the FP64 sign
__device__ __noinline__ bool exact_conflict(float4 p1, float4 p2, float4 p3, float4 e,
                                            unsigned long long* counts) {
  double bound;
  const double d = det4x4_with_bound(p1, p2, p3, e, bound);
  if (fabs(d) > bound) return d > 0.0;
  if (counts) atomicAdd(counts, 1ull);
  const int xs = det4x4_exact_sign(p1, p2, p3, e);
  if (counts && (xs > 0) != (d > 0.0)) atomicAdd(counts + 1, 1ull);
  return xs > 0;
}

// conflict of the vertex in slot vi with plane e; dup = planes identical to e
template <int PRED>
__device__ __forceinline__ bool in_conflict(const WarpCell& c, int vi, float4 e,
                                            uint64_t dup, PredCount& pc) {
  if (dup != 0ull) {  // rare: the plane equals one of the cell's
    const uchar4 v = c.ver[vi];
    if (dup & ((1ull << v.x) | (1ull << v.y) | (1ull << v.z))) return false;
  }
  ++pc.pred;
  if (uses_filter(PRED)) {
    int s = filter_sign(c.u.f.K[vi], c.u.f.M[vi], e);
    if (s != 0) return s > 0;
    ++pc.esc;
    const uchar4 v = c.ver[vi];
    if (PRED == RPD_PRED_EXACT) return exact_conflict(c.pl[v.x], c.pl[v.y], c.pl[v.z], e, pc.exact);
    return det4x4_ref(c.pl[v.x], c.pl[v.y], c.pl[v.z], e) > 0.0;
  }
  const uchar4 v = c.ver[vi];
  return det4x4_ref(c.pl[v.x], c.pl[v.y], c.pl[v.z], e) > 0.0;
}

// ------------------------------------------------------------------------
// topology update (convex_cell.cu:618-774)
// ------------------------------------------------------------------------
// cavity boundary as a circular list over plane ids (convex_cell.cu:618-678)
// (bnext must be all kEnd on entry; the warp clears it before lane 0 runs)
__device__ void compute_boundary(WarpCell& c, int nb_v, int& nb_r, int& first,
                                 int& status) {
  first = kEnd;
  int nb_iter = 0;
  int t = nb_v;
  while (nb_r > 0) {
    if (nb_iter++ > 65535) {
      status = kInconsistentBoundary;
      return;
    }
    uchar4 tr = c.ver[t];
    uint8_t p[3] = {tr.x, tr.y, tr.z};
    bool in_border[3], opp[3];
    for (int e = 0; e < 3; ++e) in_border[e] = c.bnext[p[e]] != kEnd;
    for (int e = 0; e < 3; ++e) opp[e] = c.bnext[p[(e + 1) % 3]] == p[e];
    bool simple = true;
    for (int e = 0; e < 3; ++e)
      if (!opp[e] && !opp[(e + 1) % 3] && in_border[(e + 1) % 3]) simple = false;
    if (!opp[0] && !opp[1] && !opp[2]) {
      if (first == kEnd) {
        for (int e = 0; e < 3; ++e) c.bnext[p[e]] = p[(e + 1) % 3];
        first = p[0];
      } else {
        simple = false;
      }
    }
    if (!simple) {
      t++;
      if (t == nb_v + nb_r) t = nb_v;
      continue;
    }
    for (int e = 0; e < 3; ++e)
      if (!opp[e]) c.bnext[p[e]] = p[(e + 1) % 3];
    for (int e = 0; e < 3; ++e)
      if (opp[e] && opp[(e + 1) % 3]) {
        if (first == p[(e + 1) % 3]) first = c.bnext[p[(e + 1) % 3]];
        c.bnext[p[(e + 1) % 3]] = kEnd;
      }
    int last = nb_v + nb_r - 1;
    uchar4 tmp = c.ver[t];
    c.ver[t] = c.ver[last];
    c.ver[last] = tmp;
    t = nb_v;
    nb_r--;
  }
}

// Adds plane e (already written to slot nb_p by the caller) and applies the
// clip whose conflicting vertex slots are in mask[3], by lane 0, for the box
// kernel: only the polytope (no edges, adjacency counts or perturbation
// check; the cell kernel's update is clip_full, by the whole warp).
__device__ void apply_clip_box(WarpCell& c, CellState& s, const uint32_t* mask_in) {
  // conflict bits of vertex slots 0..95 in registers (32-bit words)
  uint32_t m0 = mask_in[0], m1 = mask_in[1], m2 = mask_in[2];
  const int cur = s.nb_p;
  s.nb_p++;
  // conflict partition, the reference's swap-to-tail loop.  Only the dual
  // triangles move here; perm records where each slot's vertex came from,
  // and the warp moves the cofactors afterwards (the conflict bit of a slot
  // at or past the shrinking end is never read again)
  int nb_v = s.nb_v, nb_r = 0, i = 0;
  while (i < nb_v) {
    // the next conflicting slot from i on (bits at or past nb_v are stale
    // and end the loop)
    {
      uint32_t w = i < 32 ? m0 : (i < 64 ? m1 : m2);
      w &= ~0u << (i & 31);
      int base = i & ~31;
      while (w == 0u && base < 64) {
        base += 32;
        w = base == 32 ? m1 : m2;
      }
      if (w == 0u) break;
      i = base + __ffs(w) - 1;
      if (i >= nb_v) break;
    }
    const uint32_t wi = i < 32 ? m0 : (i < 64 ? m1 : m2);
    if ((wi >> (i & 31)) & 1u) {
      nb_v--;
      const uchar4 tv = c.ver[i];
      c.ver[i] = c.ver[nb_v];
      c.ver[nb_v] = tv;
      const uint8_t pv = c.perm[i];
      c.perm[i] = c.perm[nb_v];
      c.perm[nb_v] = pv;
      const uint32_t wn = nb_v < 32 ? m0 : (nb_v < 64 ? m1 : m2);
      const uint32_t bit = 1u << (i & 31);
      const uint32_t nw = ((wn >> (nb_v & 31)) & 1u) ? (wi | bit) : (wi & ~bit);
      if (i < 32) m0 = nw;
      else if (i < 64) m1 = nw;
      else m2 = nw;
      nb_r++;
    } else {
      i++;
    }
  }
  s.nb_v = nb_v;
  s.kept = nb_v;
  if (nb_v == 0) {
    s.status = kNoIntersection;
    return;
  }
  int first;
  if (nb_r == 1) {
    // one vertex removed: the cavity is its triangle, and the walk would
    // link its three planes in order, starting at the first
    const uchar4 tr = c.ver[nb_v];
    c.bnext[tr.x] = tr.y;
    c.bnext[tr.y] = tr.z;
    c.bnext[tr.z] = tr.x;
    first = tr.x;
  } else {
    compute_boundary(c, nb_v, nb_r, first, s.status);
  }
  if (s.status != kSuccess) return;
  if (first == kEnd) return;
  // new vertices around the cavity boundary
  int cir = first;
  do {
    const int nx = c.bnext[cir];
    if (s.nb_v + 1 >= kMaxT) {
      s.status = kTriangleOverflow;
      return;
    }
    c.ver[s.nb_v] = make_uchar4((uint8_t)cur, (uint8_t)cir, (uint8_t)nx, 0);
    s.nb_v++;
    cir = nx;
  } while (cir != first);
}

__device__ __forceinline__ void broadcast_state(CellState& s) {
  s.nb_v = __shfl_sync(0xffffffffu, s.nb_v, 0);
  s.nb_p = __shfl_sync(0xffffffffu, s.nb_p, 0);
  s.nb_e = __shfl_sync(0xffffffffu, s.nb_e, 0);
  s.status = __shfl_sync(0xffffffffu, s.status, 0);
  s.kept = __shfl_sync(0xffffffffu, s.kept, 0);
}

__device__ __forceinline__ uint64_t shfl64(uint64_t v, int src) {
  uint32_t lo = __shfl_sync(0xffffffffu, (uint32_t)v, src);
  uint32_t hi = __shfl_sync(0xffffffffu, (uint32_t)(v >> 32), src);
  return ((uint64_t)hi << 32) | lo;
}

// ------------------------------------------------------------------------
// security-radius certificate (lists in ascending bisector distance)
// ------------------------------------------------------------------------
// Every vertex x of the cell satisfies x = K_xyz / K_w (K its cofactors), so
// |x - S| <= (|K_xyz - K_w S| + e) / (|K_w| - e_w) with e, e_w the cofactor
// error bounds (gamma_5 times the permanents M) and the rounding of the
// translation.  A neighbour j whose power bisector lies at distance d_j from
// the seed S cannot clip a cell inside the ball B(S, R): every point x of
// the ball has exact bisector value >= |n_j| (d_j - |x - S|) > 0, and the
// margin below covers the float rounding of the key d_j, of the float plane
// itself (<= 9uL + 4u|w_i - w_j| / |n_j| for coordinates below L), and of the
// predicate.  Keys ascend along the list, so one test of the next key
// certifies every remaining neighbour.
__device__ __forceinline__ float vertex_radius(float4 K, float4 M, float3 S) {
  const float g = 6.0f * 5.9604645e-08f;
  float ew = g * M.w;
  float aw = fabsf(K.w);
  if (!(aw > ew)) return INFINITY;
  float nx = __fmaf_rn(-K.w, S.x, K.x), ny = __fmaf_rn(-K.w, S.y, K.y),
        nz = __fmaf_rn(-K.w, S.z, K.z);
  float ex = g * (M.x + fabsf(S.x) * M.w) + 2.4e-7f * fabsf(nx);
  float ey = g * (M.y + fabsf(S.y) * M.w) + 2.4e-7f * fabsf(ny);
  float ez = g * (M.z + fabsf(S.z) * M.w) + 2.4e-7f * fabsf(nz);
  float ax = fabsf(nx) + ex, ay = fabsf(ny) + ey, az = fabsf(nz) + ez;
  float num = sqrtf(ax * ax + ay * ay + az * az) * (1.0f + 1e-6f);
  return num / (aw - ew) * (1.0f + 1e-6f);
}

// The same bound in FP64, for a vertex whose FP32 bound is loose or void
// (|K_w| close to its error: nearly parallel planes, as at the faces of
// sliver tets).  Products of two floats are exact in double and every 3x3
// minor rounds at most 3 times, so each cofactor is within 4 eps of its
// permanent (eps = 2^-53); the translation by S and the norm add a few eps.
__device__ __noinline__ float vertex_radius_d(float4 p1, float4 p2, float4 p3, float3 S) {
  const double x1 = p1.x, y1 = p1.y, z1 = p1.z, w1 = p1.w;
  const double x2 = p2.x, y2 = p2.y, z2 = p2.z, w2 = p2.w;
  const double x3 = p3.x, y3 = p3.y, z3 = p3.z, w3 = p3.w;
  // det3 of rows (a_i, b_i, c_i) and its permanent
  auto d3 = [](double a1, double b1, double c1, double a2, double b2, double c2, double a3,
               double b3, double c3, double& perm) {
    perm = fabs(a1) * (fabs(b2 * c3) + fabs(b3 * c2)) + fabs(b1) * (fabs(a2 * c3) + fabs(a3 * c2)) +
           fabs(c1) * (fabs(a2 * b3) + fabs(a3 * b2));
    return a1 * (b2 * c3 - b3 * c2) - b1 * (a2 * c3 - a3 * c2) + c1 * (a2 * b3 - a3 * b2);
  };
  double Mx, My, Mz, Mw;
  const double Kx = -d3(y1, z1, w1, y2, z2, w2, y3, z3, w3, Mx);
  const double Ky = d3(x1, z1, w1, x2, z2, w2, x3, z3, w3, My);
  const double Kz = -d3(x1, y1, w1, x2, y2, w2, x3, y3, w3, Mz);
  const double Kw = d3(x1, y1, z1, x2, y2, z2, x3, y3, z3, Mw);
  const double eps = 1.1102230246251565e-16;
  const double ew = 4.0 * eps * Mw;
  const double aw = fabs(Kw);
  if (!(aw > 2.0 * ew)) return INFINITY;
  const double sx = S.x, sy = S.y, sz = S.z;
  const double nx = Kx - Kw * sx, ny = Ky - Kw * sy, nz = Kz - Kw * sz;
  const double ex = 4.0 * eps * (Mx + fabs(sx) * Mw) + 2.0 * eps * fabs(nx);
  const double ey = 4.0 * eps * (My + fabs(sy) * Mw) + 2.0 * eps * fabs(ny);
  const double ez = 4.0 * eps * (Mz + fabs(sz) * Mw) + 2.0 * eps * fabs(nz);
  const double ax = fabs(nx) + ex, ay = fabs(ny) + ey, az = fabs(nz) + ez;
  const double r = sqrt(ax * ax + ay * ay + az * az) * (1.0 + 8.0 * eps) / (aw - ew);
  return __double2float_ru(r * (1.0 + 8.0 * eps));
}

// the radius bound of a vertex: FP32 where it is tight (its upper and lower
// bounds within 2^-10 of each other), else FP64 -- the FP32 cofactors of
// nearly parallel planes (the faces of sliver tets) cancel, and their error
// terms can exceed the distance itself
__device__ __forceinline__ float vertex_radius_p(float4 K, float4 M, float3 S, float4 p1,
                                                 float4 p2, float4 p3) {
  const float g = 6.0f * 5.9604645e-08f;
  const float ew = g * M.w, aw = fabsf(K.w);
  if (aw > 64.0f * ew) {
    const float nx = __fmaf_rn(-K.w, S.x, K.x), ny = __fmaf_rn(-K.w, S.y, K.y),
                nz = __fmaf_rn(-K.w, S.z, K.z);
    const float e = g * (M.x + M.y + M.z + (fabsf(S.x) + fabsf(S.y) + fabsf(S.z)) * M.w) +
                    2.4e-7f * (fabsf(nx) + fabsf(ny) + fabsf(nz));
    const float n = sqrtf(nx * nx + ny * ny + nz * nz);
    if (e < n * (1.0f / 2048.0f)) return vertex_radius(K, M, S);
  }
  return vertex_radius_d(p1, p2, p3, S);
}

// the cell radius: the largest of the vertices' cached bounds
__device__ __forceinline__ float cell_radius(const WarpCell& c, int nb_v, int lane) {
  float r = 0.f;
  for (int v = lane; v < nb_v; v += 32) r = fmaxf(r, c.u.f.rad[v]);
  for (int o = 16; o > 0; o >>= 1) r = fmaxf(r, __shfl_xor_sync(0xffffffffu, r, o));
  return r;
}

// the same bound from the planes alone (no cached cofactors: plain FP64
// clipping, which keeps none)
__device__ __forceinline__ float cell_radius_fresh(const WarpCell& c, int nb_v, int lane,
                                                   float3 S) {
  float r = 0.f;
  for (int v = lane; v < nb_v; v += 32) {
    const uchar4 t = c.ver[v];
    float4 K, M;
    vertex_cofactors(c.pl[t.x], c.pl[t.y], c.pl[t.z], K, M);
    r = fmaxf(r, vertex_radius(K, M, S));
  }
  for (int o = 16; o > 0; o >>= 1) r = fmaxf(r, __shfl_xor_sync(0xffffffffu, r, o));
  return r;
}

// recompute the filter cofactors (and with RAD the radius bounds about the
// seed S) of vertex slots [from, to)
template <bool RAD>
__device__ __forceinline__ void refresh_cofactors(WarpCell& c, int from, int to, int lane,
                                                  float3 S) {
  for (int v = from + lane; v < to; v += 32) {
    uchar4 t = c.ver[v];
    float4 K, M;
    vertex_cofactors(c.pl[t.x], c.pl[t.y], c.pl[t.z], K, M);
    c.u.f.K[v] = K;
    c.u.f.M[v] = M;
    if (RAD) c.u.f.rad[v] = vertex_radius(K, M, S);
  }
}

struct Cert {
  const float* keys;  // key of each list entry (CERT), ascending
  float3 S;           // seed
  float margin;       // absolute part of the certificate's margin
  bool lazy;          // test the certificate once, after the whole (short) list
  bool certified;
  int consumed;       // list entries taken before the certificate held
  float R;            // eager: the cell radius bound after the last clip
};

__device__ __forceinline__ bool cert_holds(float key, float R, float margin) {
  return key * (1.0f - 64.0f * 5.9604645e-08f) - margin > R;
}

// ------------------------------------------------------------------------
// one clip of the cell kernel, by the whole warp
// ------------------------------------------------------------------------
// The reference's update (convex_cell.cu:618-774) is sequential: the
// swap-to-tail partition of the conflicting vertices, the walk around the
// cavity, then one edge and one vertex per boundary plane.  The warp
// computes the same result:
//  * partition: the swap-to-tail loop is a fixed permutation of the
//    conflict bits.  With n vertices, C the conflicting slots, n' = n - |C|
//    and T the surviving slots in [n', n):
//      a slot v < n' outside C keeps its vertex;
//      the j-th slot of C below n' takes the j-th highest slot of T;
//      tail slot p >= n' takes the lowest slot of C if p = n - 1, the
//      vertex of slot p + 1 if that slot conflicts, and otherwise the
//      (rho + 1)-th lowest slot of C, rho the slots of T above p;
//    each lane gathers its slot (cells of up to 32 vertices; lane 0 runs
//    the loop itself for larger ones);
//  * boundary: the cavity of one removed vertex is its triangle; otherwise
//    lane 0 walks it (compute_boundary) and lists its planes in order;
//  * lane k makes edge k and vertex k along the boundary, with the vertex's
//    cofactors and radius bound, and the status is the one the sequential
//    loop stops with: the first vertex with a zero determinant needs
//    perturbation unless a triangle overflow comes strictly before it.

// position of the j-th (1-based) lowest set bit of m (m has at least j)
__device__ __forceinline__ int select_bit(uint32_t m, int j) {
  int pos = 0;
#pragma unroll
  for (int w = 16; w > 0; w >>= 1) {
    const int c = __popc(m & ((1u << w) - 1u));
    if (c < j) {
      j -= c;
      m >>= w;
      pos += w;
    }
  }
  return pos;
}

// the swap-to-tail partition run by one thread (cells of more than 32
// vertices); returns the survivors' count
template <bool COF, bool RAD>
__device__ __noinline__ int partition_serial(WarpCell& c, int nb_v, uint32_t m0, uint32_t m1,
                                             uint32_t m2) {
  int i = 0;
  while (i < nb_v) {
    const uint32_t wi = i < 32 ? m0 : (i < 64 ? m1 : m2);
    if ((wi >> (i & 31)) & 1u) {
      nb_v--;
      const uchar4 tv = c.ver[i];
      c.ver[i] = c.ver[nb_v];
      c.ver[nb_v] = tv;
      if (COF) {
        const float4 k = c.u.f.K[i];
        c.u.f.K[i] = c.u.f.K[nb_v];
        c.u.f.K[nb_v] = k;
        const float4 mm = c.u.f.M[i];
        c.u.f.M[i] = c.u.f.M[nb_v];
        c.u.f.M[nb_v] = mm;
      }
      if (RAD) {
        const float r = c.u.f.rad[i];
        c.u.f.rad[i] = c.u.f.rad[nb_v];
        c.u.f.rad[nb_v] = r;
      }
      const uint32_t wn = nb_v < 32 ? m0 : (nb_v < 64 ? m1 : m2);
      const uint32_t bit = 1u << (i & 31);
      const uint32_t nw = ((wn >> (nb_v & 31)) & 1u) ? (wi | bit) : (wi & ~bit);
      if (i < 32) m0 = nw;
      else if (i < 64) m1 = nw;
      else m2 = nw;
    } else {
      i++;
    }
  }
  return nb_v;
}

// Adds plane e with id2 `id` as plane s.nb_p and clips the cell by it; the
// conflicting vertex slots are in mask[3] (warp-uniform).  All lanes.
template <bool COF, bool RAD>
__device__ __forceinline__ void clip_full(WarpCell& c, CellState& s, const uint32_t* mask,
                                          float4 e, int2 id, int lane, float3 S) {
  const int cur = s.nb_p;
  if (lane == 0) {
    c.pl[cur] = e;
    c.h[cur] = 1;
    c.id2[cur] = id;
  }
  s.nb_p = cur + 1;
  const int n = s.nb_v;
  int n2;
  if (n <= 32) {
    const uint32_t valid = n == 32 ? ~0u : ((1u << n) - 1u);
    const uint32_t C = mask[0] & valid;
    n2 = n - __popc(C);  // at most n - 1: the plane conflicts somewhere
    const uint32_t low = (1u << n2) - 1u;
    const uint32_t T = ~C & valid & ~low;
    const int v = lane;
    int src = v;
    if (v < n2) {
      if ((C >> v) & 1u) {
        const int j = __popc(C & ((1u << v) - 1u)) + 1;
        src = select_bit(T, __popc(T) - j + 1);
      }
    } else if (v == n - 1) {
      src = __ffs(C) - 1;
    } else if (v < n) {
      if ((C >> (v + 1)) & 1u) src = v + 1;
      else src = select_bit(C, __popc(T >> (v + 1)) + 1);
    }
    const bool move = v < n && src != v;
    uchar4 t;
    float4 K, M;
    float rd = 0.f;
    if (move) {
      t = c.ver[src];
      if (COF && v < n2) {
        K = c.u.f.K[src];
        M = c.u.f.M[src];
        if (RAD) rd = c.u.f.rad[src];
      }
    }
    __syncwarp();
    if (move) {
      c.ver[v] = t;
      if (COF && v < n2) {
        c.u.f.K[v] = K;
        c.u.f.M[v] = M;
        if (RAD) c.u.f.rad[v] = rd;
      }
    }
  } else {
    if (lane == 0) n2 = partition_serial<COF, RAD>(c, n, mask[0], mask[1], mask[2]);
    n2 = __shfl_sync(0xffffffffu, n2, 0);
  }
  __syncwarp();
  s.nb_v = n2;
  s.kept = n2;
  if (n2 == 0) {
    s.status = kNoIntersection;
    return;
  }
  const int nb_r = n - n2;
  int len = 3;
  uchar4 tr = make_uchar4(0, 0, 0, 0);
  if (nb_r == 1) {
    // the cavity is the removed vertex's triangle, its planes in order
    tr = c.ver[n2];
  } else {
    if (lane < kMaxP / 4) reinterpret_cast<uint32_t*>(c.bnext)[lane] = 0xffffffffu;
    __syncwarp();
    int st = s.status, L = 0;
    if (lane == 0) {
      int first, r = nb_r;
      compute_boundary(c, n2, r, first, st);
      if (st == kSuccess && first != kEnd) {
        // the boundary holds at most nb_p - 1 planes
        int cir = first;
        do {
          c.perm[L++] = (uint8_t)cir;
          cir = c.bnext[cir];
        } while (cir != first && L < kMaxP);
        if (cir != first) st = kInconsistentBoundary;
      }
    }
    st = __shfl_sync(0xffffffffu, st, 0);
    len = __shfl_sync(0xffffffffu, L, 0);
    s.status = st;
    if (st != kSuccess || len == 0) return;
  }
  __syncwarp();  // tr and the boundary are read before new vertices land
  if (s.nb_e + len > kMaxE) {
    s.status = kEdgeOverflow;
    return;
  }
  const uint8_t hcur = c.h[cur];
  const int nb_e = s.nb_e;
  int zero_k = kMaxP;  // first boundary vertex whose three planes are dependent
  for (int k = lane; k < len; k += 32) {
    int cir, nx;
    if (nb_r == 1) {
      cir = k == 0 ? tr.x : (k == 1 ? tr.y : tr.z);
      nx = k == 0 ? tr.y : (k == 1 ? tr.z : tr.x);
    } else {
      cir = c.perm[k];
      nx = c.perm[k + 1 == len ? 0 : k + 1];
    }
    const float4 pcir = c.pl[cir], pnx = c.pl[nx];
    const uint8_t hcir = c.h[cir], hnx = c.h[nx];
    // cur > cir: the new plane has the largest index
    c.edge[nb_e + k] = make_uchar4((uint8_t)cir, (uint8_t)cur, hcur > hcir ? hcur : hcir, 0);
    // the largest count of the vertex's three edges.  The reference looks
    // each edge up in the cell's edge list (find_edge_id,
    // convex_cell.cu:511-522); an edge's count is fixed when it is made: the
    // tet's own count for the six initial edges (convex_cell.cu:193-211),
    // max(h_a, h_b) for every edge made by new_edge (:604-616), and two
    // existing planes never become adjacent later
    uint8_t adj = hcur > hcir ? hcur : hcir;
    if (hnx > adj) adj = hnx;
    if (cir < 4 && nx < 4) {
      const uint8_t te = c.edge[cTetEdgeSlot[cir][nx]].z;
      if (te > adj) adj = te;
    }
    const int slot = n2 + k;
    if (slot + 1 < kMaxT) {
      c.ver[slot] = make_uchar4((uint8_t)cur, (uint8_t)cir, (uint8_t)nx, adj);
      if (COF) {
        float4 K, M;
        vertex_cofactors(e, pcir, pnx, K, M);
        c.u.f.K[slot] = K;
        c.u.f.M[slot] = M;
        if (RAD) c.u.f.rad[slot] = vertex_radius(K, M, S);
      }
    }
    if (det3x3_f(e, pcir, pnx) == 0.f && k < zero_k) zero_k = k;
  }
  for (int o = 16; o > 0; o >>= 1) zero_k = min(zero_k, __shfl_xor_sync(0xffffffffu, zero_k, o));
  const int k_of = max(kMaxT - 1 - n2, 0);  // first vertex that would overflow
  if (zero_k < len && zero_k <= k_of) s.status = kNeedsPerturb;
  else if (k_of < len) s.status = kTriangleOverflow;
  s.nb_e = nb_e + len;
  s.nb_v = n2 + len;
}

// ------------------------------------------------------------------------
// the neighbour loop shared by the cell kernel and the box kernel
// ------------------------------------------------------------------------
// make_plane(j) builds the plane of list entry j (bisector, or offset
// bisector for the box kernel).  With CERT the list is in ascending key
// order and clipping stops as soon as the certificate holds.
template <int PRED, bool FULL, bool CERT, class MakePlane>
__device__ void clip_list(WarpCell& c, CellState& s, const int32_t* list, int k,
                          int seed_id, MakePlane make_plane, int lane,
                          PredCount& pc, Cert& cert) {
  constexpr bool kCof = uses_filter(PRED) || CERT;
  const bool eager = CERT && !cert.lazy;
  float R = INFINITY;
  if (eager) R = cell_radius(c, s.nb_v, lane);
  cert.consumed = k;
  for (int base = 0; base < k && s.status == kSuccess; base += 32) {
    int j = (base + lane < k) ? __ldg(list + base + lane) : -1;
    uint32_t valid = __ballot_sync(0xffffffffu, j != -1);
    int count = (~valid == 0u) ? 32 : (__ffs(~valid) - 1);  // up to first -1
    float key_mine = 0.f;
    if (eager && lane < count) key_mine = __ldg(cert.keys + base + lane);
    // the lane's plane goes to shared memory (the tests read it from there;
    // no register holds it through the chunk), with the planes already in
    // the cell that equal it
    uint64_t dup_mine = 0;
    {
      float4 e_mine = make_float4(0.f, 0.f, 0.f, 0.f);
      if (lane < count) e_mine = make_plane(j);
      __syncwarp();  // the previous chunk's planes are no longer read
      c.cand[lane] = e_mine;
      for (int p = 0; p < s.nb_p; ++p)
        if (plane_eq(e_mine, c.pl[p])) dup_mine |= 1ull << p;
    }
    __syncwarp();
    bool any_dup = __any_sync(0xffffffffu, dup_mine != 0ull);
    int r = 0;
    while (r < count) {
      if (eager) {
        float kr = __shfl_sync(0xffffffffu, key_mine, r);
        if (cert_holds(kr, R, cert.margin)) {
          cert.certified = true;
          cert.consumed = base + r;
          return;
        }
      }
      if (s.nb_p >= kMaxP) {  // new_plane fails before any evaluation
        s.status = kVertexOverflow;
        break;
      }
      uint32_t mask[3] = {0u, 0u, 0u};
      int hit = -1;
      if (s.nb_v <= 32) {
        int lgV = s.nb_v <= 4 ? 2 : (s.nb_v <= 8 ? 3 : (s.nb_v <= 16 ? 4 : 5));
        int V = 1 << lgV;
        int pi = lane >> lgV, vi = lane & (V - 1);
        int pidx = r + pi;
        const float4 e = c.cand[pidx & 31];
        uint64_t dup = any_dup ? shfl64(dup_mine, pidx & 31) : 0ull;
        bool cf = false;
        if (pidx < count && vi < s.nb_v) cf = in_conflict<PRED>(c, vi, e, dup, pc);
        uint32_t m = __ballot_sync(0xffffffffu, cf);
        if (m == 0u) {
          r += 32 >> lgV;
          continue;
        }
        int pf = (__ffs(m) - 1) >> lgV;
        mask[0] = (V == 32) ? m : ((m >> (pf << lgV)) & ((1u << V) - 1u));
        hit = r + pf;
      } else {
        const float4 e = c.cand[r];
        uint64_t dup = any_dup ? shfl64(dup_mine, r) : 0ull;
        bool any = false;
        for (int w = 0; w < 3; ++w) {
          int vi = lane + 32 * w;
          bool cf = false;
          if (vi < s.nb_v) cf = in_conflict<PRED>(c, vi, e, dup, pc);
          mask[w] = __ballot_sync(0xffffffffu, cf);
          any |= mask[w] != 0u;
        }
        if (!any) {
          r += 1;
          continue;
        }
        hit = r;
      }
      // the plane of list entry `hit` clips: write it and update topology
      const float4 e = c.cand[hit];
      int jn = __shfl_sync(0xffffffffu, j, hit);
      if (FULL) {
        clip_full<kCof, CERT>(c, s, mask, e,
                              make_int2(seed_id < jn ? seed_id : jn, seed_id < jn ? jn : seed_id),
                              lane, cert.S);
        __syncwarp();
        if (eager && s.status == kSuccess) R = cell_radius(c, s.nb_v, lane);
        if (plane_eq(c.cand[lane], e)) dup_mine |= 1ull << (s.nb_p - 1);
        any_dup = __any_sync(0xffffffffu, dup_mine != 0ull);
        if (s.status != kSuccess) break;
        r = hit + 1;
        continue;
      }
      if (lane < kMaxP / 4) reinterpret_cast<uint32_t*>(c.bnext)[lane] = 0xffffffffu;
      if (kCof && !FULL)
        for (int v = lane; v < s.nb_v; v += 32) c.perm[v] = (uint8_t)v;
      __syncwarp();
      if (lane == 0) {
        const int cur = s.nb_p;
        c.pl[cur] = e;
        c.h[cur] = 1;
        c.id2[cur] = make_int2(seed_id < jn ? seed_id : jn, seed_id < jn ? jn : seed_id);
        apply_clip_box(c, s, mask);
      }
      __syncwarp();
      broadcast_state(s);
      // the surviving vertices' cofactors follow their dual triangles: a
      // survivor moved into slot v < kept came from a slot >= kept (the
      // partition only swaps with its shrinking end), so sources and
      // targets never overlap
      if (kCof && !FULL && s.status == kSuccess) {
        for (int v = lane; v < s.kept; v += 32) {
          const int src = c.perm[v];
          if (src != v) {
            c.u.f.K[v] = c.u.f.K[src];
            c.u.f.M[v] = c.u.f.M[src];
            if (CERT) c.u.f.rad[v] = c.u.f.rad[src];
          }
        }
        __syncwarp();
      }
      // the vertices created by this clip are exactly those whose first
      // plane is the new one; the surviving ones kept their cofactors
      if (kCof && s.status == kSuccess) {
        const int cur = s.nb_p - 1;
        for (int v = lane; v < s.nb_v; v += 32) {
          uchar4 t = c.ver[v];
          if (t.x == cur) {
            float4 K, M;
            vertex_cofactors(c.pl[t.x], c.pl[t.y], c.pl[t.z], K, M);
            c.u.f.K[v] = K;
            c.u.f.M[v] = M;
            if (CERT) c.u.f.rad[v] = vertex_radius(K, M, cert.S);
          }
        }
      }
      __syncwarp();
      if (eager && s.status == kSuccess) R = cell_radius(c, s.nb_v, lane);
      // later planes of this chunk identical to the new one
      if (plane_eq(c.cand[lane], e)) dup_mine |= 1ull << (s.nb_p - 1);
      any_dup = __any_sync(0xffffffffu, dup_mine != 0ull);
      if (s.status != kSuccess) break;
      r = hit + 1;
    }
    if (count < 32) {  // the list ended (-1) inside this chunk
      cert.consumed = base + count;
      break;
    }
  }
  cert.R = R;
}

// End of a cell's list without the certificate holding on the way (status
// success).  A shortened list (learned or per-site lengths) that ran out
// first: the cell is clipped again with its whole list
// (kSecurityRadiusNotReached marks it).  A whole list: the sites missing from
// it have keys >= its completeness bound, so one test against the bound can
// still certify the cell; otherwise such a site may cut it, and the cell is
// flagged, its radius recorded for a longer list.  Lists of all power
// neighbours, as libmat's triangulation gives, leave no such cells.  Out of
// line: it runs for a few cells, and keeps the hot loop's code small.
// pointers of the list metadata finish_list reads (by value: a noinline
// call must not take the address of the kernel's parameters or state)
struct ListMeta {
  const int32_t* nbr;
  const float* keys;
  const int32_t* site_row;
  const int32_t* ext_len;
  const float* ext_bound;
  const float* nbr_bound;
  unsigned long long* misses;
  int k;
};

// returns 1: flagged uncertified (recheck_cells_kernel takes it up), 2: a
// short list missed (re-clip whole), 0
template <bool CERT, bool EXT>
__device__ __forceinline__ int finish_list(const WarpCell& c, int nb_v, ListMeta m, int sid,
                                          int klen, bool lazy, float R_eager, float margin,
                                          int lane, float3 S) {
  int full;
  float bound;
  const int row = EXT ? __ldg(m.site_row + sid) : -1;
  if (row >= 0) {
    full = __ldg(m.ext_len + row);
    bound = __ldg(m.ext_bound + row);
  } else {
    full = m.k;
    bound = m.nbr_bound ? __ldg(m.nbr_bound + sid) : INFINITY;
  }
  // (only base lists are shortened)
  if (CERT && klen < full && __ldg(m.nbr + (long long)sid * m.k + klen) != -1) {
    bool ok = false;
    if (lazy) {
      // one certificate test after the whole short list
      float R = cell_radius(c, nb_v, lane);
      ok = cert_holds(__ldg(m.keys + (long long)sid * m.k + klen), R, margin);
    }
    if (ok) return 0;
    if (m.misses && lane == 0) atomicAdd(m.misses, 1ull);
    return 2;
  }
  if (klen != full || !(bound < INFINITY) || (!CERT && !m.nbr_bound)) return 0;
  // the FP32 radius bounds (cached, or from the planes): a cell they do not
  // certify is flagged, and recheck_cells_kernel bounds it again with FP64
  // where they are loose
  float R;
  if (CERT && !lazy) R = R_eager;
  else if (CERT) R = cell_radius(c, nb_v, lane);
  else R = cell_radius_fresh(c, nb_v, lane, S);
  return cert_holds(bound, R, margin) ? 0 : 1;
}

// ------------------------------------------------------------------------
// FP64-accurate reconstruction of the emitted cell
// ------------------------------------------------------------------------
// The float planes above decide the topology exactly as the reference does.
// The coordinates reported for the surviving vertices are rebuilt from the
// FP64 inputs instead: every plane is recomputed in the frame centred on the
// seed S, from double-float copies of the FP64 mesh vertices and sites
// (hi + lo, about 48 bits), and each vertex -- the intersection of its three
// planes, by Cramer's rule as in compute_vertex_coordinates
// (convex_cell.cu:319-351) -- is solved in double-float arithmetic on the
// FP32 pipe, then translated back by S and rounded to FP64 with one FP64
// add.  The cell volume uses the reference's per-vertex decomposition into
// six tets (convex_cell.cu:986-1069) in FP32, about a point of the cell
// (small coordinates, no cancellation against the scene's extent).

__device__ __forceinline__ df dmul3(df a, df b, df c) { return df_mul(df_mul(a, b), c); }

// 2x2 minor b_p c_q - b_q c_p
__device__ __forceinline__ df minor2(df bp, df bq, df cp, df cq) {
  return df_sub_s(df_mul(bp, cq), df_mul(bq, cp));
}

__device__ __forceinline__ float3 f3sub(float3 a, float3 b) {
  return make_float3(a.x - b.x, a.y - b.y, a.z - b.z);
}
__device__ __forceinline__ float f3dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float3 f3cross(float3 a, float3 b) {
  return make_float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float3 f3axpy(float a, float3 x, float3 y) {
  return make_float3(a * x.x + y.x, a * x.y + y.y, a * x.z + y.z);
}
__device__ __forceinline__ float det3f(float3 a, float3 b, float3 c) { return f3dot(a, f3cross(b, c)); }

// foot of the origin O = (0,0,0) on the plane n.x + d = 0
__device__ __forceinline__ float3 face_foot(float3 n, float d) {
  const float n2 = f3dot(n, n);
  const float lam = n2 > 0.f ? __fdividef(d, n2) : 0.f;
  return make_float3(-lam * n.x, -lam * n.y, -lam * n.z);
}

// signed volume of one vertex's six flag tets, origin O = (0,0,0): feet of
// O on the three faces (given) and on the three edge lines through A.  The
// volume is reported in FP32, so the quotients use the fast division.
__device__ float vertex_volume_f(float3 A, const float3* n, const float3* foot) {
  float3 P[6];
  for (int i = 0; i < 3; ++i) P[2 * i] = foot[i];
  for (int i = 0; i < 3; ++i) {
    float3 t = f3cross(n[i], n[(i + 1) % 3]);
    float t2 = f3dot(t, t);
    float lam = t2 > 0.f ? __fdividef(f3dot(t, A), t2) : 0.f;
    P[2 * i + 1] = f3axpy(-lam, t, A);
  }
  float3 mA = make_float3(-A.x, -A.y, -A.z);
  float v = 0.f;
  for (int i = 0; i < 6; ++i) v -= det3f(f3sub(P[i], A), f3sub(P[(i + 1) % 6], A), mA);
  return v * (1.0f / 6.0f);
}

// intersection of three float planes, double-float Cramer (box kernel):
// per coordinate a float interval [lo, hi] around the double-float value
__device__ void vertex_of_float_planes(float4 a4, float4 b4, float4 c4, float* lo, float* hi) {
  df ax = df_make(a4.x, 0.f), ay = df_make(a4.y, 0.f), az = df_make(a4.z, 0.f),
     aw = df_make(a4.w, 0.f);
  df bx = df_make(b4.x, 0.f), by = df_make(b4.y, 0.f), bz = df_make(b4.z, 0.f),
     bw = df_make(b4.w, 0.f);
  df cx = df_make(c4.x, 0.f), cy = df_make(c4.y, 0.f), cz = df_make(c4.z, 0.f),
     cw = df_make(c4.w, 0.f);
  df mxy = minor2(bx, by, cx, cy), mxz = minor2(bx, bz, cx, cz), mxw = minor2(bx, bw, cx, cw);
  df myz = minor2(by, bz, cy, cz), myw = minor2(by, bw, cy, cw), mzw = minor2(bz, bw, cz, cw);
  df Dw = df_add_s(df_sub_s(df_mul(ax, myz), df_mul(ay, mxz)), df_mul(az, mxy));
  df Dx = df_add_s(df_sub_s(df_mul(ay, mzw), df_mul(az, myw)), df_mul(aw, myz));
  df Dy = df_add_s(df_sub_s(df_mul(ax, mzw), df_mul(az, mxw)), df_mul(aw, mxz));
  df Dz = df_add_s(df_sub_s(df_mul(ax, myw), df_mul(ay, mxw)), df_mul(aw, mxy));
  const df inv = df_recip(Dw);
  const df X[3] = {df_neg(df_mul(Dx, inv)), df_mul(Dy, inv), df_neg(df_mul(Dz, inv))};
  for (int k = 0; k < 3; ++k) {
    lo[k] = __fadd_rd(X[k].hi, X[k].lo);
    hi[k] = __fadd_ru(X[k].hi, X[k].lo);
  }
}

// vertex (X, Y, Z) of the three seed-frame double-float planes pa, pb, pc
template <class Cell>
__device__ __forceinline__ void cell_vertex(const Cell& c, int pa, int pb, int pc, df& X,
                                            df& Y, df& Z) {
  df ax = c.u.g.n[pa][0], ay = c.u.g.n[pa][1], az = c.u.g.n[pa][2], aw = c.u.g.d[pa];
  df bx = c.u.g.n[pb][0], by = c.u.g.n[pb][1], bz = c.u.g.n[pb][2], bw = c.u.g.d[pb];
  df cx = c.u.g.n[pc][0], cy = c.u.g.n[pc][1], cz = c.u.g.n[pc][2], cw = c.u.g.d[pc];
  df mxy = minor2(bx, by, cx, cy), mxz = minor2(bx, bz, cx, cz), mxw = minor2(bx, bw, cx, cw);
  df myz = minor2(by, bz, cy, cz), myw = minor2(by, bw, cy, cw), mzw = minor2(bz, bw, cz, cw);
  df Dw = df_add_s(df_sub_s(df_mul(ax, myz), df_mul(ay, mxz)), df_mul(az, mxy));
  df Dx = df_add_s(df_sub_s(df_mul(ay, mzw), df_mul(az, myw)), df_mul(aw, myz));
  df Dy = df_add_s(df_sub_s(df_mul(ax, mzw), df_mul(az, mxw)), df_mul(aw, mxz));
  df Dz = df_add_s(df_sub_s(df_mul(ax, myw), df_mul(ay, mxw)), df_mul(aw, mxy));
  df inv = df_recip(Dw);
  X = df_neg(df_mul(Dx, inv));
  Y = df_mul(Dy, inv);
  Z = df_neg(df_mul(Dz, inv));
}

template <class Cell>
__device__ __forceinline__ float vertex_volume_about(const Cell& c, uchar4 tr, df X, df Y,
                                                     df Z, float3 O) {
  float3 A = make_float3(df_sub_s(X, df_make(O.x, 0.f)).hi, df_sub_s(Y, df_make(O.y, 0.f)).hi,
                         df_sub_s(Z, df_make(O.z, 0.f)).hi);
  const int pl[3] = {tr.x, tr.y, tr.z};
  float3 nn[3], ft[3];
  for (int k = 0; k < 3; ++k) {
    nn[k] = make_float3(c.u.g.n[pl[k]][0].hi, c.u.g.n[pl[k]][1].hi, c.u.g.n[pl[k]][2].hi);
    ft[k] = c.u.g.foot[pl[k]];
  }
  return vertex_volume_f(A, nn, ft);
}

__device__ __forceinline__ df ldf(const float2* p) {
  const float2 v = __ldg(p);
  return df_make(v.x, v.y);
}

// exact float -> double widening with integer operations (IEEE-754 binary32
// to binary64: same sign, exponent re-biased by 1023 - 127, fraction shifted
// by 29 bits); zeros, subnormals, infinities and NaNs take the conversion
// instruction
__device__ __forceinline__ double widen(float f) {
  const uint32_t u = __float_as_uint(f);
  const uint32_t e = (u >> 23) & 0xffu;
  if (e == 0u || e == 0xffu) return (double)f;
  const uint64_t bits = ((uint64_t)(u >> 31) << 63) | ((uint64_t)(e + 896u) << 52) |
                        ((uint64_t)(u & 0x7fffffu) << 29);
  return __longlong_as_double((long long)bits);
}

// S + X (double-float) rounded to double: hi and lo widen exactly, one add
__device__ __forceinline__ double df_translate(df S, df X) {
  const df t = df_add_s(S, X);
  return widen(t.hi) + widen(t.lo);
}

// float intersection of three planes (Cramer); used only as the origin of
// the volume decomposition, so any point near the cell will do
template <class Cell>
__device__ float3 float_vertex(const Cell& c, uchar4 tr) {
  const int pl[3] = {tr.x, tr.y, tr.z};
  float a[3][4];
  for (int k = 0; k < 3; ++k) {
    a[k][0] = c.u.g.n[pl[k]][0].hi;
    a[k][1] = c.u.g.n[pl[k]][1].hi;
    a[k][2] = c.u.g.n[pl[k]][2].hi;
    a[k][3] = c.u.g.d[pl[k]].hi;
  }
  // n_k . x = -d_k
  const float3 n0 = make_float3(a[0][0], a[0][1], a[0][2]);
  const float3 n1 = make_float3(a[1][0], a[1][1], a[1][2]);
  const float3 n2 = make_float3(a[2][0], a[2][1], a[2][2]);
  const float3 c12 = f3cross(n1, n2), c20 = f3cross(n2, n0), c01 = f3cross(n0, n1);
  const float det = f3dot(n0, c12);
  const float s = -1.0f / det;
  float3 x = make_float3(s * (a[0][3] * c12.x + a[1][3] * c20.x + a[2][3] * c01.x),
                         s * (a[0][3] * c12.y + a[1][3] * c20.y + a[2][3] * c01.y),
                         s * (a[0][3] * c12.z + a[1][3] * c20.z + a[2][3] * c01.z));
  if (!(isfinite(x.x) && isfinite(x.y) && isfinite(x.z))) x = make_float3(0.f, 0.f, 0.f);
  return x;
}

// writes xyz[3 * nb_v] and returns the cell volume; c holds the cell's
// id2 and ver, c.u.g is filled here.  W lanes (a whole warp or a half) work
// on the cell; lane is 0..W-1.  Every lane of the warp calls this the same
// number of times (its __syncwarp and shuffles span the warp); a lane group
// with no cell passes active = false.
template <int W, class Cell>
__device__ double cell_geometry(Cell& c, bool active, int nb_v, int nb_p, const float2* face2,
                                const float2* site2, int tet, int sid, int lane, double* xyz) {
  df Sx = df_make(0.f, 0.f), Sy = Sx, Sz = Sx, Sw = Sx;
  if (active) {
    const float2* S2 = site2 + 4 * (long long)sid;
    Sx = ldf(S2);
    Sy = ldf(S2 + 1);
    Sz = ldf(S2 + 2);
    Sw = ldf(S2 + 3);
  } else {
    nb_v = nb_p = 0;
  }
  for (int i = lane; i < nb_p; i += W) {
    df nx, ny, nz, d;
    if (i < 4) {
      // the tet's face plane (FP64, once per mesh), moved to the seed frame:
      // d' = d + n . S
      const float2* f = face2 + 16 * (long long)tet + 4 * i;
      nx = ldf(f);
      ny = ldf(f + 1);
      nz = ldf(f + 2);
      d = df_add_s(ldf(f + 3), df_add_s(df_add_s(df_mul(nx, Sx), df_mul(ny, Sy)), df_mul(nz, Sz)));
    } else {
      const int2 id = c.id2[i];
      const int other = id.x == sid ? id.y : id.x;
      const float2* B = site2 + 4 * (long long)other;
      // bisector in the seed frame: n = S - B, d = (|n|^2 + wS - wB) / 2
      nx = df_sub_s(Sx, ldf(B));
      ny = df_sub_s(Sy, ldf(B + 1));
      nz = df_sub_s(Sz, ldf(B + 2));
      const df n2 = df_add_s(df_add_s(df_mul(nx, nx), df_mul(ny, ny)), df_mul(nz, nz));
      d = df_add_s(n2, df_sub_s(Sw, ldf(B + 3)));
      d = df_make(0.5f * d.hi, 0.5f * d.lo);
    }
    c.u.g.n[i][0] = nx;
    c.u.g.n[i][1] = ny;
    c.u.g.n[i][2] = nz;
    c.u.g.d[i] = d;
  }
  __syncwarp();
  // volume origin O near the cell (its vertex 0, in float): the
  // decomposition's terms then scale with the cell's own size
  const float3 O = active ? float_vertex(c, c.ver[0]) : make_float3(0.f, 0.f, 0.f);
  for (int i = lane; i < nb_p; i += W) {
    const df n0 = c.u.g.n[i][0], n1 = c.u.g.n[i][1], n2 = c.u.g.n[i][2];
    const df dc = df_add_s(c.u.g.d[i], df_add_s(df_add_s(df_mul(n0, df_make(O.x, 0.f)),
                                                   df_mul(n1, df_make(O.y, 0.f))),
                                            df_mul(n2, df_make(O.z, 0.f))));
    c.u.g.foot[i] = face_foot(make_float3(n0.hi, n1.hi, n2.hi), dc.hi);
  }
  __syncwarp();
  float vol = 0.f;
  for (int v = lane; v < nb_v; v += W) {
    const uchar4 tr = c.ver[v];
    df X, Y, Z;
    cell_vertex(c, tr.x, tr.y, tr.z, X, Y, Z);
    xyz[3 * v] = df_translate(Sx, X);
    xyz[3 * v + 1] = df_translate(Sy, Y);
    xyz[3 * v + 2] = df_translate(Sz, Z);
    vol += vertex_volume_about(c, tr, X, Y, Z, O);
  }
  for (int o = W / 2; o > 0; o >>= 1) vol += __shfl_xor_sync(0xffffffffu, vol, o);
  return (double)vol;
}

// canonical topology of a cell, independent of the clipping order: the sum
// over its vertices of a hash of the sorted face keys (clip_id2) of the
// vertex's three planes and its #adjacent cells (splitmix64 mixing, Steele,
// Lea and Flood, OOPSLA 2014).  Planes that clipped intermediate vertices and
// no longer bound the cell appear in no vertex, so they do not count.
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

__device__ __forceinline__ uint64_t face_key(int2 id) {
  return ((uint64_t)(uint32_t)id.x << 32) | (uint32_t)id.y;
}

template <int W, class Cell>
__device__ uint64_t cell_topology_hash(const Cell& c, int nb_v, int lane) {
  uint64_t h = 0;
  for (int v = lane; v < nb_v; v += W) {
    uchar4 t = c.ver[v];
    uint64_t a = face_key(c.id2[t.x]), b = face_key(c.id2[t.y]), d = face_key(c.id2[t.z]), x;
    if (a > b) { x = a; a = b; b = x; }
    if (b > d) { x = b; b = d; d = x; }
    if (a > b) { x = a; a = b; b = x; }
    uint64_t hv = mix64(a);
    hv = mix64(hv ^ b);
    hv = mix64(hv ^ d);
    hv = mix64(hv ^ (uint64_t)t.w);
    h += hv;
  }
  for (int o = W / 2; o > 0; o >>= 1) h += __shfl_xor_sync(0xffffffffu, h, o);
  return h;
}

// MINB > 0 caps registers so that MINB blocks of 128 threads fit on an SM
// (occupancy variants chosen by the autotuner)
// EXT: sites may have extended rows (the exact-lists rounds); the first
// pass, on base lists only, runs without that code
template <int PRED, bool CERT, int MINB, bool EXT>
__global__ void __launch_bounds__(MINB > 0 ? 128 : kClipMaxThreads, MINB > 0 ? MINB : 1)
    clip_cells_kernel(ClipParams p) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31;
  const int wid = threadIdx.x >> 5;
  WarpCell& c = reinterpret_cast<WarpCell*>(smem_raw)[wid];
  PredCount pc = {0u, 0u, p.exact_counters};
  unsigned int n_uncert = 0;  // lane-uniform

  for (;;) {
    long long q = 0;
    if (lane == 0) q = (long long)atomicAdd(p.work, 1ull);
    q = __shfl_sync(0xffffffffu, q, 0);
    if (q >= p.n_work) break;
    if (p.pair_index) q = __ldg(p.pair_index + q);
    const int t = __ldg(p.pair_tet + q);
    const int sid = __ldg(p.pair_site + q);
    const float4 seed = __ldg(p.site4f + sid);

    // ---- cell = tet (convex_cell.cu:116-214); the tet's float vertices and
    // vertex counts come packed per tet (one dependent load less)
    if (lane < 4) {
      const float4 q0 = __ldg(p.tet_xyz + 3ll * t), q1 = __ldg(p.tet_xyz + 3ll * t + 1),
                   q2 = __ldg(p.tet_xyz + 3ll * t + 2);
      const float3 t0 = make_float3(q0.x, q0.y, q0.z), t1 = make_float3(q0.w, q1.x, q1.y),
                   t2 = make_float3(q1.z, q1.w, q2.x), t3 = make_float3(q2.y, q2.z, q2.w);
      // face `lane` (cFaceLv): (2,1,3), (0,2,3), (1,0,3), (0,1,2), selected
      // without indexing a local array by lane
      const float3 fa = lane == 0 ? t2 : (lane == 1 ? t0 : (lane == 2 ? t1 : t0));
      const float3 fb = lane == 0 ? t1 : (lane == 1 ? t2 : (lane == 2 ? t0 : t1));
      const float3 fc = lane == 3 ? t2 : t3;
      c.pl[lane] = tri2plane_f(fa, fb, fc);
      c.h[lane] = (uint8_t)__ldg(p.f_adjs + 4 * t + lane);
      c.id2[lane] = make_int2(__ldg(p.f_ids + 4 * t + lane), -1);
    } else if (lane < 8) {
      int i = lane - 4;
      const uchar4 va = __ldg(p.tet_vadj + t);
      const uint8_t vi = i == 0 ? va.x : (i == 1 ? va.y : (i == 2 ? va.z : va.w));
      c.ver[i] = make_uchar4((uint8_t)cTetTri[i][0], (uint8_t)cTetTri[i][1],
                             (uint8_t)cTetTri[i][2], vi);
    } else if (lane < 14) {
      int e = lane - 8;
      c.edge[e] = make_uchar4((uint8_t)cEdgeFaces[e][0], (uint8_t)cEdgeFaces[e][1],
                              __ldg(p.e_adj6 + 6 * (long long)t + e), 0);
    }
    __syncwarp();
    CellState s;
    s.nb_v = 4;
    s.nb_p = 4;
    s.nb_e = 6;
    s.status = kSuccess;
    if (uses_filter(PRED) || CERT) {
      refresh_cofactors<CERT>(c, 0, 4, lane, make_float3(seed.x, seed.y, seed.z));
      __syncwarp();
    }

    // ---- clip by the site's neighbour list: its base row, or the extended
    // row it was given after an earlier pass left one of its cells
    // uncertified
    const float4* site4f = p.site4f;
    auto make_plane = [&](int j) { return bisector_f(seed, __ldg(site4f + j)); };
    const int32_t* list;
    const float* keys;
    int klen;
    bool complete = false;  // a row of every site (id order, no keys)
    {
      const int row = EXT ? __ldg(p.site_row + sid) : -1;
      if (row >= 0) {
        const long long off = __ldg(p.ext_off + row);
        list = p.ext_nbr + off;
        klen = __ldg(p.ext_len + row);
        complete = !(__ldg(p.ext_bound + row) < INFINITY);
        keys = (p.ext_keys && !complete) ? p.ext_keys + off : nullptr;
      } else {
        list = p.nbr + (long long)sid * p.k;
        keys = p.keys ? p.keys + (long long)sid * p.k : nullptr;
        klen = p.k;
        if (p.site_klen) klen = min(klen, __ldg(p.site_klen + sid));
        if (p.pair_klen) klen = min(klen, __ldg(p.pair_klen + q));
      }
    }
    Cert cert;
    cert.keys = CERT ? keys : nullptr;
    cert.S = make_float3(seed.x, seed.y, seed.z);
    cert.margin = p.cert_margin;
    cert.lazy = p.lazy_cert != 0 || complete;
    cert.certified = false;
    clip_list<PRED, true, CERT>(c, s, list, klen, sid, make_plane, lane, pc, cert);
    bool uncert = false;
    if (s.status == kSuccess && !cert.certified) {
      ListMeta m;
      m.nbr = p.nbr;
      m.keys = p.keys;
      m.site_row = p.site_row;
      m.ext_len = p.ext_len;
      m.ext_bound = p.ext_bound;
      m.nbr_bound = p.nbr_bound;
      m.misses = p.misses;
      m.k = p.k;
      const int r = finish_list<CERT, EXT>(c, s.nb_v, m, sid, klen, cert.lazy, cert.R, cert.margin,
                                      lane, make_float3(seed.x, seed.y, seed.z));
      uncert = r == 1;
      if (r == 2) s.status = kSecurityRadiusNotReached;
    }
    if (p.consumed && lane == 0) p.consumed[q] = cert.consumed;
    n_uncert += uncert ? 1u : 0u;

    // ---- emit
    rpd_cell_header hd;
    hd.tet_id = t;
    hd.site_id = sid;
    hd.status = s.status;
    hd.nb_v = hd.nb_p = hd.nb_e = 0;
    hd.flags = uncert ? RPD_CELL_UNCERTIFIED : 0;
    hd.offset = 0;
    hd.volume = 0.0;
    if (s.status == kSuccess) {
      PayloadLayout L(s.nb_v, s.nb_p, s.nb_e);
      unsigned long long off = 0;
      if (lane == 0) off = atomicAdd(p.payload_cursor, (unsigned long long)L.total);
      off = __shfl_sync(0xffffffffu, off, 0);
      if (off + L.total > p.payload_cap) {
        hd.status = kPayloadFull;
      } else {
        uint8_t* dst = p.payload + off;
        for (int i = lane; i < s.nb_p; i += 32) {
          reinterpret_cast<float4*>(dst + L.plane)[i] = c.pl[i];
          reinterpret_cast<int2*>(dst + L.id2)[i] = c.id2[i];
        }
        for (int i = lane; i < s.nb_v; i += 32)
          reinterpret_cast<uchar4*>(dst + L.ver)[i] = c.ver[i];
        for (int i = lane; i < s.nb_e; i += 32)
          reinterpret_cast<uchar4*>(dst + L.edge)[i] = c.edge[i];
        for (int i = lane; i < (int)al16(s.nb_p); i += 32)
          dst[L.h + i] = i < s.nb_p ? c.h[i] : 0;
        // pad bytes of the id2 / ver / edge sections
        for (int i = 2 * s.nb_p + lane; i < (int)(al16(8u * s.nb_p) / 4); i += 32)
          reinterpret_cast<int32_t*>(dst + L.id2)[i] = 0;
        for (int i = s.nb_v + lane; i < (int)(al16(4u * s.nb_v) / 4); i += 32)
          reinterpret_cast<uint32_t*>(dst + L.ver)[i] = 0u;
        for (int i = s.nb_e + lane; i < (int)(al16(4u * s.nb_e) / 4); i += 32)
          reinterpret_cast<uint32_t*>(dst + L.edge)[i] = 0u;
        // coordinates, volume and topology hash: cell_epilogue_kernel
        hd.nb_v = (uint8_t)s.nb_v;
        hd.nb_p = (uint8_t)s.nb_p;
        hd.nb_e = (uint8_t)s.nb_e;
        hd.offset = off;
      }
    }
    if (lane == 0) p.headers[q] = hd;
    __syncwarp();
  }
  // statistics
  for (int o = 16; o > 0; o >>= 1) {
    pc.pred += __shfl_xor_sync(0xffffffffu, pc.pred, o);
    pc.esc += __shfl_xor_sync(0xffffffffu, pc.esc, o);
  }
  if (lane == 0) {
    atomicAdd(p.counters + 0, (unsigned long long)pc.pred);
    atomicAdd(p.counters + 1, (unsigned long long)pc.esc);
    if (n_uncert && p.uncertified) atomicAdd(p.uncertified, (unsigned long long)n_uncert);
  }
}

// ------------------------------------------------------------------------
// recheck of the cells flagged uncertified: the radius bound again, from
// the emitted record's planes, FP64 for the vertices whose FP32 bound is
// loose; a cell it certifies loses the flag, the others give their site's
// longer list its length (site_need, the largest radius of the site's
// flagged cells)
// ------------------------------------------------------------------------
__global__ void __launch_bounds__(128) recheck_cells_kernel(RecheckParams p) {
  const int lane = threadIdx.x & 31;
  const long long n_warps = ((long long)gridDim.x * blockDim.x) >> 5;
  const long long n = *p.n_dev;
  for (long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < n;
       w += n_warps) {
    const long long q = __ldg(p.idx + w);
    rpd_cell_header h = p.headers[q];
    const int sid = h.site_id;
    const float4 seed = __ldg(p.site4f + sid);
    const float3 S = make_float3(seed.x, seed.y, seed.z);
    const int row = p.site_row ? __ldg(p.site_row + sid) : -1;
    const float bound = row >= 0 ? __ldg(p.ext_bound + row) : __ldg(p.nbr_bound + sid);
    const PayloadLayout L(h.nb_v, h.nb_p, h.nb_e);
    const float4* pl = reinterpret_cast<const float4*>(p.payload + h.offset + L.plane);
    const uchar4* ver = reinterpret_cast<const uchar4*>(p.payload + h.offset + L.ver);
    float r = 0.f;
    for (int v = lane; v < h.nb_v; v += 32) {
      const uchar4 t = ver[v];
      const float4 a = pl[t.x], b = pl[t.y], d = pl[t.z];
      float4 K, M;
      vertex_cofactors(a, b, d, K, M);
      r = fmaxf(r, vertex_radius_p(K, M, S, a, b, d));
    }
    for (int o = 16; o > 0; o >>= 1) r = fmaxf(r, __shfl_xor_sync(0xffffffffu, r, o));
    if (lane == 0) {
      // a complete list (bound infinite) certifies any cell
      if (!(bound < INFINITY) || cert_holds(bound, r, p.margin)) {
        p.headers[q].flags = (uint8_t)(h.flags & ~RPD_CELL_UNCERTIFIED);
      } else {
        if (p.site_need) atomicMax(p.site_need + sid, __float_as_uint(r));
        if (p.kept_idx) p.kept_idx[atomicAdd(p.kept_count, 1ull)] = (int32_t)q;
      }
    }
  }
}

cudaError_t launch_recheck_cells(const RecheckParams& p, int num_sms, cudaStream_t st) {
  recheck_cells_kernel<<<(unsigned)(num_sms * 16), 128, 0, st>>>(p);
  note_launches(1);
  return cudaGetLastError();
}

// ------------------------------------------------------------------------
// epilogue: FP64-accurate coordinates and volume, canonical topology hash,
// of every emitted cell, from its record (plane ids and dual triangles)
// ------------------------------------------------------------------------
// The clip kernel leaves these to a separate pass: it keeps the clip
// kernel's code (and its instruction-cache footprint) to the topology
// update, and every warp here runs the same short program.  The first four
// planes of every record are the tet's faces, in order; the others are
// bisectors with the site pair in id2.
struct GeomCell {
  struct {
    struct {
      df n[kMaxP][3];
      df d[kMaxP];
      float3 foot[kMaxP];
    } g;
  } u;
  int2 id2[kMaxP];
  uchar4 ver[kMaxT];
};

constexpr int kEpiWarps = 4;

// two cells per warp, one per half-warp: most cells have fewer than 16
// planes and few more vertices, so 16 lanes keep busier than 32
__global__ void __launch_bounds__(kEpiWarps * 32) cell_epilogue_kernel(EpilogueParams p) {
  __shared__ GeomCell cells[2 * kEpiWarps];
  const int lane = threadIdx.x & 31;
  const int half = lane >> 4, hl = lane & 15;
  GeomCell& c = cells[2 * (threadIdx.x >> 5) + half];
  const long long n_warps = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long base = (((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 2;
       base < p.n_pairs; base += 2 * n_warps) {
    const long long q = base + half;
    rpd_cell_header hd;
    bool active = false;
    if (q < p.n_pairs) {
      hd = p.headers[q];
      active = hd.status == kSuccess;
      if (!active && p.topo_hash && hl == 0) p.topo_hash[q] = 0ull;
    }
    const int nb_v = active ? hd.nb_v : 0, nb_p = active ? hd.nb_p : 0;
    uint8_t* rec = nullptr;
    PayloadLayout L(nb_v, nb_p, active ? hd.nb_e : 0);
    if (active) {
      rec = p.payload + hd.offset;
      for (int i = hl; i < nb_p; i += 16) c.id2[i] = reinterpret_cast<const int2*>(rec + L.id2)[i];
      for (int i = hl; i < nb_v; i += 16) c.ver[i] = reinterpret_cast<const uchar4*>(rec + L.ver)[i];
    }
    __syncwarp();
    double* xyz = active ? reinterpret_cast<double*>(rec + L.xyz) : nullptr;
    double vol = 0.0;
    if (p.geometry) {
      vol = cell_geometry<16>(c, active, nb_v, nb_p, p.face2, p.site2, active ? hd.tet_id : 0,
                              active ? hd.site_id : 0, hl, xyz);
    } else if (active) {
      for (int i = hl; i < 3 * nb_v; i += 16) xyz[i] = 0.0;
    }
    uint64_t th = 0;
    if (p.topo_hash) th = cell_topology_hash<16>(c, nb_v, hl);
    if (active && hl == 0) {
      p.headers[q].volume = vol;
      if (p.topo_hash) p.topo_hash[q] = th;
    }
    __syncwarp();
  }
}

cudaError_t launch_cell_epilogue(const EpilogueParams& p, int num_sms, cudaStream_t st) {
  if (p.n_pairs <= 0) return cudaSuccess;
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, cell_epilogue_kernel, kEpiWarps * 32, 0);
  if (per_sm < 1) per_sm = 1;
  const long long want = (p.n_pairs + 2 * kEpiWarps - 1) / (2 * kEpiWarps);
  long long blocks = (long long)num_sms * per_sm * 4;
  if (blocks > want) blocks = want;
  cell_epilogue_kernel<<<(unsigned)blocks, kEpiWarps * 32, 0, st>>>(p);
  note_launches(1);
  return cudaGetLastError();
}

// face planes of every tet in FP64 (inward normals as tri2plane,
// common_cuda.h:248-254: n = (b - a) x (e - a), d = -a . n), stored as
// double-float (nx, ny, nz, d) per face
__global__ void tet_face_planes_kernel(const double* vert, const int4* tets, int n_tet, float2* out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_tet) return;
  const int4 q = tets[t];
  const int id[4] = {q.x, q.y, q.z, q.w};
  for (int i = 0; i < 4; ++i) {
    const double* a = vert + 3 * (long long)id[cFaceLv[i][0]];
    const double* b = vert + 3 * (long long)id[cFaceLv[i][1]];
    const double* e = vert + 3 * (long long)id[cFaceLv[i][2]];
    const double ux = b[0] - a[0], uy = b[1] - a[1], uz = b[2] - a[2];
    const double vx = e[0] - a[0], vy = e[1] - a[1], vz = e[2] - a[2];
    const double nx = uy * vz - uz * vy, ny = uz * vx - ux * vz, nz = ux * vy - uy * vx;
    const double d = -(a[0] * nx + a[1] * ny + a[2] * nz);
    const double v[4] = {nx, ny, nz, d};
    for (int k = 0; k < 4; ++k) {
      const df x = df_from_double(v[k]);
      out[16ll * t + 4 * i + k] = make_float2(x.hi, x.lo);
    }
  }
}

cudaError_t launch_tet_face_planes(const double* vert3d, const int4* tets, int n_tet, float2* out,
                                   cudaStream_t st) {
  if (n_tet <= 0) return cudaSuccess;
  tet_face_planes_kernel<<<(n_tet + 255) / 256, 256, 0, st>>>(vert3d, tets, n_tet, out);
  note_launches(1);
  return cudaGetLastError();
}

// ------------------------------------------------------------------------
// box kernel: bounding box of a site's cell grown by an offset, used to
// enumerate candidate tets (see rpd_pairs.cu)
// ------------------------------------------------------------------------
__global__ void __launch_bounds__(128, 6) site_box_kernel(BoxParams p) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31;
  const int wid = threadIdx.x >> 5;
  WarpCell& c = reinterpret_cast<WarpCell*>(smem_raw)[wid];
  PredCount pc = {0u, 0u, nullptr};
  const int warps_total = (gridDim.x * blockDim.x) >> 5;
  for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < p.n_site; i += warps_total) {
    float lo[3] = {p.box_lo.x, p.box_lo.y, p.box_lo.z};
    float hi[3] = {p.box_hi.x, p.box_hi.y, p.box_hi.z};
    if (p.flags[p.site_base + i] != 1u) {
      if (lane == 0) {
        p.site_box[2 * i] = make_float4(1.f, 1.f, 1.f, 0.f);  // empty box
        p.site_box[2 * i + 1] = make_float4(0.f, 0.f, 0.f, 0.f);
        p.site_nplanes[i] = 0;
      }
      continue;
    }
    const float4 seed = p.site4f[p.site_base + i];
    // box planes x>=lo, x<=hi, y>=lo, y<=hi, z>=lo, z<=hi
    if (lane < 6) {
      int ax = lane >> 1;
      float4 pl = make_float4(0.f, 0.f, 0.f, 0.f);
      float* q = reinterpret_cast<float*>(&pl);
      if ((lane & 1) == 0) {
        q[ax] = 1.f;
        pl.w = -lo[ax];
      } else {
        q[ax] = -1.f;
        pl.w = hi[ax];
      }
      c.pl[lane] = pl;
    } else if (lane < 14) {
      // corner (sx, sy, sz): planes X = sx, Y = 2 + sy, Z = 4 + sz, ordered
      // (X, Z, Y) for even parity and (X, Y, Z) for odd parity: the eight
      // dual triangles are then consistently oriented with the same sign as
      // the tet's (det4x4 of the triangle's planes with (0,0,0,1) < 0), so
      // "det > 0" means "outside" for both
      int v = lane - 6;
      int sx = v & 1, sy = (v >> 1) & 1, sz = (v >> 2) & 1;
      uint8_t X = (uint8_t)sx, Y = (uint8_t)(2 + sy), Z = (uint8_t)(4 + sz);
      c.ver[v] = ((sx + sy + sz) & 1) == 0 ? make_uchar4(X, Z, Y, 0) : make_uchar4(X, Y, Z, 0);
    }
    __syncwarp();
    CellState s;
    s.nb_v = 8;
    s.nb_p = 6;
    s.nb_e = 0;
    s.status = kSuccess;
    refresh_cofactors<false>(c, 0, 8, lane, make_float3(0.f, 0.f, 0.f));
    __syncwarp();
    const float4* site4f = p.site4f;
    const float R = p.offset_r, E = p.offset_e;
    auto make_plane = [&](int j) {
      float4 b = __ldg(site4f + j);
      float4 e = bisector_f(seed, b);
      float D = sqrtf(e.x * e.x + e.y * e.y + e.z * e.z);
      // push the plane outwards by R plus the float error of the rule's
      // power distances (E / 2D) plus a relative slack
      float slack = 1e-5f * (fabsf(e.w) + D * p.coord_scale);
      float d = e.w + R * D + 0.5f * E + slack;
      if (!(D > 0.f) || !(d < 3.0e38f)) return make_float4(0.f, 0.f, 0.f, 1.f);  // no constraint
      return make_float4(e.x, e.y, e.z, d);
    };
    // any subset of the planes gives a superset polytope; the nearest k_box
    // bisectors bound the cell well and keep the box clip small
    Cert nocert;
    nocert.keys = nullptr;
    nocert.certified = false;
    clip_list<RPD_PRED_FP32_FILTER, false, false>(c, s, p.nbr + (long long)i * p.k, p.k_box,
                                                  p.site_base + i,
                                                  make_plane, lane, pc, nocert);
    float bl[3], bh[3];
    if (s.status == kSuccess) {
      bl[0] = bl[1] = bl[2] = 3.0e38f;
      bh[0] = bh[1] = bh[2] = -3.0e38f;
      for (int v = lane; v < s.nb_v; v += 32) {
        uchar4 tr = c.ver[v];
        float xl[3], xh[3];
        vertex_of_float_planes(c.pl[tr.x], c.pl[tr.y], c.pl[tr.z], xl, xh);
        for (int k = 0; k < 3; ++k) {
          if (!(xl[k] == xl[k]) || !(xh[k] == xh[k])) {  // degenerate vertex
            xl[k] = lo[k];
            xh[k] = hi[k];
          }
          bl[k] = fminf(bl[k], xl[k]);
          bh[k] = fmaxf(bh[k], xh[k]);
        }
      }
      for (int o = 16; o > 0; o >>= 1)
        for (int k = 0; k < 3; ++k) {
          bl[k] = fminf(bl[k], __shfl_xor_sync(0xffffffffu, bl[k], o));
          bh[k] = fmaxf(bh[k], __shfl_xor_sync(0xffffffffu, bh[k], o));
        }
      for (int k = 0; k < 3; ++k) {
        float m = 1e-3f * (bh[k] - bl[k]) + p.abs_margin;
        bl[k] = fmaxf(bl[k] - m, lo[k]);
        bh[k] = fminf(bh[k] + m, hi[k]);
      }
    } else if (s.status == kNoIntersection) {
      bl[0] = bl[1] = bl[2] = 1.f;
      bh[0] = bh[1] = bh[2] = 0.f;
    } else {
      for (int k = 0; k < 3; ++k) {
        bl[k] = lo[k];
        bh[k] = hi[k];
      }
    }
    if (lane == 0) {
      p.site_box[2 * i] = make_float4(bl[0], bl[1], bl[2], (float)s.status);
      p.site_box[2 * i + 1] = make_float4(bh[0], bh[1], bh[2], 0.f);
    }
    // the planes that bound the grown cell (referenced by a vertex): the pair
    // search tests grid cells and tet centroids against them
    int npl = 0;
    if (s.status == kSuccess) {
      unsigned long long m = 0ull;
      for (int v = lane; v < s.nb_v; v += 32) {
        uchar4 tr = c.ver[v];
        m |= (1ull << tr.x) | (1ull << tr.y) | (1ull << tr.z);
      }
      uint32_t lo = __reduce_or_sync(0xffffffffu, (uint32_t)m);
      uint32_t hi = __reduce_or_sync(0xffffffffu, (uint32_t)(m >> 32));
      unsigned long long act = ((unsigned long long)hi << 32) | lo;
      // any subset of them bounds a superset of the grown cell: beyond the
      // storage, the first kBoxPlanes are kept
      npl = min(__popcll(act), kBoxPlanes);
      for (int q = lane; q < s.nb_p; q += 32) {
        const int rank = __popcll(act & ((1ull << q) - 1ull));
        if (((act >> q) & 1ull) && rank < kBoxPlanes)
          p.site_planes[(long long)i * kBoxPlanes + rank] = c.pl[q];
      }
    }
    if (lane == 0) p.site_nplanes[i] = npl;
    __syncwarp();
  }
  for (int o = 16; o > 0; o >>= 1) {
    pc.pred += __shfl_xor_sync(0xffffffffu, pc.pred, o);
    pc.esc += __shfl_xor_sync(0xffffffffu, pc.esc, o);
  }
  if (lane == 0 && p.counters) {
    atomicAdd(p.counters + 0, (unsigned long long)pc.pred);
    atomicAdd(p.counters + 1, (unsigned long long)pc.esc);
  }
}

size_t clip_smem_per_warp() { return sizeof(WarpCell); }

template <int PRED, bool CERT, int MINB>
static int occ_of(int warps) {
  size_t smem = sizeof(WarpCell) * warps;
  int n = 0;
  cudaFuncSetAttribute(clip_cells_kernel<PRED, CERT, MINB, false>,
                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, clip_cells_kernel<PRED, CERT, MINB, false>,
                                                warps * 32, smem);
  return n > 0 ? n : 1;
}

template <int PRED, bool CERT>
static int occ_variant(int variant, int warps) {
  if (variant == 1) return occ_of<PRED, CERT, 6>(4);
  if (variant == 2) return occ_of<PRED, CERT, 8>(4);
  return occ_of<PRED, CERT, 0>(warps);
}

int clip_blocks_per_sm_cert(int pred_mode, int certify, int warps, int variant) {
  if (pred_mode == RPD_PRED_FP32_FILTER)
    return certify ? occ_variant<RPD_PRED_FP32_FILTER, true>(variant, warps)
                   : occ_variant<RPD_PRED_FP32_FILTER, false>(variant, warps);
  if (pred_mode == RPD_PRED_EXACT)
    return certify ? occ_variant<RPD_PRED_EXACT, true>(variant, warps)
                   : occ_variant<RPD_PRED_EXACT, false>(variant, warps);
  return certify ? occ_variant<RPD_PRED_FP64, true>(variant, warps)
                 : occ_variant<RPD_PRED_FP64, false>(variant, warps);
}

int clip_blocks_per_sm(int pred_mode, int warps) {
  return clip_blocks_per_sm_cert(pred_mode, 0, warps, 0);
}

int box_blocks_per_sm(int warps) {
  size_t smem = sizeof(WarpCell) * warps;
  int n = 0;
  cudaFuncSetAttribute(site_box_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, site_box_kernel, warps * 32, smem);
  return n > 0 ? n : 1;
}

template <int PRED, bool CERT, int MINB, bool EXT>
static void launch_one(const ClipParams& p, int blocks, int warps, cudaStream_t st) {
  size_t smem = sizeof(WarpCell) * warps;
  cudaFuncSetAttribute(clip_cells_kernel<PRED, CERT, MINB, EXT>,
                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  clip_cells_kernel<PRED, CERT, MINB, EXT><<<blocks, warps * 32, smem, st>>>(p);
  note_launches(1);
}

// the re-clips with extended rows (few cells) use one register budget (80:
// six blocks of four warps per SM), whatever the first pass's variant
template <int PRED, bool CERT>
static void launch_variant(const ClipParams& p, int variant, int blocks, int warps,
                           cudaStream_t st) {
  if (p.site_row) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    launch_one<PRED, CERT, 6, true>(p, (sms > 0 ? sms : 1) * 6, 4, st);
  } else if (variant == 1) {
    launch_one<PRED, CERT, 6, false>(p, blocks, 4, st);
  } else if (variant == 2) {
    launch_one<PRED, CERT, 8, false>(p, blocks, 4, st);
  } else {
    launch_one<PRED, CERT, 0, false>(p, blocks, warps, st);
  }
}

cudaError_t launch_clip_cells(const ClipParams& p, int pred_mode, int certify, int variant,
                              int blocks, int warps, cudaStream_t st) {
  if (pred_mode == RPD_PRED_FP32_FILTER) {
    if (certify) launch_variant<RPD_PRED_FP32_FILTER, true>(p, variant, blocks, warps, st);
    else launch_variant<RPD_PRED_FP32_FILTER, false>(p, variant, blocks, warps, st);
  } else if (pred_mode == RPD_PRED_EXACT) {
    if (certify) launch_variant<RPD_PRED_EXACT, true>(p, variant, blocks, warps, st);
    else launch_variant<RPD_PRED_EXACT, false>(p, variant, blocks, warps, st);
  } else {
    if (certify) launch_variant<RPD_PRED_FP64, true>(p, variant, blocks, warps, st);
    else launch_variant<RPD_PRED_FP64, false>(p, variant, blocks, warps, st);
  }
  return cudaGetLastError();
}

cudaError_t launch_site_box(const BoxParams& p, int blocks, int warps, cudaStream_t st) {
  size_t smem = sizeof(WarpCell) * warps;
  cudaFuncSetAttribute(site_box_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  site_box_kernel<<<blocks, warps * 32, smem, st>>>(p);
  note_launches(1);
  return cudaGetLastError();
}

}  // namespace rpd
