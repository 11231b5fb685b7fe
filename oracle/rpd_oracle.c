/*
 * rpd_oracle.c -- CPU restatement of libmat's RPD hot path (test
 * infrastructure only; see rpd_oracle.h for the list of reference sources
 * each part follows).  Build with -ffp-contract=off: the reference's float
 * and double formulas are evaluated one IEEE-rounded operation at a time.
 */
#include "rpd_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define END ORC_END_OF_LIST

/* ------------------------------------------------------------------ */
/* payload layout                                                     */
/* ------------------------------------------------------------------ */
static size_t al16(size_t x) { return (x + 15) & ~(size_t)15; }

size_t orc_payload_bytes(int nb_v, int nb_p, int nb_e) {
  size_t b = 0;
  b += (size_t)16 * nb_p;          /* planes */
  b += al16((size_t)8 * nb_p);     /* id2 */
  b += al16((size_t)4 * nb_v);     /* ver */
  b += al16((size_t)4 * nb_e);     /* edges */
  b += al16((size_t)nb_p);         /* h */
  b += al16((size_t)24 * nb_v);    /* xyz (double) */
  return b;
}

/* ------------------------------------------------------------------ */
/* mesh adjacency (io.cxx:238-335)                                    */
/* ------------------------------------------------------------------ */
/* local faces of a tet, as the reference's tet_faces_lvid
 * (convex_cell.h:25-26): face i is opposite vertex i */
static const int kFaceLv[4][3] = {{2, 1, 3}, {0, 2, 3}, {1, 0, 3}, {0, 1, 2}};
/* local edges in the order the reference's cell constructor visits them
 * (convex_cell.cu:193-211): (0,1) (0,2) (0,3) (1,2) (1,3) (2,3) */
static const int kEdgeLv[6][2] = {{0, 1}, {0, 2}, {0, 3},
                                  {1, 2}, {1, 3}, {2, 3}};
/* the two tet faces meeting at each of those edges */
static const int kEdgeFaces[6][2] = {{2, 3}, {1, 3}, {1, 2},
                                     {0, 3}, {0, 2}, {0, 1}};

typedef struct {
  int32_t a, b, c;
  int32_t idx;
} key3;

static int cmp_key3(const void* x, const void* y) {
  const key3* p = (const key3*)x;
  const key3* q = (const key3*)y;
  if (p->a != q->a) return p->a < q->a ? -1 : 1;
  if (p->b != q->b) return p->b < q->b ? -1 : 1;
  if (p->c != q->c) return p->c < q->c ? -1 : 1;
  return p->idx < q->idx ? -1 : (p->idx > q->idx);
}

static void sort3(int32_t* v) {
  int32_t t;
  if (v[0] > v[1]) { t = v[0]; v[0] = v[1]; v[1] = t; }
  if (v[1] > v[2]) { t = v[1]; v[1] = v[2]; v[2] = t; }
  if (v[0] > v[1]) { t = v[0]; v[0] = v[1]; v[1] = t; }
}

int orc_mesh_adjacency(int n_vert, int n_tet, const int32_t* tets,
                       int32_t* v_adjs, uint8_t* e_adj6, int32_t* f_adjs,
                       int32_t* f_ids, int32_t* n_boundary_faces) {
  /* #tets per vertex */
  for (int v = 0; v < n_vert; ++v) v_adjs[v] = 0;
  for (int64_t i = 0; i < (int64_t)n_tet * 4; ++i) {
    int v = tets[i];
    if (v < 0 || v >= n_vert) return -1;
    v_adjs[v]++;
  }
  /* #tets per edge: group the 6 edges of every tet */
  int64_t ne = (int64_t)n_tet * 6;
  key3* ek = (key3*)malloc(sizeof(key3) * (size_t)(ne > 0 ? ne : 1));
  for (int t = 0; t < n_tet; ++t)
    for (int e = 0; e < 6; ++e) {
      int32_t a = tets[4 * t + kEdgeLv[e][0]], b = tets[4 * t + kEdgeLv[e][1]];
      key3* k = &ek[(int64_t)t * 6 + e];
      k->a = a < b ? a : b;
      k->b = a < b ? b : a;
      k->c = 0;
      k->idx = t * 6 + e;
    }
  qsort(ek, (size_t)ne, sizeof(key3), cmp_key3);
  for (int64_t s = 0; s < ne;) {
    int64_t r = s;
    while (r < ne && ek[r].a == ek[s].a && ek[r].b == ek[s].b) ++r;
    for (int64_t q = s; q < r; ++q) e_adj6[ek[q].idx] = (uint8_t)(r - s);
    s = r;
  }
  free(ek);
  /* faces: count and ids */
  int64_t nf = (int64_t)n_tet * 4;
  key3* fk = (key3*)malloc(sizeof(key3) * (size_t)(nf > 0 ? nf : 1));
  for (int t = 0; t < n_tet; ++t)
    for (int f = 0; f < 4; ++f) {
      int32_t v[3] = {tets[4 * t + kFaceLv[f][0]], tets[4 * t + kFaceLv[f][1]],
                      tets[4 * t + kFaceLv[f][2]]};
      sort3(v);
      key3* k = &fk[(int64_t)t * 4 + f];
      k->a = v[0];
      k->b = v[1];
      k->c = v[2];
      k->idx = t * 4 + f;
    }
  qsort(fk, (size_t)nf, sizeof(key3), cmp_key3);
  /* partner[i] = the other face slot sharing the face, -1 on the boundary */
  int32_t* partner = (int32_t*)malloc(sizeof(int32_t) * (size_t)(nf > 0 ? nf : 1));
  int bad = 0;
  for (int64_t s = 0; s < nf;) {
    int64_t r = s;
    while (r < nf && fk[r].a == fk[s].a && fk[r].b == fk[s].b &&
           fk[r].c == fk[s].c)
      ++r;
    if (r - s > 2) bad = 1;
    for (int64_t q = s; q < r; ++q) {
      f_adjs[fk[q].idx] = (int32_t)(r - s);
      partner[fk[q].idx] = (r - s == 2) ? fk[q == s ? s + 1 : s].idx : -1;
    }
    s = r;
  }
  free(fk);
  int32_t nb = 0;
  for (int64_t i = 0; i < nf; ++i)
    if (partner[i] < 0) f_ids[i] = nb++;
  int32_t next = nb;
  for (int64_t i = 0; i < nf; ++i) {
    if (partner[i] < 0) continue;
    if (partner[i] > i) f_ids[i] = next++;
    else f_ids[i] = f_ids[partner[i]];
  }
  free(partner);
  if (n_boundary_faces) *n_boundary_faces = nb;
  return bad ? -2 : 0;
}

int64_t orc_dense_e_adjs_size(int n_vert) {
  return (int64_t)n_vert * (1 + n_vert) / 2 + 1;
}

/* index of edge (v1, v2) in the dense triangular table, closed form of the
 * reference's loop (convex_cell.h:46-59) */
static int64_t dense_edge_idx(int64_t v1, int64_t v2, int64_t n) {
  int64_t lo = v1 < v2 ? v1 : v2, hi = v1 < v2 ? v2 : v1;
  return (lo + 1) * n - lo * (lo + 1) / 2 - (n - hi);
}

void orc_dense_e_adjs(int n_vert, int n_tet, const int32_t* tets,
                      const uint8_t* e_adj6, int32_t* e_adjs) {
  int64_t n = orc_dense_e_adjs_size(n_vert);
  for (int64_t i = 0; i < n; ++i) e_adjs[i] = -1;
  for (int t = 0; t < n_tet; ++t)
    for (int e = 0; e < 6; ++e)
      e_adjs[dense_edge_idx(tets[4 * t + kEdgeLv[e][0]],
                            tets[4 * t + kEdgeLv[e][1]], n_vert)] =
          e_adj6[6 * t + e];
}

/* ------------------------------------------------------------------ */
/* neighbour lists                                                    */
/* ------------------------------------------------------------------ */
float orc_bisector_key(const float* si, const float* sj) {
  float dx = sj[0] - si[0], dy = sj[1] - si[1], dz = sj[2] - si[2];
  float d2 = dx * dx + dy * dy + dz * dz;
  if (d2 == 0.0f) return sj[3] > si[3] ? -INFINITY : INFINITY;
  float num = (d2 - sj[3]) + si[3];
  float den = 2.0f * sqrtf(d2);
  return num / den;
}

typedef struct {
  float key;
  int32_t id;
} kv;

static int kv_less(float ka, int32_t ia, float kb, int32_t ib) {
  return ka < kb || (ka == kb && ia < ib);
}

void orc_knn(int n_site, const float* site4, int k, int32_t* nbr, float* keys,
             int n_threads) {
#ifdef _OPENMP
  if (n_threads > 0) omp_set_num_threads(n_threads);
#pragma omp parallel
#endif
  {
    kv* best = (kv*)malloc(sizeof(kv) * (size_t)(k > 0 ? k : 1));
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 64)
#endif
    for (int i = 0; i < n_site; ++i) {
      /* the k smallest (key, id) kept sorted by insertion */
      int m = 0;
      for (int j = 0; j < n_site; ++j) {
        if (j == i) continue;
        float key = orc_bisector_key(site4 + 4 * (int64_t)i, site4 + 4 * (int64_t)j);
        if (m == k && !kv_less(key, j, best[k - 1].key, best[k - 1].id)) continue;
        int pos = m < k ? m : k - 1;
        while (pos > 0 && kv_less(key, j, best[pos - 1].key, best[pos - 1].id)) {
          best[pos] = best[pos - 1];
          --pos;
        }
        best[pos].key = key;
        best[pos].id = j;
        if (m < k) ++m;
      }
      for (int r = 0; r < k; ++r) {
        nbr[(int64_t)i * k + r] = r < m ? best[r].id : -1;
        if (keys) keys[(int64_t)i * k + r] = r < m ? best[r].key : INFINITY;
      }
    }
    free(best);
  }
}

/* ------------------------------------------------------------------ */
/* candidate pairs: voronoi.cu:154-193, knncuda.cu:21-94 + :130-160   */
/* ------------------------------------------------------------------ */
/* power distance of mesh vertex v to site s, in the reference's order:
 * ((0 + t0^2) + t1^2) + t2^2, then minus the weight */
static float pow_dist(const float* s, const float* v) {
  float ssd = 0.0f, t;
  t = s[0] - v[0];
  ssd = ssd + t * t;
  t = s[1] - v[1];
  ssd = ssd + t * t;
  t = s[2] - v[2];
  ssd = ssd + t * t;
  return ssd - s[3];
}

int64_t orc_candidate_pairs(int n_vert, const float* vert3, int n_tet,
                            const int32_t* tets, int n_site,
                            const float* site4, const uint32_t* flags,
                            const int32_t* nbr, int k, int32_t* tet_offsets,
                            int32_t* pair_sites, int64_t capacity,
                            int n_threads) {
  (void)n_vert;
  int32_t* cnt = (int32_t*)calloc((size_t)n_tet + 1, sizeof(int32_t));
  uint8_t* rel = NULL;
  /* first pass: counts; second pass: fill (same deterministic test) */
  for (int pass = 0; pass < 2; ++pass) {
#ifdef _OPENMP
    if (n_threads > 0) omp_set_num_threads(n_threads);
#pragma omp parallel for schedule(dynamic, 64)
#endif
    for (int t = 0; t < n_tet; ++t) {
      const float* tv[4];
      for (int q = 0; q < 4; ++q) tv[q] = vert3 + 3 * (int64_t)tets[4 * t + q];
      int32_t c = 0;
      int32_t base = pass ? tet_offsets[t] : 0;
      for (int i = 0; i < n_site; ++i) {
        if (flags[i] != 1u) continue;
        float pdi[4];
        for (int q = 0; q < 4; ++q) pdi[q] = pow_dist(site4 + 4 * (int64_t)i, tv[q]);
        int ok = 1;
        for (int r = 0; r < k && ok; ++r) {
          int m = nbr[(int64_t)i * k + r];
          if (m == -1) continue; /* voronoi.cu:171 skips, does not stop */
          int hit = 0;
          for (int q = 0; q < 4 && !hit; ++q)
            if (pow_dist(site4 + 4 * (int64_t)m, tv[q]) > pdi[q]) hit = 1;
          ok = hit;
        }
        if (ok) {
          if (pass && base + c < capacity) pair_sites[base + c] = i;
          ++c;
        }
      }
      if (!pass) cnt[t] = c;
    }
    if (!pass) {
      tet_offsets[0] = 0;
      for (int t = 0; t < n_tet; ++t) tet_offsets[t + 1] = tet_offsets[t] + cnt[t];
      if (tet_offsets[n_tet] > capacity) {
        free(cnt);
        return -1;
      }
    }
  }
  (void)rel;
  free(cnt);
  return tet_offsets[n_tet];
}

/* ------------------------------------------------------------------ */
/* the convex cell (convex_cell.h:117-185, convex_cell.cu:116-774)    */
/* ------------------------------------------------------------------ */
typedef struct {
  float pl[ORC_MAX_P][4];
  int32_t id2[ORC_MAX_P][2];
  uint8_t h[ORC_MAX_P];
  uint8_t ver[ORC_MAX_T][4];
  uint8_t edge[ORC_MAX_E][3];
  uint8_t bnext[ORC_MAX_P];
  int nb_v, nb_p, nb_e, nb_r;
  int first;
  int status;
  float seed[4];
  int seed_id;
  int pred_mode;
  int64_t n_pred, n_esc, n_unc, n_flip;
} cell_t;

/* include/common_cuda.h:195-213 in double */
static double det4x4d(double a11, double a12, double a13, double a14,
                      double a21, double a22, double a23, double a24,
                      double a31, double a32, double a33, double a34,
                      double a41, double a42, double a43, double a44) {
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

double orc_det4x4_ref(const float* p1, const float* p2, const float* p3,
                      const float* e) {
  return det4x4d(p1[0], p2[0], p3[0], e[0], p1[1], p2[1], p3[1], e[1], p1[2],
                 p2[2], p3[2], e[2], p1[3], p2[3], p3[3], e[3]);
}

/* include/common_cuda.h:153-166 in float */
static float det2x2f(float a11, float a12, float a21, float a22) {
  return a11 * a22 - a12 * a21;
}
static float det3x3f(float a11, float a12, float a13, float a21, float a22,
                     float a23, float a31, float a32, float a33) {
  return a11 * det2x2f(a22, a23, a32, a33) - a21 * det2x2f(a12, a13, a32, a33) +
         a31 * det2x2f(a12, a13, a22, a23);
}

/* FP32 static filter.  det4x4(p1,p2,p3,e) = sum_r e_r K_r where K_r are the
 * signed 3x3 minors of the three vertex planes.  K_r is evaluated in FP32
 * with FMA (error <= gamma_5 * permanent), the dot with e adds gamma_4.  The
 * bound also covers the reference's own FP64 evaluation error (gamma_9 of
 * double precision times the 4x4 permanent), so a decided sign equals the
 * sign the reference's FP64 determinant returns. */
static void minor3(float a1, float b1, float c1, float a2, float b2, float c2,
                   float a3, float b3, float c3, float* det, float* perm) {
  float u1 = fmaf(b2, c3, -(b3 * c2));
  float u2 = fmaf(a2, c3, -(a3 * c2));
  float u3 = fmaf(a2, b3, -(a3 * b2));
  *det = fmaf(a1, u1, fmaf(-b1, u2, c1 * u3));
  float v1 = fmaf(fabsf(b2), fabsf(c3), fabsf(b3) * fabsf(c2));
  float v2 = fmaf(fabsf(a2), fabsf(c3), fabsf(a3) * fabsf(c2));
  float v3 = fmaf(fabsf(a2), fabsf(b3), fabsf(a3) * fabsf(b2));
  *perm = fmaf(fabsf(a1), v1, fmaf(fabsf(b1), v2, fabsf(c1) * v3));
}

/* cofactors K[4] of the vertex (p1,p2,p3) and the matching 3x3 permanents
 * M[4] */
static void vertex_cofactors(const float* p1, const float* p2, const float* p3,
                             float* K, float* M) {
  float d;
  /* rows y z w */
  minor3(p1[1], p1[2], p1[3], p2[1], p2[2], p2[3], p3[1], p3[2], p3[3], &d, &M[0]);
  K[0] = -d;
  /* rows x z w */
  minor3(p1[0], p1[2], p1[3], p2[0], p2[2], p2[3], p3[0], p3[2], p3[3], &d, &M[1]);
  K[1] = d;
  /* rows x y w */
  minor3(p1[0], p1[1], p1[3], p2[0], p2[1], p2[3], p3[0], p3[1], p3[3], &d, &M[2]);
  K[2] = -d;
  /* rows x y z */
  minor3(p1[0], p1[1], p1[2], p2[0], p2[1], p2[2], p3[0], p3[1], p3[2], &d, &M[3]);
  K[3] = d;
}

/* filter constants: 5u for the dot, 6u for the cofactor and FP64 terms,
 * u = 2^-24; absolute floor for underflow */
#define FILT_C1 (5.0f * 5.9604645e-08f)
#define FILT_C2 (6.0f * 5.9604645e-08f)
#define FILT_ABS 1e-30f

/* bound: c1 sum|e_r K_r| + c2 sum|e_r| M_r (the 4x4 permanent) */
static int filter_sign_k(const float* K, const float* M, const float* e) {
  float s = fmaf(e[3], K[3], fmaf(e[2], K[2], fmaf(e[1], K[1], e[0] * K[0])));
  float t = fmaf(fabsf(e[3]), fabsf(K[3]),
                 fmaf(fabsf(e[2]), fabsf(K[2]),
                      fmaf(fabsf(e[1]), fabsf(K[1]), fabsf(e[0]) * fabsf(K[0]))));
  float pm = fmaf(fabsf(e[3]), M[3],
                  fmaf(fabsf(e[2]), M[2], fmaf(fabsf(e[1]), M[1], fabsf(e[0]) * M[0])));
  float b = fmaf(FILT_C1, t, FILT_C2 * pm) + FILT_ABS;
  if (s > b) return 1;
  if (s < -b) return -1;
  return 0;
}

int orc_filter_sign(const float* p1, const float* p2, const float* p3,
                    const float* e) {
  float K[4], M[4];
  vertex_cofactors(p1, p2, p3, K, M);
  return filter_sign_k(K, M, e);
}

/* ---- RPD_PRED_EXACT (an extension, not in the reference): det4x4_ref's
 * FP64 value with an error bound, and the exact sign of the determinant by
 * floating-point expansions (Shewchuk, Discrete Comput. Geom. 18, 1997:
 * TwoSum, TwoProduct via fma, FAST-EXPANSION-SUM and SCALE-EXPANSION with
 * zero elimination).  This file is compiled with -ffp-contract=off. */
double orc_det4x4_bound(const float* p1, const float* p2, const float* p3, const float* e,
                        double* bound) {
  const double a11 = p1[0], a12 = p2[0], a13 = p3[0], a14 = e[0];
  const double a21 = p1[1], a22 = p2[1], a23 = p3[1], a24 = e[1];
  const double a31 = p1[2], a32 = p2[2], a33 = p3[2], a34 = e[2];
  const double a41 = p1[3], a42 = p2[3], a43 = p3[3], a44 = e[3];
  const double P12 = fabs(a21 * a12) + fabs(a11 * a22), P13 = fabs(a31 * a12) + fabs(a11 * a32);
  const double P14 = fabs(a41 * a12) + fabs(a11 * a42), P23 = fabs(a31 * a22) + fabs(a21 * a32);
  const double P24 = fabs(a41 * a22) + fabs(a21 * a42), P34 = fabs(a41 * a32) + fabs(a31 * a42);
  const double P123 = P23 * fabs(a13) + P13 * fabs(a23) + P12 * fabs(a33);
  const double P124 = P24 * fabs(a13) + P14 * fabs(a23) + P12 * fabs(a43);
  const double P134 = P34 * fabs(a13) + P14 * fabs(a33) + P13 * fabs(a43);
  const double P234 = P34 * fabs(a23) + P24 * fabs(a33) + P23 * fabs(a43);
  const double P = P234 * fabs(a14) + P134 * fabs(a24) + P124 * fabs(a34) + P123 * fabs(a44);
  *bound = 10.0 * 1.1102230246251565e-16 * P + 1e-300;
  return orc_det4x4_ref(p1, p2, p3, e);
}

static void x_two_sum(double a, double b, double* x, double* y) {
  *x = a + b;
  double bv = *x - a, av = *x - bv;
  *y = (a - av) + (b - bv);
}
static void x_fast_two_sum(double a, double b, double* x, double* y) {
  *x = a + b;
  *y = b - (*x - a);
}
static void x_two_prod(double a, double b, double* x, double* y) {
  *x = a * b;
  *y = fma(a, b, -*x);
}

static int x_sum(int elen, const double* e, int flen, const double* f, double* h) {
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
      x_fast_two_sum(en, Q, &Qn, &hh);
      en = ++ei < elen ? e[ei] : 0.0;
    } else {
      x_fast_two_sum(fn, Q, &Qn, &hh);
      fn = ++fi < flen ? f[fi] : 0.0;
    }
    Q = Qn;
    if (hh != 0.0) h[hi++] = hh;
    while (ei < elen && fi < flen) {
      if ((fn > en) == (fn > -en)) {
        x_two_sum(Q, en, &Qn, &hh);
        en = ++ei < elen ? e[ei] : 0.0;
      } else {
        x_two_sum(Q, fn, &Qn, &hh);
        fn = ++fi < flen ? f[fi] : 0.0;
      }
      Q = Qn;
      if (hh != 0.0) h[hi++] = hh;
    }
  }
  while (ei < elen) {
    x_two_sum(Q, en, &Qn, &hh);
    en = ++ei < elen ? e[ei] : 0.0;
    Q = Qn;
    if (hh != 0.0) h[hi++] = hh;
  }
  while (fi < flen) {
    x_two_sum(Q, fn, &Qn, &hh);
    fn = ++fi < flen ? f[fi] : 0.0;
    Q = Qn;
    if (hh != 0.0) h[hi++] = hh;
  }
  if (Q != 0.0 || hi == 0) h[hi++] = Q;
  return hi;
}

static int x_scale(int elen, const double* e, double b, double* h) {
  int hi = 0;
  double Q, hh, p1, p0, sum;
  x_two_prod(e[0], b, &Q, &hh);
  if (hh != 0.0) h[hi++] = hh;
  for (int i = 1; i < elen; ++i) {
    x_two_prod(e[i], b, &p1, &p0);
    x_two_sum(Q, p0, &sum, &hh);
    if (hh != 0.0) h[hi++] = hh;
    x_fast_two_sum(p1, sum, &Q, &hh);
    if (hh != 0.0) h[hi++] = hh;
  }
  if (Q != 0.0 || hi == 0) h[hi++] = Q;
  return hi;
}

static int x_minor2(double a, double b, double c, double d, double* h) {
  double x, y;
  x_two_sum(a * b, -(c * d), &x, &y);
  int n = 0;
  if (y != 0.0) h[n++] = y;
  if (x != 0.0 || n == 0) h[n++] = x;
  return n;
}

static int x_combine3(const double* u, int lu, double a, const double* v, int lv, double b,
                      const double* w, int lw, double c, double* h) {
  double t1[24], t2[24], t3[24], t12[48];
  int n1 = x_scale(lu, u, a, t1), n2 = x_scale(lv, v, -b, t2), n3 = x_scale(lw, w, c, t3);
  int n12 = x_sum(n1, t1, n2, t2, t12);
  return x_sum(n12, t12, n3, t3, h);
}

int orc_det4x4_exact_sign(const float* p1, const float* p2, const float* p3, const float* e) {
  const double a11 = p1[0], a12 = p2[0], a13 = p3[0], a14 = e[0];
  const double a21 = p1[1], a22 = p2[1], a23 = p3[1], a24 = e[1];
  const double a31 = p1[2], a32 = p2[2], a33 = p3[2], a34 = e[2];
  const double a41 = p1[3], a42 = p2[3], a43 = p3[3], a44 = e[3];
  double m12[2], m13[2], m14[2], m23[2], m24[2], m34[2];
  int l12 = x_minor2(a21, a12, a11, a22, m12), l13 = x_minor2(a31, a12, a11, a32, m13);
  int l14 = x_minor2(a41, a12, a11, a42, m14), l23 = x_minor2(a31, a22, a21, a32, m23);
  int l24 = x_minor2(a41, a22, a21, a42, m24), l34 = x_minor2(a41, a32, a31, a42, m34);
  double m123[12], m124[12], m134[12], m234[12];
  int l123 = x_combine3(m23, l23, a13, m13, l13, a23, m12, l12, a33, m123);
  int l124 = x_combine3(m24, l24, a13, m14, l14, a23, m12, l12, a43, m124);
  int l134 = x_combine3(m34, l34, a13, m14, l14, a33, m13, l13, a43, m134);
  int l234 = x_combine3(m34, l34, a23, m24, l24, a33, m23, l23, a43, m234);
  double t1[24], t2[24], t3[24], t4[24], s12[48], s34[48], d[96];
  int n1 = x_scale(l234, m234, a14, t1), n2 = x_scale(l134, m134, -a24, t2);
  int n3 = x_scale(l124, m124, a34, t3), n4 = x_scale(l123, m123, -a44, t4);
  int n12 = x_sum(n1, t1, n2, t2, s12), n34 = x_sum(n3, t3, n4, t4, s34);
  int n = x_sum(n12, s12, n34, s34, d);
  double top = d[n - 1];
  return top > 0.0 ? 1 : (top < 0.0 ? -1 : 0);
}

static int plane_eq(const float* a, const float* b) {
  return a[0] == b[0] && a[1] == b[1] && a[2] == b[2] && a[3] == b[3];
}

/* convex_cell.cu:437-500 (cc_vertex_is_in_conflict_double) */
static int in_conflict(cell_t* c, const uint8_t* v, const float* e) {
  const float* p1 = c->pl[v[0]];
  const float* p2 = c->pl[v[1]];
  const float* p3 = c->pl[v[2]];
  if (plane_eq(e, p1) || plane_eq(e, p2) || plane_eq(e, p3)) return 0;
  c->n_pred++;
  if (c->pred_mode == 1 || c->pred_mode == 2) {
    int s = orc_filter_sign(p1, p2, p3, e);
    if (s != 0) return s > 0;
    c->n_esc++;
  }
  if (c->pred_mode == 2) {
    double bound, d = orc_det4x4_bound(p1, p2, p3, e, &bound);
    if (fabs(d) > bound) return d > 0.0;
    c->n_unc++;
    int xs = orc_det4x4_exact_sign(p1, p2, p3, e);
    if ((xs > 0) != (d > 0.0)) c->n_flip++;
    return xs > 0;
  }
  double det = orc_det4x4_ref(p1, p2, p3, e);
  return det > 0.0;
}

/* tri2plane (common_cuda.h:248-254) on the face vertices */
static void tri2plane_f(const float* v0, const float* v1, const float* v2,
                        float* out) {
  float ax = v1[0] - v0[0], ay = v1[1] - v0[1], az = v1[2] - v0[2];
  float bx = v2[0] - v0[0], by = v2[1] - v0[1], bz = v2[2] - v0[2];
  float nx = ay * bz - az * by;
  float ny = az * bx - ax * bz;
  float nz = ax * by - ay * bx;
  out[0] = nx;
  out[1] = ny;
  out[2] = nz;
  out[3] = -(v0[0] * nx + v0[1] * ny + v0[2] * nz);
}

/* new_plane (convex_cell.cu:561-592): bisector of seed S and site B, normal
 * towards S, weights added for the power diagram */
static void bisector_f(const float* S, const float* B, float* out) {
  float dx = S[0] - B[0], dy = S[1] - B[1], dz = S[2] - B[2];
  float ax = S[0] + B[0], ay = S[1] + B[1], az = S[2] + B[2];
  float dot = (ax * dx + ay * dy + az * dz) + (B[3] - S[3]);
  out[0] = dx;
  out[1] = dy;
  out[2] = dz;
  out[3] = -dot / 2.f;
}

static void cell_init(cell_t* c, const float* vert3, const int32_t* tv,
                      const int32_t* v_adjs, const uint8_t* e6,
                      const int32_t* fa, const int32_t* fi) {
  c->first = END;
  memset(c->bnext, END, sizeof(c->bnext));
  c->status = ORC_SUCCESS;
  for (int i = 0; i < 4; ++i) {
    tri2plane_f(vert3 + 3 * (int64_t)tv[kFaceLv[i][0]],
                vert3 + 3 * (int64_t)tv[kFaceLv[i][1]],
                vert3 + 3 * (int64_t)tv[kFaceLv[i][2]], c->pl[i]);
    c->h[i] = (uint8_t)fa[i];
    c->id2[i][0] = fi[i];
    c->id2[i][1] = -1;
  }
  c->nb_p = 4;
  static const uint8_t tri[4][3] = {{1, 3, 2}, {0, 2, 3}, {0, 3, 1}, {0, 1, 2}};
  for (int i = 0; i < 4; ++i) {
    c->ver[i][0] = tri[i][0];
    c->ver[i][1] = tri[i][1];
    c->ver[i][2] = tri[i][2];
    c->ver[i][3] = (uint8_t)v_adjs[tv[i]];
  }
  c->nb_v = 4;
  for (int e = 0; e < 6; ++e) {
    c->edge[e][0] = (uint8_t)kEdgeFaces[e][0];
    c->edge[e][1] = (uint8_t)kEdgeFaces[e][1];
    c->edge[e][2] = e6[e];
  }
  c->nb_e = 6;
}

static int find_edge(const cell_t* c, int p1, int p2) {
  int lo = p1 < p2 ? p1 : p2, hi = p1 < p2 ? p2 : p1;
  for (int e = 0; e < c->nb_e; ++e)
    if (c->edge[e][0] == lo && c->edge[e][1] == hi) return e;
  return -1;
}

static void swap_ver(cell_t* c, int a, int b) {
  uint8_t t[4];
  memcpy(t, c->ver[a], 4);
  memcpy(c->ver[a], c->ver[b], 4);
  memcpy(c->ver[b], t, 4);
}

/* convex_cell.cu:618-678 */
static void compute_boundary(cell_t* c) {
  memset(c->bnext, END, sizeof(c->bnext));
  c->first = END;
  int nb_iter = 0;
  int t = c->nb_v;
  while (c->nb_r > 0) {
    if (nb_iter++ > 65535) {
      c->status = ORC_INCONSISTENT_BOUNDARY;
      return;
    }
    const uint8_t* tr = c->ver[t];
    int in_border[3], opp[3];
    for (int e = 0; e < 3; ++e) in_border[e] = c->bnext[tr[e]] != END;
    for (int e = 0; e < 3; ++e) opp[e] = c->bnext[tr[(e + 1) % 3]] == tr[e];
    int simple = 1;
    for (int e = 0; e < 3; ++e)
      if (!opp[e] && !opp[(e + 1) % 3] && in_border[(e + 1) % 3]) simple = 0;
    if (!opp[0] && !opp[1] && !opp[2]) {
      if (c->first == END) {
        for (int e = 0; e < 3; ++e) c->bnext[tr[e]] = tr[(e + 1) % 3];
        c->first = tr[0];
      } else {
        simple = 0;
      }
    }
    if (!simple) {
      t++;
      if (t == c->nb_v + c->nb_r) t = c->nb_v;
      continue;
    }
    for (int e = 0; e < 3; ++e)
      if (!opp[e]) c->bnext[tr[e]] = tr[(e + 1) % 3];
    for (int e = 0; e < 3; ++e)
      if (opp[e] && opp[(e + 1) % 3]) {
        if (c->first == tr[(e + 1) % 3]) c->first = c->bnext[tr[(e + 1) % 3]];
        c->bnext[tr[(e + 1) % 3]] = END;
      }
    swap_ver(c, t, c->nb_v + c->nb_r - 1);
    t = c->nb_v;
    c->nb_r--;
  }
}

/* convex_cell.cu:274-316: a new vertex whose three planes have a zero
 * float 3x3 determinant cannot be represented */
static void check_perturb(cell_t* c, int i, int j, int k) {
  const float* a = c->pl[i];
  const float* b = c->pl[j];
  const float* d = c->pl[k];
  float w = det3x3f(a[0], a[1], a[2], b[0], b[1], b[2], d[0], d[1], d[2]);
  if (w == 0.f) c->status = ORC_NEEDS_PERTURB;
}

/* convex_cell.cu:680-774 */
static void clip_by_site(cell_t* c, const float* site4, int nid) {
  if (c->nb_p >= ORC_MAX_P) {
    c->status = ORC_VERTEX_OVERFLOW;
    return;
  }
  int cur = c->nb_p;
  const float* B = site4 + 4 * (int64_t)nid;
  bisector_f(c->seed, B, c->pl[cur]);
  c->h[cur] = 1;
  c->id2[cur][0] = c->seed_id < nid ? c->seed_id : nid;
  c->id2[cur][1] = c->seed_id < nid ? nid : c->seed_id;
  c->nb_p++;
  const float* e = c->pl[cur];
  c->nb_r = 0;
  int i = 0;
  while (i < c->nb_v) {
    if (in_conflict(c, c->ver[i], e)) {
      c->nb_v--;
      swap_ver(c, i, c->nb_v);
      c->nb_r++;
    } else {
      i++;
    }
  }
  if (c->nb_r == 0) {
    c->nb_p--;
    return;
  }
  if (c->nb_v == 0) {
    c->status = ORC_NO_INTERSECTION;
    return;
  }
  compute_boundary(c);
  if (c->status != ORC_SUCCESS) return;
  if (c->first == END) return;
  int cir = c->first;
  do {
    if (c->nb_e >= ORC_MAX_E) {
      c->status = ORC_EDGE_OVERFLOW;
      return;
    }
    int lo = cur < cir ? cur : cir, hi = cur < cir ? cir : cur;
    uint8_t ha = c->h[cur], hb = c->h[cir];
    c->edge[c->nb_e][0] = (uint8_t)lo;
    c->edge[c->nb_e][1] = (uint8_t)hi;
    c->edge[c->nb_e][2] = ha > hb ? ha : hb;
    c->nb_e++;
    cir = c->bnext[cir];
  } while (cir != c->first);
  cir = c->first;
  do {
    int nx = c->bnext[cir];
    if (c->nb_v + 1 >= ORC_MAX_T) {
      c->status = ORC_TRIANGLE_OVERFLOW;
    } else {
      int e1 = find_edge(c, cur, cir), e2 = find_edge(c, cur, nx),
          e3 = find_edge(c, cir, nx);
      if (e1 < 0 || e2 < 0 || e3 < 0) {
        /* the reference reads out of bounds here (assert compiled out);
         * treat as an inconsistent cell */
        c->status = ORC_INCONSISTENT_BOUNDARY;
        return;
      }
      uint8_t adj = c->edge[e1][2];
      if (c->edge[e2][2] > adj) adj = c->edge[e2][2];
      if (c->edge[e3][2] > adj) adj = c->edge[e3][2];
      c->ver[c->nb_v][0] = (uint8_t)cur;
      c->ver[c->nb_v][1] = (uint8_t)cir;
      c->ver[c->nb_v][2] = (uint8_t)nx;
      c->ver[c->nb_v][3] = adj;
      c->nb_v++;
    }
    check_perturb(c, cur, cir, nx);
    if (c->status != ORC_SUCCESS) return;
    cir = nx;
  } while (cir != c->first);
}

/* ------------------------------------------------------------------ */
/* FP64 reconstruction                                                */
/* ------------------------------------------------------------------ */
static void tri2plane_d(const double* v0, const double* v1, const double* v2,
                        double* out) {
  double ax = v1[0] - v0[0], ay = v1[1] - v0[1], az = v1[2] - v0[2];
  double bx = v2[0] - v0[0], by = v2[1] - v0[1], bz = v2[2] - v0[2];
  double nx = ay * bz - az * by;
  double ny = az * bx - ax * bz;
  double nz = ax * by - ay * bx;
  out[0] = nx;
  out[1] = ny;
  out[2] = nz;
  out[3] = -(v0[0] * nx + v0[1] * ny + v0[2] * nz);
}

static void bisector_d(const double* S, const double* B, double* out) {
  double dx = S[0] - B[0], dy = S[1] - B[1], dz = S[2] - B[2];
  double ax = S[0] + B[0], ay = S[1] + B[1], az = S[2] + B[2];
  double dot = (ax * dx + ay * dy + az * dz) + (B[3] - S[3]);
  out[0] = dx;
  out[1] = dy;
  out[2] = dz;
  out[3] = -dot * 0.5;
}

static double det3d(double a11, double a12, double a13, double a21, double a22,
                    double a23, double a31, double a32, double a33) {
  return a11 * (a22 * a33 - a23 * a32) - a21 * (a12 * a33 - a13 * a32) +
         a31 * (a12 * a23 - a13 * a22);
}

/* intersection of three planes (homogeneous Cramer, as the reference's
 * compute_vertex_coordinates, convex_cell.cu:319-351) */
static void vertex_d(const double* a, const double* b, const double* c,
                     double* out) {
  double x = -det3d(a[3], a[1], a[2], b[3], b[1], b[2], c[3], c[1], c[2]);
  double y = -det3d(a[0], a[3], a[2], b[0], b[3], b[2], c[0], c[3], c[2]);
  double z = -det3d(a[0], a[1], a[3], b[0], b[1], b[3], c[0], c[1], c[3]);
  double w = det3d(a[0], a[1], a[2], b[0], b[1], b[2], c[0], c[1], c[2]);
  out[0] = x / w;
  out[1] = y / w;
  out[2] = z / w;
}

static void project_d(const double* P, const double* pl, double* out) {
  double n2 = pl[0] * pl[0] + pl[1] * pl[1] + pl[2] * pl[2];
  double lam =
      n2 > 0.0 ? (pl[0] * P[0] + pl[1] * P[1] + pl[2] * P[2] + pl[3]) / n2 : 0.0;
  out[0] = P[0] - lam * pl[0];
  out[1] = P[1] - lam * pl[1];
  out[2] = P[2] - lam * pl[2];
}

/* signed volume of one vertex's 6 flag tets (convex_cell.cu:986-1069):
 * C = seed, A = vertex, P[2i] = foot of C on face i, P[2i+1] = foot of C on
 * the edge line between faces i and i+1 */
static double vertex_volume_d(const double* C, const double* A,
                              const double* f0, const double* f1,
                              const double* f2) {
  const double* f[3] = {f0, f1, f2};
  double P[6][3];
  for (int i = 0; i < 3; ++i) project_d(C, f[i], P[2 * i]);
  for (int i = 0; i < 3; ++i) {
    /* the edge between faces i and i+1 runs along n_i x n_(i+1); the foot of
     * C on that line is the projection of A onto the plane through C with
     * that normal */
    const double* u = f[i];
    const double* v = f[(i + 1) % 3];
    double n[4] = {u[1] * v[2] - u[2] * v[1], u[2] * v[0] - u[0] * v[2],
                   u[0] * v[1] - u[1] * v[0], 0.0};
    n[3] = -(C[0] * n[0] + C[1] * n[1] + C[2] * n[2]);
    project_d(A, n, P[2 * i + 1]);
  }
  double vol = 0.0;
  for (int i = 0; i < 6; ++i) {
    const double* p = P[i];
    const double* q = P[(i + 1) % 6];
    double a0 = p[0] - A[0], a1 = p[1] - A[1], a2 = p[2] - A[2];
    double b0 = q[0] - A[0], b1 = q[1] - A[1], b2 = q[2] - A[2];
    double c0 = C[0] - A[0], c1 = C[1] - A[1], c2 = C[2] - A[2];
    vol += -det3d(a0, a1, a2, b0, b1, b2, c0, c1, c2) / 6.0;
  }
  return vol;
}

/* ------------------------------------------------------------------ */
/* per-pair driver (convex_cell.cu:1166-1337)                         */
/* ------------------------------------------------------------------ */
static int64_t emit_payload(const cell_t* c, const double* vert3d,
                            const int32_t* tv, const double* site4d,
                            uint8_t* out, double* volume) {
  int np = c->nb_p, nv = c->nb_v, ne = c->nb_e;
  uint8_t* p = out;
  memcpy(p, c->pl, (size_t)16 * np);
  p += 16 * np;
  memset(p, 0, al16((size_t)8 * np));
  memcpy(p, c->id2, (size_t)8 * np);
  p += al16((size_t)8 * np);
  memset(p, 0, al16((size_t)4 * nv));
  memcpy(p, c->ver, (size_t)4 * nv);
  p += al16((size_t)4 * nv);
  memset(p, 0, al16((size_t)4 * ne));
  for (int e = 0; e < ne; ++e) {
    p[4 * e + 0] = c->edge[e][0];
    p[4 * e + 1] = c->edge[e][1];
    p[4 * e + 2] = c->edge[e][2];
    p[4 * e + 3] = 0;
  }
  p += al16((size_t)4 * ne);
  memset(p, 0, al16((size_t)np));
  memcpy(p, c->h, (size_t)np);
  p += al16((size_t)np);
  /* FP64 planes from FP64 inputs */
  double pd[ORC_MAX_P][4];
  for (int i = 0; i < 4 && i < np; ++i)
    tri2plane_d(vert3d + 3 * (int64_t)tv[kFaceLv[i][0]],
                vert3d + 3 * (int64_t)tv[kFaceLv[i][1]],
                vert3d + 3 * (int64_t)tv[kFaceLv[i][2]], pd[i]);
  const double* S = site4d + 4 * (int64_t)c->seed_id;
  for (int i = 4; i < np; ++i) {
    int other = c->id2[i][0] == c->seed_id ? c->id2[i][1] : c->id2[i][0];
    bisector_d(S, site4d + 4 * (int64_t)other, pd[i]);
  }
  double* xyz = (double*)p;
  double vol = 0.0;
  for (int v = 0; v < nv; ++v) {
    const uint8_t* t = c->ver[v];
    vertex_d(pd[t[0]], pd[t[1]], pd[t[2]], xyz + 3 * v);
    vol += vertex_volume_d(S, xyz + 3 * v, pd[t[0]], pd[t[1]], pd[t[2]]);
  }
  p += al16((size_t)24 * nv);
  *volume = vol;
  return (int64_t)(p - out);
}

typedef struct {
  uint8_t* buf;
  int64_t size, cap;
} tbuf_t;

static uint8_t* tbuf_reserve(tbuf_t* b, int64_t n) {
  if (b->size + n > b->cap) {
    int64_t nc = b->cap ? b->cap * 2 : (1 << 20);
    while (nc < b->size + n) nc *= 2;
    b->buf = (uint8_t*)realloc(b->buf, (size_t)nc);
    b->cap = nc;
  }
  return b->buf + b->size;
}

int64_t orc_clip_cells(int n_vert, const float* vert3, const double* vert3d,
                       int n_tet, const int32_t* tets, const int32_t* v_adjs,
                       const uint8_t* e_adj6, const int32_t* f_adjs,
                       const int32_t* f_ids, int n_site, const float* site4,
                       const double* site4d, const int32_t* nbr, int k,
                       const int32_t* tet_offsets, const int32_t* pair_sites,
                       int pred_mode, orc_cell_header* headers,
                       uint8_t* payload, int64_t payload_capacity,
                       int64_t* stats, int n_threads) {
  (void)n_vert;
  (void)n_site;
  int64_t n_pairs = tet_offsets[n_tet];
  int nthr = 1;
#ifdef _OPENMP
  if (n_threads > 0) omp_set_num_threads(n_threads);
  nthr = omp_get_max_threads();
#endif
  tbuf_t* tb = (tbuf_t*)calloc((size_t)nthr, sizeof(tbuf_t));
  /* per pair: owning thread and offset in that thread's buffer */
  int32_t* own = (int32_t*)malloc(sizeof(int32_t) * (size_t)(n_pairs > 0 ? n_pairs : 1));
  int64_t* loff = (int64_t*)malloc(sizeof(int64_t) * (size_t)(n_pairs > 0 ? n_pairs : 1));
  int64_t tot_pred = 0, tot_esc = 0, tot_unc = 0, tot_flip = 0;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 16) reduction(+ : tot_pred, tot_esc, tot_unc, tot_flip)
#endif
  for (int t = 0; t < n_tet; ++t) {
    int me = 0;
#ifdef _OPENMP
    me = omp_get_thread_num();
#endif
    cell_t c;
    for (int32_t q = tet_offsets[t]; q < tet_offsets[t + 1]; ++q) {
      int s = pair_sites[q];
      c.pred_mode = pred_mode;
      c.n_pred = c.n_esc = c.n_unc = c.n_flip = 0;
      c.seed_id = s;
      memcpy(c.seed, site4 + 4 * (int64_t)s, sizeof(float) * 4);
      cell_init(&c, vert3, tets + 4 * (int64_t)t, v_adjs, e_adj6 + 6 * (int64_t)t,
                f_adjs + 4 * (int64_t)t, f_ids + 4 * (int64_t)t);
      for (int r = 0; r < k; ++r) {
        int nid = nbr[(int64_t)s * k + r];
        if (nid == -1) break;
        clip_by_site(&c, site4, nid);
        if (c.status != ORC_SUCCESS) break;
      }
      tot_pred += c.n_pred;
      tot_esc += c.n_esc;
      tot_unc += c.n_unc;
      tot_flip += c.n_flip;
      orc_cell_header* h = &headers[q];
      h->tet_id = t;
      h->site_id = s;
      h->status = c.status;
      h->flags = 0;
      h->offset = 0;
      h->volume = 0.0;
      h->nb_v = h->nb_p = h->nb_e = 0;
      own[q] = me;
      loff[q] = -1;
      if (c.status == ORC_SUCCESS) {
        h->nb_v = (uint8_t)c.nb_v;
        h->nb_p = (uint8_t)c.nb_p;
        h->nb_e = (uint8_t)c.nb_e;
        int64_t need = (int64_t)orc_payload_bytes(c.nb_v, c.nb_p, c.nb_e);
        uint8_t* dst = tbuf_reserve(&tb[me], need);
        double vol = 0.0;
        emit_payload(&c, vert3d, tets + 4 * (int64_t)t, site4d, dst, &vol);
        h->volume = vol;
        loff[q] = tb[me].size;
        tb[me].size += need;
      }
    }
  }
  int64_t off = 0;
  for (int64_t q = 0; q < n_pairs; ++q) {
    headers[q].offset = (uint64_t)off;
    if (headers[q].status == ORC_SUCCESS)
      off += (int64_t)orc_payload_bytes(headers[q].nb_v, headers[q].nb_p,
                                        headers[q].nb_e);
  }
  if (stats) {
    stats[0] = tot_pred;
    stats[1] = tot_esc;
    stats[2] = tot_unc;
    stats[3] = tot_flip;
  }
  if (off <= payload_capacity && payload) {
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int64_t q = 0; q < n_pairs; ++q) {
      if (headers[q].status != ORC_SUCCESS) continue;
      memcpy(payload + headers[q].offset, tb[own[q]].buf + loff[q],
             orc_payload_bytes(headers[q].nb_v, headers[q].nb_p,
                               headers[q].nb_e));
    }
  }
  for (int i = 0; i < nthr; ++i) free(tb[i].buf);
  free(tb);
  free(own);
  free(loff);
  return off <= payload_capacity ? off : -1;
}

/* ------------------------------------------------------------------------
 * Per-cell topology of emitted cells: restates ConvexCellHost's host-side
 * reconstruction (src/rpd3d_base/voronoi_defs.cxx) on the packed record.
 * ---------------------------------------------------------------------- */
size_t orc_topo_bytes(int nb_v, int nb_p, int nb_e) {
  return al16((size_t)6 * nb_p + (size_t)nb_e + (size_t)3 * nb_v);
}

/* include/common_cxx.h:128-135 */
static float orc_cdet2(float a11, float a12, float a21, float a22) {
  return a11 * a22 - a12 * a21;
}
static float orc_cdet3(float a11, float a12, float a13, float a21, float a22,
                       float a23, float a31, float a32, float a33) {
  return a11 * orc_cdet2(a22, a23, a32, a33) - a21 * orc_cdet2(a12, a13, a32, a33) +
         a31 * orc_cdet2(a12, a13, a22, a23);
}

/* compute_vertex_coordinates with the perspective divide
 * (voronoi_defs.cxx:33-74): is any coordinate NaN? */
static int orc_vertex_null(const float* p1, const float* p2, const float* p3) {
  float x = -orc_cdet3(p1[3], p1[1], p1[2], p2[3], p2[1], p2[2], p3[3], p3[1], p3[2]);
  float y = -orc_cdet3(p1[0], p1[3], p1[2], p2[0], p2[3], p2[2], p3[0], p3[3], p3[2]);
  float z = -orc_cdet3(p1[0], p1[1], p1[3], p2[0], p2[1], p2[3], p3[0], p3[1], p3[3]);
  float w = orc_cdet3(p1[0], p1[1], p1[2], p2[0], p2[1], p2[2], p3[0], p3[1], p3[2]);
  float px = x / w, py = y / w, pz = z / w;
  return isnan(px) || isnan(py) || isnan(pz);
}

static int orc_on_plane(const uint8_t* v, int p) { return v[0] == p || v[1] == p || v[2] == p; }

static void orc_one_topology(const orc_cell_header* h, const uint8_t* rec,
                             orc_topo_header* th, uint8_t* out) {
  const int nv = h->nb_v, np = h->nb_p, ne = h->nb_e;
  const size_t o_id2 = (size_t)16 * np, o_ver = o_id2 + al16((size_t)8 * np),
               o_edge = o_ver + al16((size_t)4 * nv), o_h = o_edge + al16((size_t)4 * ne);
  const float* pl = (const float*)rec;
  const int32_t* id2 = (const int32_t*)(rec + o_id2);
  const uint8_t* ver = rec + o_ver;
  const uint8_t* edge = rec + o_edge;
  const uint8_t* hh = rec + o_h;
  float* facet = (float*)out;
  uint8_t* act = out + (size_t)4 * np;
  int8_t* lf2a = (int8_t*)(act + np);
  uint8_t* acte = act + (size_t)2 * np;
  uint8_t* faces = acte + ne;
  int cnt[ORC_MAX_P];
  int tab_v[ORC_MAX_T], tab_lp[ORC_MAX_T];
  memset(out, 0, orc_topo_bytes(nv, np, ne));
  th->flags = 0;
  th->pad[0] = th->pad[1] = 0;

  /* reload_active (:76-106): vertices per plane, then edges whose two
   * planes are active and share at least two vertices */
  for (int p = 0; p < np; ++p) cnt[p] = 0;
  for (int t = 0; t < nv; ++t)
    for (int k = 0; k < 3; ++k)
      if (ver[4 * t + k] < np) cnt[ver[4 * t + k]]++;
  for (int e = 0; e < ne; ++e) {
    const int x = edge[4 * e], y = edge[4 * e + 1];
    acte[e] = 0;
    if (x >= np || y >= np || cnt[x] <= 0 || cnt[y] <= 0) continue;
    int common = 0;
    for (int t = 0; t < nv; ++t)
      if (orc_on_plane(ver + 4 * t, x) && orc_on_plane(ver + 4 * t, y)) common++;
    if (common >= 2) acte[e] = 1;
  }

  /* reload_pc_explicit (:108-188): a NaN vertex stops it before the faces */
  int vnull = 0;
  for (int t = 0; t < nv && !vnull; ++t) {
    const uint8_t* v = ver + 4 * t;
    if (v[0] < np && v[1] < np && v[2] < np)
      vnull = orc_vertex_null(pl + 4 * v[0], pl + 4 * v[1], pl + 4 * v[2]);
  }
  int lf = 0, slot = 0;
  for (int plane = 0; plane < np; ++plane) {
    act[plane] = (uint8_t)cnt[plane];
    lf2a[plane] = -1;
    if (cnt[plane] <= 0) continue;
    if (!vnull) {
      int n = 0;
      for (int t = 0; t < nv; ++t) {
        const uint8_t* v = ver + 4 * t;
        if (v[0] == plane) { tab_v[n] = t; tab_lp[n++] = 0; }
        else if (v[1] == plane) { tab_v[n] = t; tab_lp[n++] = 1; }
        else if (v[2] == plane) { tab_v[n] = t; tab_lp[n++] = 2; }
      }
      /* from the first vertex, the next is the first j whose plane before
       * `plane` is the plane after it in vertex i */
      int i = 0, got = 0;
      while (got < n) {
        const int ind_i = (tab_lp[i] + 1) % 3;
        int j = 0;
        for (; j < n; ++j) {
          const int ind_j = (tab_lp[j] + 2) % 3;
          if (ver[4 * tab_v[i] + ind_i] == ver[4 * tab_v[j] + ind_j]) break;
        }
        if (j == n) { /* the cycle does not close: the reference reads past
                         its list here */
          th->flags |= 2;
          for (int r = got; r < n; ++r) faces[slot + r] = 255;
          break;
        }
        faces[slot + got++] = (uint8_t)tab_v[i];
        i = j;
      }
      lf2a[plane] = (int8_t)lf;
      lf++;
    }
    slot += cnt[plane];
  }
  if (vnull) {
    memset(faces, 255, (size_t)3 * nv);
    th->flags |= 1;
    lf = 0;
  }
  th->n_faces = (uint8_t)lf;

  /* cal_cell_euler (:190-222) */
  double sum_v = 0.0, sum_f = 0.0, sum_e = 0.0;
  for (int t = 0; t < nv; ++t) {
    const int v_adj = ver[4 * t + 3];
    sum_v += 1.f / v_adj;
  }
  for (int p = 0; p < np; ++p)
    if (cnt[p] > 0) sum_f += 1. / (float)hh[p];
  for (int e = 0; e < ne; ++e)
    if (acte[e] > 0) sum_e += 1. / edge[4 * e + 2];
  th->euler = (float)(sum_v - sum_e + sum_f);

  /* cal_halfplane_facet_euler (:224-266) for every active bisector plane:
   * the face is the first active plane whose id pair holds the neighbour */
  for (int p = 0; p < np; ++p) {
    facet[p] = 0.f;
    if (cnt[p] <= 0 || id2[2 * p + 1] == -1) continue;
    const int nb = id2[2 * p] == h->site_id ? id2[2 * p + 1] : id2[2 * p];
    int clip = -1;
    for (int r = 0; r < np; ++r) {
      if (cnt[r] <= 0) continue;
      if (id2[2 * r] == nb || id2[2 * r + 1] == nb) { clip = r; break; }
    }
    double sv = 0.0, se = 0.0, sf = 1.0;
    for (int t = 0; t < nv; ++t) {
      if (!orc_on_plane(ver + 4 * t, clip)) continue;
      const int v_adj = ver[4 * t + 3];
      sv += 1.f / v_adj;
    }
    for (int e = 0; e < ne; ++e) {
      if (edge[4 * e] != clip && edge[4 * e + 1] != clip) continue;
      if (acte[e] <= 0) continue;
      se += 1. / edge[4 * e + 2];
    }
    facet[p] = (float)(sv - se + sf);
  }
}

int64_t orc_cell_topology(int64_t n_cells, const orc_cell_header* cells,
                          const uint8_t* payload, orc_topo_header* headers,
                          uint8_t* out, int64_t capacity) {
  int64_t off = 0;
  for (int64_t q = 0; q < n_cells; ++q) {
    if (headers) headers[q].offset = (uint64_t)off;
    off += (int64_t)orc_topo_bytes(cells[q].nb_v, cells[q].nb_p, cells[q].nb_e);
  }
  if (!out || !headers) return off;
  if (off > capacity) return -1;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 256)
#endif
  for (int64_t q = 0; q < n_cells; ++q)
    orc_one_topology(cells + q, payload + cells[q].offset, headers + q, out + headers[q].offset);
  return off;
}

/* ------------------------------------------------------------------------
 * Polygon soup: restates get_one_convex_cell_faces_const
 * (src/IO/IO_CUDA/io_cuda.cxx:21-141) on the packed records, cell after cell.
 * ---------------------------------------------------------------------- */
/* compute_vertex_coordinates of vertex t (voronoi_defs.cxx:33-74), float */
static void orc_float_vertex(const float* pl, const uint8_t* ver, int t, float* out) {
  const float* p1 = pl + 4 * ver[4 * t];
  const float* p2 = pl + 4 * ver[4 * t + 1];
  const float* p3 = pl + 4 * ver[4 * t + 2];
  float x = -orc_cdet3(p1[3], p1[1], p1[2], p2[3], p2[1], p2[2], p3[3], p3[1], p3[2]);
  float y = -orc_cdet3(p1[0], p1[3], p1[2], p2[0], p2[3], p2[2], p3[0], p3[3], p3[2]);
  float z = -orc_cdet3(p1[0], p1[1], p1[3], p2[0], p2[1], p2[3], p3[0], p3[1], p3[3]);
  float w = orc_cdet3(p1[0], p1[1], p1[2], p2[0], p2[1], p2[2], p3[0], p3[1], p3[2]);
  out[0] = x / w;
  out[1] = y / w;
  out[2] = z / w;
}

/* save_convex_cells_houdini's slicing (io_cuda.cxx:166-170): the cell's
 * barycenter, compute_cell_barycenter (io_cuda.cxx:6-17: float sum of the
 * float vertices, divided by (float) nb_v), and is_slice_by_plane
 * (io.cxx:810-820: dot(bary - pos, normal) >= 0 in double, GEO::dot's
 * order) with plane = {pos, normal} */
static int orc_sliced(const float* pl, const uint8_t* ver, int nv, const double* plane) {
  float b[3] = {0.f, 0.f, 0.f}, v[3];
  for (int t = 0; t < nv; ++t) {
    orc_float_vertex(pl, ver, t, v);
    for (int k = 0; k < 3; ++k) b[k] = v[k] + b[k];
  }
  for (int k = 0; k < 3; ++k) b[k] = b[k] / (float)nv;
  const double dx = (double)b[0] - plane[0], dy = (double)b[1] - plane[1],
               dz = (double)b[2] - plane[2];
  const double dist = dx * plane[3] + dy * plane[4] + dz * plane[5];
  return dist >= 0;
}

int orc_cell_polygons(int64_t n_cells, const orc_cell_header* cells,
                      const uint8_t* payload, int triangulate, int boundary_only,
                      int max_sf_fid, const double* slice, float* points, int64_t max_points,
                      int64_t* poly_offsets, uint32_t* indices, int64_t max_indices,
                      int32_t* poly_site, int32_t* poly_adj_site, int64_t max_polys,
                      int64_t* counts) {
  int64_t n_pts = 0, n_poly = 0, n_idx = 0;
  const int write = points != NULL;
  int tab_v[ORC_MAX_T], tab_lp[ORC_MAX_T], cyc[ORC_MAX_T];
  for (int64_t q = 0; q < n_cells; ++q) {
    const orc_cell_header* h = cells + q;
    const int nv = h->nb_v, np = h->nb_p, ne = h->nb_e;
    const uint8_t* rec = payload + h->offset;
    const size_t o_id2 = (size_t)16 * np, o_ver = o_id2 + al16((size_t)8 * np);
    const float* pl = (const float*)rec;
    const int32_t* id2 = (const int32_t*)(rec + o_id2);
    const uint8_t* ver = rec + o_ver;
    (void)ne;
    if (slice && orc_sliced(pl, ver, nv, slice)) continue;
    const int64_t row = n_pts;
    /* the cell's vertices; a NaN one ends the cell */
    int null_seen = 0;
    for (int t = 0; t < nv; ++t) {
      float xyz[3];
      orc_float_vertex(pl, ver, t, xyz);
      const float px = xyz[0], py = xyz[1], pz = xyz[2];
      if (isnan(px) || isnan(py) || isnan(pz)) { null_seen = 1; break; }
      if (write) {
        if (n_pts >= max_points) return -1;
        points[3 * n_pts] = px;
        points[3 * n_pts + 1] = py;
        points[3 * n_pts + 2] = pz;
      }
      n_pts++;
    }
    if (null_seen) continue;
    /* active planes: vertices per plane (reload_active) */
    int cnt[ORC_MAX_P];
    for (int p = 0; p < np; ++p) cnt[p] = 0;
    for (int t = 0; t < nv; ++t)
      for (int k = 0; k < 3; ++k)
        if (ver[4 * t + k] < np) cnt[ver[4 * t + k]]++;
    for (int plane = 0; plane < np; ++plane) {
      if (cnt[plane] <= 0) continue;
      const int hx = id2[2 * plane], hy = id2[2 * plane + 1];
      if (boundary_only && !(hy != -1 || (hy == -1 && hx < max_sf_fid))) continue;
      int n = 0;
      for (int t = 0; t < nv; ++t) {
        const uint8_t* v = ver + 4 * t;
        if (v[0] == plane) { tab_v[n] = t; tab_lp[n++] = 0; }
        else if (v[1] == plane) { tab_v[n] = t; tab_lp[n++] = 1; }
        else if (v[2] == plane) { tab_v[n] = t; tab_lp[n++] = 2; }
      }
      int i = 0, got = 0;
      while (got < n) {
        const int ind_i = (tab_lp[i] + 1) % 3;
        int j = 0;
        for (; j < n; ++j)
          if (ver[4 * tab_v[i] + ind_i] == ver[4 * tab_v[j] + (tab_lp[j] + 2) % 3]) break;
        if (j == n) break; /* open cycle: not a valid cell */
        cyc[got++] = tab_v[i];
        i = j;
      }
      const int adj = hy != -1 ? (hx == h->site_id ? hy : hx) : -1;
      if (triangulate) {
        for (int k = 1; k < got - 1; ++k) {
          if (write) {
            if (n_poly >= max_polys || n_idx + 3 > max_indices) return -1;
            poly_offsets[n_poly] = n_idx;
            indices[n_idx] = (uint32_t)(row + cyc[0]);
            indices[n_idx + 1] = (uint32_t)(row + cyc[k]);
            indices[n_idx + 2] = (uint32_t)(row + cyc[(k + 1) % got]);
            poly_site[n_poly] = h->site_id;
            poly_adj_site[n_poly] = adj;
          }
          n_poly++;
          n_idx += 3;
        }
      } else {
        if (write) {
          if (n_poly >= max_polys || n_idx + got > max_indices) return -1;
          poly_offsets[n_poly] = n_idx;
          for (int k = 0; k < got; ++k) indices[n_idx + k] = (uint32_t)(row + cyc[k]);
          poly_site[n_poly] = h->site_id;
          poly_adj_site[n_poly] = adj;
        }
        n_poly++;
        n_idx += got;
      }
    }
  }
  if (write) {
    if (n_poly + 1 > max_polys + 1) return -1;
    poly_offsets[n_poly] = n_idx;
  }
  if (counts) {
    counts[0] = n_pts;
    counts[1] = n_poly;
    counts[2] = n_idx;
  }
  return 0;
}

/* ------------------------------------------------------------------ */
/* power neighbours: the stand-in for libmat's regular-triangulation   */
/* neighbour lists (src/rpd3d_base/triangulation.cxx:62-144, :442-558) */
/* ------------------------------------------------------------------ */
typedef struct {
  double key;
  int32_t id;
} pn_kv;

static int pn_less(const pn_kv* a, const pn_kv* b) {
  return a->key < b->key || (a->key == b->key && a->id < b->id);
}

static int pn_cmp(const void* x, const void* y) {
  const pn_kv* a = (const pn_kv*)x;
  const pn_kv* b = (const pn_kv*)y;
  return pn_less(a, b) ? -1 : (pn_less(b, a) ? 1 : 0);
}

/* v[0..n) rearranged so that its m smallest entries come first (any order) */
static void pn_select(pn_kv* v, int64_t n, int64_t m) {
  int64_t lo = 0, hi = n - 1;
  while (lo < hi) {
    pn_kv piv = v[lo + (hi - lo) / 2];
    int64_t i = lo, j = hi;
    while (i <= j) {
      while (pn_less(&v[i], &piv)) ++i;
      while (pn_less(&piv, &v[j])) --j;
      if (i <= j) {
        pn_kv t = v[i];
        v[i] = v[j];
        v[j] = t;
        ++i;
        --j;
      }
    }
    if (m - 1 <= j) hi = j;
    else if (m - 1 >= i) lo = i;
    else break;
  }
}

/* largest distance from the seed to a vertex of the cell, vertices solved
 * in double from the float planes */
static double pn_radius(const cell_t* c) {
  double r = 0.0;
  for (int v = 0; v < c->nb_v; ++v) {
    double a[4], b[4], d[4], x[3];
    for (int q = 0; q < 4; ++q) {
      a[q] = c->pl[c->ver[v][0]][q];
      b[q] = c->pl[c->ver[v][1]][q];
      d[q] = c->pl[c->ver[v][2]][q];
    }
    vertex_d(a, b, d, x);
    double dx = x[0] - c->seed[0], dy = x[1] - c->seed[1], dz = x[2] - c->seed[2];
    double r2 = sqrt(dx * dx + dy * dy + dz * dz);
    if (!(r2 <= r)) r = r2;  /* NaN propagates as "unbounded" */
  }
  return r;
}

/* drops the planes no vertex uses and rebuilds the edge list from the
 * vertices (the clipper never deletes either): only the cell's current
 * faces and edges stay, so a long clip sequence fits the capacities.  Edge
 * and face adjacency counts are not kept (the neighbour lists do not use
 * them). */
static void pn_compact(cell_t* c) {
  uint8_t map[ORC_MAX_P];
  memset(map, END, sizeof(map));
  for (int v = 0; v < c->nb_v; ++v)
    for (int q = 0; q < 3; ++q) map[c->ver[v][q]] = 0;
  int np = 0;
  for (int p = 0; p < c->nb_p; ++p) {
    if (map[p] == END && p >= 4) continue;  /* the region's faces stay at 0..3 */
    map[p] = (uint8_t)np;
    if (np != p) {
      memcpy(c->pl[np], c->pl[p], sizeof(c->pl[p]));
      c->id2[np][0] = c->id2[p][0];
      c->id2[np][1] = c->id2[p][1];
      c->h[np] = c->h[p];
    }
    ++np;
  }
  c->nb_p = np;
  c->nb_e = 0;
  for (int v = 0; v < c->nb_v; ++v) {
    for (int q = 0; q < 3; ++q) c->ver[v][q] = map[c->ver[v][q]];
    for (int q = 0; q < 3; ++q) {
      int a = c->ver[v][q], b = c->ver[v][(q + 1) % 3];
      int lo = a < b ? a : b, hi = a < b ? b : a;
      if (find_edge(c, lo, hi) >= 0) continue;
      c->edge[c->nb_e][0] = (uint8_t)lo;
      c->edge[c->nb_e][1] = (uint8_t)hi;
      c->edge[c->nb_e][2] = 1;
      c->nb_e++;
    }
  }
}

/* one region tet: 4 float vertices, positively oriented (the clipper's
 * face planes point inwards) */
typedef struct {
  float v[12];
} pn_tet;

static void pn_orient(pn_tet* t) {
  /* the centroid must lie on the inner side of the clipper's first face
   * plane; otherwise two vertices swap */
  const int32_t tv[4] = {0, 1, 2, 3};
  const int32_t vad[4] = {1, 1, 1, 1}, fa[4] = {1, 1, 1, 1}, fi[4] = {-1, -1, -1, -1};
  const uint8_t e6[6] = {1, 1, 1, 1, 1, 1};
  cell_t c;
  cell_init(&c, t->v, tv, vad, e6, fa, fi);
  double cen[3] = {0, 0, 0};
  for (int v = 0; v < 4; ++v)
    for (int k = 0; k < 3; ++k) cen[k] += 0.25 * t->v[3 * v + k];
  if ((double)c.pl[0][0] * cen[0] + (double)c.pl[0][1] * cen[1] + (double)c.pl[0][2] * cen[2] +
          (double)c.pl[0][3] < 0.0) {
    for (int k = 0; k < 3; ++k) {
      const float x = t->v[k];
      t->v[k] = t->v[3 + k];
      t->v[3 + k] = x;
    }
  }
}

/* the 8 tets of the midpoint subdivision: 4 at the corners, 4 around the
 * octahedron's diagonal m02-m13 */
static void pn_split(const pn_tet* t, pn_tet out[8]) {
  float m[4][4][3];
  for (int a = 0; a < 4; ++a)
    for (int b = 0; b < 4; ++b)
      for (int k = 0; k < 3; ++k)
        m[a][b][k] = (float)(0.5 * ((double)t->v[3 * a + k] + (double)t->v[3 * b + k]));
  static const int ix[8][4][2] = {
      {{0, 0}, {0, 1}, {0, 2}, {0, 3}}, {{0, 1}, {1, 1}, {1, 2}, {1, 3}},
      {{0, 2}, {1, 2}, {2, 2}, {2, 3}}, {{0, 3}, {1, 3}, {2, 3}, {3, 3}},
      {{0, 2}, {1, 3}, {0, 1}, {0, 3}}, {{0, 2}, {1, 3}, {0, 3}, {2, 3}},
      {{0, 2}, {1, 3}, {2, 3}, {1, 2}}, {{0, 2}, {1, 3}, {1, 2}, {0, 1}}};
  for (int q = 0; q < 8; ++q) {
    for (int v = 0; v < 4; ++v)
      for (int k = 0; k < 3; ++k) out[q].v[3 * v + k] = m[ix[q][v][0]][ix[q][v][1]][k];
    pn_orient(&out[q]);
  }
}

static int pn_meets_box(const pn_tet* t, const double* box) {
  for (int k = 0; k < 3; ++k) {
    double lo = t->v[k], hi = t->v[k];
    for (int v = 1; v < 4; ++v) {
      lo = fmin(lo, t->v[3 * v + k]);
      hi = fmax(hi, t->v[3 * v + k]);
    }
    if (hi < box[k] || lo > box[3 + k]) return 0;
  }
  return 1;
}

/* clips region tet t by the sites in ascending key (kv[0..m), sorted on
 * demand in chunks) until the next key exceeds the cell's radius; marks the
 * sites of the final cell's bisector faces in `hit`.  Returns the cell's
 * status. */
static int pn_clip_region(cell_t* c, const pn_tet* t, const float* site4, int i, pn_kv* kv,
                          int64_t m, int64_t* sorted, double margin, uint8_t* hit) {
  const int32_t tv[4] = {0, 1, 2, 3};
  const int32_t vad[4] = {1, 1, 1, 1}, fa[4] = {1, 1, 1, 1}, fi[4] = {-1, -1, -1, -1};
  const uint8_t e6[6] = {1, 1, 1, 1, 1, 1};
  c->pred_mode = 2;
  c->n_pred = c->n_esc = c->n_unc = c->n_flip = 0;
  c->seed_id = i;
  memcpy(c->seed, site4 + 4 * (int64_t)i, sizeof(float) * 4);
  cell_init(c, t->v, tv, vad, e6, fa, fi);
  double R = pn_radius(c);
  int64_t pos = 0;
  while (pos < m && c->status == ORC_SUCCESS) {
    if (pos == *sorted) {
      /* next chunk of the smallest keys */
      int64_t want = *sorted == 0 ? 256 : (m - *sorted);
      if (want > m - *sorted) want = m - *sorted;
      pn_select(kv + *sorted, m - *sorted, want);
      qsort(kv + *sorted, (size_t)want, sizeof(pn_kv), pn_cmp);
      *sorted += want;
    }
    if (kv[pos].key * (1.0 - 1e-9) - margin > R) break;
    if (c->nb_p > ORC_MAX_P - 8 || c->nb_e > ORC_MAX_E - 48) pn_compact(c);
    const int nb_p0 = c->nb_p;
    clip_by_site(c, site4, kv[pos].id);
    if (c->status == ORC_SUCCESS && c->nb_p > nb_p0) R = pn_radius(c);
    ++pos;
  }
  if (c->status != ORC_SUCCESS) return c->status;
  uint8_t used[ORC_MAX_P];
  memset(used, 0, sizeof(used));
  for (int v = 0; v < c->nb_v; ++v)
    for (int q = 0; q < 3; ++q) used[c->ver[v][q]] = 1;
  for (int p = 4; p < c->nb_p; ++p)
    if (used[p]) hit[c->id2[p][0] == i ? c->id2[p][1] : c->id2[p][0]] = 1;
  return ORC_SUCCESS;
}

int orc_power_neighbors(int n_site, const float* site4, const double* region, int max_nbr,
                        int32_t* nbr, int32_t* count, int n_threads) {
  /* a regular tet around the region's box: vertices c + s (+-1, +-1, +-1)
   * with an even number of minus signs; its inradius s / sqrt(3) exceeds
   * the box's half diagonal.  A cell beyond the clipper's capacities (a
   * large power cell with many faces) is computed again on the 8 tets of
   * the region's midpoint subdivision (those that meet the box), recursively:
   * a face of the cell inside the box lies in one of them, so the union of
   * their neighbours is the cell's. */
  double c0[3], h2 = 0.0, L = 0.0;
  for (int a = 0; a < 3; ++a) {
    c0[a] = 0.5 * (region[a] + region[3 + a]);
    h2 += 0.25 * (region[3 + a] - region[a]) * (region[3 + a] - region[a]);
    L = fmax(L, fmax(fabs(region[a]), fabs(region[3 + a])));
  }
  const double s = sqrt(h2) * sqrt(3.0) * 1.05 + 1.0;
  static const double sg[4][3] = {{1, 1, 1}, {1, -1, -1}, {-1, 1, -1}, {-1, -1, 1}};
  pn_tet root;
  for (int v = 0; v < 4; ++v)
    for (int a = 0; a < 3; ++a) root.v[3 * v + a] = (float)(c0[a] + s * sg[v][a]);
  pn_orient(&root);
  /* rounding of the float bisector planes against the exact keys, and of
   * the radius: a site whose key exceeds R + margin cannot cut the cell */
  const double margin = 1e-5 * (L + 2.0 * sqrt(h2)) + 1e-12;
  enum { kMaxDepth = 7, kStack = 8 * kMaxDepth + 1 };
  int bad = 0;
#ifdef _OPENMP
  if (n_threads > 0) omp_set_num_threads(n_threads);
#pragma omp parallel reduction(+ : bad)
#endif
  {
    pn_kv* kv = (pn_kv*)malloc(sizeof(pn_kv) * (size_t)(n_site > 0 ? n_site : 1));
    uint8_t* hit = (uint8_t*)calloc((size_t)(n_site > 0 ? n_site : 1), 1);
    cell_t* c = (cell_t*)malloc(sizeof(cell_t));
    pn_tet stack[kStack];
    int depth_of[kStack];
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 16)
#endif
    for (int i = 0; i < n_site; ++i) {
      const float* si = site4 + 4 * (int64_t)i;
      int64_t m = 0;
      int hidden = 0;
      for (int j = 0; j < n_site; ++j) {
        if (j == i) continue;
        const float* sj = site4 + 4 * (int64_t)j;
        double dx = (double)sj[0] - si[0], dy = (double)sj[1] - si[1], dz = (double)sj[2] - si[2];
        double d2 = dx * dx + dy * dy + dz * dz;
        if (d2 == 0.0) {
          if ((double)sj[3] > (double)si[3]) hidden = 1;
          continue;
        }
        kv[m].key = (d2 - (double)sj[3] + (double)si[3]) / (2.0 * sqrt(d2));
        kv[m].id = j;
        ++m;
      }
      int32_t* row = nbr + (int64_t)i * max_nbr;
      for (int r = 0; r < max_nbr; ++r) row[r] = -1;
      if (hidden) {
        count[i] = -1;
        continue;
      }
      int64_t sorted = 0;
      int nonempty = 0, failed = 0, top = 0;
      stack[top] = root;
      depth_of[top++] = 0;
      while (top > 0 && !failed) {
        const pn_tet t = stack[--top];
        const int depth = depth_of[top];
        const int st = pn_clip_region(c, &t, site4, i, kv, m, &sorted, margin, hit);
        if (st == ORC_SUCCESS) {
          nonempty = 1;
        } else if (st != ORC_NO_INTERSECTION) {
          if (depth >= kMaxDepth) {
            failed = 1;
            break;
          }
          pn_tet sub[8];
          pn_split(&t, sub);
          for (int q = 0; q < 8; ++q) {
            if (!pn_meets_box(&sub[q], region)) continue;
            stack[top] = sub[q];
            depth_of[top++] = depth + 1;
          }
        }
      }
      /* the marked sites (all among the clipped, kv[0..sorted)), and the
       * marks cleared */
      int n = 0, over = 0;
      for (int64_t q = 0; q < sorted; ++q) {
        const int j = kv[q].id;
        if (!hit[j]) continue;
        hit[j] = 0;
        if (n < max_nbr) row[n] = j;
        else over = 1;
        ++n;
      }
      if (failed) {
        count[i] = -2;
        ++bad;
        for (int r = 0; r < max_nbr; ++r) row[r] = -1;
        continue;
      }
      if (over) {
        count[i] = -3;
        ++bad;
        for (int r = 0; r < max_nbr; ++r) row[r] = -1;
        continue;
      }
      if (!nonempty) {
        count[i] = -1;
        continue;
      }
      for (int a = 1; a < n; ++a) {
        int32_t x = row[a];
        int b = a - 1;
        while (b >= 0 && row[b] > x) {
          row[b + 1] = row[b];
          --b;
        }
        row[b + 1] = x;
      }
      count[i] = n;
    }
    free(c);
    free(hit);
    free(kv);
  }
  return bad;
}

/* ------------------------------------------------------------------ */
/* canonical topology hash of emitted cells: the sum over vertices of  */
/* a splitmix64 chain over the sorted face keys (id2) of the vertex's  */
/* three planes and its #adj -- independent of plane and vertex order */
/* ------------------------------------------------------------------ */
static uint64_t orc_mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

void orc_topology_hashes(int64_t n, const orc_cell_header* h, const uint8_t* payload,
                         uint64_t* out) {
  for (int64_t q = 0; q < n; ++q) {
    out[q] = 0;
    if (h[q].status != ORC_SUCCESS) continue;
    const int nb_v = h[q].nb_v, nb_p = h[q].nb_p;
    const uint8_t* rec = payload + h[q].offset;
    const int32_t* id2 = (const int32_t*)(rec + 16 * (size_t)nb_p);
    const uint8_t* ver = rec + 16 * (size_t)nb_p + al16(8 * (size_t)nb_p);
    uint64_t sum = 0;
    for (int v = 0; v < nb_v; ++v) {
      uint64_t k[3];
      for (int a = 0; a < 3; ++a) {
        const int p = ver[4 * v + a];
        k[a] = ((uint64_t)(uint32_t)id2[2 * p] << 32) | (uint32_t)id2[2 * p + 1];
      }
      for (int a = 1; a < 3; ++a)
        for (int b = a; b > 0 && k[b - 1] > k[b]; --b) {
          uint64_t t = k[b];
          k[b] = k[b - 1];
          k[b - 1] = t;
        }
      uint64_t hv = orc_mix64(k[0]);
      hv = orc_mix64(hv ^ k[1]);
      hv = orc_mix64(hv ^ k[2]);
      hv = orc_mix64(hv ^ (uint64_t)ver[4 * v + 3]);
      sum += hv;
    }
    out[q] = sum;
  }
}
