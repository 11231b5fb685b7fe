// rpd_api.cpp -- the C ABI of include/rpd_gb300.h: context, device buffers,
// one CUDA stream, and the orchestration of the kernels.
//
// Replaces the host driver compute_clipped_voro_diagram_GPU
// (src/rpd3d/voronoi.cu:455-795): instead of pitched AoS->SoA copies, dense
// n_site x n_tet relation matrices, a host gather loop and a copy of every
// 3.4 KB thread slot back to the host, everything stays on the device --
// neighbour lists, candidate pairs (per-tet CSR), cells (compact records) --
// and only emitted cells are copied out on request.  Errors are returned,
// never exit()ed (the reference exits on CUDA errors, voronoi.cu:31-37).

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <random>
#include <string>
#include <vector>

#include "../../include/rpd_gb300.h"
#include "rpd_common.cuh"
#include "rpd_kernels.cuh"

using namespace rpd;

#include "rpd_ctx.hpp"

namespace {

rpd_status fail(rpd_ctx* c, rpd_status s, const std::string& msg) {
  if (c) c->err = msg;
  return s;
}

rpd_status cuda_fail(rpd_ctx* c, cudaError_t e, const char* where) {
  cudaGetLastError();  // clear non-sticky errors
  return fail(c, e == cudaErrorMemoryAllocation ? RPD_ERR_OUT_OF_MEMORY : RPD_ERR_CUDA,
              std::string(where) + ": " + cudaGetErrorString(e));
}

// The small device->host reads of set-up and compute (counts, sizes,
// statistics).  add() queues a one-block kernel that stores the bytes into
// the context's page-locked, device-mapped staging memory, in stream order
// like cudaMemcpyAsync; wait() synchronizes the stream and hands them to
// their destinations.  The copy engines are not involved, so another
// context's bulk copy of its cells (queued on an engine) holds none of
// them up.
struct SmallReads {
  rpd_ctx* c;
  cudaStream_t st;
  struct Read {
    void* dst;
    size_t off, n;
  } r[8];
  int nr = 0;
  size_t used = 0;
  SmallReads(rpd_ctx* ctx, cudaStream_t s) : c(ctx), st(s) {}
  cudaError_t add(void* dst, const void* src, size_t n) {
    const size_t off = (used + 15) & ~(size_t)15;
    if (nr == 8 || off + n > rpd_ctx::kStageBytes) return cudaErrorInvalidValue;
    const cudaError_t e = launch_stage_bytes(src, c->stage_dev + off, n, st);
    if (e != cudaSuccess) return e;
    r[nr++] = {dst, off, n};
    used = off + n;
    return cudaSuccess;
  }
  cudaError_t wait() {
    const cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return e;
    for (int i = 0; i < nr; ++i) std::memcpy(r[i].dst, c->stage_host + r[i].off, r[i].n);
    nr = 0;
    used = 0;
    return cudaSuccess;
  }
};

#define CK(expr, where)                          \
  do {                                           \
    cudaError_t _e = (expr);                     \
    if (_e != cudaSuccess) return cuda_fail(c, _e, where); \
  } while (0)

// double -> (hi, lo) float pair, hi + lo ~ x to about 48 bits
float2 split_df(double x) {
  const float h = (float)x;
  return make_float2(h, (float)(x - (double)h));
}

Grid make_grid(const double* lo, const double* hi, long long n_items, double per_cell) {
  Grid g;
  double ext[3], vol = 1.0;
  for (int a = 0; a < 3; ++a) {
    ext[a] = std::max(hi[a] - lo[a], 1e-9);
    vol *= ext[a];
  }
  double cell = std::cbrt(vol * per_cell / (double)std::max<long long>(n_items, 1));
  double maxe = std::max(ext[0], std::max(ext[1], ext[2]));
  cell = std::max(cell, maxe / 512.0);
  int n[3];
  for (int a = 0; a < 3; ++a) n[a] = std::max(1, (int)std::ceil(ext[a] / cell));
  while ((long long)n[0] * n[1] * n[2] > (1ll << 26)) {
    cell *= 1.25;
    for (int a = 0; a < 3; ++a) n[a] = std::max(1, (int)std::ceil(ext[a] / cell));
  }
  g.lo = make_float3((float)lo[0], (float)lo[1], (float)lo[2]);
  g.cell = (float)cell;
  g.inv_cell = (float)(1.0 / cell);
  g.nx = n[0];
  g.ny = n[1];
  g.nz = n[2];
  return g;
}

// bf16 features of n_rows pairs (pair_index[0..n_rows), or all pairs) into
// c->feat; with `target`, the labels log2(max(consumed, 1)) as well
rpd_status pair_features(rpd_ctx* c, const int32_t* pair_index, long long n_rows, float* target) {
  cudaStream_t st = c->stream;
  if (c->n_bverts < 0) {  // boundary vertices, from the marks of rpd_set_mesh
    CK(c->bverts.ensure((size_t)c->n_vert), "alloc");
    CK(c->prep_hist.ensure(kRadiusBins), "alloc");
    CK(boundary_list(c->bmark.ptr, c->vert3f.ptr, c->n_vert, c->bverts.ptr, c->prep_hist.ptr, st),
       "boundary");
    int32_t nb = 0;
    CK(cudaMemcpyAsync(&nb, c->prep_hist.ptr, sizeof(nb), cudaMemcpyDeviceToHost, st), "D2H");
    CK(cudaStreamSynchronize(st), "boundary sync");
    c->n_bverts = nb;
  }
  if (!c->bdist_valid) {
    CK(c->site_bdist.ensure((size_t)c->n_site), "alloc");
    CK(launch_boundary_distance(c->site4f.ptr, c->n_site, c->bverts.ptr, c->n_bverts,
                                c->site_bdist.ptr, st), "boundary distance");
    c->bdist_valid = true;
  }
  CK(c->feat.ensure((size_t)std::max<long long>(n_rows, 1) * kMlpFeatures), "alloc features");
  FeatureParams fp;
  fp.pair_tet = c->pair_tet.ptr;
  fp.pair_site = c->pair_site.ptr;
  fp.pair_index = pair_index;
  fp.n_pairs = n_rows;
  fp.site4f = c->site4f.ptr;
  fp.vert3f = c->vert3f.ptr;
  fp.tets = c->tets.ptr;
  fp.centroid = c->centroid.ptr;
  fp.keys = c->nbr_keys.ptr;
  fp.k = c->k;
  fp.cell_of = c->s_cell_of.ptr;
  fp.cell_count = c->s_cell_count.ptr;
  fp.site_bdist = c->site_bdist.ptr;
  const double h = std::cbrt(std::max(c->mesh_volume, 1e-300) / (double)std::max(c->n_site, 1));
  fp.inv_h = (float)(1.0 / h);
  fp.X = c->feat.ptr;
  fp.consumed = target ? c->consumed.ptr : nullptr;
  fp.target = target;
  CK(launch_pair_features(fp, st), "features");
  c->n_feat_rows = n_rows;
  return RPD_OK;
}

bool certify_on(const rpd_ctx* c) { return c->cfg.certify != 0; }

MlpWeights mlp_view(const rpd_ctx* c) {
  return mlp_weights_view(c->mlp_params.ptr, c->mlp_W1T.ptr, c->mlp_W2.ptr, c->mlp_W2T.ptr);
}

rpd_status mlp_alloc(rpd_ctx* c) {
  CK(c->mlp_params.ensure(kMlpParams), "alloc");
  CK(c->mlp_grads.ensure(kMlpParams), "alloc");
  CK(c->mlp_m.ensure(kMlpParams), "alloc");
  CK(c->mlp_v.ensure(kMlpParams), "alloc");
  CK(c->mlp_W1T.ensure(kMlpFeatures * kMlpHidden), "alloc");
  CK(c->mlp_W2.ensure(kMlpHidden * kMlpHidden), "alloc");
  CK(c->mlp_W2T.ensure(kMlpHidden * kMlpHidden), "alloc");
  return RPD_OK;
}

}  // namespace

extern "C" {

const char* rpd_status_string(rpd_status s) {
  switch (s) {
    case RPD_OK: return "ok";
    case RPD_ERR_INVALID_ARGUMENT: return "invalid argument";
    case RPD_ERR_CUDA: return "CUDA error";
    case RPD_ERR_OUT_OF_MEMORY: return "out of device memory";
    case RPD_ERR_NOT_READY: return "inputs not set";
    case RPD_ERR_CAPACITY: return "capacity exceeded";
    case RPD_ERR_NO_DEVICE: return "no CUDA device";
  }
  return "unknown status";
}

size_t rpd_payload_bytes(int nb_v, int nb_p, int nb_e) {
  return PayloadLayout(nb_v, nb_p, nb_e).total;
}

size_t rpd_topo_bytes(int nb_v, int nb_p, int nb_e) { return TopoLayout(nb_v, nb_p, nb_e).total; }

void rpd_config_default(rpd_config* cfg) {
  if (!cfg) return;
  std::memset(cfg, 0, sizeof(*cfg));
  cfg->device = 0;
  cfg->predicate_mode = RPD_PRED_FP32_FILTER;
  cfg->neighbor_source = RPD_NEIGH_KNN;
  cfg->knn_k = 64;
  cfg->clip_order = RPD_ORDER_SITE_ID;
  cfg->compute_geometry = 1;
  cfg->warps_per_block = 0;
  cfg->blocks_per_sm = 0;
  cfg->topology_hash = 1;
  cfg->exact_lists = 1;
}

static bool config_valid(const rpd_config& c0) {
  if (c0.predicate_mode != RPD_PRED_FP64 && c0.predicate_mode != RPD_PRED_FP32_FILTER &&
      c0.predicate_mode != RPD_PRED_EXACT)
    return false;
  if (c0.neighbor_source != RPD_NEIGH_USER && c0.neighbor_source != RPD_NEIGH_KNN) return false;
  if (c0.neighbor_source == RPD_NEIGH_KNN && (c0.knn_k < 1 || c0.knn_k > 128)) return false;
  if (c0.warps_per_block < 0 || c0.warps_per_block > kClipMaxThreads / 32 || c0.blocks_per_sm < 0)
    return false;
  if (c0.certify && c0.neighbor_source != RPD_NEIGH_KNN) return false;
  if (c0.clip_variant < 0 || c0.clip_variant > 2) return false;
  if (c0.box_planes < 0 || c0.box_planes > 128) return false;
  if (c0.learned_k < 0 || c0.learned_k > 1 || (c0.learned_k && !c0.certify)) return false;
  if (c0.topology_hash < 0 || c0.topology_hash > 1) return false;
  if (c0.exact_lists < 0 || c0.exact_lists > 1) return false;
  return true;
}

rpd_status rpd_create(const rpd_config* cfg, rpd_ctx** out) {
  if (!out) return RPD_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  rpd_config c0;
  rpd_config_default(&c0);
  if (cfg) c0 = *cfg;
  if (!config_valid(c0)) return RPD_ERR_INVALID_ARGUMENT;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) {
    cudaGetLastError();
    return RPD_ERR_NO_DEVICE;
  }
  if (c0.device < 0 || c0.device >= ndev) return RPD_ERR_INVALID_ARGUMENT;
  rpd_ctx* c = new rpd_ctx();
  c->cfg = c0;
  c->device = c0.device;
  if (cudaSetDevice(c->device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    delete c;
    return RPD_ERR_CUDA;
  }
  for (int i = 0; i < kEvCount; ++i) cudaEventCreate(&c->ev[i]);
  cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, c->device);
  void* stage = nullptr;
  if (cudaHostAlloc(&stage, rpd_ctx::kStageBytes, cudaHostAllocMapped) != cudaSuccess ||
      cudaHostGetDevicePointer((void**)&c->stage_dev, stage, 0) != cudaSuccess) {
    cudaGetLastError();
    if (stage) cudaFreeHost(stage);
    cudaStreamDestroy(c->stream);
    for (int i = 0; i < kEvCount; ++i)
      if (c->ev[i]) cudaEventDestroy(c->ev[i]);
    delete c;
    return RPD_ERR_CUDA;
  }
  c->stage_host = static_cast<uint8_t*>(stage);
  *out = c;
  return RPD_OK;
}

void rpd_destroy(rpd_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  c->vert3f.release(); c->vert3d.release(); c->tets.release(); c->v_adjs.release();
  c->f_adjs.release(); c->f_ids.release(); c->e_adj6.release(); c->tet_class.release();
  c->site4f.release(); c->site4d.release(); c->flags.release();
  c->nbr.release(); c->nbr_dist.release(); c->site_klen.release(); c->reclip_idx.release();
  c->topo_hash.release(); c->nbr_ref_tmp.release(); c->knn_status.release(); c->nbr_keys.release();
  c->nbr_bound.release(); c->site_need.release(); c->site_row.release(); c->ext_sites.release();
  c->site_flag.release(); c->site_pos.release(); c->ext_idx.release(); c->ext_nbr.release();
  c->ext_len.release();
  c->ext_keys.release(); c->ext_bound.release(); c->ext_off.release();
  c->s_cell_of.release(); c->s_cell_count.release(); c->s_cell_start.release();
  c->s_cell_fill.release(); c->s_cell_items.release();
  c->t_cell_of.release(); c->t_cell_count.release(); c->t_cell_start.release();
  c->t_cell_fill.release(); c->t_cell_items.release();
  c->centroid.release(); c->site_box.release(); c->site_planes.release();
  c->site_nplanes.release(); c->pair_ntasks.release(); c->pair_taskoff.release(); c->scan_tmp.release();
  c->pair_buf.release(); c->tet_count.release(); c->tet_offsets.release();
  c->tet_fill.release(); c->pair_site.release(); c->pair_tet.release();
  c->pair_headers.release(); c->cells.release(); c->payload.release();
  c->flag_tmp.release(); c->pos_tmp.release(); c->scratch.release(); c->n_out.release();
  for (int i = 0; i < kEvCount; ++i)
    if (c->ev[i]) cudaEventDestroy(c->ev[i]);
  if (c->stream) cudaStreamDestroy(c->stream);
  if (c->stage_host) cudaFreeHost(c->stage_host);
  delete c;
}

rpd_status rpd_get_config(const rpd_ctx* c, rpd_config* cfg) {
  if (!c || !cfg) return RPD_ERR_INVALID_ARGUMENT;
  *cfg = c->cfg;
  return RPD_OK;
}

rpd_status rpd_get_mesh_info(const rpd_ctx* c, rpd_mesh_info* info) {
  if (!c || !info) return RPD_ERR_INVALID_ARGUMENT;
  if (!c->has_mesh) return RPD_ERR_NOT_READY;
  *info = rpd_mesh_info{};
  info->n_vert = c->n_vert;
  info->n_tet = c->n_tet;
  for (int a = 0; a < 3; ++a) {
    info->lo[a] = c->mesh_lo[a];
    info->hi[a] = c->mesh_hi[a];
  }
  info->volume = c->mesh_volume;
  info->tet_radius = c->tet_radius;
  for (int k = 0; k < 2; ++k) {
    info->class_count[k] = c->class_count[k];
    info->class_radius[k] = c->class_radius[k];
  }
  return RPD_OK;
}

rpd_status rpd_set_config(rpd_ctx* c, const rpd_config* cfg) {
  if (!c || !cfg) return RPD_ERR_INVALID_ARGUMENT;
  if (!config_valid(*cfg)) return fail(c, RPD_ERR_INVALID_ARGUMENT, "rpd_set_config: invalid configuration");
  if (cfg->device != c->device)
    return fail(c, RPD_ERR_INVALID_ARGUMENT, "rpd_set_config: a context stays on its device");
  if (cfg->neighbor_source != c->cfg.neighbor_source || cfg->knn_k != c->cfg.knn_k)
    c->has_site_klen = false;
  c->cfg = *cfg;
  c->has_result = false;
  return RPD_OK;
}

const char* rpd_last_error(const rpd_ctx* c) { return c ? c->err.c_str() : "no context"; }

rpd_status rpd_set_mesh(rpd_ctx* c, const double* xyz, int n_vert, const int32_t* tets, int n_tet,
                        const int32_t* v_adjs, const uint8_t* e_adj6, const int32_t* f_adjs,
                        const int32_t* f_ids) {
  if (!c) return RPD_ERR_INVALID_ARGUMENT;
  if (n_vert <= 0 || n_tet <= 0 || !xyz || !tets || !v_adjs || !e_adj6 || !f_adjs || !f_ids)
    return fail(c, RPD_ERR_INVALID_ARGUMENT, "rpd_set_mesh: empty mesh or null buffer");
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  c->has_mesh = false;
  c->has_result = false;
  c->cells_for_mesh = false;
  cudaStream_t st = c->stream;
  // the raw arrays go to the device; everything derived is computed there
  CK(c->vert3d.ensure((size_t)n_vert * 3), "alloc vert3d");
  CK(c->vert3f.ensure((size_t)n_vert * 3), "alloc vert3f");
  CK(c->vert2.ensure((size_t)n_vert * 3), "alloc vert2");
  CK(c->tets.ensure(n_tet), "alloc tets");
  CK(c->v_adjs.ensure(n_vert), "alloc v_adjs");
  CK(c->e_adj6.ensure((size_t)n_tet * 6), "alloc e_adj6");
  CK(c->f_adjs.ensure((size_t)n_tet * 4), "alloc f_adjs");
  CK(c->f_ids.ensure((size_t)n_tet * 4), "alloc f_ids");
  CK(c->tet_class.ensure(n_tet), "alloc classes");
  CK(c->tet_rad.ensure(n_tet), "alloc radii");
  CK(c->bmark.ensure(n_vert), "alloc marks");
  CK(c->face2.ensure((size_t)n_tet * 16), "alloc faces");
  CK(c->prep.ensure(1), "alloc");
  CK(c->prep_hist.ensure(kRadiusBins), "alloc");
  CK(cudaMemcpyAsync(c->vert3d.ptr, xyz, (size_t)n_vert * 24, cudaMemcpyHostToDevice, st), "H2D vert");
  CK(cudaMemcpyAsync(c->tets.ptr, tets, (size_t)n_tet * 16, cudaMemcpyHostToDevice, st), "H2D tets");
  CK(cudaMemcpyAsync(c->v_adjs.ptr, v_adjs, (size_t)n_vert * 4, cudaMemcpyHostToDevice, st), "H2D v_adjs");
  CK(cudaMemcpyAsync(c->e_adj6.ptr, e_adj6, (size_t)n_tet * 6, cudaMemcpyHostToDevice, st), "H2D e_adj6");
  CK(cudaMemcpyAsync(c->f_adjs.ptr, f_adjs, (size_t)n_tet * 16, cudaMemcpyHostToDevice, st), "H2D f_adjs");
  CK(cudaMemcpyAsync(c->f_ids.ptr, f_ids, (size_t)n_tet * 16, cudaMemcpyHostToDevice, st), "H2D f_ids");
  CK(mesh_prep_init(c->prep.ptr, st), "prep");
  CK(mesh_prep_geometry(c->vert3d.ptr, n_vert, c->tets.ptr, c->f_adjs.ptr, n_tet, c->vert3f.ptr,
                        c->vert2.ptr, c->tet_rad.ptr, c->bmark.ptr, c->prep.ptr, st), "prep");
  MeshPrepOut po;
  SmallReads rd(c, st);
  CK(rd.add(&po, c->prep.ptr, sizeof(po)), "D2H");
  CK(rd.wait(), "set_mesh sync");
  if (po.bad & 1u) return fail(c, RPD_ERR_INVALID_ARGUMENT, "rpd_set_mesh: non-finite vertex");
  if (po.bad & 2u) return fail(c, RPD_ERR_INVALID_ARGUMENT, "rpd_set_mesh: vertex id out of range");
  const double rmax = key_to_double(po.rmax_key);
  // two radius classes: up to the 99.5th-percentile radius (upper edge of
  // its histogram bin), and the rest
  std::vector<int32_t> hist(kRadiusBins);
  CK(mesh_prep_histogram(c->tet_rad.ptr, n_tet, rmax, c->prep_hist.ptr, st), "histogram");
  CK(rd.add(hist.data(), c->prep_hist.ptr, sizeof(int32_t) * kRadiusBins), "D2H");
  CK(rd.wait(), "set_mesh sync");
  const long long want = std::min<long long>(n_tet, (long long)std::ceil(0.995 * (double)n_tet));
  long long acc = 0;
  int bin = kRadiusBins - 1;
  for (int b = 0; b < kRadiusBins; ++b) {
    acc += hist[(size_t)b];
    if (acc >= want) {
      bin = b;
      break;
    }
  }
  const double r0 = rmax * (double)(bin + 1) / (double)kRadiusBins;
  CK(mesh_prep_classify(c->tet_rad.ptr, n_tet, r0, c->tet_class.ptr, c->prep.ptr, st), "classes");
  CK(launch_tet_face_planes(c->vert3d.ptr, c->tets.ptr, n_tet, c->face2.ptr, st), "face planes");
  CK(rd.add(&po, c->prep.ptr, sizeof(po)), "D2H");
  CK(rd.wait(), "set_mesh sync");
  for (int k = 0; k < rpd_ctx::kClasses; ++k) {
    c->class_count[k] = k < 2 ? po.class_count[k] : 0;
    c->class_radius[k] = k < 2 && po.class_count[k] > 0 ? key_to_double(po.class_rmax_key[k]) : 0.0;
  }
  c->n_vert = n_vert;
  c->n_tet = n_tet;
  for (int a = 0; a < 3; ++a) {
    c->mesh_lo[a] = key_to_double(po.lo_key[a]);
    c->mesh_hi[a] = key_to_double(po.hi_key[a]);
  }
  c->tet_radius = rmax;
  c->mesh_volume = po.volume;
  c->n_bverts = -1;  // boundary vertex list built on first use
  c->bdist_valid = false;
  c->has_mesh = true;
  return RPD_OK;
}

rpd_status rpd_set_sites(rpd_ctx* c, const double* xyzw, int n_site, const uint32_t* flags) {
  if (!c) return RPD_ERR_INVALID_ARGUMENT;
  if (n_site <= 0 || !xyzw) return fail(c, RPD_ERR_INVALID_ARGUMENT, "rpd_set_sites: no sites");
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  std::vector<float> sf((size_t)n_site * 4);
  std::vector<uint32_t> fl((size_t)n_site, 1u);
  double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  float wmax = -INFINITY;
  for (long long i = 0; i < n_site; ++i) {
    for (int a = 0; a < 4; ++a) {
      double v = xyzw[4 * i + a];
      if (!std::isfinite(v)) return fail(c, RPD_ERR_INVALID_ARGUMENT, "rpd_set_sites: non-finite site");
      sf[4 * i + a] = (float)v;
    }
    for (int a = 0; a < 3; ++a) {
      lo[a] = std::min(lo[a], xyzw[4 * i + a]);
      hi[a] = std::max(hi[a], xyzw[4 * i + a]);
    }
    wmax = std::max(wmax, sf[4 * i + 3]);
    if (flags) fl[i] = flags[i];
  }
  CK(c->site4f.ensure(n_site), "alloc sites");
  CK(c->site4d.ensure((size_t)n_site * 4), "alloc sites");
  CK(c->site2.ensure((size_t)n_site * 4), "alloc sites");
  std::vector<float2> s2((size_t)n_site * 4);
  for (size_t i = 0; i < s2.size(); ++i) s2[i] = split_df(xyzw[i]);
  CK(c->flags.ensure(n_site), "alloc flags");
  cudaStream_t st = c->stream;
  CK(cudaMemcpyAsync(c->site4f.ptr, sf.data(), sf.size() * 4, cudaMemcpyHostToDevice, st), "H2D sites");
  CK(cudaMemcpyAsync(c->site4d.ptr, xyzw, (size_t)n_site * 32, cudaMemcpyHostToDevice, st), "H2D sites");
  CK(cudaMemcpyAsync(c->site2.ptr, s2.data(), s2.size() * sizeof(float2), cudaMemcpyHostToDevice, st), "H2D sites");
  CK(cudaMemcpyAsync(c->flags.ptr, fl.data(), (size_t)n_site * 4, cudaMemcpyHostToDevice, st), "H2D flags");
  CK(cudaStreamSynchronize(st), "set_sites sync");
  if (c->n_site != n_site) {
    c->has_user_nbr = false;
    c->has_site_klen = false;
    c->cells_for_mesh = false;  // site ids of the previous cells no longer apply
  }
  c->n_site = n_site;
  c->has_site_range = false;  // (a batch sets its meshes' ranges after this)
  for (int a = 0; a < 3; ++a) {
    c->site_lo[a] = lo[a];
    c->site_hi[a] = hi[a];
  }
  c->w_max = wmax;
  c->bdist_valid = false;
  c->has_sites = true;
  c->has_result = false;
  return RPD_OK;
}

rpd_status rpd_set_neighbors(rpd_ctx* c, const int32_t* nbr, int k, int layout) {
  if (!c) return RPD_ERR_INVALID_ARGUMENT;
  if (!c->has_sites) return fail(c, RPD_ERR_NOT_READY, "rpd_set_neighbors: set the sites first");
  if (!nbr || k < 0 || (layout != 0 && layout != 1))
    return fail(c, RPD_ERR_INVALID_ARGUMENT, "rpd_set_neighbors: bad arguments");
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  long long n = (long long)c->n_site * k;
  long long n_in = layout == 1 ? (long long)c->n_site * (k + 1) : n;
  for (long long i = 0; i < n_in; ++i)
    if (nbr[i] < -1 || nbr[i] >= c->n_site)
      return fail(c, RPD_ERR_INVALID_ARGUMENT, "rpd_set_neighbors: site id out of range");
  int kk = std::max(k, 1);
  CK(c->nbr.ensure((size_t)c->n_site * kk), "alloc nbr");
  cudaStream_t st = c->stream;
  if (k == 0) {
    CK(cudaMemsetAsync(c->nbr.ptr, 0xff, sizeof(int32_t) * (size_t)c->n_site, st), "memset nbr");
  } else if (layout == 0) {
    CK(cudaMemcpyAsync(c->nbr.ptr, nbr, sizeof(int32_t) * (size_t)n, cudaMemcpyHostToDevice, st), "H2D nbr");
  } else {
    CK(c->nbr_ref_tmp.ensure((size_t)n_in), "alloc nbr");
    CK(cudaMemcpyAsync(c->nbr_ref_tmp.ptr, nbr, sizeof(int32_t) * (size_t)n_in, cudaMemcpyHostToDevice, st), "H2D nbr");
    CK(neighbors_from_reference(c->nbr_ref_tmp.ptr, k, c->n_site, c->nbr.ptr, st), "nbr transpose");
  }
  CK(cudaStreamSynchronize(st), "set_neighbors sync");
  c->k = kk;
  c->has_user_nbr = true;
  c->has_result = false;
  return RPD_OK;
}

// CSR of the pairs, clipping (+ re-clip), epilogue, compaction and the
// statistics: the part of a compute after the candidate pairs are in
// pair_buf / tet_count (n_pairs of them)
// exact lists: rounds of longer lists for the sites whose cells the pass
// before left uncertified (list lengths of the rounds; the last round gives
// every site, which certifies any cell)
constexpr int kExtRounds = 3;
constexpr int kExtK[kExtRounds - 1] = {512, 4096};

static rpd_status finish_compute(rpd_ctx* c, bool knn, bool learned, rpd_stats* stats,
                                 bool extend_ok) {
  cudaStream_t st = c->stream;
  const int n_tet = c->n_tet;
  const int n_site = c->n_site;
  // lists the GPU built: bounds are known, and uncertified cells can be
  // given longer lists
  const bool extend = extend_ok && knn && c->cfg.exact_lists != 0;
  c->ext_valid = false;
  CK(c->tet_offsets.ensure((size_t)n_tet + 1), "alloc");
  CK(c->tet_fill.ensure(n_tet), "alloc");
  CK(c->scan_tmp.ensure(scan_temp_ints(std::max<long long>(c->n_pairs, n_tet)) + 16), "alloc");
  CK(scan_exclusive(c->tet_count.ptr, c->tet_offsets.ptr, n_tet, c->scan_tmp.ptr, st), "scan");
  CK(c->pair_site.ensure((size_t)c->n_pairs), "alloc");
  CK(c->pair_tet.ensure((size_t)c->n_pairs), "alloc");
  CK(pairs_to_csr(c->pair_buf.ptr, c->n_pairs, n_tet, c->tet_offsets.ptr, c->tet_fill.ptr,
                  c->pair_site.ptr, c->pair_tet.ptr,
                  reinterpret_cast<int32_t*>(c->scratch.ptr + 5), st), "csr");
  CK(cudaEventRecord(c->ev[kEvPairs], st), "event");

  // ---- learned list lengths: features and inference per pair
  const long long n_pairs = c->n_pairs;
  CK(cudaEventRecord(c->ev[kEvPred0], st), "event");
  if (learned && n_pairs > 0) {
    rpd_status fs = pair_features(c, nullptr, n_pairs, nullptr);
    if (fs != RPD_OK) return fs;
    CK(c->pair_klen.ensure((size_t)n_pairs), "alloc");
    CK(launch_mlp_predict(c->feat.ptr, nullptr, n_pairs, mlp_view(c), c->mlp_margin, 1, c->k,
                          c->pair_klen.ptr, nullptr, st), "predict");
  }
  const bool use_pair_k = !learned && certify_on(c) && c->n_user_pair_k >= 0;
  if (use_pair_k && c->n_user_pair_k != n_pairs)
    return fail(c, RPD_ERR_INVALID_ARGUMENT, "rpd_compute: rpd_set_pair_k lengths do not match the pairs");
  CK(cudaEventRecord(c->ev[kEvPred1], st), "event");
  c->last_learned = learned;
  if (c->want_consumed) CK(c->consumed.ensure((size_t)std::max<long long>(n_pairs, 1)), "alloc");

  // ---- clipping
  CK(c->pair_headers.ensure((size_t)std::max<long long>(n_pairs, 1)), "alloc headers");
  CK(c->topo_hash.ensure((size_t)std::max<long long>(n_pairs, 1)), "alloc hashes");
  long long pcap = c->payload_cap_hint > 0 ? c->payload_cap_hint
                                           : std::max<long long>(1 << 24, 640ll * n_pairs);
  const int warps = c->cfg.warps_per_block > 0 ? c->cfg.warps_per_block : 4;
  const int certify = c->cfg.certify ? 1 : 0;
  int bps = c->cfg.blocks_per_sm;
  const int variant = c->cfg.clip_variant;
  if (bps <= 0) bps = clip_blocks_per_sm_cert(c->cfg.predicate_mode, certify, warps, variant);
  int blocks = std::max(1, c->num_sms * bps);
  // certificate margin: 16u (L + D), L the largest coordinate magnitude,
  // D the largest distance between two sites
  double L = 0.0, D2 = 0.0;
  for (int a = 0; a < 3; ++a) {
    L = std::max(L, std::max(std::fabs(c->site_lo[a]), std::fabs(c->site_hi[a])));
    L = std::max(L, std::max(std::fabs(c->mesh_lo[a]), std::fabs(c->mesh_hi[a])));
    D2 += (c->site_hi[a] - c->site_lo[a]) * (c->site_hi[a] - c->site_lo[a]);
  }
  const float cert_margin = (float)(16.0 * std::ldexp(1.0, -24) * (L + std::sqrt(D2)) + 1e-30);
  c->n_reclipped = 0;
  long long n_ext_sites = 0, n_cert_reclipped = 0;
  int n_ext_rounds = 0, ext_longest = 0;
  float ms_ext_lists = 0.f;
  if (extend) {
    CK(c->site_need.ensure((size_t)n_site), "alloc");
    CK(c->site_row.ensure((size_t)n_site), "alloc");
    CK(c->ext_sites.ensure((size_t)n_site), "alloc");
    CK(c->site_flag.ensure((size_t)n_site), "alloc");
    CK(c->site_pos.ensure((size_t)n_site + 1), "alloc");
    CK(c->scan_tmp.ensure(scan_temp_ints(std::max<long long>(std::max<long long>(n_pairs, n_tet),
                                                             n_site)) + 16), "alloc");
  }
  for (int attempt = 0; attempt < 3; ++attempt) {
    CK(cudaMemsetAsync(c->scratch.ptr + 28, 0, 4 * sizeof(unsigned long long), st), "memset");
    if (extend) {
      CK(cudaMemsetAsync(c->site_need.ptr, 0, sizeof(unsigned int) * (size_t)n_site, st), "memset");
      CK(cudaMemsetAsync(c->site_row.ptr, 0xff, sizeof(int32_t) * (size_t)n_site, st), "memset");
      c->ext_used = 0;
      c->ext_rows = 0;
      n_ext_sites = n_cert_reclipped = 0;
      n_ext_rounds = ext_longest = 0;
      ms_ext_lists = 0.f;
    }
    CK(c->payload.ensure((size_t)pcap), "alloc payload");
    CK(cudaMemsetAsync(c->scratch.ptr, 0, 4 * sizeof(unsigned long long), st), "memset");
    ClipParams p;
    p.vert3f = c->vert3f.ptr;
    p.vert3d = c->vert3d.ptr;
    p.tets = c->tets.ptr;
    p.v_adjs = c->v_adjs.ptr;
    p.tet_xyz = c->tet_xyz.ptr;
    p.tet_vadj = c->tet_vadj.ptr;
    p.e_adj6 = c->e_adj6.ptr;
    p.f_adjs = c->f_adjs.ptr;
    p.f_ids = c->f_ids.ptr;
    p.site4f = c->site4f.ptr;
    p.site4d = c->site4d.ptr;
    p.vert2 = c->vert2.ptr;
    p.site2 = c->site2.ptr;
    p.nbr = certify ? c->nbr_dist.ptr : c->nbr.ptr;
    p.k = c->k;
    p.pair_tet = c->pair_tet.ptr;
    p.pair_site = c->pair_site.ptr;
    p.n_pairs = n_pairs;
    p.headers = c->pair_headers.ptr;
    p.payload = c->payload.ptr;
    p.payload_cursor = c->scratch.ptr + 0;
    p.payload_cap = (unsigned long long)c->payload.cap;
    p.work = c->scratch.ptr + 1;
    p.counters = c->scratch.ptr + 2;
    p.exact_counters = c->scratch.ptr + 29;
    p.geometry = c->cfg.compute_geometry;
    p.keys = certify ? c->nbr_keys.ptr : nullptr;
    p.site_klen = (certify && c->has_site_klen && !learned && !use_pair_k) ? c->site_klen.ptr : nullptr;
    p.pair_klen = learned ? c->pair_klen.ptr : (use_pair_k ? c->user_pair_k.ptr : nullptr);
    p.lazy_cert = (learned || use_pair_k) ? 1 : 0;
    p.misses = c->scratch.ptr + 28;
    p.uncertified = c->scratch.ptr + 31;
    p.consumed = (certify && c->want_consumed) ? c->consumed.ptr : nullptr;
    p.cert_margin = cert_margin;
    p.pair_index = nullptr;
    p.n_work = n_pairs;
    p.topo_hash = c->cfg.topology_hash ? c->topo_hash.ptr : nullptr;
    p.uncertified = nullptr;  // counted at the compaction, after every round
    p.nbr_bound = knn ? c->nbr_bound.ptr : nullptr;
    p.site_row = nullptr;  // base lists only in the first pass
    p.ext_nbr = nullptr;
    p.ext_keys = nullptr;
    p.ext_off = nullptr;
    p.ext_len = nullptr;
    p.ext_bound = nullptr;
    CK(cudaEventRecord(c->ev[kEvClipK0], st), "event");
    if (n_pairs > 0) CK(launch_clip_cells(p, c->cfg.predicate_mode, certify, variant, blocks, warps, st), "clip");
    CK(cudaEventRecord(c->ev[kEvClipK1], st), "event");
    if ((p.site_klen || p.pair_klen) && n_pairs > 0) {
      // cells whose shortened list was not enough: clip them again whole
      CK(c->flag_tmp.ensure((size_t)n_pairs + 1), "alloc");
      CK(c->pos_tmp.ensure((size_t)n_pairs + 1), "alloc");
      CK(c->reclip_idx.ensure((size_t)n_pairs), "alloc");
      CK(c->scan_tmp.ensure(scan_temp_ints(std::max<long long>(n_pairs, n_tet)) + 16), "alloc");
      CK(select_pairs(c->pair_headers.ptr, n_pairs, kSecurityRadiusNotReached, c->flag_tmp.ptr,
                      c->pos_tmp.ptr, c->scan_tmp.ptr, c->reclip_idx.ptr, st), "select");
      int32_t n_re = 0;
      SmallReads rd(c, st);
      CK(rd.add(&n_re, c->pos_tmp.ptr + n_pairs, sizeof(n_re)), "D2H");
      CK(rd.wait(), "reclip sync");
      c->n_reclipped = n_re;
      if (n_re > 0) {
        CK(cudaMemsetAsync(c->scratch.ptr + 1, 0, sizeof(unsigned long long), st), "memset");
        p.site_klen = nullptr;
        p.pair_klen = nullptr;
        p.lazy_cert = 0;
        p.pair_index = c->reclip_idx.ptr;
        p.n_work = n_re;
        CK(launch_clip_cells(p, c->cfg.predicate_mode, certify, variant, blocks, warps, st), "reclip");
      }
    }
    // ---- the cells the clip kernel flagged uncertified, bounded again from
    // their records (FP64 where the FP32 bound is loose): the flag stays
    // where the certificate still fails, and with exact lists the cell's
    // radius goes into its site's site_need
    CK(cudaEventRecord(c->ev[kEvExt0], st), "event");
    // (scratch[32]: cells still flagged after a recheck, compacted into
    // ext_idx; the selection's count is read on the device)
    CK(c->flag_tmp.ensure((size_t)n_pairs + 1), "alloc");
    CK(c->pos_tmp.ensure((size_t)n_pairs + 1), "alloc");
    CK(c->reclip_idx.ensure((size_t)std::max<long long>(n_pairs, 1)), "alloc");
    CK(c->ext_idx.ensure((size_t)std::max<long long>(n_pairs, 1)), "alloc");
    auto recheck = [&](bool rows) -> rpd_status {
      CK(select_uncertified(c->pair_headers.ptr, n_pairs, c->flag_tmp.ptr, c->pos_tmp.ptr,
                            c->scan_tmp.ptr, c->reclip_idx.ptr, st), "select cells");
      CK(cudaMemsetAsync(c->scratch.ptr + 32, 0, sizeof(unsigned long long), st), "memset");
      RecheckParams rp;
      rp.headers = c->pair_headers.ptr;
      rp.idx = c->reclip_idx.ptr;
      rp.n_dev = c->pos_tmp.ptr + n_pairs;
      rp.payload = c->payload.ptr;
      rp.site4f = c->site4f.ptr;
      rp.site_row = rows ? c->site_row.ptr : nullptr;
      rp.ext_bound = c->ext_bound.ptr;
      rp.nbr_bound = c->nbr_bound.ptr;
      rp.margin = cert_margin;
      rp.site_need = extend ? c->site_need.ptr : nullptr;
      rp.kept_idx = c->ext_idx.ptr;
      rp.kept_count = c->scratch.ptr + 32;
      CK(launch_recheck_cells(rp, c->num_sms, st), "recheck");
      return RPD_OK;
    };
    if (knn && n_pairs > 0) {
      rpd_status rs = recheck(false);
      if (rs != RPD_OK) return rs;
    }
    // ---- exact lists: the sites of uncertified cells get every site whose
    // key lies below the cells' radius bound (at most kExtK entries), and
    // those cells are clipped again; a round's re-clip can leave a cell
    // uncertified (its list was cut at kExtK), which the next round takes up
    for (int round = 0; extend && n_pairs > 0 && round < kExtRounds; ++round) {
      CK(select_sites(c->site_need.ptr, n_site, c->site_flag.ptr, c->site_pos.ptr, c->scan_tmp.ptr,
                      c->ext_sites.ptr, st), "select sites");
      int32_t n_f = 0;
      unsigned long long n_flag = 0;
      SmallReads rd(c, st);
      CK(rd.add(&n_f, c->site_pos.ptr + n_site, sizeof(n_f)), "D2H");
      CK(rd.add(&n_flag, c->scratch.ptr + 32, sizeof(n_flag)), "D2H");
      CK(rd.wait(), "extend sync");
      if (round > 0) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, c->ev[kEvExtR0], c->ev[kEvExtK]);
        ms_ext_lists += ms;
      }
      if (n_f == 0 || n_flag == 0) break;
      const bool last = round == kExtRounds - 1;
      const int KL = last ? n_site
                          : std::min(kExtK[round], std::min(knn_max_k(), std::max(n_site - 1, 1)));
      const long long need = c->ext_used + (last ? (long long)n_site : (long long)n_f * KL);
      CK(c->ext_nbr.grow_keep((size_t)need, (size_t)c->ext_used, st), "alloc ext");
      CK(c->ext_keys.grow_keep((size_t)need, (size_t)c->ext_used, st), "alloc ext");
      CK(c->ext_len.grow_keep((size_t)c->ext_rows + n_f, (size_t)c->ext_rows, st), "alloc ext");
      CK(c->ext_bound.grow_keep((size_t)c->ext_rows + n_f, (size_t)c->ext_rows, st), "alloc ext");
      CK(c->ext_off.grow_keep((size_t)c->ext_rows + n_f, (size_t)c->ext_rows, st), "alloc ext");
      CK(cudaEventRecord(c->ev[kEvExtR0], st), "event");
      if (last) {
        CK(complete_rows(c->ext_sites.ptr, n_f, c->ext_rows, c->ext_used, n_site, c->site_row.ptr,
                         c->ext_off.ptr, c->ext_len.ptr, c->ext_bound.ptr, c->ext_nbr.ptr, st,
                         c->has_site_range ? c->site_range.ptr : nullptr),
           "complete rows");
      } else {
        Grid g = c->has_site_range ? make_grid(c->grid_lo, c->grid_hi, n_site, 2.0)
                                   : make_grid(c->site_lo, c->site_hi, n_site, 2.0);
        KnnArgs ka = {};
        ka.site4f = c->site4f.ptr;
        ka.n_rows = n_f;
        ka.g = g;
        ka.cell_start = c->s_cell_start.ptr;
        ka.cell_items = c->s_cell_items.ptr;
        ka.site_range = c->has_site_range ? c->site_range.ptr : nullptr;
        ka.grid_pos = c->has_site_range ? c->site_gridpos.ptr : nullptr;
        ka.k = KL;
        ka.w_max = c->w_max;
        // ascending key in every mode: in site-id order the hundreds of
        // entries would clip the cell with many sites that are not its
        // neighbours before those that are, past the 64-plane capacity
        ka.order_by_id = 0;
        ka.nbr = c->ext_nbr.ptr + c->ext_used;
        ka.keys = c->ext_keys.ptr + c->ext_used;
        ka.subset = c->ext_sites.ptr;
        // every key up to the radius bound of the site's uncertified cells:
        // the certificate then holds at the end of the list, since clipping
        // with more planes only shrinks the cells (the slack covers the
        // rounding of the radius bounds and of the certificate's test)
        ka.radius = c->site_need.ptr;
        ka.bound_scale = 1.0f + 1.0f / 512.0f;
        ka.bound_abs = 2.0f * cert_margin;
        ka.len_out = c->ext_len.ptr + c->ext_rows;
        ka.bound_out = c->ext_bound.ptr + c->ext_rows;
        CK(launch_knn(ka, st), "extended lists");
        CK(assign_rows(c->ext_sites.ptr, n_f, c->ext_rows, c->ext_used, KL, c->site_row.ptr,
                       c->ext_off.ptr, st), "rows");
      }
      CK(cudaEventRecord(c->ev[kEvExtK], st), "event");
      c->ext_used = need;
      c->ext_rows += n_f;
      // the still uncertified cells, clipped again with the new rows
      CK(cudaMemsetAsync(c->site_need.ptr, 0, sizeof(unsigned int) * (size_t)n_site, st), "memset");
      CK(cudaMemsetAsync(c->scratch.ptr + 1, 0, sizeof(unsigned long long), st), "memset");
      ClipParams pe = p;
      pe.site_klen = nullptr;
      pe.pair_klen = nullptr;
      pe.lazy_cert = 0;
      pe.consumed = nullptr;
      pe.pair_index = c->ext_idx.ptr;
      pe.n_work = (long long)n_flag;
      pe.site_row = c->site_row.ptr;
      pe.ext_nbr = c->ext_nbr.ptr;
      pe.ext_keys = c->ext_keys.ptr;
      pe.ext_off = c->ext_off.ptr;
      pe.ext_len = c->ext_len.ptr;
      pe.ext_bound = c->ext_bound.ptr;
      CK(launch_clip_cells(pe, c->cfg.predicate_mode, certify, variant, blocks, warps, st),
         "reclip extended");
      ++n_ext_rounds;
      n_ext_sites += n_f;
      n_cert_reclipped += (long long)n_flag;
      ext_longest = std::max(ext_longest, KL);
      rpd_status rs = recheck(true);
      if (rs != RPD_OK) return rs;
      if (round == kExtRounds - 1) {
        CK(cudaStreamSynchronize(st), "extend sync");
        float ms = 0.f;
        cudaEventElapsedTime(&ms, c->ev[kEvExtR0], c->ev[kEvExtK]);
        ms_ext_lists += ms;
      }
    }
    CK(cudaEventRecord(c->ev[kEvExt1], st), "event");
    c->ext_valid = extend;
    unsigned long long cur = 0;
    SmallReads rd(c, st);
    CK(rd.add(&cur, c->scratch.ptr, sizeof(cur)), "D2H");
    CK(rd.wait(), "clip sync");
    c->payload_bytes = (long long)cur;
    if ((long long)cur <= (long long)c->payload.cap) break;
    pcap = (long long)cur + (long long)cur / 8 + (1 << 20);
    if (attempt == 2) return fail(c, RPD_ERR_CAPACITY, "rpd_compute: payload buffer");
  }
  c->payload_cap_hint = std::max<long long>(c->payload_cap_hint, c->payload_bytes + c->payload_bytes / 8 + (1 << 20));
  // coordinates, volumes and topology hashes of the emitted cells
  CK(cudaEventRecord(c->ev[kEvEpi0], st), "event");
  {
    EpilogueParams ep;
    ep.headers = c->pair_headers.ptr;
    ep.n_pairs = n_pairs;
    ep.payload = c->payload.ptr;
    ep.face2 = c->face2.ptr;
    ep.site2 = c->site2.ptr;
    ep.geometry = c->cfg.compute_geometry;
    ep.topo_hash = c->cfg.topology_hash ? c->topo_hash.ptr : nullptr;
    CK(launch_cell_epilogue(ep, c->num_sms, st), "epilogue");
  }
  CK(cudaEventRecord(c->ev[kEvClip], st), "event");

  // ---- compaction
  CK(c->cells.ensure((size_t)std::max<long long>(n_pairs, 1)), "alloc cells");
  CK(c->flag_tmp.ensure((size_t)n_pairs + 1), "alloc");
  CK(c->pos_tmp.ensure((size_t)n_pairs + 1), "alloc");
  CK(c->scan_tmp.ensure(scan_temp_ints(std::max<long long>(n_pairs, n_tet)) + 16), "alloc");
  CK(c->n_out.ensure(1), "alloc");
  CK(cudaMemsetAsync(c->scratch.ptr + 31, 0, sizeof(unsigned long long), st), "memset");
  CK(compact_cells(c->pair_headers.ptr, n_pairs, c->flag_tmp.ptr, c->pos_tmp.ptr, c->scan_tmp.ptr,
                   c->cells.ptr, c->n_out.ptr, c->scratch.ptr + 8, st, c->scratch.ptr + 31),
     "compact");
  CK(cudaEventRecord(c->ev[kEvEnd], st), "event");
  unsigned long long host_scratch[40];
  long long n_cells = 0;
  {
    SmallReads rd(c, st);
    CK(rd.add(host_scratch, c->scratch.ptr, sizeof(host_scratch)), "D2H");
    CK(rd.add(&n_cells, c->n_out.ptr, sizeof(n_cells)), "D2H");
    CK(rd.wait(), "compute sync");
  }
  c->n_cells = n_cells;
  c->tet_k = (int)reinterpret_cast<int32_t*>(host_scratch + 5)[0];
  c->has_result = true;
  c->has_topology = false;
  c->has_polygons = false;
  c->has_power_cells = false;
  c->cells_for_mesh = false;
  if (host_scratch[8 + 10] != 0)
    return fail(c, RPD_ERR_CAPACITY, "rpd_compute: cells lost to a full payload buffer");
  c->cells_for_mesh = true;
  if (stats) {
    std::memset(stats, 0, sizeof(*stats));
    stats->n_pairs = n_pairs;
    stats->n_cells = n_cells;
    for (int i = 0; i < 10; ++i) stats->status_counts[i] = (int64_t)host_scratch[8 + i];
    stats->n_predicates = (int64_t)host_scratch[2];
    stats->n_escalated = (int64_t)host_scratch[3];
    stats->payload_bytes = c->payload_bytes;
    stats->tet_k = c->tet_k;
    stats->knn_k = c->k;
    cudaEventElapsedTime(&stats->ms_total, c->ev[kEvStart], c->ev[kEvEnd]);
    cudaEventElapsedTime(&stats->ms_knn, c->ev[kEvStart], c->ev[kEvKnn]);
    cudaEventElapsedTime(&stats->ms_pairs, c->ev[kEvKnn], c->ev[kEvPairs]);
    cudaEventElapsedTime(&stats->ms_clip, c->ev[kEvPairs], c->ev[kEvClip]);
    cudaEventElapsedTime(&stats->ms_compact, c->ev[kEvClip], c->ev[kEvEnd]);
    cudaEventElapsedTime(&stats->ms_clip_kernel, c->ev[kEvClipK0], c->ev[kEvClipK1]);
    stats->n_launches = take_launches();
    for (int i = 0; i < 6; ++i) stats->search[i] = (int64_t)host_scratch[20 + i];
    stats->search[4] = c->n_pairs;
    stats->n_reclipped = c->n_reclipped;
    cudaEventElapsedTime(&stats->ms_predict, c->ev[kEvPred0], c->ev[kEvPred1]);
    stats->learned = learned ? 1 : 0;
    stats->n_fp64_uncertain = (int64_t)host_scratch[29];
    stats->n_exact_flips = (int64_t)host_scratch[30];
    stats->n_uncertified = (int64_t)host_scratch[31];
    cudaEventElapsedTime(&stats->ms_epilogue, c->ev[kEvEpi0], c->ev[kEvClip]);
    stats->n_extended_sites = n_ext_sites;
    stats->n_cert_reclipped = n_cert_reclipped;
    stats->n_extend_rounds = n_ext_rounds;
    stats->ext_longest = ext_longest;
    stats->ms_extend_lists = ms_ext_lists;
    cudaEventElapsedTime(&stats->ms_extend, c->ev[kEvExt0], c->ev[kEvExt1]);
  }
  return RPD_OK;
}

rpd_status rpd_compute(rpd_ctx* c, rpd_stats* stats) {
  if (!c) return RPD_ERR_INVALID_ARGUMENT;
  if (!c->has_mesh || !c->has_sites) return fail(c, RPD_ERR_NOT_READY, "rpd_compute: mesh and sites required");
  const bool knn = c->cfg.neighbor_source == RPD_NEIGH_KNN;
  if (!knn && !c->has_user_nbr)
    return fail(c, RPD_ERR_NOT_READY, "rpd_compute: neighbour lists required (rpd_set_neighbors)");
  const bool learned = c->cfg.learned_k != 0;
  if (learned && (!c->cfg.certify || !knn))
    return fail(c, RPD_ERR_INVALID_ARGUMENT, "rpd_compute: learned_k needs certify and GPU-built lists");
  if (learned && !c->mlp_ready)
    return fail(c, RPD_ERR_NOT_READY,
                "rpd_compute: learned_k needs a predictor (rpd_mlp_train or rpd_mlp_set_params)");
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  cudaStream_t st = c->stream;
  const int n_site = c->n_site, n_tet = c->n_tet;
  CK(c->scratch.ensure(40), "alloc scratch");
  CK(cudaMemsetAsync(c->scratch.ptr, 0, 32 * sizeof(unsigned long long), st), "memset");
  take_launches();
  CK(cudaEventRecord(c->ev[kEvStart], st), "event");

  // ---- neighbour lists
  if (knn) {
    c->k = c->cfg.knn_k;
    Grid g = make_grid(c->site_lo, c->site_hi, n_site, 2.0);
    long long nc = (long long)g.nx * g.ny * g.nz;
    CK(c->s_cell_of.ensure(n_site), "alloc");
    CK(c->s_cell_count.ensure(nc), "alloc");
    CK(c->s_cell_start.ensure(nc + 1), "alloc");
    CK(c->s_cell_fill.ensure(nc), "alloc");
    CK(c->s_cell_items.ensure(n_site), "alloc");
    CK(c->scan_tmp.ensure(scan_temp_ints(std::max<long long>(nc, n_tet)) + 16), "alloc");
    CK(c->nbr.ensure((size_t)n_site * c->k), "alloc nbr");
    CK(c->nbr_keys.ensure((size_t)n_site * c->k), "alloc nbr");
    CK(c->nbr_dist.ensure((size_t)n_site * c->k), "alloc nbr");
    CK(c->knn_status.ensure(n_site), "alloc");
    CK(grid_build_sites(c->site4f.ptr, n_site, g, c->s_cell_of.ptr, c->s_cell_count.ptr,
                        c->s_cell_start.ptr, c->s_cell_fill.ptr, c->s_cell_items.ptr,
                        c->scan_tmp.ptr, st), "site grid");
    CK(c->nbr_bound.ensure((size_t)n_site), "alloc nbr");
    CK(launch_knn(c->site4f.ptr, n_site, g, c->s_cell_start.ptr, c->s_cell_items.ptr, c->k,
                  c->w_max, c->cfg.clip_order == RPD_ORDER_SITE_ID ? 1 : 0, c->nbr.ptr,
                  c->nbr_keys.ptr, c->nbr_dist.ptr, c->knn_status.ptr, st, 0,
                  c->nbr_bound.ptr), "knn");
  }
  CK(cudaEventRecord(c->ev[kEvKnn], st), "event");

  // ---- candidate pairs
  {
    CK(c->centroid.ensure(n_tet), "alloc");
    CK(c->t_cell_of.ensure(n_tet), "alloc");
    CK(c->t_cell_items.ensure(n_tet), "alloc");
    CK(c->tet_xyz.ensure((size_t)n_tet * 3), "alloc");
    CK(c->tet_vadj.ensure((size_t)n_tet), "alloc");
    CK(tet_centroids(c->vert3f.ptr, c->tets.ptr, n_tet, c->centroid.ptr, st, c->tet_xyz.ptr,
                     c->v_adjs.ptr, c->tet_vadj.ptr),
       "centroids");
    double diag2 = 0.0, cs = 0.0;
    for (int a = 0; a < 3; ++a) {
      double l = std::min(c->mesh_lo[a], c->site_lo[a]), h = std::max(c->mesh_hi[a], c->site_hi[a]);
      diag2 += (h - l) * (h - l);
      cs = std::max(cs, std::max(std::fabs(l), std::fabs(h)));
    }
    const double u = std::ldexp(1.0, -24);
    double ext = 0.0;
    for (int a = 0; a < 3; ++a) ext = std::max(ext, c->mesh_hi[a] - c->mesh_lo[a]);
    const double margin = 1e-4 * ext + 1e-6 * cs;
    // the nearest bisectors bound each cell; with a GPU-built list the
    // distance-ordered copy gives them first, a user list is used whole
    const int32_t* box_list = knn ? c->nbr_dist.ptr : c->nbr.ptr;
    const int box0 = c->cfg.box_planes > 0 ? c->cfg.box_planes : kDefaultBoxPlanes;
    CK(c->site_box.ensure((size_t)n_site * 2), "alloc");
    CK(c->site_planes.ensure((size_t)n_site * kBoxPlanes), "alloc");
    CK(c->site_nplanes.ensure((size_t)n_site), "alloc");
    CK(c->tet_count.ensure(n_tet), "alloc");
    CK(c->tet_offsets.ensure((size_t)n_tet + 1), "alloc");
    CK(c->tet_fill.ensure(n_tet), "alloc");
    long long cap = c->pair_cap_hint > 0 ? c->pair_cap_hint : std::max<long long>(1 << 20, 16ll * n_tet);
    for (int attempt = 0; attempt < 3; ++attempt) {
      CK(c->pair_buf.ensure((size_t)cap), "alloc pairs");
      CK(cudaMemsetAsync(c->tet_count.ptr, 0, sizeof(int32_t) * (size_t)n_tet, st), "memset");
      CK(cudaMemsetAsync(c->scratch.ptr + 4, 0, sizeof(unsigned long long), st), "memset");
      CK(cudaMemsetAsync(c->scratch.ptr + 20, 0, 6 * sizeof(unsigned long long), st), "memset");
      for (int cl = 0; cl < rpd_ctx::kClasses; ++cl) {
        if (c->class_count[cl] == 0) continue;
        Grid tg = make_grid(c->mesh_lo, c->mesh_hi, c->class_count[cl], kTetsPerCell);
        long long nc = (long long)tg.nx * tg.ny * tg.nz;
        CK(c->t_cell_count.ensure(nc), "alloc");
        CK(c->t_cell_rmax.ensure(nc), "alloc");
        CK(c->t_cell_start.ensure(nc + 1), "alloc");
        CK(c->t_cell_fill.ensure(nc), "alloc");
        CK(c->scan_tmp.ensure(scan_temp_ints(std::max<long long>(nc, n_tet)) + 16), "alloc");
        CK(grid_build_tets(c->centroid.ptr, n_tet, c->tet_class.ptr, cl, tg, c->t_cell_of.ptr,
                           c->t_cell_count.ptr, c->t_cell_start.ptr, c->t_cell_fill.ptr,
                           c->t_cell_items.ptr, c->scan_tmp.ptr, st, c->t_cell_rmax.ptr), "tet grid");
        // per-site boxes: every tet of this class that passes the rule has
        // its centroid in the site's cell pushed out by the class radius
        const double R = c->class_radius[cl] * (1.0 + 1e-5) + 1e-6 * cs;
        BoxParams bp;
        bp.site4f = c->site4f.ptr;
        bp.flags = c->flags.ptr;
        bp.site_base = 0;
        bp.nbr = box_list;
        bp.k = c->k;
        // the nearest bisectors (distance-ordered GPU lists) for the common
        // tets; the class of the largest tets has few tets, so a looser
        // region costs little in the search and its box is cheap to clip
        bp.k_box = knn ? std::min(c->k, cl == 0 ? box0 : std::min(box0, 12)) : c->k;
        bp.n_site = n_site;
        bp.box_lo = make_float4((float)(c->mesh_lo[0] - margin), (float)(c->mesh_lo[1] - margin),
                                (float)(c->mesh_lo[2] - margin), 0.f);
        bp.box_hi = make_float4((float)(c->mesh_hi[0] + margin), (float)(c->mesh_hi[1] + margin),
                                (float)(c->mesh_hi[2] + margin), 0.f);
        bp.offset_r = (float)R;
        bp.offset_e = (float)(48.0 * u * (diag2 + std::fabs((double)c->w_max)));
        bp.coord_scale = (float)cs;
        bp.abs_margin = (float)margin;
        bp.site_box = c->site_box.ptr;
        bp.site_planes = c->site_planes.ptr;
        bp.site_nplanes = c->site_nplanes.ptr;
        bp.counters = nullptr;
        int bw = 4;
        int bblocks = std::max(1, std::min((n_site + bw - 1) / bw, c->num_sms * box_blocks_per_sm(bw)));
        CK(launch_site_box(bp, bblocks, bw, st), "site boxes");
        PairParams pp;
        pp.vert3f = c->vert3f.ptr;
        pp.tets = c->tets.ptr;
        pp.centroid = c->centroid.ptr;
        pp.tet_xyz = c->tet_xyz.ptr;
        pp.tet_base = 0;
        pp.site_base = 0;
        pp.tg = tg;
        pp.tcell_start = c->t_cell_start.ptr;
        pp.tcell_items = c->t_cell_items.ptr;
        pp.tcell_rmax = c->t_cell_rmax.ptr;
        pp.site4f = c->site4f.ptr;
        pp.flags = c->flags.ptr;
        pp.nbr = c->nbr.ptr;
        pp.rule_nbr = knn ? c->nbr_dist.ptr : nullptr;
        pp.k = c->k;
        pp.n_site = n_site;
        pp.site_box = c->site_box.ptr;
        pp.offset_r = bp.offset_r;
        pp.rule_keys = knn ? c->nbr_keys.ptr : nullptr;
        pp.accept_margin = (float)(16.0 * u * (cs + std::sqrt(diag2)));
        pp.accept_err = 1.01f * bp.offset_e;
        pp.site_planes = c->site_planes.ptr;
        pp.site_nplanes = c->site_nplanes.ptr;
        pp.coord_scale = (float)cs;
        pp.pair_buf = c->pair_buf.ptr;
        pp.pair_cursor = c->scratch.ptr + 4;
        pp.pair_cap = (long long)c->pair_buf.cap;
        pp.tet_count = c->tet_count.ptr;
        pp.diag = c->scratch.ptr + 20;
        CK(c->pair_ntasks.ensure((size_t)n_site), "alloc");
        CK(c->pair_taskoff.ensure((size_t)n_site + 1), "alloc");
        CK(c->scan_tmp.ensure(scan_temp_ints(std::max<long long>(std::max<long long>(nc, n_tet), n_site)) + 16), "alloc");
        CK(launch_pairs(pp, c->pair_ntasks.ptr, c->pair_taskoff.ptr, c->scan_tmp.ptr,
                        c->scratch.ptr + 27, c->num_sms, st), "pairs");
      }
      unsigned long long np = 0;
      SmallReads rd(c, st);
      CK(rd.add(&np, c->scratch.ptr + 4, sizeof(np)), "D2H");
      CK(rd.wait(), "pairs sync");
      c->n_pairs = (long long)np;
      if ((long long)np <= (long long)c->pair_buf.cap) break;
      cap = (long long)np + (long long)np / 8 + 1024;
      if (attempt == 2) return fail(c, RPD_ERR_CAPACITY, "rpd_compute: pair buffer");
    }
    if (c->n_pairs > INT32_MAX) return fail(c, RPD_ERR_CAPACITY, "rpd_compute: more than 2^31 pairs");
    c->pair_cap_hint = std::max<long long>(c->pair_cap_hint, c->n_pairs + c->n_pairs / 8 + 1024);
  }
  return finish_compute(c, knn, learned, stats, true);
}

rpd_status rpd_autotune(rpd_ctx* c, int repeats, rpd_tuning* result) {
  if (!c) return RPD_ERR_INVALID_ARGUMENT;
  if (repeats < 1) repeats = 1;
  struct Cand {
    int warps, variant, bucket;
  };
  std::vector<Cand> cands;
  const int w0 = c->cfg.warps_per_block > 0 ? c->cfg.warps_per_block : 4;
  cands.push_back({w0, c->cfg.clip_variant, 0});
  const int wlist[3] = {2, 4, 8};
  for (int w : wlist) cands.push_back({w, 0, 0});
  cands.push_back({4, 1, 0});
  cands.push_back({4, 2, 0});
  const rpd_config saved = c->cfg;
  const bool saved_klen = c->has_site_klen;
  std::vector<int32_t> saved_k;
  if (saved_klen) {
    saved_k.resize((size_t)c->n_site);
    CK(cudaMemcpy(saved_k.data(), c->site_klen.ptr, sizeof(int32_t) * saved_k.size(),
                  cudaMemcpyDeviceToHost), "D2H");
  }
  // first-pass list lengths: 0 = the whole list (certificate tested as the
  // cell is clipped), 16 / 32 for every site (misses re-clipped), and -1 =
  // the k-predictor's per-cell lengths when one is trained
  int buckets[4] = {0, 0, 0, 0};
  int nb = 1;
  if (c->cfg.certify && c->cfg.neighbor_source == RPD_NEIGH_KNN) {
    buckets[1] = 16;
    buckets[2] = 32;
    nb = 3;
    if (c->mlp_ready) buckets[nb++] = -1;
  }
  float best = INFINITY, first = 0.f;
  Cand best_c = cands[0];
  int tried = 0;
  for (int bi = 0; bi < nb; ++bi) {
    for (size_t ci = 0; ci < cands.size(); ++ci) {
      if (bi > 0 && ci == 0) continue;
      Cand cd = cands[ci];
      cd.bucket = buckets[bi];
      c->cfg.warps_per_block = cd.warps;
      c->cfg.clip_variant = cd.variant;
      c->cfg.blocks_per_sm = 0;
      c->cfg.learned_k = cd.bucket < 0 ? 1 : 0;
      if (cd.bucket > 0) {
        std::vector<int32_t> kk((size_t)c->n_site, cd.bucket);
        rpd_status s = rpd_set_site_k(c, kk.data(), 0);
        if (s != RPD_OK) return s;
      } else {
        c->has_site_klen = false;
      }
      std::vector<float> t;
      for (int r = 0; r < repeats + 1; ++r) {
        rpd_stats st;
        rpd_status s = rpd_compute(c, &st);
        if (s != RPD_OK) {
          c->cfg = saved;
          return s;
        }
        if (r > 0) t.push_back(st.ms_clip);
      }
      std::sort(t.begin(), t.end());
      float med = t[t.size() / 2];
      if (tried == 0) first = med;
      ++tried;
      if (med < best) {
        best = med;
        best_c = cd;
      }
    }
  }
  c->cfg = saved;
  c->cfg.warps_per_block = best_c.warps;
  c->cfg.clip_variant = best_c.variant;
  c->cfg.blocks_per_sm = 0;
  c->cfg.learned_k = best_c.bucket < 0 ? 1 : 0;
  if (best_c.bucket > 0) {
    std::vector<int32_t> kk((size_t)c->n_site, best_c.bucket);
    rpd_status s = rpd_set_site_k(c, kk.data(), 0);
    if (s != RPD_OK) return s;
  } else if (saved_klen) {
    rpd_status s = rpd_set_site_k(c, saved_k.data(), 0);
    if (s != RPD_OK) return s;
  } else {
    c->has_site_klen = false;
  }
  // base list length of GPU-built exact lists: longer base lists cost the
  // kNN and the pair rule more, and leave fewer cells to the longer-list
  // rounds; the cells are the same, so the whole compute decides
  float best_total = INFINITY;
  if (c->cfg.neighbor_source == RPD_NEIGH_KNN && c->cfg.certify && c->cfg.exact_lists) {
    const int k0 = c->cfg.knn_k;
    const int ks[4] = {k0, 64, 96, 128};
    int best_k = k0;
    for (int i = 0; i < 4; ++i) {
      if (i > 0 && ks[i] == k0) continue;
      c->cfg.knn_k = ks[i];
      std::vector<float> t;
      for (int r = 0; r < repeats + 1; ++r) {
        rpd_stats st;
        rpd_status s = rpd_compute(c, &st);
        if (s != RPD_OK) {
          c->cfg.knn_k = k0;
          return s;
        }
        if (r > 0) t.push_back(st.ms_total);
      }
      std::sort(t.begin(), t.end());
      const float med = t[t.size() / 2];
      ++tried;
      if (med < best_total) {
        best_total = med;
        best_k = ks[i];
      }
    }
    c->cfg.knn_k = best_k;
  }
  c->has_result = false;
  if (result) {
    result->warps_per_block = best_c.warps;
    result->clip_variant = best_c.variant;
    result->k_bucket = best_c.bucket > 0 ? best_c.bucket : 0;
    result->learned_k = best_c.bucket < 0 ? 1 : 0;
    result->n_candidates = tried;
    result->ms_clip_best = best;
    result->ms_clip_first = first;
    result->knn_k = c->cfg.knn_k;
    result->ms_total_best = best_total;
  }
  return RPD_OK;
}

rpd_status rpd_get_cells(rpd_ctx* c, rpd_cells_view* v) {
  if (!c || !v) return RPD_ERR_INVALID_ARGUMENT;
  if (!c->has_result) return fail(c, RPD_ERR_NOT_READY, "rpd_get_cells: no result");
  v->n_cells = c->n_cells;
  v->headers = c->cells.ptr;
  v->payload = c->payload.ptr;
  v->payload_bytes = c->payload_bytes;
  v->n_pairs = c->n_pairs;
  v->pair_headers = c->pair_headers.ptr;
  return RPD_OK;
}

rpd_status rpd_copy_cells_to_host(rpd_ctx* c, rpd_cell_header* headers, int64_t max_cells,
                                  void* payload, int64_t payload_capacity, int64_t* n_cells,
                                  int64_t* payload_bytes) {
  const rpd_status s = rpd_copy_cells_to_host_async(c, headers, max_cells, payload,
                                                    payload_capacity, n_cells, payload_bytes);
  if (s != RPD_OK || (!headers && !payload)) return s;
  return rpd_synchronize(c);
}

rpd_status rpd_synchronize(rpd_ctx* c) {
  if (!c) return RPD_ERR_INVALID_ARGUMENT;
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  CK(cudaStreamSynchronize(c->stream), "sync");
  return RPD_OK;
}

rpd_status rpd_copy_cells_to_host_async(rpd_ctx* c, rpd_cell_header* headers, int64_t max_cells,
                                        void* payload, int64_t payload_capacity,
                                        int64_t* n_cells, int64_t* payload_bytes) {
  if (!c) return RPD_ERR_INVALID_ARGUMENT;
  if (!c->has_result) return fail(c, RPD_ERR_NOT_READY, "rpd_copy_cells_to_host: no result");
  if (n_cells) *n_cells = c->n_cells;
  if (payload_bytes) *payload_bytes = c->payload_bytes;
  if (!headers && !payload) return RPD_OK;
  if ((headers && max_cells < c->n_cells) || (payload && payload_capacity < c->payload_bytes))
    return fail(c, RPD_ERR_CAPACITY, "rpd_copy_cells_to_host: buffers too small");
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  cudaStream_t st = c->stream;
  if (headers && c->n_cells > 0)
    CK(cudaMemcpyAsync(headers, c->cells.ptr, sizeof(rpd_cell_header) * (size_t)c->n_cells,
                       cudaMemcpyDeviceToHost, st), "D2H cells");
  if (payload && c->payload_bytes > 0)
    CK(cudaMemcpyAsync(payload, c->payload.ptr, (size_t)c->payload_bytes, cudaMemcpyDeviceToHost, st),
       "D2H payload");
  return RPD_OK;
}

rpd_status rpd_set_site_k(rpd_ctx* c, const int32_t* k_per_site, int on_device) {
  if (!c) return RPD_ERR_INVALID_ARGUMENT;
  if (!k_per_site) {
    c->has_site_klen = false;
    return RPD_OK;
  }
  if (!c->has_sites) return fail(c, RPD_ERR_NOT_READY, "rpd_set_site_k: set the sites first");
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  CK(c->site_klen.ensure((size_t)c->n_site), "alloc");
  CK(cudaMemcpyAsync(c->site_klen.ptr, k_per_site, sizeof(int32_t) * (size_t)c->n_site,
                     on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, c->stream),
     "copy site k");
  CK(cudaStreamSynchronize(c->stream), "sync");
  c->has_site_klen = true;
  c->has_result = false;
  return RPD_OK;
}

rpd_status rpd_set_pair_k(rpd_ctx* c, const int32_t* k_per_pair, int64_t n_pairs) {
  if (!c) return RPD_ERR_INVALID_ARGUMENT;
  if (!k_per_pair) {
    c->n_user_pair_k = -1;
    return RPD_OK;
  }
  if (!c->cfg.certify) return fail(c, RPD_ERR_INVALID_ARGUMENT, "rpd_set_pair_k: needs certify");
  if (n_pairs < 0) return fail(c, RPD_ERR_INVALID_ARGUMENT, "rpd_set_pair_k: n_pairs < 0");
  for (int64_t i = 0; i < n_pairs; ++i)
    if (k_per_pair[i] < 1) return fail(c, RPD_ERR_INVALID_ARGUMENT, "rpd_set_pair_k: lengths must be >= 1");
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  CK(c->user_pair_k.ensure((size_t)std::max<int64_t>(n_pairs, 1)), "alloc");
  if (n_pairs > 0)
    CK(cudaMemcpy(c->user_pair_k.ptr, k_per_pair, sizeof(int32_t) * (size_t)n_pairs, cudaMemcpyHostToDevice), "H2D");
  c->n_user_pair_k = n_pairs;
  return RPD_OK;
}

// ---- per-cell topology of the emitted cells ------------------------------
rpd_status rpd_compute_topology(rpd_ctx* c, float* ms) {
  if (!c) return RPD_ERR_INVALID_ARGUMENT;
  if (!c->has_result) return fail(c, RPD_ERR_NOT_READY, "rpd_compute_topology: no result");
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  cudaStream_t st = c->stream;
  const long long n = c->n_cells;
  CK(c->topo_units.ensure((size_t)std::max(n, 1ll)), "alloc");
  CK(c->topo_off.ensure((size_t)n + 1), "alloc");
  CK(c->topo_h.ensure((size_t)std::max(n, 1ll)), "alloc");
  CK(c->scan_tmp.ensure(scan_temp_ints(std::max(n, 1ll))), "alloc");
  CK(cudaEventRecord(c->ev[kEvTopo0], st), "event");
  CK(topo_units(c->cells.ptr, n, c->topo_units.ptr, st), "topology sizes");
  CK(scan_exclusive(c->topo_units.ptr, c->topo_off.ptr, n, c->scan_tmp.ptr, st), "topology scan");
  int32_t units = 0;
  CK(cudaMemcpyAsync(&units, c->topo_off.ptr + n, sizeof(units), cudaMemcpyDeviceToHost, st), "D2H");
  CK(cudaStreamSynchronize(st), "topology sync");
  const long long bytes = 16ll * units;
  CK(c->topo_buf.ensure((size_t)std::max(bytes, 16ll)), "alloc");
  CK(topo_fill(c->cells.ptr, n, c->payload.ptr, c->topo_off.ptr, c->topo_h.ptr, c->topo_buf.ptr,
               c->num_sms, st), "topology");
  CK(cudaEventRecord(c->ev[kEvTopo1], st), "event");
  CK(cudaStreamSynchronize(st), "topology sync");
  if (ms) CK(cudaEventElapsedTime(ms, c->ev[kEvTopo0], c->ev[kEvTopo1]), "event time");
  c->topo_bytes = bytes;
  c->has_topology = true;
  return RPD_OK;
}

rpd_status rpd_get_topology(rpd_ctx* c, rpd_topo_view* v) {
  if (!c || !v) return RPD_ERR_INVALID_ARGUMENT;
  if (!c->has_result || !c->has_topology)
    return fail(c, RPD_ERR_NOT_READY, "rpd_get_topology: call rpd_compute_topology first");
  v->n_cells = c->n_cells;
  v->headers = c->topo_h.ptr;
  v->records = c->topo_buf.ptr;
  v->bytes = c->topo_bytes;
  return RPD_OK;
}

rpd_status rpd_copy_topology_to_host(rpd_ctx* c, rpd_topo_header* headers, int64_t max_cells,
                                     void* records, int64_t capacity, int64_t* n_cells,
                                     int64_t* bytes) {
  if (!c) return RPD_ERR_INVALID_ARGUMENT;
  if (!c->has_result || !c->has_topology)
    return fail(c, RPD_ERR_NOT_READY, "rpd_copy_topology_to_host: call rpd_compute_topology first");
  if (n_cells) *n_cells = c->n_cells;
  if (bytes) *bytes = c->topo_bytes;
  if (!headers && !records) return RPD_OK;
  if ((headers && max_cells < c->n_cells) || (records && capacity < c->topo_bytes))
    return fail(c, RPD_ERR_CAPACITY, "rpd_copy_topology_to_host: buffers too small");
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  cudaStream_t st = c->stream;
  if (headers && c->n_cells > 0)
    CK(cudaMemcpyAsync(headers, c->topo_h.ptr, sizeof(rpd_topo_header) * (size_t)c->n_cells,
                       cudaMemcpyDeviceToHost, st), "D2H topology");
  if (records && c->topo_bytes > 0)
    CK(cudaMemcpyAsync(records, c->topo_buf.ptr, (size_t)c->topo_bytes, cudaMemcpyDeviceToHost, st),
       "D2H topology");
  CK(cudaStreamSynchronize(st), "copy sync");
  return RPD_OK;
}

// ---- power cells of the emitted cells -------------------------------------
rpd_status rpd_set_feature_edges(rpd_ctx* c, const rpd_feature_edge* fe, int64_t n) {
  if (!c) return RPD_ERR_INVALID_ARGUMENT;
  if (n < 0 || (n > 0 && !fe)) return fail(c, RPD_ERR_INVALID_ARGUMENT, "rpd_set_feature_edges: bad arguments");
  for (int64_t i = 0; i < n; ++i)
    if (fe[i].tet_id < 0 || fe[i].lf_min < 0 || fe[i].lf_min >= fe[i].lf_max || fe[i].lf_max > 3)
      return fail(c, RPD_ERR_INVALID_ARGUMENT, "rpd_set_feature_edges: bad tet id or local faces");
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  // keys in ascending order; of equal keys the last record (a map's last
  // assignment)
  std::vector<unsigned long long> key((size_t)n);
  for (int64_t i = 0; i < n; ++i)
    key[i] = ((unsigned long long)(uint32_t)fe[i].tet_id << 4) | (unsigned)(fe[i].lf_min << 2) |
             (unsigned)fe[i].lf_max;
  std::vector<int64_t> order((size_t)n);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) { return key[a] < key[b]; });
  std::vector<unsigned long long> uk;
  std::vector<int32_t> uv;
  for (size_t j = 0; j < order.size(); ++j) {
    if (j + 1 < order.size() && key[order[j + 1]] == key[order[j]]) continue;
    const rpd_feature_edge& r = fe[order[j]];
    uk.push_back(key[order[j]]);
    uv.push_back(r.fe_type);
    uv.push_back(r.fe_id);
    uv.push_back(r.fe_line_id);
  }
  const long long m = (long long)uk.size();
  CK(c->fe_keys.ensure((size_t)std::max(m, 1ll)), "alloc");
  CK(c->fe_vals.ensure((size_t)std::max(3 * m, 3ll)), "alloc");
  if (m > 0) {
    CK(cudaMemcpyAsync(c->fe_keys.ptr, uk.data(), sizeof(unsigned long long) * (size_t)m,
                       cudaMemcpyHostToDevice, c->stream), "H2D");
    CK(cudaMemcpyAsync(c->fe_vals.ptr, uv.data(), sizeof(int32_t) * (size_t)(3 * m),
                       cudaMemcpyHostToDevice, c->stream), "H2D");
  }
  CK(cudaStreamSynchronize(c->stream), "sync");
  c->n_fe = m;
  c->has_power_cells = false;
  return RPD_OK;
}

rpd_status rpd_set_surface_mesh(rpd_ctx* c, const int32_t* facet_adj, int32_t n_faces,
                                const int32_t* no_cross, int64_t n_pairs) {
  if (!c) return RPD_ERR_INVALID_ARGUMENT;
  if (n_faces < 0 || n_pairs < 0 || (n_faces > 0 && !facet_adj) || (n_pairs > 0 && !no_cross))
    return fail(c, RPD_ERR_INVALID_ARGUMENT, "rpd_set_surface_mesh: bad arguments");
  for (long long f = 0; f < n_faces; ++f)
    for (int le = 0; le < 3; ++le) {
      const int32_t g = facet_adj[3 * f + le];
      if (g < -1 || g >= n_faces)
        return fail(c, RPD_ERR_INVALID_ARGUMENT, "rpd_set_surface_mesh: face id out of range");
      if (g >= 0 && facet_adj[3 * g] != f && facet_adj[3 * g + 1] != f && facet_adj[3 * g + 2] != f)
        return fail(c, RPD_ERR_INVALID_ARGUMENT, "rpd_set_surface_mesh: adjacency not symmetric");
    }
  std::vector<unsigned long long> keys((size_t)n_pairs);
  for (int64_t i = 0; i < n_pairs; ++i) {
    const int32_t a = no_cross[2 * i], b = no_cross[2 * i + 1];
    if (a < 0 || b < 0 || a >= n_faces || b >= n_faces)
      return fail(c, RPD_ERR_INVALID_ARGUMENT, "rpd_set_surface_mesh: pair face id out of range");
    keys[i] = ((unsigned long long)(uint32_t)std::min(a, b) << 32) | (uint32_t)std::max(a, b);
  }
  std::sort(keys.begin(), keys.end());
  keys.erase(std::unique(keys.begin(), keys.end()), keys.end());
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  CK(c->sf_adj.ensure((size_t)std::max(3ll * n_faces, 3ll)), "alloc");
  CK(c->sf_no_cross.ensure(std::max(keys.size(), (size_t)1)), "alloc");
  if (n_faces > 0)
    CK(cudaMemcpyAsync(c->sf_adj.ptr, facet_adj, sizeof(int32_t) * 3 * (size_t)n_faces,
                       cudaMemcpyHostToDevice, c->stream), "H2D");
  if (!keys.empty())
    CK(cudaMemcpyAsync(c->sf_no_cross.ptr, keys.data(), sizeof(unsigned long long) * keys.size(),
                       cudaMemcpyHostToDevice, c->stream), "H2D");
  CK(cudaStreamSynchronize(c->stream), "sync");
  c->sf_faces = n_faces;
  c->sf_n_no_cross = (long long)keys.size();
  c->has_power_cells = false;
  return RPD_OK;
}

rpd_status rpd_compute_power_cells(rpd_ctx* c, int max_sf_fid, float* ms) {
  if (!c) return RPD_ERR_INVALID_ARGUMENT;
  if (!c->has_result) return fail(c, RPD_ERR_NOT_READY, "rpd_compute_power_cells: no result");
  if (!c->has_topology) {
    const rpd_status s = rpd_compute_topology(c, nullptr);
    if (s != RPD_OK) return s;
  }
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  cudaStream_t st = c->stream;
  const long long n = c->n_cells;
  const int n_site = c->n_site;
  if (n > 0x7fffffffll) return fail(c, RPD_ERR_CAPACITY, "rpd_compute_power_cells: too many cells");
  CK(cudaEventRecord(c->ev[kEvTopo0], st), "event");
  CK(c->pc_cnt.ensure((size_t)std::max(8 * n, 8ll)), "alloc");
  CK(c->pc_off.ensure((size_t)(8 * (n + 1))), "alloc");
  CK(c->pc_scan.ensure(scan64_temp(std::max(n, 1ll)) + 16), "alloc");
  PowerCellParams p = {};
  p.cells = c->cells.ptr;
  p.n = n;
  p.payload = c->payload.ptr;
  p.topo_h = c->topo_h.ptr;
  p.topo = c->topo_buf.ptr;
  p.max_sf_fid = max_sf_fid;
  p.cnt = c->pc_cnt.ptr;
  p.off = c->pc_off.ptr;
  p.fe_keys = c->fe_keys.ptr;
  p.fe_vals = c->fe_vals.ptr;
  p.n_fe = c->n_fe;
  CK(pc_count(p, st), "power cell counts");
  // feature-edge rows only with a map set; else their offsets are all 0
  const int n_rows = c->n_fe > 0 ? 8 : 5;
  if (c->n_fe > 0) CK(pc_feature_edges(p, 0, st), "feature edge counts");
  else CK(cudaMemsetAsync(c->pc_off.ptr + 5 * (n + 1), 0, sizeof(long long) * (size_t)(3 * (n + 1)), st),
          "memset");
  for (int k = 0; k < n_rows; ++k)
    CK(scan64_exclusive(c->pc_cnt.ptr + k * n, c->pc_off.ptr + k * (n + 1), n, c->pc_scan.ptr, st),
       "power cell scan");
  long long tot[8];
  for (int k = 0; k < 8; ++k)
    CK(cudaMemcpyAsync(&tot[k], c->pc_off.ptr + k * (n + 1) + n, sizeof(long long),
                       cudaMemcpyDeviceToHost, st), "D2H");
  CK(cudaStreamSynchronize(st), "sync");
  const long long n_tf = tot[0], n_fa = tot[1], n_ed = tot[2], n_vx = tot[3], n_sf = tot[4];
  const long long n_se = tot[5], n_ce = tot[6], n_end = tot[7];
  // key / value segments: tet faces, facets, edges, sites
  const long long seg[4] = {n_tf, n_fa, n_ed, n};
  const long long n_keys = n_tf + n_fa + n_ed + n;
  const long long max_seg = std::max(std::max(n_tf, n_fa), std::max(n_ed, n));
  if (max_seg > 0x7fffffffll) return fail(c, RPD_ERR_CAPACITY, "rpd_compute_power_cells: too many records");
  CK(c->pc_keys.ensure((size_t)std::max(n_keys, 1ll)), "alloc");
  CK(c->pc_vals.ensure((size_t)std::max(n_keys, 1ll)), "alloc");
  CK(c->pc_keys_tmp.ensure((size_t)std::max(max_seg, 1ll)), "alloc");
  CK(c->pc_vals_tmp.ensure((size_t)std::max(max_seg, 1ll)), "alloc");
  const size_t nh = radix_hist_ints(std::max(max_seg, 1ll));
  CK(c->pc_hist.ensure(nh), "alloc");
  CK(c->pc_scan_i.ensure(scan_temp_ints((long long)nh) + 16), "alloc");
  CK(c->pc_tf_fid.ensure((size_t)std::max(n_tf, 1ll)), "alloc");
  CK(c->pc_ed_fields.ensure((size_t)std::max(6 * n_ed, 6ll)), "alloc");
  CK(c->pc_ed_out.ensure((size_t)std::max(7 * n_ed, 7ll)), "alloc");
  CK(c->pc_vx_i.ensure((size_t)std::max(6 * n_vx, 6ll)), "alloc");
  CK(c->pc_vx_pos.ensure((size_t)std::max(3 * n_vx, 3ll)), "alloc");
  CK(c->pc_sf_i.ensure((size_t)std::max(2 * n_sf, 2ll)), "alloc");
  CK(c->pc_sf_pos.ensure((size_t)std::max(3 * n_sf, 3ll)), "alloc");
  CK(c->pc_site_off.ensure((size_t)(3 * ((long long)n_site + 1))), "alloc");
  CK(c->pc_nbr_cnt.ensure((size_t)std::max(n, 1ll)), "alloc");
  CK(c->pc_nbr_fill.ensure((size_t)std::max(n, 1ll)), "alloc");
  CK(c->pc_nbr_off.ensure((size_t)n + 1), "alloc");
  CK(c->pc_fe_i.ensure((size_t)std::max(5 * n_se + 5 * n_ce + 4 * n_end, 1ll)), "alloc");
  CK(c->pc_fe_pos.ensure((size_t)std::max(3 * n_end, 3ll)), "alloc");
  unsigned long long* keys[4];
  uint32_t* vals[4];
  long long at = 0;
  for (int k = 0; k < 4; ++k) {
    keys[k] = c->pc_keys.ptr + at;
    vals[k] = c->pc_vals.ptr + at;
    at += seg[k];
  }
  p.tf_fid = c->pc_tf_fid.ptr;
  p.tf_key = keys[0];
  p.tf_val = vals[0];
  p.fa_key = keys[1];
  p.fa_val = vals[1];
  p.ed_key = keys[2];
  p.ed_val = vals[2];
  int32_t* ef = c->pc_ed_fields.ptr;
  p.ed_site = ef;
  p.ed_n0 = ef + n_ed;
  p.ed_n1 = ef + 2 * n_ed;
  p.ed_cell = ef + 3 * n_ed;
  p.ed_lv0 = ef + 4 * n_ed;
  p.ed_lv1 = ef + 5 * n_ed;
  p.ed_out = c->pc_ed_out.ptr;
  int32_t* vi = c->pc_vx_i.ptr;
  p.vx_cell = vi;
  p.vx_lvid = vi + n_vx;
  p.vx_sfid = vi + 2 * n_vx;
  p.vx_ids = vi + 3 * n_vx;
  p.vx_pos = c->pc_vx_pos.ptr;
  p.sf_cell = c->pc_sf_i.ptr;
  p.sf_fid = c->pc_sf_i.ptr + n_sf;
  p.sf_pos = c->pc_sf_pos.ptr;
  p.site_key = keys[3];
  p.site_val = vals[3];
  p.nbr_cnt = c->pc_nbr_cnt.ptr;
  p.nbr_fill = c->pc_nbr_fill.ptr;
  p.nbr_off = c->pc_nbr_off.ptr;
  CK(pc_fill(p, st), "power cell records");
  p.se = c->pc_fe_i.ptr;
  p.ce = p.se + 5 * n_se;
  p.se_end = p.ce + 5 * n_ce;
  p.se_end_pos = c->pc_fe_pos.ptr;
  if (n_se + n_ce + n_end > 0) CK(pc_feature_edges(p, 1, st), "feature edge records");
  // stable sorts: by (site, key) for faces and facets; edges by the
  // neighbour pair, then by site; cells by site
  int site_bits = 1;
  while ((1ll << site_bits) < (long long)std::max(n_site, 1)) ++site_bits;
  auto sort = [&](int k, int bits) {
    return radix_sort_pairs(keys[k], vals[k], seg[k], bits, c->pc_keys_tmp.ptr, c->pc_vals_tmp.ptr,
                            c->pc_hist.ptr, c->pc_scan_i.ptr, st);
  };
  CK(sort(0, 32 + site_bits), "sort");
  CK(sort(1, 32 + site_bits), "sort");
  CK(sort(2, 32 + site_bits), "sort");
  CK(pc_edges_finish(p, n_ed, 0, st), "edge keys");
  CK(sort(2, site_bits), "sort");
  CK(pc_edges_finish(p, n_ed, 1, st), "edge gather");
  CK(sort(3, site_bits), "sort");
  long long* so = c->pc_site_off.ptr;
  CK(pc_site_offsets(keys[3], n, n_site, 0, so, st), "offsets");
  CK(pc_site_offsets(keys[1], n_fa, n_site, 32, so + (n_site + 1), st), "offsets");
  CK(pc_site_offsets(keys[2], n_ed, n_site, 0, so + 2 * (n_site + 1), st), "offsets");
  // neighbour cells across tet faces
  CK(cudaMemsetAsync(c->pc_nbr_cnt.ptr, 0, sizeof(int32_t) * (size_t)std::max(n, 1ll), st), "memset");
  CK(cudaMemsetAsync(c->pc_nbr_fill.ptr, 0, sizeof(int32_t) * (size_t)std::max(n, 1ll), st), "memset");
  CK(pc_neighbours(p, n_tf, 0, st), "neighbours");
  CK(scan64_exclusive(c->pc_nbr_cnt.ptr, c->pc_nbr_off.ptr, n, c->pc_scan.ptr, st), "scan");
  long long n_nbr = 0;
  CK(cudaMemcpyAsync(&n_nbr, c->pc_nbr_off.ptr + n, sizeof(n_nbr), cudaMemcpyDeviceToHost, st), "D2H");
  CK(cudaStreamSynchronize(st), "sync");
  CK(c->pc_nbr.ensure((size_t)std::max(n_nbr, 1ll)), "alloc");
  p.nbr = c->pc_nbr.ptr;
  CK(pc_neighbours(p, n_tf, 1, st), "neighbours");
  CK(pc_neighbours(p, n_tf, 2, st), "neighbours");
  // connected components: cc_cells, facet_cc_cells, edge_cc_cells
  const long long n_all = n + n_fa + n_ed;
  if (n_all > 0x7fffffffll) return fail(c, RPD_ERR_CAPACITY, "rpd_compute_power_cells: too many records");
  // int32: parent, root, rank, flag, croot (n_all each), size (n_fa), the
  // three labels (n_all); int64: pos, gstart (n_all + 1), gid (n_all)
  CK(c->pc_cc_i.ensure((size_t)(6 * n_all + n_fa + 1)), "alloc");
  CK(c->pc_cc_l.ensure((size_t)(3 * n_all + 2 + power_cell_components_temp(n_all))), "alloc");
  CK(c->pc_cc_err.ensure(1), "alloc");
  CK(cudaMemsetAsync(c->pc_cc_err.ptr, 0, sizeof(unsigned int), st), "memset");
  CcParams cp = {};
  cp.n = n;
  cp.n_fa = n_fa;
  cp.n_ed = n_ed;
  cp.nbr_off = c->pc_nbr_off.ptr;
  cp.nbrs = c->pc_nbr.ptr;
  cp.site_key = keys[3];
  cp.site_cells = vals[3];
  cp.facet_keys = keys[1];
  cp.facet_cells = vals[1];
  cp.edges = c->pc_ed_out.ptr;
  cp.parent = c->pc_cc_i.ptr;
  cp.root = cp.parent + n_all;
  cp.rank = cp.root + n_all;
  cp.flag = cp.rank + n_all;
  cp.croot = cp.flag + n_all;
  cp.size = cp.croot + n_all;
  cp.cell_cc = cp.size + n_fa;
  cp.facet_cc = cp.cell_cc + n;
  cp.edge_cc = cp.facet_cc + n_fa;
  cp.pos = c->pc_cc_l.ptr;
  cp.gstart = cp.pos + (n_all + 1);
  cp.gid = cp.gstart + (n_all + 1);
  cp.scan_tmp = cp.gid + n_all;
  cp.err = c->pc_cc_err.ptr;
  CK(power_cell_components(cp, st), "components");
  // surface groups (update_sphere_surf_v2fids), with a surface mesh set
  const long long n_sg = c->sf_faces > 0 ? n_sf : 0;
  const size_t sg_hist = radix_hist_ints(std::max(n_sg, 1ll));
  CK(c->sfg_k.ensure((size_t)std::max(3 * n_sg, 3ll)), "alloc");
  CK(c->sfg_v.ensure((size_t)std::max(2 * n_sg, 2ll)), "alloc");
  CK(c->sfg_i.ensure((size_t)std::max(8 * n_sg, 8ll) + sg_hist + scan_temp_ints((long long)sg_hist) + 16),
     "alloc");
  CK(c->sfg_l.ensure((size_t)(n_sg + 1 + (n_site + 1) + scan64_temp(std::max(n_sg, 1ll)) + 16)), "alloc");
  SurfaceGroupParams sg = {};
  sg.n_sf = n_sg;
  sg.n_site = n_site;
  sg.site_bits = site_bits;
  sg.cells = c->cells.ptr;
  sg.surface_cell = p.sf_cell;
  sg.surface_fid = p.sf_fid;
  sg.facet_adj = c->sf_adj.ptr;
  sg.n_faces = c->sf_faces;
  sg.no_cross = c->sf_no_cross.ptr;
  sg.n_no_cross = c->sf_n_no_cross;
  const long long m = std::max(n_sg, 1ll);
  sg.keys = c->sfg_k.ptr;
  sg.keys_tmp = sg.keys + m;
  sg.ekey = sg.keys_tmp + m;
  sg.vals = c->sfg_v.ptr;
  sg.vals_tmp = sg.vals + m;
  sg.flag = c->sfg_i.ptr;
  sg.erec = sg.flag + m;
  sg.parent = sg.erec + m;
  sg.root = sg.parent + m;
  sg.rank = sg.root + m;
  sg.out_group = sg.rank + m;
  sg.out_fid = sg.out_group + m;
  sg.out_rec = sg.out_fid + m;
  sg.hist = sg.out_rec + m;
  sg.hist_tmp = sg.hist + sg_hist;
  sg.pos = c->sfg_l.ptr;
  sg.site_off = sg.pos + (m + 1);
  sg.scan_tmp = sg.site_off + (n_site + 1);
  sg.err = c->pc_cc_err.ptr;
  long long n_sfg = 0;
  CK(surface_groups(sg, &n_sfg, st), "surface groups");
  unsigned int cc_err = 0;
  CK(cudaMemcpyAsync(&cc_err, c->pc_cc_err.ptr, sizeof(cc_err), cudaMemcpyDeviceToHost, st), "D2H");
  CK(cudaEventRecord(c->ev[kEvTopo1], st), "event");
  CK(cudaStreamSynchronize(st), "sync");
  if (cc_err) return fail(c, RPD_ERR_CUDA, "rpd_compute_power_cells: component search did not finish");
  if (ms) CK(cudaEventElapsedTime(ms, c->ev[kEvTopo0], c->ev[kEvTopo1]), "event time");
  rpd_power_cells_view& v = c->pc_view;
  v.n_site = n_site;
  v.n_cells = n;
  v.site_cell_off = reinterpret_cast<const int64_t*>(so);
  v.site_cells = vals[3];
  v.cell_nbr_off = reinterpret_cast<const int64_t*>(c->pc_nbr_off.ptr);
  v.cell_nbrs = c->pc_nbr.ptr;
  v.cell_tfid_off = reinterpret_cast<const int64_t*>(c->pc_off.ptr);
  v.cell_tfids = c->pc_tf_fid.ptr;
  v.n_facets = n_fa;
  v.site_facet_off = reinterpret_cast<const int64_t*>(so + (n_site + 1));
  v.facet_keys = reinterpret_cast<const uint64_t*>(keys[1]);
  v.facet_cells = vals[1];
  v.n_edges = n_ed;
  v.site_edge_off = reinterpret_cast<const int64_t*>(so + 2 * (n_site + 1));
  v.edges = c->pc_ed_out.ptr;
  v.n_vertices = n_vx;
  v.cell_vertex_off = reinterpret_cast<const int64_t*>(c->pc_off.ptr + 3 * (n + 1));
  v.vertex_cell = p.vx_cell;
  v.vertex_lvid = p.vx_lvid;
  v.vertex_ids = p.vx_ids;
  v.vertex_pos = p.vx_pos;
  v.vertex_sfid = p.vx_sfid;
  v.n_surface = n_sf;
  v.cell_surface_off = reinterpret_cast<const int64_t*>(c->pc_off.ptr + 4 * (n + 1));
  v.surface_cell = p.sf_cell;
  v.surface_fid = p.sf_fid;
  v.surface_pos = p.sf_pos;
  v.n_se_covered = n_se;
  v.cell_se_covered_off = reinterpret_cast<const int64_t*>(c->pc_off.ptr + 5 * (n + 1));
  v.se_covered = p.se;
  v.n_ce_covered = n_ce;
  v.cell_ce_covered_off = reinterpret_cast<const int64_t*>(c->pc_off.ptr + 6 * (n + 1));
  v.ce_covered = p.ce;
  v.n_se_line_end = n_end;
  v.cell_se_line_end_off = reinterpret_cast<const int64_t*>(c->pc_off.ptr + 7 * (n + 1));
  v.se_line_end = p.se_end;
  v.se_line_end_pos = p.se_end_pos;
  v.n_sfg = n_sfg;
  v.site_sfg_off = reinterpret_cast<const int64_t*>(sg.site_off);
  v.sfg_group = sg.out_group;
  v.sfg_fid = sg.out_fid;
  v.sfg_record = sg.out_rec;
  v.cell_cc = cp.cell_cc;
  v.facet_cc = cp.facet_cc;
  v.edge_cc = cp.edge_cc;
  c->pc_n_nbr = n_nbr;
  c->has_power_cells = true;
  return RPD_OK;
}

rpd_status rpd_get_power_cells(rpd_ctx* c, rpd_power_cells_view* v) {
  if (!c || !v) return RPD_ERR_INVALID_ARGUMENT;
  if (!c->has_result || !c->has_power_cells)
    return fail(c, RPD_ERR_NOT_READY, "rpd_get_power_cells: call rpd_compute_power_cells first");
  *v = c->pc_view;
  return RPD_OK;
}

rpd_status rpd_copy_device_to_host(rpd_ctx* c, void* dst, const void* src, int64_t bytes) {
  if (!c || bytes < 0 || (bytes > 0 && (!dst || !src))) return RPD_ERR_INVALID_ARGUMENT;
  if (bytes == 0) return RPD_OK;
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  CK(cudaMemcpyAsync(dst, src, (size_t)bytes, cudaMemcpyDeviceToHost, c->stream), "D2H");
  CK(cudaStreamSynchronize(c->stream), "copy sync");
  return RPD_OK;
}

// ---- incremental update ---------------------------------------------------
rpd_status rpd_compute_partial(rpd_ctx* c, const uint32_t* recompute, rpd_stats* stats) {
  if (!c || !recompute) return RPD_ERR_INVALID_ARGUMENT;
  if (!c->cells_for_mesh)
    return fail(c, RPD_ERR_NOT_READY,
                "rpd_compute_partial: needs the cells of a previous rpd_compute on this mesh and "
                "site count");
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  cudaStream_t st = c->stream;
  const int n_site = c->n_site;
  // the previous cells move aside; the partial compute runs with the
  // recomputed sites' flags (and the caller's: unselected sites stay so)
  c->cells.swap(c->prev_cells);
  c->payload.swap(c->prev_payload);
  const long long n_old = c->n_cells;
  c->cells_for_mesh = false;
  CK(c->partial_flags.ensure((size_t)n_site), "alloc");
  CK(c->user_flags.ensure((size_t)n_site), "alloc");
  std::vector<uint32_t> rf((size_t)n_site), uf((size_t)n_site);
  CK(cudaMemcpyAsync(uf.data(), c->flags.ptr, sizeof(uint32_t) * (size_t)n_site,
                     cudaMemcpyDeviceToHost, st), "D2H flags");
  CK(cudaStreamSynchronize(st), "sync");
  for (int i = 0; i < n_site; ++i) {
    rf[(size_t)i] = recompute[i] ? 1u : 0u;
    uf[(size_t)i] = uf[(size_t)i] == 1u && rf[(size_t)i] ? 1u : 0u;
  }
  CK(cudaMemcpyAsync(c->partial_flags.ptr, rf.data(), sizeof(uint32_t) * (size_t)n_site,
                     cudaMemcpyHostToDevice, st), "H2D flags");
  CK(cudaMemcpyAsync(c->user_flags.ptr, uf.data(), sizeof(uint32_t) * (size_t)n_site,
                     cudaMemcpyHostToDevice, st), "H2D flags");
  c->flags.swap(c->user_flags);  // user_flags now holds the caller's flags
  rpd_status s = rpd_compute(c, stats);
  c->flags.swap(c->user_flags);
  if (s != RPD_OK) return s;
  // merge: kept old cells (sites not recomputed) and the new cells, in
  // (tet, site) order
  const long long n_new = c->n_cells, n = n_old + n_new;
  CK(c->merge_keep.ensure((size_t)std::max(n_old, 1ll)), "alloc");
  CK(c->merge_keep_pos.ensure((size_t)n_old + 1), "alloc");
  CK(c->scan_tmp.ensure(scan_temp_ints(std::max(n_old, 1ll)) + 16), "alloc");
  CK(merge_keep(c->prev_cells.ptr, n_old, c->partial_flags.ptr, c->merge_keep.ptr, st), "merge");
  CK(scan_exclusive(c->merge_keep.ptr, c->merge_keep_pos.ptr, n_old, c->scan_tmp.ptr, st), "merge scan");
  int32_t n_kept = 0;
  CK(cudaMemcpyAsync(&n_kept, c->merge_keep_pos.ptr + n_old, sizeof(n_kept), cudaMemcpyDeviceToHost,
                     st), "D2H");
  CK(cudaStreamSynchronize(st), "sync");
  const long long n_out = n_kept + n_new;
  if (n_out > n) return fail(c, RPD_ERR_CUDA, "rpd_compute_partial: inconsistent merge");
  CK(c->merge_src.ensure((size_t)std::max(n_out, 1ll)), "alloc");
  CK(c->merge_units.ensure((size_t)std::max(n_out, 1ll)), "alloc");
  CK(c->merge_off.ensure((size_t)n_out + 1), "alloc");
  CK(c->merge_scan.ensure(scan64_temp(std::max(n_out, 1ll))), "alloc");
  CK(merge_slots(c->prev_cells.ptr, n_old, c->merge_keep.ptr, c->merge_keep_pos.ptr, c->cells.ptr,
                 n_new, n_out, c->merge_src.ptr, c->merge_units.ptr, st), "merge slots");
  CK(scan64_exclusive(c->merge_units.ptr, c->merge_off.ptr, n_out, c->merge_scan.ptr, st),
     "merge scan");
  long long units = 0;
  CK(cudaMemcpyAsync(&units, c->merge_off.ptr + n_out, sizeof(units), cudaMemcpyDeviceToHost, st),
     "D2H");
  CK(cudaStreamSynchronize(st), "sync");
  CK(c->merged_cells.ensure((size_t)std::max(n_out, 1ll)), "alloc");
  CK(c->merged_payload.ensure((size_t)std::max(16 * units, 16ll)), "alloc");
  CK(merge_gather(c->merge_src.ptr, n_out, c->merge_off.ptr, c->prev_cells.ptr, c->prev_payload.ptr,
                  c->cells.ptr, c->payload.ptr, c->merged_cells.ptr, c->merged_payload.ptr,
                  c->num_sms, st), "merge gather");
  CK(cudaStreamSynchronize(st), "sync");
  c->cells.swap(c->merged_cells);
  c->payload.swap(c->merged_payload);
  c->n_cells = n_out;
  c->payload_bytes = 16 * units;
  c->cells_for_mesh = true;
  return RPD_OK;
}

// ---- distance to local medial primitives ---------------------------------
rpd_status rpd_dist2mat(rpd_ctx* c, const float* spheres, int n_spheres, const float* samples,
                        int n_samples, const uint32_t* offsets, const uint32_t* counts,
                        const int32_t* prims, int64_t n_prims, float* dist, int32_t* closest,
                        int on_device) {
  if (!c) return RPD_ERR_INVALID_ARGUMENT;
  if (n_samples < 0 || n_spheres < 0 || n_prims < 0 || (n_samples > 0 && (!samples || !offsets ||
      !counts || !dist || !closest)) || (n_prims > 0 && (!prims || !spheres)))
    return fail(c, RPD_ERR_INVALID_ARGUMENT, "rpd_dist2mat: missing input");
  if (n_samples == 0) return RPD_OK;
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  cudaStream_t st = c->stream;
  const float4* d_sph = reinterpret_cast<const float4*>(spheres);
  const float3* d_smp = reinterpret_cast<const float3*>(samples);
  const int3* d_prm = reinterpret_cast<const int3*>(prims);
  const uint32_t *d_off = offsets, *d_cnt = counts;
  float* d_dist = dist;
  int32_t* d_cl = closest;
  auto h2d = [&](void* dst, const void* src, size_t bytes) {
    return bytes ? cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st) : cudaSuccess;
  };
  if (!on_device || (reinterpret_cast<uintptr_t>(spheres) & 15u)) {
    CK(c->d2m_spheres.ensure((size_t)std::max(n_spheres, 1)), "alloc");
    if (n_spheres > 0)
      CK(cudaMemcpyAsync(c->d2m_spheres.ptr, spheres, sizeof(float4) * (size_t)n_spheres,
                         on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, st),
         "copy spheres");
    d_sph = c->d2m_spheres.ptr;
  }
  if (!on_device) {
    CK(c->d2m_samples.ensure((size_t)n_samples), "alloc");
    CK(c->d2m_prims.ensure((size_t)std::max<int64_t>(n_prims, 1)), "alloc");
    CK(c->d2m_offsets.ensure((size_t)n_samples), "alloc");
    CK(c->d2m_counts.ensure((size_t)n_samples), "alloc");
    CK(c->d2m_dist.ensure((size_t)n_samples), "alloc");
    CK(c->d2m_closest.ensure((size_t)n_samples), "alloc");
    CK(h2d(c->d2m_samples.ptr, samples, sizeof(float3) * (size_t)n_samples), "H2D");
    CK(h2d(c->d2m_prims.ptr, prims, sizeof(int3) * (size_t)n_prims), "H2D");
    CK(h2d(c->d2m_offsets.ptr, offsets, sizeof(uint32_t) * (size_t)n_samples), "H2D");
    CK(h2d(c->d2m_counts.ptr, counts, sizeof(uint32_t) * (size_t)n_samples), "H2D");
    d_smp = c->d2m_samples.ptr;
    d_prm = c->d2m_prims.ptr;
    d_off = c->d2m_offsets.ptr;
    d_cnt = c->d2m_counts.ptr;
    d_dist = c->d2m_dist.ptr;
    d_cl = c->d2m_closest.ptr;
  }
  CK(c->d2m_bad.ensure(1), "alloc");
  CK(check_dist2mat(d_prm, n_prims, n_spheres, d_off, d_cnt, n_samples, c->d2m_bad.ptr, st),
     "dist2mat check");
  unsigned int bad = 0;
  CK(cudaMemcpyAsync(&bad, c->d2m_bad.ptr, sizeof(bad), cudaMemcpyDeviceToHost, st), "D2H");
  CK(cudaStreamSynchronize(st), "dist2mat sync");
  if (bad) return fail(c, RPD_ERR_INVALID_ARGUMENT, "rpd_dist2mat: sphere id or list out of range");
  CK(launch_dist2mat(d_smp, n_samples, d_sph, d_prm, d_off, d_cnt, d_dist, d_cl, st), "dist2mat");
  if (!on_device) {
    CK(cudaMemcpyAsync(dist, d_dist, sizeof(float) * (size_t)n_samples, cudaMemcpyDeviceToHost, st),
       "D2H");
    CK(cudaMemcpyAsync(closest, d_cl, sizeof(int32_t) * (size_t)n_samples, cudaMemcpyDeviceToHost,
                       st), "D2H");
  }
  CK(cudaStreamSynchronize(st), "dist2mat sync");
  return RPD_OK;
}

// ---- polygon soup of the emitted cells ----------------------------------
rpd_status rpd_compute_polygons(rpd_ctx* c, int triangulate, int boundary_only, int max_sf_fid,
                                float* ms) {
  if (!c) return RPD_ERR_INVALID_ARGUMENT;
  if (!c->has_result) return fail(c, RPD_ERR_NOT_READY, "rpd_compute_polygons: no result");
  if (!c->has_topology) {
    const rpd_status s = rpd_compute_topology(c, nullptr);
    if (s != RPD_OK) return s;
  }
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  cudaStream_t st = c->stream;
  const long long n = c->n_cells;
  CK(c->poly_cnt.ensure((size_t)std::max(3 * n, 3ll)), "alloc");
  CK(c->poly_off.ensure((size_t)(3 * (n + 1))), "alloc");
  CK(c->poly_scan_tmp.ensure(scan64_temp(std::max(n, 1ll))), "alloc");
  PolyParams p;
  p.cells = c->cells.ptr;
  p.n = n;
  p.payload = c->payload.ptr;
  p.topo_h = c->topo_h.ptr;
  p.topo = c->topo_buf.ptr;
  p.triangulate = triangulate != 0;
  p.boundary_only = boundary_only != 0;
  p.max_sf_fid = max_sf_fid;
  p.slice = c->poly_slice;
  for (int k = 0; k < 6; ++k) p.slice_plane[k] = c->poly_slice_plane[k];
  p.cnt_points = c->poly_cnt.ptr;
  p.cnt_polys = c->poly_cnt.ptr + n;
  p.cnt_indices = c->poly_cnt.ptr + 2 * n;
  long long* off = c->poly_off.ptr;
  p.off_points = off;
  p.off_polys = off + (n + 1);
  p.off_indices = off + 2 * (n + 1);
  CK(cudaEventRecord(c->ev[kEvTopo0], st), "event");
  CK(poly_count(p, st), "polygon counts");
  for (int k = 0; k < 3; ++k)
    CK(scan64_exclusive(c->poly_cnt.ptr + k * n, off + k * (n + 1), n, c->poly_scan_tmp.ptr, st),
       "polygon scan");
  long long tot[3];
  for (int k = 0; k < 3; ++k)
    CK(cudaMemcpyAsync(&tot[k], off + k * (n + 1) + n, sizeof(long long), cudaMemcpyDeviceToHost,
                       st), "D2H");
  CK(cudaStreamSynchronize(st), "polygon sync");
  if (tot[0] > 0xffffffffll)
    return fail(c, RPD_ERR_CAPACITY, "rpd_compute_polygons: more than 2^32 points");
  CK(c->poly_points.ensure((size_t)std::max(3 * tot[0], 3ll)), "alloc");
  CK(c->poly_offsets.ensure((size_t)tot[1] + 1), "alloc");
  CK(c->poly_indices.ensure((size_t)std::max(tot[2], 1ll)), "alloc");
  CK(c->poly_site.ensure((size_t)std::max(tot[1], 1ll)), "alloc");
  CK(c->poly_adj.ensure((size_t)std::max(tot[1], 1ll)), "alloc");
  p.points = c->poly_points.ptr;
  p.poly_offsets = c->poly_offsets.ptr;
  p.indices = c->poly_indices.ptr;
  p.poly_site = c->poly_site.ptr;
  p.poly_adj_site = c->poly_adj.ptr;
  CK(poly_fill(p, st), "polygons");
  CK(cudaMemcpyAsync(c->poly_offsets.ptr + tot[1], off + 2 * (n + 1) + n, sizeof(long long),
                     cudaMemcpyDeviceToDevice, st), "polygon end");
  CK(cudaEventRecord(c->ev[kEvTopo1], st), "event");
  CK(cudaStreamSynchronize(st), "polygon sync");
  if (ms) CK(cudaEventElapsedTime(ms, c->ev[kEvTopo0], c->ev[kEvTopo1]), "event time");
  c->n_poly_points = tot[0];
  c->n_polys = tot[1];
  c->n_poly_indices = tot[2];
  c->has_polygons = true;
  return RPD_OK;
}

rpd_status rpd_set_polygon_slice(rpd_ctx* c, int enable, const double* pos, const double* normal) {
  if (!c) return RPD_ERR_INVALID_ARGUMENT;
  if (!enable) {
    c->poly_slice = 0;
    return RPD_OK;
  }
  if (!pos || !normal) return fail(c, RPD_ERR_INVALID_ARGUMENT, "rpd_set_polygon_slice: no plane");
  for (int k = 0; k < 3; ++k)
    if (!std::isfinite(pos[k]) || !std::isfinite(normal[k]))
      return fail(c, RPD_ERR_INVALID_ARGUMENT, "rpd_set_polygon_slice: non-finite plane");
  for (int k = 0; k < 3; ++k) {
    c->poly_slice_plane[k] = pos[k];
    c->poly_slice_plane[3 + k] = normal[k];
  }
  c->poly_slice = 1;
  return RPD_OK;
}

namespace {
void be32(uint8_t* d, uint32_t v) {
  d[0] = (uint8_t)(v >> 24);
  d[1] = (uint8_t)(v >> 16);
  d[2] = (uint8_t)(v >> 8);
  d[3] = (uint8_t)v;
}
}  // namespace

rpd_status rpd_write_polygons_bgeo(rpd_ctx* c, const char* path, int64_t* bytes) {
  if (!c || !path) return RPD_ERR_INVALID_ARGUMENT;
  if (!c->has_result || !c->has_polygons)
    return fail(c, RPD_ERR_NOT_READY, "rpd_write_polygons_bgeo: call rpd_compute_polygons first");
  const long long n_pts = c->n_poly_points, n_polys = c->n_polys, n_idx = c->n_poly_indices;
  if (n_pts == 0) return fail(c, RPD_ERR_INVALID_ARGUMENT, "rpd_write_polygons_bgeo: no points");
  if (n_pts > 0x7fffffffll || n_polys > 0x7fffffffll)
    return fail(c, RPD_ERR_CAPACITY, "rpd_write_polygons_bgeo: counts above the format's int range");
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  cudaStream_t st = c->stream;
  const int wide = n_pts > (1ll << 16);
  const long long hdr = 41, pts = 16 * n_pts, attr = 20, polys = 13 * n_polys + (wide ? 4 : 2) * n_idx;
  const long long total = hdr + pts + attr + polys + 2;
  CK(c->bgeo_img.ensure((size_t)total), "alloc");
  uint8_t* img = c->bgeo_img.ptr;
  // header: 'Bgeo', 'V', version 5, points, polygons, point groups, primitive
  // groups, point attributes besides P, vertex attributes, primitive
  // attributes (PrimAttr), detail attributes
  uint8_t h[41];
  h[0] = 'B';
  h[1] = 'g';
  h[2] = 'e';
  h[3] = 'o';
  h[4] = 'V';
  const uint32_t hv[9] = {5u, (uint32_t)n_pts, (uint32_t)n_polys, 0u, 0u, 0u, 0u, 1u, 0u};
  for (int k = 0; k < 9; ++k) be32(h + 5 + 4 * k, hv[k]);
  // PrimAttr: name length, name, size 1, type integer, default 0
  uint8_t a[20] = {0, 8, 'P', 'r', 'i', 'm', 'A', 't', 't', 'r', 0, 1};
  be32(a + 12, 1u);
  be32(a + 16, 0u);
  const uint8_t foot[2] = {0x00, 0xff};
  CK(cudaMemcpyAsync(img, h, sizeof(h), cudaMemcpyHostToDevice, st), "H2D");
  CK(cudaMemcpyAsync(img + hdr + pts, a, sizeof(a), cudaMemcpyHostToDevice, st), "H2D");
  CK(cudaMemcpyAsync(img + total - 2, foot, sizeof(foot), cudaMemcpyHostToDevice, st), "H2D");
  CK(bgeo_fill(c->poly_points.ptr, n_pts, c->poly_offsets.ptr, c->poly_indices.ptr, c->poly_site.ptr,
               n_polys, wide, img + hdr, img + hdr + pts + attr, c->num_sms, st),
     "bgeo image");
  CK(cudaStreamSynchronize(st), "bgeo sync");
  FILE* f = std::fopen(path, "wb");
  if (!f) return fail(c, RPD_ERR_INVALID_ARGUMENT, "rpd_write_polygons_bgeo: cannot open the file");
  // through a pinned staging buffer, 32 MB at a time
  const size_t chunk = (size_t)32 << 20;
  void* stage = nullptr;
  if (cudaMallocHost(&stage, chunk) != cudaSuccess) {
    std::fclose(f);
    return fail(c, RPD_ERR_OUT_OF_MEMORY, "rpd_write_polygons_bgeo: pinned staging buffer");
  }
  rpd_status res = RPD_OK;
  for (long long at = 0; at < total && res == RPD_OK; at += (long long)chunk) {
    const size_t nb = (size_t)std::min((long long)chunk, total - at);
    if (cudaMemcpyAsync(stage, img + at, nb, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
      res = fail(c, RPD_ERR_CUDA, "rpd_write_polygons_bgeo: D2H");
    else if (std::fwrite(stage, 1, nb, f) != nb)
      res = fail(c, RPD_ERR_INVALID_ARGUMENT, "rpd_write_polygons_bgeo: write failed");
  }
  cudaFreeHost(stage);
  if (std::fclose(f) != 0 && res == RPD_OK)
    res = fail(c, RPD_ERR_INVALID_ARGUMENT, "rpd_write_polygons_bgeo: write failed");
  if (res == RPD_OK && bytes) *bytes = total;
  return res;
}

rpd_status rpd_get_polygons(rpd_ctx* c, rpd_polygon_view* v) {
  if (!c || !v) return RPD_ERR_INVALID_ARGUMENT;
  if (!c->has_result || !c->has_polygons)
    return fail(c, RPD_ERR_NOT_READY, "rpd_get_polygons: call rpd_compute_polygons first");
  v->n_points = c->n_poly_points;
  v->points = c->poly_points.ptr;
  v->n_polys = c->n_polys;
  v->poly_offsets = reinterpret_cast<const int64_t*>(c->poly_offsets.ptr);
  v->n_indices = c->n_poly_indices;
  v->indices = c->poly_indices.ptr;
  v->poly_site = c->poly_site.ptr;
  v->poly_adj_site = c->poly_adj.ptr;
  return RPD_OK;
}

rpd_status rpd_copy_polygons_to_host(rpd_ctx* c, float* points, int64_t max_points,
                                     int64_t* poly_offsets, uint32_t* indices, int64_t max_indices,
                                     int32_t* poly_site, int32_t* poly_adj_site, int64_t max_polys,
                                     int64_t* n_points, int64_t* n_polys, int64_t* n_indices) {
  if (!c) return RPD_ERR_INVALID_ARGUMENT;
  if (!c->has_result || !c->has_polygons)
    return fail(c, RPD_ERR_NOT_READY, "rpd_copy_polygons_to_host: call rpd_compute_polygons first");
  if (n_points) *n_points = c->n_poly_points;
  if (n_polys) *n_polys = c->n_polys;
  if (n_indices) *n_indices = c->n_poly_indices;
  if (!points && !poly_offsets && !indices && !poly_site && !poly_adj_site) return RPD_OK;
  if ((points && max_points < c->n_poly_points) || (indices && max_indices < c->n_poly_indices) ||
      ((poly_offsets || poly_site || poly_adj_site) && max_polys < c->n_polys))
    return fail(c, RPD_ERR_CAPACITY, "rpd_copy_polygons_to_host: buffers too small");
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  cudaStream_t st = c->stream;
  auto d2h = [&](void* dst, const void* src, size_t bytes) {
    return bytes ? cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, st) : cudaSuccess;
  };
  if (points) CK(d2h(points, c->poly_points.ptr, sizeof(float) * 3 * (size_t)c->n_poly_points), "D2H");
  if (poly_offsets)
    CK(d2h(poly_offsets, c->poly_offsets.ptr, sizeof(long long) * ((size_t)c->n_polys + 1)), "D2H");
  if (indices) CK(d2h(indices, c->poly_indices.ptr, sizeof(uint32_t) * (size_t)c->n_poly_indices), "D2H");
  if (poly_site) CK(d2h(poly_site, c->poly_site.ptr, sizeof(int32_t) * (size_t)c->n_polys), "D2H");
  if (poly_adj_site) CK(d2h(poly_adj_site, c->poly_adj.ptr, sizeof(int32_t) * (size_t)c->n_polys), "D2H");
  CK(cudaStreamSynchronize(st), "copy sync");
  return RPD_OK;
}

rpd_status rpd_copy_topology_hashes_to_host(rpd_ctx* c, uint64_t* hashes, int64_t capacity,
                                            int64_t* n_pairs) {
  if (!c) return RPD_ERR_INVALID_ARGUMENT;
  if (!c->has_result) return fail(c, RPD_ERR_NOT_READY, "rpd_copy_topology_hashes_to_host: no result");
  if (!c->cfg.topology_hash)
    return fail(c, RPD_ERR_NOT_READY, "rpd_copy_topology_hashes_to_host: topology_hash is off");
  if (n_pairs) *n_pairs = c->n_pairs;
  if (!hashes) return RPD_OK;
  if (capacity < c->n_pairs) return fail(c, RPD_ERR_CAPACITY, "rpd_copy_topology_hashes_to_host: buffer too small");
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  if (c->n_pairs > 0)
    CK(cudaMemcpyAsync(hashes, c->topo_hash.ptr, sizeof(uint64_t) * (size_t)c->n_pairs,
                       cudaMemcpyDeviceToHost, c->stream), "D2H");
  CK(cudaStreamSynchronize(c->stream), "sync");
  return RPD_OK;
}

rpd_status rpd_copy_pair_headers_to_host(rpd_ctx* c, rpd_cell_header* headers, int64_t capacity,
                                         int64_t* n_pairs) {
  if (!c) return RPD_ERR_INVALID_ARGUMENT;
  if (!c->has_result) return fail(c, RPD_ERR_NOT_READY, "rpd_copy_pair_headers_to_host: no result");
  if (n_pairs) *n_pairs = c->n_pairs;
  if (!headers) return RPD_OK;
  if (capacity < c->n_pairs) return fail(c, RPD_ERR_CAPACITY, "rpd_copy_pair_headers_to_host: buffer too small");
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  if (c->n_pairs > 0)
    CK(cudaMemcpyAsync(headers, c->pair_headers.ptr, sizeof(rpd_cell_header) * (size_t)c->n_pairs,
                       cudaMemcpyDeviceToHost, c->stream), "D2H");
  CK(cudaStreamSynchronize(c->stream), "sync");
  return RPD_OK;
}

rpd_status rpd_copy_neighbors_to_host(rpd_ctx* c, int32_t* nbr, int64_t capacity, int* k_out) {
  if (!c) return RPD_ERR_INVALID_ARGUMENT;
  if (k_out) *k_out = c->k;
  if (!nbr) return RPD_OK;
  long long n = (long long)c->n_site * c->k;
  if (capacity < n) return fail(c, RPD_ERR_CAPACITY, "rpd_copy_neighbors_to_host: buffer too small");
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  CK(cudaMemcpyAsync(nbr, c->nbr.ptr, sizeof(int32_t) * (size_t)n, cudaMemcpyDeviceToHost, c->stream), "D2H");
  CK(cudaStreamSynchronize(c->stream), "sync");
  return RPD_OK;
}

rpd_status rpd_copy_site_lists_to_host(rpd_ctx* c, int64_t* offsets, int32_t* ids,
                                       int64_t capacity, int64_t* n_total) {
  if (!c || !n_total) return RPD_ERR_INVALID_ARGUMENT;
  if (!c->has_result) return fail(c, RPD_ERR_NOT_READY, "rpd_copy_site_lists_to_host: no compute yet");
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  cudaStream_t st = c->stream;
  const int n_site = c->n_site, k = c->k;
  // the base lists in clip order: certified clipping reads the key-ordered
  // copy (GPU-built lists only)
  const bool knn = c->cfg.neighbor_source == RPD_NEIGH_KNN;
  const int32_t* base = (knn && c->cfg.certify) ? c->nbr_dist.ptr : c->nbr.ptr;
  std::vector<int32_t> nb((size_t)n_site * k), row((size_t)n_site, -1);
  CK(cudaMemcpyAsync(nb.data(), base, sizeof(int32_t) * nb.size(), cudaMemcpyDeviceToHost, st), "D2H");
  std::vector<long long> eoff;
  std::vector<int32_t> elen, enbr;
  if (c->ext_valid && c->ext_rows > 0) {
    eoff.resize((size_t)c->ext_rows);
    elen.resize((size_t)c->ext_rows);
    enbr.resize((size_t)c->ext_used);
    CK(cudaMemcpyAsync(row.data(), c->site_row.ptr, sizeof(int32_t) * (size_t)n_site,
                       cudaMemcpyDeviceToHost, st), "D2H");
    CK(cudaMemcpyAsync(eoff.data(), c->ext_off.ptr, sizeof(long long) * eoff.size(),
                       cudaMemcpyDeviceToHost, st), "D2H");
    CK(cudaMemcpyAsync(elen.data(), c->ext_len.ptr, sizeof(int32_t) * elen.size(),
                       cudaMemcpyDeviceToHost, st), "D2H");
    CK(cudaMemcpyAsync(enbr.data(), c->ext_nbr.ptr, sizeof(int32_t) * enbr.size(),
                       cudaMemcpyDeviceToHost, st), "D2H");
  }
  CK(cudaStreamSynchronize(st), "sync");
  long long pos = 0;
  for (int i = 0; i < n_site; ++i) {
    if (offsets) offsets[i] = pos;
    const int r = row[(size_t)i];
    const int32_t* L = r >= 0 ? enbr.data() + eoff[(size_t)r] : nb.data() + (size_t)i * k;
    const int n = r >= 0 ? elen[(size_t)r] : k;
    for (int q = 0; q < n; ++q) {
      const int32_t j = L[q];
      if (j < 0 || j == i) continue;  // holes, and the seed in a complete row
      if (ids) {
        if (pos >= capacity) return fail(c, RPD_ERR_CAPACITY, "rpd_copy_site_lists_to_host: buffer too small");
        ids[pos] = j;
      }
      ++pos;
    }
  }
  if (offsets) offsets[n_site] = pos;
  *n_total = pos;
  return RPD_OK;
}

rpd_status rpd_copy_pairs_to_host(rpd_ctx* c, int32_t* tet_offsets, int32_t* pair_sites,
                                  int64_t capacity, int64_t* n_pairs) {
  if (!c) return RPD_ERR_INVALID_ARGUMENT;
  if (!c->has_result) return fail(c, RPD_ERR_NOT_READY, "rpd_copy_pairs_to_host: no result");
  if (n_pairs) *n_pairs = c->n_pairs;
  if (!tet_offsets && !pair_sites) return RPD_OK;
  if (pair_sites && capacity < c->n_pairs) return fail(c, RPD_ERR_CAPACITY, "rpd_copy_pairs_to_host: buffer too small");
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  if (tet_offsets)
    CK(cudaMemcpyAsync(tet_offsets, c->tet_offsets.ptr, sizeof(int32_t) * ((size_t)c->n_tet + 1),
                       cudaMemcpyDeviceToHost, c->stream), "D2H");
  if (pair_sites && c->n_pairs > 0)
    CK(cudaMemcpyAsync(pair_sites, c->pair_site.ptr, sizeof(int32_t) * (size_t)c->n_pairs,
                       cudaMemcpyDeviceToHost, c->stream), "D2H");
  CK(cudaStreamSynchronize(c->stream), "sync");
  return RPD_OK;
}

// ---------------------------------------------------------------------------
// learned list length
// ---------------------------------------------------------------------------
rpd_status rpd_mlp_collect(rpd_ctx* c, int64_t max_samples, int64_t* n_total) {
  if (!c) return RPD_ERR_INVALID_ARGUMENT;
  if (max_samples < 0) return fail(c, RPD_ERR_INVALID_ARGUMENT, "rpd_mlp_collect: max_samples < 0");
  if (!c->cfg.certify || c->cfg.neighbor_source != RPD_NEIGH_KNN)
    return fail(c, RPD_ERR_INVALID_ARGUMENT, "rpd_mlp_collect: needs certify and GPU-built lists");
  // the plain method's cells: whole lists, certificate tested as it goes
  const rpd_config saved = c->cfg;
  const bool saved_klen = c->has_site_klen;
  const long long saved_pair_k = c->n_user_pair_k;
  c->cfg.learned_k = 0;
  c->has_site_klen = false;
  c->n_user_pair_k = -1;
  c->want_consumed = true;
  rpd_status s = rpd_compute(c, nullptr);
  c->want_consumed = false;
  c->cfg = saved;
  c->has_site_klen = saved_klen;
  c->n_user_pair_k = saved_pair_k;
  if (s != RPD_OK) return s;
  cudaStream_t st = c->stream;
  const long long n_pairs = c->n_pairs;
  if (n_pairs > 0 && max_samples > 0) {
    CK(c->reclip_idx.ensure((size_t)n_pairs), "alloc");
    CK(select_pairs(c->pair_headers.ptr, n_pairs, kSuccess, c->flag_tmp.ptr, c->pos_tmp.ptr,
                    c->scan_tmp.ptr, c->reclip_idx.ptr, st), "select");
    int32_t n_sel = 0;
    CK(cudaMemcpyAsync(&n_sel, c->pos_tmp.ptr + n_pairs, sizeof(n_sel), cudaMemcpyDeviceToHost, st), "D2H");
    CK(cudaStreamSynchronize(st), "collect sync");
    if (n_sel > 0) {
      // every stride-th emitted cell in (tet, site) order
      const long long stride = (n_sel + max_samples - 1) / max_samples;
      const long long take = (n_sel + stride - 1) / stride;
      std::vector<int32_t> sel((size_t)n_sel), sub((size_t)take);
      CK(cudaMemcpy(sel.data(), c->reclip_idx.ptr, sizeof(int32_t) * sel.size(), cudaMemcpyDeviceToHost), "D2H");
      for (long long q = 0; q < take; ++q) sub[(size_t)q] = sel[(size_t)(q * stride)];
      CK(c->sample_idx.ensure((size_t)take), "alloc");
      CK(c->mlp_target.ensure((size_t)take), "alloc");
      CK(cudaMemcpyAsync(c->sample_idx.ptr, sub.data(), sizeof(int32_t) * sub.size(), cudaMemcpyHostToDevice, st), "H2D");
      s = pair_features(c, c->sample_idx.ptr, take, c->mlp_target.ptr);
      if (s != RPD_OK) return s;
      const size_t nf = kMlpFeatures;
      CK(c->train_X.grow_keep((size_t)(c->n_train + take) * nf, (size_t)c->n_train * nf, st), "alloc");
      CK(c->train_y.grow_keep((size_t)(c->n_train + take), (size_t)c->n_train, st), "alloc");
      CK(cudaMemcpyAsync(c->train_X.ptr + (size_t)c->n_train * nf, c->feat.ptr,
                         sizeof(uint16_t) * nf * (size_t)take, cudaMemcpyDeviceToDevice, st), "D2D");
      CK(cudaMemcpyAsync(c->train_y.ptr + c->n_train, c->mlp_target.ptr, sizeof(float) * (size_t)take,
                         cudaMemcpyDeviceToDevice, st), "D2D");
      CK(cudaStreamSynchronize(st), "collect sync");
      c->n_train += take;
    }
  }
  if (n_total) *n_total = c->n_train;
  return RPD_OK;
}

rpd_status rpd_mlp_clear_samples(rpd_ctx* c) {
  if (!c) return RPD_ERR_INVALID_ARGUMENT;
  c->n_train = 0;
  return RPD_OK;
}

rpd_status rpd_mlp_copy_samples(rpd_ctx* c, uint16_t* x, float* y, int64_t capacity,
                                int64_t* n_samples) {
  if (!c) return RPD_ERR_INVALID_ARGUMENT;
  if (n_samples) *n_samples = c->n_train;
  if (!x && !y) return RPD_OK;
  if (capacity < c->n_train) return fail(c, RPD_ERR_CAPACITY, "rpd_mlp_copy_samples: buffer too small");
  if (c->n_train == 0) return RPD_OK;
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  if (x)
    CK(cudaMemcpy(x, c->train_X.ptr, sizeof(uint16_t) * kMlpFeatures * (size_t)c->n_train,
                  cudaMemcpyDeviceToHost), "D2H");
  if (y) CK(cudaMemcpy(y, c->train_y.ptr, sizeof(float) * (size_t)c->n_train, cudaMemcpyDeviceToHost), "D2H");
  return RPD_OK;
}

rpd_status rpd_mlp_train(rpd_ctx* c, int epochs, int batch, float lr, float miss_target,
                         uint64_t seed, rpd_mlp_report* report) {
  if (!c) return RPD_ERR_INVALID_ARGUMENT;
  if (epochs < 1 || batch < 16 || !(lr > 0.f) || !(miss_target > 0.f && miss_target < 1.f))
    return fail(c, RPD_ERR_INVALID_ARGUMENT, "rpd_mlp_train: bad arguments");
  if (c->n_train < 64) return fail(c, RPD_ERR_NOT_READY, "rpd_mlp_train: collect samples first");
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  cudaStream_t st = c->stream;
  rpd_status s = mlp_alloc(c);
  if (s != RPD_OK) return s;
  const long long n = c->n_train;
  std::vector<float> y_all((size_t)n);
  CK(cudaMemcpy(y_all.data(), c->train_y.ptr, sizeof(float) * (size_t)n, cudaMemcpyDeviceToHost), "D2H");
  // initialisation: uniform(+-sqrt(6 / fan_in)) weights (fan_in 12 for the
  // used features), zero biases, b3 = mean label
  std::mt19937_64 rng(seed);
  std::vector<float> prm((size_t)kMlpParams, 0.f);
  {
    std::uniform_real_distribution<float> u1(-std::sqrt(6.f / 12.f), std::sqrt(6.f / 12.f));
    std::uniform_real_distribution<float> u2(-std::sqrt(6.f / 64.f), std::sqrt(6.f / 64.f));
    std::uniform_real_distribution<float> u3(-std::sqrt(1.f / 64.f), std::sqrt(1.f / 64.f));
    size_t o = 0;
    for (int f = 0; f < kMlpFeatures; ++f)
      for (int h = 0; h < kMlpHidden; ++h) prm[o++] = f < 12 ? u1(rng) : 0.f;
    o += kMlpHidden;  // b1
    for (int e = 0; e < kMlpHidden * kMlpHidden; ++e) prm[o++] = u2(rng);
    o += kMlpHidden;  // b2
    for (int e = 0; e < kMlpHidden; ++e) prm[o++] = u3(rng);
    double mean = 0.0;
    for (float v : y_all) mean += v;
    prm[o] = (float)(mean / (double)n);
  }
  CK(cudaMemcpyAsync(c->mlp_params.ptr, prm.data(), sizeof(float) * prm.size(), cudaMemcpyHostToDevice, st), "H2D");
  CK(cudaMemsetAsync(c->mlp_grads.ptr, 0, sizeof(float) * kMlpParams, st), "memset");
  CK(cudaMemsetAsync(c->mlp_m.ptr, 0, sizeof(float) * kMlpParams, st), "memset");
  CK(cudaMemsetAsync(c->mlp_v.ptr, 0, sizeof(float) * kMlpParams, st), "memset");
  CK(launch_mlp_sync_operands(c->mlp_params.ptr, c->mlp_W1T.ptr, c->mlp_W2.ptr, c->mlp_W2T.ptr, st), "sync");
  // a random tenth held out for the margin
  std::vector<int32_t> perm((size_t)n);
  std::iota(perm.begin(), perm.end(), 0);
  std::shuffle(perm.begin(), perm.end(), rng);
  const long long n_cal = std::max<long long>(16, n / 10);
  const long long n_tr = n - n_cal;
  std::vector<int32_t> cal(perm.begin(), perm.begin() + n_cal), tr(perm.begin() + n_cal, perm.end());
  CK(c->train_idx.ensure((size_t)n), "alloc");
  CK(c->mlp_loss.ensure((size_t)epochs), "alloc");
  CK(cudaMemsetAsync(c->mlp_loss.ptr, 0, sizeof(float) * (size_t)epochs, st), "memset");
  const MlpWeights w = mlp_view(c);
  CK(cudaEventRecord(c->ev[kEvStart], st), "event");
  int step = 0;
  for (int e = 0; e < epochs; ++e) {
    std::shuffle(tr.begin(), tr.end(), rng);
    // pageable source: the call returns once the indices are staged
    CK(cudaMemcpyAsync(c->train_idx.ptr, tr.data(), sizeof(int32_t) * tr.size(), cudaMemcpyHostToDevice, st), "H2D");
    for (long long b = 0; b < n_tr; b += batch) {
      const long long nb = std::min<long long>(batch, n_tr - b);
      CK(launch_mlp_grad(c->train_X.ptr, c->train_y.ptr, c->train_idx.ptr + b, nb, 1.0f / (float)nb,
                         w, c->mlp_grads.ptr, c->mlp_loss.ptr + e, st), "grad");
      CK(launch_mlp_adam(c->mlp_params.ptr, c->mlp_grads.ptr, c->mlp_m.ptr, c->mlp_v.ptr, ++step, lr,
                         c->mlp_W1T.ptr, c->mlp_W2.ptr, c->mlp_W2T.ptr, st), "adam");
    }
    CK(cudaStreamSynchronize(st), "epoch sync");  // tr is reshuffled next
  }
  CK(cudaEventRecord(c->ev[kEvEnd], st), "event");
  std::vector<float> losses((size_t)epochs);
  CK(cudaMemcpyAsync(losses.data(), c->mlp_loss.ptr, sizeof(float) * losses.size(), cudaMemcpyDeviceToHost, st), "D2H");
  // held-out predictions
  CK(c->sample_idx.ensure((size_t)n_cal), "alloc");
  CK(c->mlp_y.ensure((size_t)n_cal), "alloc");
  CK(cudaMemcpyAsync(c->sample_idx.ptr, cal.data(), sizeof(int32_t) * cal.size(), cudaMemcpyHostToDevice, st), "H2D");
  CK(launch_mlp_predict(c->train_X.ptr, c->sample_idx.ptr, n_cal, w, 0.f, 1, 1 << 20, nullptr,
                        c->mlp_y.ptr, st), "predict");
  std::vector<float> yc((size_t)n_cal);
  CK(cudaMemcpyAsync(yc.data(), c->mlp_y.ptr, sizeof(float) * yc.size(), cudaMemcpyDeviceToHost, st), "D2H");
  CK(cudaStreamSynchronize(st), "train sync");
  float ms = 0.f;
  cudaEventElapsedTime(&ms, c->ev[kEvStart], c->ev[kEvEnd]);
  // margin: the (1 - miss_target) quantile of label - prediction
  std::vector<float> resid((size_t)n_cal);
  std::vector<int> kstar((size_t)n_cal);
  double cal_loss = 0.0;
  for (long long q = 0; q < n_cal; ++q) {
    const float t = y_all[(size_t)cal[(size_t)q]];
    resid[(size_t)q] = t - yc[(size_t)q];
    cal_loss += (double)resid[(size_t)q] * resid[(size_t)q];
    kstar[(size_t)q] = (int)std::lround(std::exp2((double)t));
  }
  std::vector<float> rs(resid);
  std::sort(rs.begin(), rs.end());
  const long long qi = std::min<long long>(n_cal - 1, (long long)std::ceil((1.0 - miss_target) * (double)n_cal) - 1);
  const float margin = rs[(size_t)std::max<long long>(qi, 0)] + 1e-4f;
  const int kmax = std::max(c->k, 1);
  long long miss = 0;
  double sum_k = 0.0;
  for (long long q = 0; q < n_cal; ++q) {
    int kk = (int)std::ceil(std::exp2(std::min(yc[(size_t)q] + margin, 10.0f)));
    kk = std::min(std::max(kk, 1), kmax);
    sum_k += kk;
    if (kstar[(size_t)q] > kk) ++miss;
  }
  std::vector<int> ks(kstar);
  std::sort(ks.begin(), ks.end());
  const int const_k = ks[(size_t)std::max<long long>(qi, 0)];
  c->mlp_margin = margin;
  c->mlp_ready = true;
  if (report) {
    std::memset(report, 0, sizeof(*report));
    report->n_train = n_tr;
    report->n_calib = n_cal;
    report->loss_first = losses.front() / (float)n_tr;
    report->loss_last = losses.back() / (float)n_tr;
    report->calib_loss = (float)(cal_loss / (double)n_cal);
    report->margin = margin;
    report->calib_miss_rate = (float)miss / (float)n_cal;
    report->calib_mean_k = (float)(sum_k / (double)n_cal);
    report->const_k = (float)std::min(const_k, kmax);
    report->ms_train = ms;
    report->steps = step;
    report->epochs = epochs;
    double mu = 0.0, m2 = 0.0;
    for (float v : y_all) mu += v;
    mu /= (double)n;
    for (float v : y_all) m2 += ((double)v - mu) * ((double)v - mu);
    report->label_var = (float)(m2 / (double)n);
  }
  return RPD_OK;
}

rpd_status rpd_mlp_enable(rpd_ctx* c, int on) {
  if (!c) return RPD_ERR_INVALID_ARGUMENT;
  if (on != 0 && on != 1) return fail(c, RPD_ERR_INVALID_ARGUMENT, "rpd_mlp_enable: on must be 0 or 1");
  if (on && !c->cfg.certify) return fail(c, RPD_ERR_INVALID_ARGUMENT, "rpd_mlp_enable: needs certify");
  c->cfg.learned_k = on;
  return RPD_OK;
}

rpd_status rpd_mlp_get_params(rpd_ctx* c, float* params, int n_params, float* margin) {
  if (!c) return RPD_ERR_INVALID_ARGUMENT;
  if (!c->mlp_ready) return fail(c, RPD_ERR_NOT_READY, "rpd_mlp_get_params: no predictor");
  if (params && n_params < kMlpParams) return fail(c, RPD_ERR_CAPACITY, "rpd_mlp_get_params: buffer too small");
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  if (params)
    CK(cudaMemcpy(params, c->mlp_params.ptr, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost), "D2H");
  if (margin) *margin = c->mlp_margin;
  return RPD_OK;
}

rpd_status rpd_mlp_set_params(rpd_ctx* c, const float* params, int n_params, float margin) {
  if (!c) return RPD_ERR_INVALID_ARGUMENT;
  if (!params || n_params != kMlpParams || !std::isfinite(margin))
    return fail(c, RPD_ERR_INVALID_ARGUMENT, "rpd_mlp_set_params: expected RPD_MLP_PARAMS floats");
  for (int i = 0; i < n_params; ++i)
    if (!std::isfinite(params[i])) return fail(c, RPD_ERR_INVALID_ARGUMENT, "rpd_mlp_set_params: non-finite parameter");
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  rpd_status s = mlp_alloc(c);
  if (s != RPD_OK) return s;
  cudaStream_t st = c->stream;
  CK(cudaMemcpyAsync(c->mlp_params.ptr, params, sizeof(float) * kMlpParams, cudaMemcpyHostToDevice, st), "H2D");
  CK(launch_mlp_sync_operands(c->mlp_params.ptr, c->mlp_W1T.ptr, c->mlp_W2.ptr, c->mlp_W2T.ptr, st), "sync");
  CK(cudaStreamSynchronize(st), "set_params sync");
  c->mlp_margin = margin;
  c->mlp_ready = true;
  return RPD_OK;
}

rpd_status rpd_mlp_forward(rpd_ctx* c, const uint16_t* x, int64_t n, float* y) {
  if (!c) return RPD_ERR_INVALID_ARGUMENT;
  if (n < 0 || (n > 0 && (!x || !y))) return fail(c, RPD_ERR_INVALID_ARGUMENT, "rpd_mlp_forward: bad arguments");
  if (!c->mlp_ready) return fail(c, RPD_ERR_NOT_READY, "rpd_mlp_forward: no predictor");
  if (n == 0) return RPD_OK;
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  cudaStream_t st = c->stream;
  CK(c->feat.ensure((size_t)n * kMlpFeatures), "alloc");
  CK(c->mlp_y.ensure((size_t)n), "alloc");
  CK(cudaMemcpyAsync(c->feat.ptr, x, sizeof(uint16_t) * kMlpFeatures * (size_t)n, cudaMemcpyHostToDevice, st), "H2D");
  c->n_feat_rows = n;
  CK(launch_mlp_predict(c->feat.ptr, nullptr, n, mlp_view(c), 0.f, 1, 1 << 20, nullptr, c->mlp_y.ptr, st), "predict");
  CK(cudaMemcpyAsync(y, c->mlp_y.ptr, sizeof(float) * (size_t)n, cudaMemcpyDeviceToHost, st), "D2H");
  CK(cudaStreamSynchronize(st), "forward sync");
  return RPD_OK;
}

rpd_status rpd_mlp_gradient(rpd_ctx* c, const uint16_t* x, const float* target, int64_t n,
                            float* grads, float* loss) {
  if (!c) return RPD_ERR_INVALID_ARGUMENT;
  if (n <= 0 || !x || !target || !grads) return fail(c, RPD_ERR_INVALID_ARGUMENT, "rpd_mlp_gradient: bad arguments");
  if (!c->mlp_ready) return fail(c, RPD_ERR_NOT_READY, "rpd_mlp_gradient: no parameters");
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  cudaStream_t st = c->stream;
  CK(c->feat.ensure((size_t)n * kMlpFeatures), "alloc");
  CK(c->mlp_target.ensure((size_t)n), "alloc");
  CK(c->mlp_loss.ensure(1), "alloc");
  CK(cudaMemcpyAsync(c->feat.ptr, x, sizeof(uint16_t) * kMlpFeatures * (size_t)n, cudaMemcpyHostToDevice, st), "H2D");
  CK(cudaMemcpyAsync(c->mlp_target.ptr, target, sizeof(float) * (size_t)n, cudaMemcpyHostToDevice, st), "H2D");
  CK(cudaMemsetAsync(c->mlp_grads.ptr, 0, sizeof(float) * kMlpParams, st), "memset");
  CK(cudaMemsetAsync(c->mlp_loss.ptr, 0, sizeof(float), st), "memset");
  c->n_feat_rows = n;
  CK(launch_mlp_grad(c->feat.ptr, c->mlp_target.ptr, nullptr, n, 1.0f / (float)n, mlp_view(c),
                     c->mlp_grads.ptr, c->mlp_loss.ptr, st), "grad");
  float l = 0.f;
  CK(cudaMemcpyAsync(grads, c->mlp_grads.ptr, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost, st), "D2H");
  CK(cudaMemcpyAsync(&l, c->mlp_loss.ptr, sizeof(float), cudaMemcpyDeviceToHost, st), "D2H");
  CK(cudaMemsetAsync(c->mlp_grads.ptr, 0, sizeof(float) * kMlpParams, st), "memset");
  CK(cudaStreamSynchronize(st), "gradient sync");
  if (loss) *loss = l / (float)n;
  return RPD_OK;
}

rpd_status rpd_mlp_copy_features(rpd_ctx* c, uint16_t* x, int64_t capacity, int64_t* n_rows) {
  if (!c) return RPD_ERR_INVALID_ARGUMENT;
  if (n_rows) *n_rows = c->n_feat_rows;
  if (!x) return RPD_OK;
  if (capacity < c->n_feat_rows) return fail(c, RPD_ERR_CAPACITY, "rpd_mlp_copy_features: buffer too small");
  if (c->n_feat_rows == 0) return RPD_OK;
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  CK(cudaMemcpy(x, c->feat.ptr, sizeof(uint16_t) * kMlpFeatures * (size_t)c->n_feat_rows,
                cudaMemcpyDeviceToHost), "D2H");
  return RPD_OK;
}

rpd_status rpd_mlp_copy_klen(rpd_ctx* c, int32_t* klen, int64_t capacity, int64_t* n_pairs) {
  if (!c) return RPD_ERR_INVALID_ARGUMENT;
  if (!c->has_result || !c->last_learned)
    return fail(c, RPD_ERR_NOT_READY, "rpd_mlp_copy_klen: no learned_k result");
  if (n_pairs) *n_pairs = c->n_pairs;
  if (!klen) return RPD_OK;
  if (capacity < c->n_pairs) return fail(c, RPD_ERR_CAPACITY, "rpd_mlp_copy_klen: buffer too small");
  if (c->n_pairs == 0) return RPD_OK;
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  CK(cudaMemcpy(klen, c->pair_klen.ptr, sizeof(int32_t) * (size_t)c->n_pairs, cudaMemcpyDeviceToHost), "D2H");
  return RPD_OK;
}

void* rpd_host_alloc(size_t bytes) {
  void* p = nullptr;
  if (cudaMallocHost(&p, bytes) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  // every page written once here: the first device->host copies into
  // pages never touched from the host ran at about 40 % of the link rate
  std::memset(p, 0, bytes);
  return p;
}

void rpd_host_free(void* p) {
  if (p) cudaFreeHost(p);
}

}  // extern "C"

rpd_status rpd_fail(rpd_ctx* c, rpd_status s, const std::string& msg) { return fail(c, s, msg); }
rpd_status rpd_cuda_fail(rpd_ctx* c, cudaError_t e, const char* where) { return cuda_fail(c, e, where); }
Grid rpd_make_grid(const double* lo, const double* hi, long long n_items, double per_cell) {
  return make_grid(lo, hi, n_items, per_cell);
}
rpd_status rpd_finish_compute(rpd_ctx* c, bool knn, bool learned, rpd_stats* stats, bool extend) {
  return finish_compute(c, knn, learned, stats, extend);
}
