// rpd_ctx.hpp -- the engine context behind the C ABI (host side, internal):
// device buffers, the stream, the events and the results of the last
// compute.  Shared by rpd_api.cpp (single meshes) and rpd_batch.cpp (batches
// of meshes).
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <utility>
#include <cstdint>
#include <string>

#include "../../include/rpd_gb300.h"
#include "rpd_common.cuh"
#include "rpd_kernels.cuh"

using namespace rpd;

namespace rpd_host {

template <class T>
struct DevBuf {
  T* ptr = nullptr;
  size_t cap = 0;  // elements
  cudaError_t ensure(size_t n) {
    if (n <= cap && ptr) return cudaSuccess;
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    cap = 0;
    size_t want = std::max<size_t>(n, 1);
    cudaError_t e = cudaMalloc((void**)&ptr, want * sizeof(T));
    if (e == cudaSuccess) cap = want;
    return e;
  }
  // grows to n elements keeping the first `keep` (stream-ordered copy)
  cudaError_t grow_keep(size_t n, size_t keep, cudaStream_t st) {
    if (n <= cap && ptr) return cudaSuccess;
    T* old = ptr;
    size_t want = std::max<size_t>(n, std::max<size_t>(2 * cap, 1));
    T* fresh = nullptr;
    cudaError_t e = cudaMalloc((void**)&fresh, want * sizeof(T));
    if (e != cudaSuccess) return e;
    if (old && keep) {
      e = cudaMemcpyAsync(fresh, old, keep * sizeof(T), cudaMemcpyDeviceToDevice, st);
      if (e == cudaSuccess) e = cudaStreamSynchronize(st);
      if (e != cudaSuccess) {
        cudaFree(fresh);
        return e;
      }
    }
    if (old) cudaFree(old);
    ptr = fresh;
    cap = want;
    return cudaSuccess;
  }
  void release() {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    cap = 0;
  }
  void swap(DevBuf& o) {
    std::swap(ptr, o.ptr);
    std::swap(cap, o.cap);
  }
  ~DevBuf() { release(); }
};

enum Ev {
  kEvStart, kEvKnn, kEvPairs, kEvPred0, kEvPred1, kEvClipK0, kEvClipK1, kEvEpi0, kEvClip, kEvEnd,
  kEvTopo0, kEvTopo1, kEvExt0, kEvExt1, kEvExtR0, kEvExtK, kEvCount
};

}  // namespace rpd_host

using namespace rpd_host;

struct rpd_ctx {
  rpd_config cfg;
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev[kEvCount] = {};
  std::string err;
  // page-locked, device-mapped staging for the small device->host reads of
  // set-up and compute (SmallReads): stores from a kernel, not the copy
  // engines, so another context's bulk copy does not hold them up
  static constexpr size_t kStageBytes = 64 << 10;
  uint8_t* stage_host = nullptr;
  uint8_t* stage_dev = nullptr;

  // mesh
  int n_vert = 0, n_tet = 0;
  DevBuf<float> vert3f;
  DevBuf<double> vert3d;
  DevBuf<float2> vert2;  // double-float copies (geometry epilogue)
  DevBuf<float2> face2;  // double-float face planes of every tet (geometry epilogue)
  DevBuf<int4> tets;
  DevBuf<int32_t> v_adjs, f_adjs, f_ids;
  DevBuf<uint8_t> e_adj6;
  double mesh_lo[3] = {0, 0, 0}, mesh_hi[3] = {0, 0, 0};
  double tet_radius = 0.0;
  // tets grouped by radius (largest vertex distance to the centroid): the
  // candidate search offsets each site's cell by its class's largest radius
  static constexpr int kClasses = 8;
  DevBuf<uint8_t> tet_class;
  int class_count[kClasses] = {0};
  double class_radius[kClasses] = {0};
  bool has_mesh = false;

  // sites
  int n_site = 0;
  DevBuf<float4> site4f;
  DevBuf<double> site4d;
  DevBuf<float2> site2;
  DevBuf<uint32_t> flags;
  double site_lo[3] = {0, 0, 0}, site_hi[3] = {0, 0, 0};
  float w_max = 0.f;
  bool has_sites = false;

  // neighbour lists
  int k = 0;
  DevBuf<int32_t> nbr, nbr_dist, nbr_ref_tmp, knn_status, site_klen, reclip_idx;
  bool has_site_klen = false;
  DevBuf<unsigned long long> topo_hash;
  long long n_reclipped = 0;
  DevBuf<float> nbr_keys;
  bool has_user_nbr = false;
  // per site: the ids its lists may hold (a batch: its mesh's sites); the
  // exact-lists rounds search the whole-context site grid with it
  DevBuf<int2> site_range;
  bool has_site_range = false;
  // per site: its place in the exact-lists rounds' site grid (a batch: its
  // mesh moved to a slot of its own), over [grid_lo, grid_hi]
  DevBuf<float4> site_gridpos;
  double grid_lo[3] = {0, 0, 0}, grid_hi[3] = {0, 0, 0};
  // exact lists (rpd_config.exact_lists): the completeness bound of every
  // base list, and the longer lists given to sites whose cells a pass left
  // uncertified -- row r of the extended lists starts at ext_off[r]
  DevBuf<float> nbr_bound;          // n_site
  DevBuf<unsigned int> site_need;   // n_site: radius bound (float bits), 0 = none
  DevBuf<int32_t> site_row;         // n_site: extended row, -1 = base list
  DevBuf<int32_t> ext_sites, site_flag, site_pos, ext_idx;
  DevBuf<int32_t> ext_nbr, ext_len;
  DevBuf<float> ext_keys, ext_bound;
  DevBuf<long long> ext_off;
  long long ext_used = 0;           // entries of ext_nbr / ext_keys in use
  int ext_rows = 0;                 // rows in use
  bool ext_valid = false;           // site_row / ext_* describe the last compute's lists

  // grids
  DevBuf<int32_t> s_cell_of, s_cell_count, s_cell_start, s_cell_fill, s_cell_items;
  DevBuf<int32_t> t_cell_of, t_cell_count, t_cell_start, t_cell_fill, t_cell_items;
  DevBuf<float> t_cell_rmax;
  DevBuf<float4> centroid, site_box, site_planes, tet_xyz;
  DevBuf<uchar4> tet_vadj;
  DevBuf<int32_t> site_nplanes, pair_ntasks, pair_taskoff;
  DevBuf<int32_t> scan_tmp;

  // pairs
  DevBuf<int2> pair_buf;
  DevBuf<int32_t> tet_count, tet_offsets, tet_fill, pair_site, pair_tet;
  long long pair_cap_hint = 0;

  // cells
  DevBuf<rpd_cell_header> pair_headers, cells;
  // per-cell topology of the emitted cells (rpd_compute_topology)
  DevBuf<int32_t> topo_units, topo_off;
  DevBuf<rpd_topo_header> topo_h;
  DevBuf<uint8_t> topo_buf;
  long long topo_bytes = 0;
  bool has_topology = false;
  // polygon soup of the emitted cells (rpd_compute_polygons)
  DevBuf<int32_t> poly_cnt;        // 3 x n_cells: points, polygons, indices per cell
  DevBuf<long long> poly_off;      // 3 x (n_cells + 1)
  DevBuf<long long> poly_scan_tmp;
  DevBuf<float> poly_points;
  DevBuf<long long> poly_offsets;
  DevBuf<uint32_t> poly_indices;
  DevBuf<int32_t> poly_site, poly_adj;
  long long n_poly_points = 0, n_polys = 0, n_poly_indices = 0;
  bool has_polygons = false;
  int poly_slice = 0;               // rpd_set_polygon_slice
  double poly_slice_plane[6] = {};  // pos, normal
  DevBuf<uint8_t> bgeo_img;         // Houdini file image
  // rpd_compute_partial: the previous cells, the merge's buffers, the
  // recomputed sites' flags
  bool cells_for_mesh = false;  // cells / payload hold every cell of the current mesh and sites
  DevBuf<rpd_cell_header> prev_cells, merged_cells;
  DevBuf<uint8_t> prev_payload, merged_payload;
  DevBuf<int32_t> merge_keep, merge_keep_pos, merge_units;
  DevBuf<long long> merge_src, merge_off, merge_scan;
  DevBuf<uint32_t> partial_flags, user_flags;
  // rpd_compute_power_cells
  DevBuf<int32_t> pc_cnt, pc_tf_fid, pc_ed_fields, pc_ed_out, pc_vx_i, pc_sf_i, pc_nbr_cnt,
      pc_nbr_fill, pc_nbr, pc_hist, pc_scan_i;
  DevBuf<long long> pc_off, pc_scan, pc_site_off, pc_nbr_off;
  DevBuf<unsigned long long> pc_keys, pc_keys_tmp;
  DevBuf<uint32_t> pc_vals, pc_vals_tmp;
  DevBuf<float> pc_vx_pos, pc_sf_pos;
  DevBuf<int32_t> pc_fe_i;
  DevBuf<int32_t> pc_cc_i;      // union-find arrays and the component labels
  DevBuf<long long> pc_cc_l;    // their scans and group ranges
  DevBuf<unsigned int> pc_cc_err;
  // surface mesh for the surface groups (rpd_set_surface_mesh) and scratch
  DevBuf<int32_t> sf_adj;
  DevBuf<unsigned long long> sf_no_cross;
  int sf_faces = 0;
  long long sf_n_no_cross = 0;
  DevBuf<unsigned long long> sfg_k;
  DevBuf<uint32_t> sfg_v;
  DevBuf<int32_t> sfg_i;
  DevBuf<long long> sfg_l;
  DevBuf<float> pc_fe_pos;
  // TetMesh::tet_es2fe_map: sorted unique keys and (type, id, line) values
  DevBuf<unsigned long long> fe_keys;
  DevBuf<int32_t> fe_vals;
  long long n_fe = 0;
  long long pc_n[5] = {0, 0, 0, 0, 0};
  long long pc_n_nbr = 0;
  bool has_power_cells = false;
  rpd_power_cells_view pc_view = {};
  // rpd_dist2mat scratch (host inputs are copied here)
  DevBuf<float4> d2m_spheres;
  DevBuf<float3> d2m_samples;
  DevBuf<int3> d2m_prims;
  DevBuf<uint32_t> d2m_offsets, d2m_counts;
  DevBuf<float> d2m_dist;
  DevBuf<int32_t> d2m_closest;
  DevBuf<unsigned int> d2m_bad;
  DevBuf<uint8_t> payload;
  DevBuf<int32_t> flag_tmp, pos_tmp;
  DevBuf<unsigned long long> scratch;  // [0] payload cursor [1] work [2..3] counters
                                       // [4] pair cursor [8..18] status hist
                                       // [32] cells still uncertified
  DevBuf<long long> n_out;
  long long payload_cap_hint = 0;

  // learned list length: features, predictor, training set
  double mesh_volume = 0.0;
  DevBuf<double> tet_rad;       // FP64 radius of every tet
  DevBuf<uint8_t> bmark;        // boundary vertex marks
  DevBuf<MeshPrepOut> prep;
  DevBuf<int32_t> prep_hist;
  DevBuf<float4> bverts;        // boundary vertices
  int n_bverts = 0;
  DevBuf<float> site_bdist;     // site -> nearest boundary vertex distance
  bool bdist_valid = false;
  DevBuf<uint16_t> feat;        // bf16 rows of the last features launch
  long long n_feat_rows = 0;
  DevBuf<int32_t> pair_klen, consumed, sample_idx;
  bool want_consumed = false;
  bool last_learned = false;
  DevBuf<int32_t> user_pair_k;   // rpd_set_pair_k
  long long n_user_pair_k = -1;
  DevBuf<float> mlp_params, mlp_grads, mlp_m, mlp_v, mlp_loss, mlp_y, mlp_target;
  DevBuf<uint16_t> mlp_W1T, mlp_W2, mlp_W2T;
  float mlp_margin = 0.f;
  bool mlp_ready = false;
  DevBuf<uint16_t> train_X;
  DevBuf<float> train_y;
  DevBuf<int32_t> train_idx;
  long long n_train = 0;

  // results of the last compute
  long long n_pairs = 0, n_cells = 0, payload_bytes = 0;
  int tet_k = 0;
  bool has_result = false;
};

// internal helpers of rpd_api.cpp used by the batch code
rpd_status rpd_fail(rpd_ctx* c, rpd_status s, const std::string& msg);
rpd_status rpd_cuda_fail(rpd_ctx* c, cudaError_t e, const char* where);
Grid rpd_make_grid(const double* lo, const double* hi, long long n_items, double per_cell);
// tets per cell of the pair search's tet grids: coarser cells mean fewer cell
// tests and more centroid tests; swept on the 1M-tet workload (k = 128), the
// pair stage takes 9.66 / 7.61 / 6.59 / 6.42 / 6.26 / 6.52 / 6.62 ms with 1 /
// 2 / 4 / 6 / 8 / 12 / 16, identical pairs
constexpr double kTetsPerCell = 8.0;
// CSR, clipping, epilogue, compaction and statistics once pair_buf /
// tet_count hold the candidate pairs (c->n_pairs of them)
rpd_status rpd_finish_compute(rpd_ctx* c, bool knn, bool learned, rpd_stats* stats,
                              bool extend = false);

#define RPD_CK(ctx, expr, where)                                      \
  do {                                                                \
    cudaError_t _e = (expr);                                          \
    if (_e != cudaSuccess) return rpd_cuda_fail((ctx), _e, (where));  \
  } while (0)
