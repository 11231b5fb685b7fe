/*
 * rpd_gb300_compat.hpp -- libmat's C++ entry point on top of the C ABI.
 *
 * Provides, with the exact signature of src/rpd3d/voronoi.h:52-61,
 *
 *   std::vector<ConvexCellHost> compute_clipped_voro_diagram_GPU(...)
 *
 * so RPD3D_GPU::calculate / calculate_partial (src/rpd3d_api/rpd_api.cxx:117,
 * :275) and every consumer of ConvexCellHost (rpd_update, matfun_fix,
 * IO_CUDA) keep working when libmat's src/rpd3d is replaced by
 * librpd_gb300.so.  Header-only on purpose: it fills the caller's own
 * ConvexCellHost type, so include libmat's voronoi_defs.h (ConvexCellHost,
 * cuchar4, cfloat5, cint2, cuchar3, Status) before this header.
 *
 * Inputs keep the reference's layouts: AoS float vertices, AoS tet indices,
 * the dense triangular e_adjs table (io.cxx:264-281), SoA float sites
 * (3 x n_site), float weights (r^2), site_knn with (site_k + 1) rows.
 * Behaviour kept: only flagged sites get cells; each neighbour list is
 * clipped in its order up to the first -1; cells whose clipping fails
 * (overflow, needs_perturb, ...) are dropped; the result is ordered by
 * (tet, site) with id = index; thread_id = tet * tet_k + slot.
 * Differences: errors throw std::runtime_error instead of exit(); `site`
 * is left unchanged (the reference copies it back unchanged);
 * site_cell_vol receives the FP64 volume of each site's cells (the
 * reference zeroes it).  num_itr_global, v2tets, nb_Lloyd_iter and
 * preferred_tet_k are unused, as in the reference.
 *
 * Topology: the cells come back with what update_power_cells
 * (src/rpd3d_base/rpd_update.cxx:568-638) would otherwise rebuild on the
 * host -- reload_active's active_clipping_planes / active_edges and
 * reload_pc_explicit's pc_local_active_faces / pc_lf2active_map / pc_points
 * (src/rpd3d_base/voronoi_defs.cxx:76-188) -- computed on the device by
 * rpd_compute_topology, with is_active_updated and is_pc_explicit set, so
 * the consumer skips both.  pc_points are filled by the caller's own
 * ConvexCellHost::compute_vertex_coordinates.  A cell with a NaN vertex is
 * left as the reference returns it (the consumer's reload_pc_explicit then
 * reports it).  euler stays -1, as in the reference's records
 * (cal_cell_euler computes it on demand).  Define
 * RPD_GB300_COMPAT_NO_TOPOLOGY to return the cells without topology.
 */
#ifndef RPD_GB300_COMPAT_HPP
#define RPD_GB300_COMPAT_HPP

#include <cstring>
#include <map>
#include <set>
#include <stdexcept>
#include <string>
#include <vector>

#include "rpd_gb300.h"

namespace rpd_gb300_detail {

inline void check(rpd_status s, rpd_ctx* ctx, const char* what) {
  if (s != RPD_OK) {
    std::string msg = std::string(what) + ": " + rpd_status_string(s);
    if (ctx) msg += std::string(" (") + rpd_last_error(ctx) + ")";
    throw std::runtime_error(msg);
  }
}

struct CtxGuard {
  rpd_ctx* c = nullptr;
  ~CtxGuard() { rpd_destroy(c); }
};

/* index of edge (v1, v2) in libmat's dense triangular table
 * (closed form of get_edge_idx, convex_cell.h:46-59) */
inline long long dense_edge_index(long long v1, long long v2, long long n) {
  long long lo = v1 < v2 ? v1 : v2, hi = v1 < v2 ? v2 : v1;
  return (lo + 1) * n - lo * (lo + 1) / 2 - (n - hi);
}

}  // namespace rpd_gb300_detail

inline std::vector<ConvexCellHost> compute_clipped_voro_diagram_GPU(
    const int num_itr_global, const std::vector<float>& vertices,
    const std::vector<int>& indices, const std::map<int, std::set<int>>& v2tets,
    const std::vector<int>& v_adjs, const std::vector<int>& e_adjs,
    const std::vector<int>& f_adjs, const std::vector<int>& f_ids,
    std::vector<float>& site, const int n_site,
    const std::vector<float>& site_weights, const std::vector<uint>& site_flags,
    const std::vector<int>& site_knn, const int site_k,
    std::vector<float>& site_cell_vol, const bool site_is_transposed,
    int nb_Lloyd_iter = 1, int preferred_tet_k = 0) {
  using namespace rpd_gb300_detail;
  (void)num_itr_global;
  (void)v2tets;
  (void)nb_Lloyd_iter;
  (void)preferred_tet_k;
  (void)site_is_transposed;
  const int n_vert = (int)(vertices.size() / 3);
  const int n_tet = (int)(indices.size() / 4);
  if (site.size() < (size_t)3 * n_site || site_weights.size() < (size_t)n_site ||
      site_flags.size() < (size_t)n_site || site_knn.size() < (size_t)(site_k + 1) * n_site)
    throw std::runtime_error("compute_clipped_voro_diagram_GPU: inconsistent input sizes");

  std::vector<double> xyz(vertices.begin(), vertices.begin() + 3 * (size_t)n_vert);
  std::vector<uint8_t> e_adj6((size_t)n_tet * 6);
  static const int kEdgeLv[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};
  for (long long t = 0; t < n_tet; ++t)
    for (int e = 0; e < 6; ++e)
      e_adj6[6 * t + e] = (uint8_t)e_adjs[(size_t)dense_edge_index(
          indices[4 * t + kEdgeLv[e][0]], indices[4 * t + kEdgeLv[e][1]], n_vert)];
  std::vector<double> xyzw((size_t)n_site * 4);
  for (long long i = 0; i < n_site; ++i) {
    xyzw[4 * i + 0] = site[i];
    xyzw[4 * i + 1] = site[i + n_site];
    xyzw[4 * i + 2] = site[i + 2 * (size_t)n_site];
    xyzw[4 * i + 3] = site_weights[i];
  }

  CtxGuard g;
  rpd_config cfg;
  rpd_config_default(&cfg);
  cfg.neighbor_source = RPD_NEIGH_USER;
  check(rpd_create(&cfg, &g.c), nullptr, "rpd_create");
  check(rpd_set_mesh(g.c, xyz.data(), n_vert, indices.data(), n_tet, v_adjs.data(),
                     e_adj6.data(), f_adjs.data(), f_ids.data()), g.c, "rpd_set_mesh");
  check(rpd_set_sites(g.c, xyzw.data(), n_site, site_flags.data()), g.c, "rpd_set_sites");
  check(rpd_set_neighbors(g.c, site_knn.data(), site_k, 1), g.c, "rpd_set_neighbors");
  rpd_stats st;
  check(rpd_compute(g.c, &st), g.c, "rpd_compute");
  int64_t n_cells = 0, n_bytes = 0, n_pairs = 0;
  check(rpd_copy_cells_to_host(g.c, nullptr, 0, nullptr, 0, &n_cells, &n_bytes), g.c, "copy");
  std::vector<rpd_cell_header> hd((size_t)n_cells);
  std::vector<uint8_t> pay((size_t)n_bytes + 16);
  check(rpd_copy_cells_to_host(g.c, hd.data(), n_cells, pay.data(), (int64_t)pay.size(),
                               &n_cells, &n_bytes), g.c, "copy");
  check(rpd_copy_pairs_to_host(g.c, nullptr, nullptr, 0, &n_pairs), g.c, "pairs");
  std::vector<int32_t> offs((size_t)n_tet + 1), psites((size_t)n_pairs + 1);
  check(rpd_copy_pairs_to_host(g.c, offs.data(), psites.data(), (int64_t)psites.size(), &n_pairs),
        g.c, "pairs");

  site_cell_vol.assign((size_t)n_site, 0.f);
  std::vector<double> vol_acc((size_t)n_site, 0.0);
  std::vector<ConvexCellHost> out((size_t)n_cells);
  for (long long q = 0; q < n_cells; ++q) {
    const rpd_cell_header& h = hd[q];
    ConvexCellHost& cc = out[q];
    const int nv = h.nb_v, np = h.nb_p, ne = h.nb_e;
    const size_t a16p = (8u * np + 15u) & ~15u, a16v = (4u * nv + 15u) & ~15u,
                 a16e = (4u * ne + 15u) & ~15u;
    const uint8_t* base = pay.data() + h.offset;
    const float* pl = reinterpret_cast<const float*>(base);
    const int32_t* id2 = reinterpret_cast<const int32_t*>(base + 16u * np);
    const uint8_t* ver = base + 16u * np + a16p;
    const uint8_t* edg = ver + a16v;
    const uint8_t* hh = edg + a16e;
    int slot = 0;
    for (int32_t r = offs[h.tet_id]; r < offs[h.tet_id + 1]; ++r)
      if (psites[r] == h.site_id) slot = r - offs[h.tet_id];
    cc.is_active = true;
    cc.status = static_cast<decltype(cc.status)>(h.status);
    cc.thread_id = h.tet_id * st.tet_k + slot;
    cc.voro_id = h.site_id;
    cc.tet_id = h.tet_id;
    cc.euler = -1.f;
    cc.weight = site_weights[h.site_id];
    cc.nb_v = (unsigned char)nv;
    cc.nb_p = (unsigned char)np;
    cc.nb_e = (unsigned char)ne;
    for (int i = 0; i < nv; ++i) {
      cc.ver_data_trans[i].x = ver[4 * i];
      cc.ver_data_trans[i].y = ver[4 * i + 1];
      cc.ver_data_trans[i].z = ver[4 * i + 2];
      cc.ver_data_trans[i].w = ver[4 * i + 3];
    }
    for (int i = 0; i < np; ++i) {
      cc.clip_data_trans[i].x = pl[4 * i];
      cc.clip_data_trans[i].y = pl[4 * i + 1];
      cc.clip_data_trans[i].z = pl[4 * i + 2];
      cc.clip_data_trans[i].w = pl[4 * i + 3];
      cc.clip_data_trans[i].h = (float)hh[i];
      cc.clip_id2_data_trans[i].x = id2[2 * i];
      cc.clip_id2_data_trans[i].y = id2[2 * i + 1];
    }
    for (int i = 0; i < ne; ++i) {
      cc.edge_data[i].x = edg[4 * i];
      cc.edge_data[i].y = edg[4 * i + 1];
      cc.edge_data[i].z = edg[4 * i + 2];
    }
    cc.cell_vol = -1.f;
    cc.id = (int)q;
    vol_acc[h.site_id] += h.volume;
  }
  for (int i = 0; i < n_site; ++i) site_cell_vol[i] = (float)vol_acc[i];
#ifndef RPD_GB300_COMPAT_NO_TOPOLOGY
  check(rpd_compute_topology(g.c, nullptr), g.c, "rpd_compute_topology");
  int64_t n_topo = 0, topo_bytes = 0;
  check(rpd_copy_topology_to_host(g.c, nullptr, 0, nullptr, 0, &n_topo, &topo_bytes), g.c,
        "topology");
  std::vector<rpd_topo_header> th((size_t)n_topo + 1);
  std::vector<uint8_t> trec((size_t)topo_bytes + 16);
  check(rpd_copy_topology_to_host(g.c, th.data(), n_topo, trec.data(), (int64_t)trec.size(),
                                  &n_topo, &topo_bytes), g.c, "topology");
  for (long long q = 0; q < n_cells; ++q) {
    ConvexCellHost& cc = out[q];
    const int nv = cc.nb_v, np = cc.nb_p, ne = cc.nb_e;
    const uint8_t* r = trec.data() + th[q].offset;
    const uint8_t* act = r + 4 * np;
    const int8_t* lf2a = reinterpret_cast<const int8_t*>(act + np);
    const uint8_t* acte = act + 2 * np;
    const uint8_t* faces = acte + ne;
    cc.active_clipping_planes.assign((size_t)np + 1, 0);
    for (int p = 0; p < np; ++p) cc.active_clipping_planes[p] = act[p];
    cc.active_edges.assign((size_t)ne + 1, 0);
    for (int e = 0; e < ne; ++e) cc.active_edges[e] = acte[e];
    cc.is_active_updated = true;
    if (th[q].flags & RPD_TOPO_VERTEX_NULL) continue;
    cc.pc_points.clear();
    for (int i = 0; i < nv; ++i) {
      const auto v = cc.compute_vertex_coordinates(cmake_uchar3(cc.ver_data_trans[i]));
      cc.pc_points.push_back(cmake_float3(v.x, v.y, v.z));
    }
    cc.pc_local_active_faces.assign(th[q].n_faces, std::vector<int>());
    cc.pc_lf2active_map.assign((size_t)np, -1);
    size_t slot = 0;
    for (int p = 0; p < np; ++p) {
      if (act[p] == 0) continue;
      cc.pc_lf2active_map[p] = lf2a[p];
      std::vector<int>& f = cc.pc_local_active_faces[(size_t)lf2a[p]];
      for (int k = 0; k < act[p]; ++k) f.push_back(faces[slot + k]);
      slot += act[p];
    }
    cc.is_pc_explicit = true;
  }
#endif
  return out;
}

#endif
