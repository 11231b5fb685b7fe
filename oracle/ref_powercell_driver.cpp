/*
 * ref_powercell_driver.cpp -- runs libmat's own power-cell construction on
 * the CPU: get_all_voro_info, update_sphere_surf_v2fids, update_pc_cc_info,
 * update_pc_facet_cc_info and update_pc_edge_cc_info
 * (src/rpd3d_base/rpd_update.cxx:80-521), per sphere in the order
 * update_power_cells calls them (:568-638), on cells in the packed record
 * layout of rpd_oracle.h, after the reference's own reload_active and
 * reload_pc_explicit (voronoi_defs.cxx).  The PowerCell maps come out as the
 * flat arrays of the oracle's power_cells (oracle/powercell_oracle.py).
 *
 * Test infrastructure: oracle/build.py compiles rpd_update.cxx:1-521 (the
 * three helpers, get_all_voro_info, the surface groups and the component
 * updates; the rest of the file needs the sphere model and geogram) from the
 * reference sources in place, read into the compiler's standard input, with
 * ref_pc_shim/ standing in for medial_sphere.h and input_types.h.  Never
 * shipped, used only to pin the oracle.
 */
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <exception>
#include <map>
#include <set>
#include <vector>

#include "medial_sphere.h"
#include "rpd_oracle.h"

void get_all_voro_info(const std::vector<ConvexCellHost>& voro_convex_cells,
                       PowerCell& powercell, const uint max_surf_fid,
                       const std::map<aint3, aint3>& tet_es2fe_map);
void update_sphere_surf_v2fids(const SurfaceMesh& sf_mesh, MedialSphere& msphere,
                               bool is_debug);
void update_pc_cc_info(PowerCell& pcell);
void update_pc_facet_cc_info(PowerCell& pcell, const int msphere_id);
void update_pc_edge_cc_info(PowerCell& pcell);

namespace {

size_t al16(size_t x) { return (x + 15) & ~(size_t)15; }

ConvexCellHost make_cell(const orc_cell_header& h, const uint8_t* rec, int id) {
  const int nv = h.nb_v, np = h.nb_p, ne = h.nb_e;
  const size_t o_id2 = (size_t)16 * np, o_ver = o_id2 + al16((size_t)8 * np),
               o_edge = o_ver + al16((size_t)4 * nv), o_h = o_edge + al16((size_t)4 * ne);
  ConvexCellHost cc;
  cc.status = Status::success;
  cc.is_active = true;
  cc.voro_id = h.site_id;
  cc.tet_id = h.tet_id;
  cc.id = id;
  cc.nb_v = (uchar)nv;
  cc.nb_p = (uchar)np;
  cc.nb_e = (uchar)ne;
  for (int i = 0; i < np; ++i) {
    float f[4];
    int32_t id2[2];
    std::memcpy(f, rec + 16 * i, 16);
    std::memcpy(id2, rec + o_id2 + 8 * i, 8);
    cc.clip_data_trans[i] = cmake_float5(f[0], f[1], f[2], f[3], (float)rec[o_h + i]);
    cc.clip_id2_data_trans[i] = cmake_int2(id2[0], id2[1]);
  }
  for (int i = 0; i < nv; ++i) {
    const uint8_t* v = rec + o_ver + 4 * i;
    cc.ver_data_trans[i] = cmake_uchar4(v[0], v[1], v[2], v[3]);
  }
  for (int i = 0; i < ne; ++i) {
    const uint8_t* e = rec + o_edge + 4 * i;
    cc.edge_data[i] = cmake_uchar3(e[0], e[1], e[2]);
  }
  cc.reload_active();
  cc.reload_pc_explicit();
  return cc;
}

// index of the set in `groups` that holds `x`, -1 if none
template <class G>
int group_of(const G& groups, int x) {
  for (size_t j = 0; j < groups.size(); ++j)
    if (groups[j].count(x)) return (int)j;
  return -1;
}

void put3(std::vector<float>& out, const Vector3& p) {
  out.push_back((float)p.x);
  out.push_back((float)p.y);
  out.push_back((float)p.z);
}

struct Result {
  // the oracle's record arrays (per-cell / per-site offsets are rebuilt from
  // these by the caller)
  std::vector<int32_t> site_cells;                        // per site, cells ascending
  std::vector<int32_t> nbr_cell, nbr;                     // (cell, neighbour) rows
  std::vector<int32_t> tfid_cell, tfid;                   // (cell, tet face) rows
  std::vector<int64_t> facet_keys;                        // site << 32 | neighbour
  std::vector<int32_t> facet_cells, facet_cc;
  std::vector<int32_t> cell_cc;                           // per cell
  std::vector<int32_t> edges, edge_cc;                    // 7 ints per edge row
  std::vector<int32_t> vertex_cell, vertex_lvid, vertex_ids, vertex_sfid;
  std::vector<float> vertex_pos;
  std::vector<int32_t> surface_cell, surface_fid;
  std::vector<float> surface_pos;
  std::vector<int32_t> sfg;                               // (site, group, fid, record)
  std::vector<int32_t> se_covered, ce_covered;            // 5 ints per row
  std::vector<int32_t> se_line_end;                       // 4 ints per row
  std::vector<float> se_line_end_pos;
  int64_t n_failed = 0;                                   // spheres that threw
  int64_t n_mismatch = 0;                                 // inconsistent maps
};

}  // namespace

extern "C" {

/* Runs the reference on the emitted cells (status success) of `headers`
 * (HEADER layout of rpd_oracle.h), in output order; cell ids are positions
 * among them.  fe: n_fe records (tet, lf_min, lf_max, fe_type, fe_id,
 * fe_line_id), later records replacing earlier ones with the same key.
 * sf_adj: n_faces x 3 face neighbours (-1 none) or NULL for no surface
 * groups; no_cross: n_nc face pairs across sharp edges.  Returns a handle
 * for ref_pc_get / ref_pc_free. */
void* ref_pc_run(int64_t n_headers, const orc_cell_header* headers, const uint8_t* payload,
                 int n_site, int max_sf_fid, int64_t n_fe, const int32_t* fe, int n_faces,
                 const int32_t* sf_adj, int64_t n_nc, const int32_t* no_cross) {
  Result* r = new Result();
  std::vector<const orc_cell_header*> cells;
  for (int64_t q = 0; q < n_headers; ++q)
    if (headers[q].status == ORC_SUCCESS) cells.push_back(headers + q);
  const int n = (int)cells.size();
  std::vector<ConvexCellHost> host(n);
  std::vector<std::vector<int>> by_site(n_site);
  for (int q = 0; q < n; ++q) {
    host[q] = make_cell(*cells[q], payload + cells[q]->offset, q);
    by_site[cells[q]->site_id].push_back(q);
  }
  std::map<aint3, aint3> fe_map;
  for (int64_t i = 0; i < n_fe; ++i) {
    const int32_t* x = fe + 6 * i;
    fe_map[aint3{{x[0], x[1], x[2]}}] = aint3{{x[3], x[4], x[5]}};
  }
  SurfaceMesh sf;
  sf.facets.adj = sf_adj;
  sf.facets.n = sf_adj ? n_faces : 0;
  for (int64_t i = 0; i < n_nc; ++i) {
    aint2 pr = {{no_cross[2 * i], no_cross[2 * i + 1]}};
    std::sort(pr.begin(), pr.end());
    sf.fe_sf_fs_pairs.insert(pr);
  }
  std::vector<std::set<int>> nbrs(n), tfids(n);
  std::vector<std::set<aint5>> se_cov(n), ce_cov(n);
  std::map<aint2, std::pair<aint3, v2int>> verts;  // (cell, lvid)
  std::map<int, std::vector<v2int>> surf;          // cell -> records
  std::map<aint4, Vector3> se_end;
  r->cell_cc.assign(n, -1);
  struct SiteOut {
    std::vector<std::pair<int64_t, int>> facets;  // (key, cell) with cc
    std::vector<int> facet_cc;
    std::vector<std::array<int, 7>> edges;
    std::vector<int> edge_cc;
    std::vector<std::vector<v2int>> groups;
  };
  std::vector<SiteOut> per_site(n_site);
  for (int s = 0; s < n_site; ++s) {
    for (int q : by_site[s]) r->site_cells.push_back(q);
    if (by_site[s].empty()) continue;
    std::vector<ConvexCellHost> ccells;
    MedialSphere ms;
    ms.id = s;
    for (int q : by_site[s]) {
      ccells.push_back(host[q]);
      ms.pcell.cell_ids.insert(q);
      ms.pcell.tet_ids.insert(host[q].tet_id);
    }
    ms.pcell.voro_id = s;
    try {
      get_all_voro_info(ccells, ms.pcell, (uint)max_sf_fid, fe_map);
      if (sf_adj) update_sphere_surf_v2fids(sf, ms, false);
      update_pc_cc_info(ms.pcell);
      update_pc_facet_cc_info(ms.pcell, ms.id);
      update_pc_edge_cc_info(ms.pcell);
    } catch (const std::exception&) {
      ++r->n_failed;
      continue;
    }
    const PowerCell& pc = ms.pcell;
    for (const auto& kv : pc.cell_neighbors) nbrs[kv.first].insert(kv.second.begin(), kv.second.end());
    for (const auto& kv : pc.cell_to_tfids) tfids[kv.first].insert(kv.second.begin(), kv.second.end());
    for (int q : by_site[s]) r->cell_cc[q] = group_of(pc.cc_cells, q);
    SiteOut& so = per_site[s];
    for (const auto& kv : pc.facet_neigh_to_cells) {
      const auto it = pc.facet_cc_cells.find(kv.first);
      for (int q : kv.second) {
        so.facets.emplace_back(((int64_t)s << 32) | (int64_t)(uint32_t)kv.first, q);
        so.facet_cc.push_back(it == pc.facet_cc_cells.end() ? -1 : group_of(it->second, q));
      }
    }
    for (const auto& kv : pc.edge_2endvertices) {
      const auto it = pc.edge_cc_cells.find(kv.first);
      for (const auto& ends : kv.second) {
        if (ends[0][0] != ends[1][0]) ++r->n_mismatch;  // both ends in one cell
        so.edges.push_back({s, kv.first[0], kv.first[1], ends[0][0], ends[0][1], ends[1][1], 0});
        so.edge_cc.push_back(it == pc.edge_cc_cells.end() ? -1 : group_of(it->second, ends[0][0]));
      }
    }
    for (const auto& kv : pc.vertex_2id) {
      const auto it = pc.vertex_2pos.find(kv.first);
      if (it == pc.vertex_2pos.end()) {
        ++r->n_mismatch;
        continue;
      }
      verts[kv.first] = std::make_pair(kv.second, it->second);
    }
    if (pc.vertex_2pos.size() != pc.vertex_2id.size()) ++r->n_mismatch;
    for (const auto& kv : pc.cell_to_surfv2fid) surf[kv.first] = kv.second;
    for (const auto& row : pc.se_covered_lvids) se_cov[row[0]].insert(row);
    for (const auto& row : pc.ce_covered_lvids) ce_cov[row[0]].insert(row);
    for (const auto& kv : pc.se_line_endpos) se_end[kv.first] = kv.second;
    so.groups = pc.surf_v2fid_in_groups;
  }
  for (int q = 0; q < n; ++q) {
    for (int x : nbrs[q]) {
      r->nbr_cell.push_back(q);
      r->nbr.push_back(x);
    }
    for (int x : tfids[q]) {
      r->tfid_cell.push_back(q);
      r->tfid.push_back(x);
    }
    for (const auto& row : se_cov[q]) r->se_covered.insert(r->se_covered.end(), row.begin(), row.end());
    for (const auto& row : ce_cov[q]) r->ce_covered.insert(r->ce_covered.end(), row.begin(), row.end());
  }
  for (int s = 0; s < n_site; ++s) {
    const SiteOut& so = per_site[s];
    for (size_t i = 0; i < so.facets.size(); ++i) {
      r->facet_keys.push_back(so.facets[i].first);
      r->facet_cells.push_back(so.facets[i].second);
      r->facet_cc.push_back(so.facet_cc[i]);
    }
    for (size_t i = 0; i < so.edges.size(); ++i) {
      r->edges.insert(r->edges.end(), so.edges[i].begin(), so.edges[i].end());
      r->edge_cc.push_back(so.edge_cc[i]);
    }
  }
  for (const auto& kv : verts) {
    r->vertex_cell.push_back(kv.first[0]);
    r->vertex_lvid.push_back(kv.first[1]);
    for (int a = 0; a < 3; ++a) r->vertex_ids.push_back(kv.second.first[a]);
    put3(r->vertex_pos, kv.second.second.first);
    r->vertex_sfid.push_back(kv.second.second.second);
  }
  // surface records in cell order; a group entry names the last record of
  // its face among the site's records
  std::vector<std::map<int, int>> last_rec(n_site);
  int rec = 0;
  for (const auto& kv : surf) {
    for (const auto& v2 : kv.second) {
      r->surface_cell.push_back(kv.first);
      r->surface_fid.push_back(v2.second);
      put3(r->surface_pos, v2.first);
      last_rec[cells[kv.first]->site_id][v2.second] = rec++;
    }
  }
  for (int s = 0; s < n_site; ++s) {
    const auto& groups = per_site[s].groups;
    for (size_t j = 0; j < groups.size(); ++j) {
      for (const auto& v2 : groups[j]) {
        const auto it = last_rec[s].find(v2.second);
        int at = -1;
        if (it != last_rec[s].end()) {
          at = it->second;
          const float* p = &r->surface_pos[3 * (size_t)at];
          if (p[0] != (float)v2.first.x || p[1] != (float)v2.first.y || p[2] != (float)v2.first.z)
            ++r->n_mismatch;
        }
        r->sfg.insert(r->sfg.end(), {s, (int32_t)j, v2.second, at});
      }
    }
  }
  for (const auto& kv : se_end) {
    r->se_line_end.insert(r->se_line_end.end(), kv.first.begin(), kv.first.end());
    put3(r->se_line_end_pos, kv.second);
  }
  return r;
}

/* Array `which` of a run (the order of REF_PC_ARRAYS in oracle.py): its
 * element count, copied to `out` when out is not NULL and cap suffices. */
int64_t ref_pc_get(void* handle, int which, void* out, int64_t cap) {
  const Result* r = static_cast<const Result*>(handle);
  const void* src = nullptr;
  int64_t n = 0;
  size_t es = 4;
  auto pick = [&](const auto& v) {
    src = v.data();
    n = (int64_t)v.size();
    es = sizeof(v[0]);
  };
  switch (which) {
    case 0: pick(r->site_cells); break;
    case 1: pick(r->nbr_cell); break;
    case 2: pick(r->nbr); break;
    case 3: pick(r->tfid_cell); break;
    case 4: pick(r->tfid); break;
    case 5: pick(r->facet_keys); break;
    case 6: pick(r->facet_cells); break;
    case 7: pick(r->facet_cc); break;
    case 8: pick(r->cell_cc); break;
    case 9: pick(r->edges); break;
    case 10: pick(r->edge_cc); break;
    case 11: pick(r->vertex_cell); break;
    case 12: pick(r->vertex_lvid); break;
    case 13: pick(r->vertex_ids); break;
    case 14: pick(r->vertex_pos); break;
    case 15: pick(r->vertex_sfid); break;
    case 16: pick(r->surface_cell); break;
    case 17: pick(r->surface_fid); break;
    case 18: pick(r->surface_pos); break;
    case 19: pick(r->sfg); break;
    case 20: pick(r->se_covered); break;
    case 21: pick(r->ce_covered); break;
    case 22: pick(r->se_line_end); break;
    case 23: pick(r->se_line_end_pos); break;
    case 24: return r->n_failed;
    case 25: return r->n_mismatch;
    default: return -1;
  }
  if (out && n <= cap && n > 0) std::memcpy(out, src, (size_t)n * es);
  return n;
}

void ref_pc_free(void* handle) { delete static_cast<Result*>(handle); }

}  // extern "C"
