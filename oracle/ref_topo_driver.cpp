/*
 * ref_topo_driver.cpp -- runs libmat's own host-side cell topology,
 * ConvexCellHost::reload_active, reload_pc_explicit, cal_cell_euler and
 * cal_halfplane_facet_euler (src/rpd3d_base/voronoi_defs.cxx:76-266), on
 * cells in the packed record layout of rpd_oracle.h, and writes what they
 * compute in the topology record layout of rpd_oracle.h.  Test
 * infrastructure: built by oracle/build.py into oracle/_ref/ together with
 * the reference's voronoi_defs.cxx (compiled in place, never copied) when
 * the reference sources are present; used only to pin the oracle.
 */
#include "voronoi_defs.h"

#include <cstring>
#include <thread>
#include <vector>

#include "rpd_oracle.h"

namespace {
size_t al16(size_t x) { return (x + 15) & ~(size_t)15; }

/* the record sizes of rpd_oracle.h, restated so this library stays
 * independent of the oracle */
size_t topo_bytes(int nb_v, int nb_p, int nb_e) {
  return al16((size_t)6 * nb_p + (size_t)nb_e + (size_t)3 * nb_v);
}

void one_cell(const orc_cell_header& h, const uint8_t* rec, orc_topo_header* th,
              uint8_t* out) {
  const int nv = h.nb_v, np = h.nb_p, ne = h.nb_e;
  const size_t o_id2 = (size_t)16 * np, o_ver = o_id2 + al16((size_t)8 * np),
               o_edge = o_ver + al16((size_t)4 * nv), o_h = o_edge + al16((size_t)4 * ne);
  ConvexCellHost cc;
  cc.status = Status::success;
  cc.voro_id = h.site_id;
  cc.tet_id = h.tet_id;
  cc.nb_v = (uchar)nv;
  cc.nb_p = (uchar)np;
  cc.nb_e = (uchar)ne;
  for (int i = 0; i < np; ++i) {
    float f[4];
    int32_t id[2];
    std::memcpy(f, rec + 16 * i, 16);
    std::memcpy(id, rec + o_id2 + 8 * i, 8);
    cc.clip_data_trans[i] = cmake_float5(f[0], f[1], f[2], f[3], (float)rec[o_h + i]);
    cc.clip_id2_data_trans[i] = cmake_int2(id[0], id[1]);
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
  const float euler = (float)cc.cal_cell_euler();

  std::memset(out, 0, topo_bytes(nv, np, ne));
  float* facet = reinterpret_cast<float*>(out);
  uint8_t* act = out + (size_t)4 * np;
  int8_t* lf2a = reinterpret_cast<int8_t*>(act + np);
  uint8_t* acte = act + (size_t)2 * np;
  uint8_t* faces = acte + ne;
  for (int p = 0; p < np; ++p) {
    act[p] = (uint8_t)cc.active_clipping_planes[p];
    lf2a[p] = cc.is_vertex_null ? -1 : (int8_t)cc.pc_lf2active_map[p];
    facet[p] = 0.f;
    const cint2 id = cc.clip_id2_const(p);
    if (cc.active_clipping_planes[p] > 0 && id.y != -1) {
      const int nb = id.x == cc.voro_id ? id.y : id.x;
      facet[p] = (float)cc.cal_halfplane_facet_euler(nb);
    }
  }
  for (int e = 0; e < ne; ++e) acte[e] = (uint8_t)cc.active_edges[e];
  size_t slot = 0;
  if (cc.is_vertex_null) {
    std::memset(faces, 255, (size_t)3 * nv);
  } else {
    for (const auto& f : cc.pc_local_active_faces)
      for (int v : f) faces[slot++] = (uint8_t)v;
  }
  th->euler = euler;
  th->n_faces = cc.is_vertex_null ? 0 : (uint8_t)cc.pc_local_active_faces.size();
  th->flags = cc.is_vertex_null ? 1 : 0;
  th->pad[0] = th->pad[1] = 0;
}
}  // namespace

extern "C" int64_t ref_cell_topology(int64_t n_cells, const orc_cell_header* cells,
                                     const uint8_t* payload, orc_topo_header* headers,
                                     uint8_t* out, int64_t capacity, int n_threads) {
  int64_t off = 0;
  for (int64_t q = 0; q < n_cells; ++q) {
    headers[q].offset = (uint64_t)off;
    off += (int64_t)topo_bytes(cells[q].nb_v, cells[q].nb_p, cells[q].nb_e);
  }
  if (off > capacity) return -1;
  if (n_threads < 1) n_threads = 1;
  std::vector<std::thread> th;
  for (int w = 0; w < n_threads; ++w)
    th.emplace_back([&, w] {
      for (int64_t q = w; q < n_cells; q += n_threads)
        one_cell(cells[q], payload + cells[q].offset, headers + q, out + headers[q].offset);
    });
  for (auto& t : th) t.join();
  return off;
}
