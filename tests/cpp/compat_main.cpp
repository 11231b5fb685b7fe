// Drives compute_clipped_voro_diagram_GPU through rpd_gb300_compat.hpp the way
// libmat's RPD3D_GPU does, with stand-ins for the libmat types the shim fills
// (field names of src/rpd3d_base/voronoi_defs.h, src/include/common_cxx.h).
//
//   compat_main <input.bin> <output.bin>
// input:  int32 n_vert, n_tet, n_site, site_k; float vertices[3 n_vert];
//         int32 indices[4 n_tet], v_adjs[n_vert], n_e_adjs, e_adjs[n_e_adjs],
//         f_adjs[4 n_tet], f_ids[4 n_tet]; float site[3 n_site] (SoA),
//         weights[n_site]; uint32 flags[n_site]; int32 site_knn[(k+1) n_site]
// output: int32 n_cells, then per cell: status, thread_id, voro_id, tet_id,
//         id, nb_v, nb_p, nb_e, then ver (4 B each), planes (5 floats),
//         ids (2 int32), edges (3 B each), then int32 is_active_updated,
//         is_pc_explicit, #faces, active_clipping_planes[nb_p + 1],
//         active_edges[nb_e + 1], per face (length, vertex slots),
//         pc_lf2active_map[nb_p], float pc_points[nb_v][3];
//         then float site_cell_vol[n_site]
#include <cstdint>
#include <cstdio>
#include <map>
#include <set>
#include <vector>

typedef unsigned int uint;
typedef unsigned char uchar;
struct cint2 { int x, y; };
struct cuchar3 { uchar x, y, z; };
struct cuchar4 { uchar x, y, z, w; };
struct cfloat3 { float x, y, z; };
struct cfloat4 { float x, y, z, w; };
struct cfloat5 { float x, y, z, w, h; };
inline cuchar3 cmake_uchar3(cuchar4 v) { return cuchar3{v.x, v.y, v.z}; }
inline cfloat3 cmake_float3(float x, float y, float z) { return cfloat3{x, y, z}; }
inline float cdet2x2(float a11, float a12, float a21, float a22) { return a11 * a22 - a12 * a21; }
inline float cdet3x3(float a11, float a12, float a13, float a21, float a22, float a23, float a31,
                     float a32, float a33) {
  return a11 * cdet2x2(a22, a23, a32, a33) - a21 * cdet2x2(a12, a13, a32, a33) +
         a31 * cdet2x2(a12, a13, a22, a23);
}
enum Status { early_return = -1, triangle_overflow = 0, vertex_overflow = 1,
              inconsistent_boundary = 2, security_radius_not_reached = 3, success = 4,
              needs_exact_predicates = 5, no_intersection = 6, edge_overflow = 7,
              needs_perturb = 8 };
struct ConvexCellHost {
  Status status;
  int thread_id;
  int voro_id;
  int tet_id;
  float weight = -1;
  bool is_active = false;
  uchar nb_v, nb_p, nb_e;
  cuchar4 ver_data_trans[96];
  cfloat5 clip_data_trans[64];
  cint2 clip_id2_data_trans[64];
  cuchar3 edge_data[152];
  float euler = -1;
  float cell_vol = -1;
  int id = -1;
  // topology members the shim fills (voronoi_defs.h)
  bool is_active_updated = false;
  std::vector<int> active_clipping_planes;
  std::vector<int> active_edges;
  bool is_pc_explicit = false;
  std::vector<cfloat3> pc_points;
  std::vector<std::vector<int>> pc_local_active_faces;
  std::vector<int> pc_lf2active_map;
  bool is_vertex_null = false;
  // vertex of three planes by Cramer's rule with the perspective divide
  // (the reference's member, voronoi_defs.cxx:33-74)
  cfloat4 compute_vertex_coordinates(cuchar3 t, bool persp_divide = true) const {
    const cfloat5 a = clip_data_trans[t.x], b = clip_data_trans[t.y], c = clip_data_trans[t.z];
    cfloat4 r;
    r.x = -cdet3x3(a.w, a.y, a.z, b.w, b.y, b.z, c.w, c.y, c.z);
    r.y = -cdet3x3(a.x, a.w, a.z, b.x, b.w, b.z, c.x, c.w, c.z);
    r.z = -cdet3x3(a.x, a.y, a.w, b.x, b.y, b.w, c.x, c.y, c.w);
    r.w = cdet3x3(a.x, a.y, a.z, b.x, b.y, b.z, c.x, c.y, c.z);
    if (!persp_divide) return r;
    return cfloat4{r.x / r.w, r.y / r.w, r.z / r.w, 1.f};
  }
};

#include "rpd_gb300_compat.hpp"

template <class T>
static bool rd(FILE* f, std::vector<T>& v, size_t n) {
  v.resize(n);
  return fread(v.data(), sizeof(T), n, f) == n;
}

int main(int argc, char** argv) {
  if (argc != 3) return 2;
  FILE* f = fopen(argv[1], "rb");
  if (!f) return 2;
  int32_t hdr[4];
  if (fread(hdr, 4, 4, f) != 4) return 2;
  int n_vert = hdr[0], n_tet = hdr[1], n_site = hdr[2], site_k = hdr[3];
  std::vector<float> vert, site, w;
  std::vector<int> idx, v_adjs, e_adjs, f_adjs, f_ids, knn;
  std::vector<uint> flags;
  int32_t n_e;
  bool ok = rd(f, vert, 3 * (size_t)n_vert) && rd(f, idx, 4 * (size_t)n_tet) &&
            rd(f, v_adjs, n_vert) && fread(&n_e, 4, 1, f) == 1 && rd(f, e_adjs, n_e) &&
            rd(f, f_adjs, 4 * (size_t)n_tet) && rd(f, f_ids, 4 * (size_t)n_tet) &&
            rd(f, site, 3 * (size_t)n_site) && rd(f, w, n_site) && rd(f, flags, n_site) &&
            rd(f, knn, (size_t)(site_k + 1) * n_site);
  fclose(f);
  if (!ok) return 3;
  std::map<int, std::set<int>> v2tets;  // unused by the engine, as by the reference
  std::vector<float> cell_vol;
  std::vector<ConvexCellHost> cells;
  try {
    cells = compute_clipped_voro_diagram_GPU(0, vert, idx, v2tets, v_adjs, e_adjs, f_adjs, f_ids,
                                             site, n_site, w, flags, knn, site_k, cell_vol, true);
  } catch (const std::exception& e) {
    fprintf(stderr, "error: %s\n", e.what());
    return 4;
  }
  FILE* o = fopen(argv[2], "wb");
  int32_t n = (int32_t)cells.size();
  fwrite(&n, 4, 1, o);
  for (const auto& c : cells) {
    int32_t h[8] = {(int32_t)c.status, c.thread_id, c.voro_id, c.tet_id, c.id,
                    c.nb_v, c.nb_p, c.nb_e};
    fwrite(h, 4, 8, o);
    fwrite(c.ver_data_trans, 4, c.nb_v, o);
    for (int i = 0; i < c.nb_p; ++i) fwrite(&c.clip_data_trans[i], 4, 5, o);
    fwrite(c.clip_id2_data_trans, 8, c.nb_p, o);
    fwrite(c.edge_data, 3, c.nb_e, o);
    // topology: flags, active planes / edges, faces, face map, points
    int32_t fl[3] = {c.is_active_updated, c.is_pc_explicit, (int32_t)c.pc_local_active_faces.size()};
    fwrite(fl, 4, 3, o);
    fwrite(c.active_clipping_planes.data(), 4, c.active_clipping_planes.size(), o);
    fwrite(c.active_edges.data(), 4, c.active_edges.size(), o);
    for (const auto& f : c.pc_local_active_faces) {
      int32_t m = (int32_t)f.size();
      fwrite(&m, 4, 1, o);
      fwrite(f.data(), 4, f.size(), o);
    }
    fwrite(c.pc_lf2active_map.data(), 4, c.pc_lf2active_map.size(), o);
    fwrite(c.pc_points.data(), 12, c.pc_points.size(), o);
  }
  fwrite(cell_vol.data(), 4, cell_vol.size(), o);
  fclose(o);
  return 0;
}
