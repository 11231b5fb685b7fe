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
//         ids (2 int32), edges (3 B each); then float site_cell_vol[n_site]
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
struct cfloat5 { float x, y, z, w, h; };
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
  }
  fwrite(cell_vol.data(), 4, cell_vol.size(), o);
  fclose(o);
  return 0;
}
