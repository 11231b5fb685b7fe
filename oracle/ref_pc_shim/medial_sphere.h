/*
 * Stand-in for libmat's src/matbase/medial_sphere.h when
 * ref_powercell_driver compiles the reference's rpd_update.cxx:1-521 for the
 * CPU (test infrastructure): the PowerCell members that get_all_voro_info
 * and the component updates fill, with the member names and container types
 * of the reference's PowerCell (medial_sphere.h:145-275), a double 3-vector
 * for geogram's vec3 (stored, copied and read by component there), and a sphere that holds
 * its power cell.
 */
#pragma once

#include <array>
#include <map>
#include <set>
#include <utility>
#include <vector>

#include "input_types.h"
#include "voronoi_defs.h"

struct Vector3 {
  double x = 0.0, y = 0.0, z = 0.0;
  Vector3() {}
  Vector3(double a, double b, double c) : x(a), y(b), z(c) {}
  double operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
typedef std::pair<Vector3, int> v2int;

inline Vector3 to_vec(const cfloat4& v) { return Vector3(v.x, v.y, v.z); }

struct PowerCell {
  int voro_id = -1;
  float pcell_vol = -1;
  std::set<int> cell_ids;
  std::set<int> tet_ids;
  std::map<int, std::set<int>> cell_neighbors;
  std::map<int, std::set<int>> cell_to_tfids;
  std::map<int, std::vector<v2int>> cell_to_surfv2fid;
  std::vector<std::set<int>> cc_cells;
  std::vector<std::vector<v2int>> cc_surf_v2fids;
  std::map<int, std::set<int>> facet_neigh_to_cells;
  std::map<int, bool> facet_neigh_is_fixed;
  std::map<int, std::vector<std::set<int>>> facet_cc_cells;
  std::map<int, std::vector<std::vector<v2int>>> facet_cc_surf_v2fids;
  std::map<aint2, std::set<int>> e_to_cells;
  std::map<aint2, bool> e_is_fixed;
  std::map<aint2, std::vector<std::set<int>>> edge_cc_cells;
  std::map<aint2, std::vector<std::array<aint2, 2>>> edge_2endvertices;
  std::map<aint2, aint3> vertex_2id;
  std::map<aint2, v2int> vertex_2pos;
  std::set<aint5> se_covered_lvids;
  std::map<aint4, Vector3> se_line_endpos;
  std::set<aint5> ce_covered_lvids;
  std::vector<std::vector<v2int>> surf_v2fid_in_groups;
};

struct MedialSphere {
  int id = -1;
  PowerCell pcell;
};
