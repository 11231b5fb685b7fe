// rpd_mesh.cpp -- mesh adjacency counts and face ids on the host.
//
// Same results as libmat's load_tet_adj_info (src/IO/IO_CXX/io.cxx:238-335):
// #tets per vertex (v_adjs), per edge and per face, and a unique id per face
// (boundary faces: the surface facet ids; interior faces: ids from
// n_boundary_faces up, numbered at their first occurrence).  The reference
// intersects std::set<int> vertex stars for every query and keeps edge
// counts in a dense n_vert(n_vert+1)/2 table; here edges and faces are
// grouped by sorting packed 64-bit keys, and edge counts are kept per tet
// (6 bytes), which is all the clipper reads (convex_cell.cu:193-211).
// Boundary faces are numbered in scan order (tet ascending, face i opposite
// vertex i) -- the surface mesh's facet numbering when the boundary faces
// are the surface mesh.

#include <algorithm>
#include <cstdint>
#include <vector>

#include "../../include/rpd_gb300.h"

namespace {
const int kFaceLv[4][3] = {{2, 1, 3}, {0, 2, 3}, {1, 0, 3}, {0, 1, 2}};
const int kEdgeLv[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};

struct Key {
  uint64_t hi, lo;  // (a, b) and c, compared lexicographically
  int64_t slot;
};
bool operator<(const Key& x, const Key& y) {
  if (x.hi != y.hi) return x.hi < y.hi;
  if (x.lo != y.lo) return x.lo < y.lo;
  return x.slot < y.slot;
}
}  // namespace

extern "C" rpd_status rpd_build_mesh_adjacency(int n_vert, const int32_t* tets, int n_tet,
                                               int32_t* v_adjs, uint8_t* e_adj6,
                                               int32_t* f_adjs, int32_t* f_ids,
                                               int32_t* n_boundary_faces) {
  if (n_vert <= 0 || n_tet <= 0 || !tets || !v_adjs || !e_adj6 || !f_adjs || !f_ids)
    return RPD_ERR_INVALID_ARGUMENT;
  std::fill(v_adjs, v_adjs + n_vert, 0);
  for (int64_t i = 0; i < (int64_t)n_tet * 4; ++i) {
    if (tets[i] < 0 || tets[i] >= n_vert) return RPD_ERR_INVALID_ARGUMENT;
    v_adjs[tets[i]]++;
  }
  // edges
  {
    std::vector<Key> k((size_t)n_tet * 6);
    for (int64_t t = 0; t < n_tet; ++t)
      for (int e = 0; e < 6; ++e) {
        uint32_t a = (uint32_t)tets[4 * t + kEdgeLv[e][0]], b = (uint32_t)tets[4 * t + kEdgeLv[e][1]];
        if (a > b) std::swap(a, b);
        k[6 * t + e] = Key{((uint64_t)a << 32) | b, 0, 6 * t + e};
      }
    std::sort(k.begin(), k.end());
    for (size_t s = 0; s < k.size();) {
      size_t r = s;
      while (r < k.size() && k[r].hi == k[s].hi) ++r;
      uint8_t cnt = (uint8_t)std::min<size_t>(r - s, 255);
      for (size_t q = s; q < r; ++q) e_adj6[k[q].slot] = cnt;
      s = r;
    }
  }
  // faces
  std::vector<int64_t> partner((size_t)n_tet * 4, -1);
  {
    std::vector<Key> k((size_t)n_tet * 4);
    for (int64_t t = 0; t < n_tet; ++t)
      for (int f = 0; f < 4; ++f) {
        uint32_t v[3] = {(uint32_t)tets[4 * t + kFaceLv[f][0]], (uint32_t)tets[4 * t + kFaceLv[f][1]],
                         (uint32_t)tets[4 * t + kFaceLv[f][2]]};
        std::sort(v, v + 3);
        k[4 * t + f] = Key{((uint64_t)v[0] << 32) | v[1], v[2], 4 * t + f};
      }
    std::sort(k.begin(), k.end());
    for (size_t s = 0; s < k.size();) {
      size_t r = s;
      while (r < k.size() && k[r].hi == k[s].hi && k[r].lo == k[s].lo) ++r;
      if (r - s > 2) return RPD_ERR_INVALID_ARGUMENT;  // non-manifold face
      for (size_t q = s; q < r; ++q) {
        f_adjs[k[q].slot] = (int32_t)(r - s);
        if (r - s == 2) partner[k[q].slot] = k[q == s ? s + 1 : s].slot;
      }
      s = r;
    }
  }
  int32_t nb = 0;
  for (size_t i = 0; i < partner.size(); ++i)
    if (partner[i] < 0) f_ids[i] = nb++;
  int32_t next = nb;
  for (size_t i = 0; i < partner.size(); ++i) {
    if (partner[i] < 0) continue;
    if (partner[i] > (int64_t)i) f_ids[i] = next++;
    else f_ids[i] = f_ids[partner[i]];
  }
  if (n_boundary_faces) *n_boundary_faces = nb;
  return RPD_OK;
}
