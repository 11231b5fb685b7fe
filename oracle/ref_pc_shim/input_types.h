/*
 * Stand-in for libmat's src/inputs/input_types.h when ref_powercell_driver
 * compiles the reference's rpd_update.cxx:1-521 for the CPU (test
 * infrastructure): the feature-edge kinds and a triangle surface mesh that
 * answers what update_sphere_surf_v2fids asks of its GEO::Mesh -- facet
 * adjacency and the pairs of faces across a sharp edge -- from plain arrays.
 */
#pragma once

#include <iostream>  // common_cxx.h prints with std::cout
#include <set>

#include "common_cxx.h"

namespace GEO {
typedef unsigned int index_t;
const index_t NO_FACET = ~index_t(0);
}  // namespace GEO

enum EdgeType { UE = -1, SE = 1, CE = 2 };

struct SurfaceMesh {
  struct Facets {
    const int* adj = nullptr;  // three neighbours per triangle, -1 for none
    int n = 0;
    GEO::index_t nb() const { return (GEO::index_t)n; }
    GEO::index_t nb_vertices(GEO::index_t) const { return 3; }
    // a face beyond the mesh has no neighbours
    GEO::index_t adjacent(GEO::index_t f, GEO::index_t le) const {
      if (f >= (GEO::index_t)n) return GEO::NO_FACET;
      const int a = adj[3 * (size_t)f + le];
      return a < 0 ? GEO::NO_FACET : (GEO::index_t)a;
    }
  } facets;
  std::set<aint2> fe_sf_fs_pairs;  // sorted face pairs across a sharp edge
};
