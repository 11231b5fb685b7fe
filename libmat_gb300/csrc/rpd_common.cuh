// rpd_common.cuh -- shared definitions of the GB300 RPD engine.
//
// Capacities, status codes and the packed cell record.  The capacities and
// status values are those of libmat's preset 3 and Status enum
// (src/rpd3d_base/voronoi_common.h:8-63); the record is this engine's own
// compact layout (one 32-byte header per (tet, site) pair plus a variable
// payload per emitted cell), from which the reference's ConvexCellHost
// (src/rpd3d_base/voronoi_defs.h:19-100) is expanded on the host.
#pragma once

#include <cstdint>

#include "../../include/rpd_gb300.h"

namespace rpd {

constexpr int kMaxP = 64;   // planes per cell (_MAX_P_)
constexpr int kMaxT = 96;   // vertices (dual triangles) per cell (_MAX_T_)
constexpr int kMaxE = 152;  // edges per cell (_MAX_E_)
constexpr uint8_t kEnd = 255;

enum CellStatus : int32_t {
  kEarlyReturn = -1,
  kTriangleOverflow = 0,
  kVertexOverflow = 1,
  kInconsistentBoundary = 2,
  kSecurityRadiusNotReached = 3,
  kSuccess = 4,
  kNeedsExactPredicates = 5,
  kNoIntersection = 6,
  kEdgeOverflow = 7,
  kNeedsPerturb = 8,
  // engine-only: the payload buffer was too small (cell is re-run)
  kPayloadFull = 100,
};

static_assert(sizeof(rpd_cell_header) == 32, "header layout");

__host__ __device__ inline uint32_t al16(uint32_t x) { return (x + 15u) & ~15u; }

// payload layout (all sections 16-byte aligned):
//   float4 plane[nb_p] | int2 id2[nb_p] | uchar4 ver[nb_v] | uchar4 edge[nb_e]
//   | uint8 h[nb_p] | double xyz[nb_v][3]
struct PayloadLayout {
  uint32_t plane, id2, ver, edge, h, xyz, total;
  __host__ __device__ PayloadLayout(int nv, int np, int ne) {
    plane = 0;
    id2 = plane + 16u * np;
    ver = id2 + al16(8u * np);
    edge = ver + al16(4u * nv);
    h = edge + al16(4u * ne);
    xyz = h + al16((uint32_t)np);
    total = xyz + al16(24u * nv);
  }
};

// per-cell topology record (rpd_topo_header): sections in this order
struct TopoLayout {
  uint32_t facet_euler, active, lf2active, active_e, faces, total;
  __host__ __device__ TopoLayout(int nv, int np, int ne) {
    facet_euler = 0;
    active = 4u * np;
    lf2active = active + np;
    active_e = lf2active + np;
    faces = active_e + ne;
    total = al16(faces + 3u * nv);
  }
};

}  // namespace rpd
