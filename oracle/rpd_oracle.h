/*
 * rpd_oracle.h -- CPU restatement of libmat's restricted-power-diagram (RPD)
 * hot path.  TEST INFRASTRUCTURE ONLY: the tests, the smoke check and the
 * CPU-baseline leg of bench.py call it as the checker.  The product path
 * (libmat_gb300/csrc) never links or calls anything here.
 *
 * What it restates (file:line in the libmat sources):
 *   - per-(tet, site) convex-cell clipping, status codes, capacities and drop
 *     rules: src/rpd3d/convex_cell.cu:116-214 (cell = tet), :437-500 (FP64
 *     conflict predicate on float planes, tie = no conflict), :524-616 (new
 *     vertex / plane / edge), :618-678 (cavity boundary walk), :680-774
 *     (clip sequence), :1166-1337 (per-pair driver);
 *     src/rpd3d_base/voronoi_common.h:8-63 (Status, _MAX_P_/_MAX_T_/_MAX_E_)
 *   - float plane formulas: include/common_cuda.h:153-213 (det3x3, det4x4),
 *     :248-254 (tri2plane)
 *   - candidate (tet, site) rule: src/rpd3d/voronoi.cu:154-193 and the
 *     host loop :284-317 (ascending site id per tet); power distances as in
 *     src/rpd3d/kNN-CUDA/knncuda.cu:21-94 + :130-160
 *   - mesh adjacency counts: src/IO/IO_CXX/io.cxx:238-335
 *   - FP64 cell volume: the per-vertex 6-tet decomposition of
 *     src/rpd3d/convex_cell.cu:986-1069, evaluated in double.
 *
 * All float/double arithmetic is written in the reference's operation order
 * and must be compiled with -ffp-contract=off so that every operation is a
 * single IEEE-rounded step (the reference's source semantics).
 */
#ifndef RPD_ORACLE_H
#define RPD_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* capacities of the reference preset 3 (voronoi_common.h:55-62) */
#define ORC_MAX_P 64
#define ORC_MAX_T 96
#define ORC_MAX_E 152
#define ORC_END_OF_LIST 255

/* reference Status enum values (voronoi_common.h:10-25) */
enum {
  ORC_EARLY_RETURN = -1,
  ORC_TRIANGLE_OVERFLOW = 0,
  ORC_VERTEX_OVERFLOW = 1,
  ORC_INCONSISTENT_BOUNDARY = 2,
  ORC_SECURITY_RADIUS_NOT_REACHED = 3,
  ORC_SUCCESS = 4,
  ORC_NEEDS_EXACT_PREDICATES = 5,
  ORC_NO_INTERSECTION = 6,
  ORC_EDGE_OVERFLOW = 7,
  ORC_NEEDS_PERTURB = 8
};

/* Packed cell record, byte-identical to the CUDA path's output. */
typedef struct {
  int32_t tet_id;
  int32_t site_id;
  int32_t status;
  uint8_t nb_v, nb_p, nb_e, flags;
  uint64_t offset; /* byte offset of the payload (16-byte aligned) */
  double volume;   /* FP64 volume of the cell (0 when not emitted) */
} orc_cell_header;

/* Payload layout at `offset` (all sections 16-byte aligned):
 *   float  plane[nb_p][4]   (a, b, c, d), float, reference rounding
 *   int32  id2[nb_p][2]     (fid, -1) for tet faces, (min, max) site ids
 *   uint8  ver[nb_v][4]     (plane1, plane2, plane3, #adjacent cells)
 *   uint8  edge[nb_e][4]    (plane_min, plane_max, #adjacent cells, 0)
 *   uint8  h[nb_p]          (#adjacent cells of the face) padded to 16
 *   double xyz[nb_v][3]     FP64 vertex coordinates */
size_t orc_payload_bytes(int nb_v, int nb_p, int nb_e);

/* ---- mesh adjacency (io.cxx:238-335), per-tet edge counts instead of the
 * dense n_vert^2/2 matrix.  Boundary faces are numbered in scan order
 * (tet asc, face asc) starting at 0 -- the stand-in for the surface-mesh
 * facet ids -- and interior faces from n_boundary_faces up. */
int orc_mesh_adjacency(int n_vert, int n_tet, const int32_t* tets,
                       int32_t* v_adjs, uint8_t* e_adj6, int32_t* f_adjs,
                       int32_t* f_ids, int32_t* n_boundary_faces);
int64_t orc_dense_e_adjs_size(int n_vert);
void orc_dense_e_adjs(int n_vert, int n_tet, const int32_t* tets,
                      const uint8_t* e_adj6, int32_t* e_adjs);

/* ---- neighbour lists: k smallest power-bisector distances
 * key(i,j) = ((|cj-ci|^2 - wj) + wi) / (2 |cj-ci|), ties by site id */
float orc_bisector_key(const float* si, const float* sj);
void orc_knn(int n_site, const float* site4, int k, int32_t* nbr,
             float* keys, int n_threads);

/* ---- candidate (tet, site) pairs, the reference rule, brute force.
 * Returns the number of pairs (or -1 if capacity is too small); writes the
 * per-tet CSR (tet_offsets[n_tet+1]) with sites ascending per tet. */
int64_t orc_candidate_pairs(int n_vert, const float* vert3, int n_tet,
                            const int32_t* tets, int n_site,
                            const float* site4, const uint32_t* flags,
                            const int32_t* nbr, int k, int32_t* tet_offsets,
                            int32_t* pair_sites, int64_t capacity,
                            int n_threads);

/* ---- clipping of every pair.  pred_mode 0: FP64 determinant on every
 * predicate (reference); 1: FP32 filter, FP64 determinant when undecided.
 * vert3d/site4d are the FP64 inputs used for the vertex reconstruction and
 * the cell volume.  headers[n_pairs] receives one record per pair;
 * payload[] is filled sequentially for emitted cells.  Returns the payload
 * bytes used, or -1 if payload_capacity is too small.  stats (may be NULL):
 * [0] predicates, [1] escalated to FP64. */
int64_t orc_clip_cells(int n_vert, const float* vert3, const double* vert3d,
                       int n_tet, const int32_t* tets, const int32_t* v_adjs,
                       const uint8_t* e_adj6, const int32_t* f_adjs,
                       const int32_t* f_ids, int n_site, const float* site4,
                       const double* site4d, const int32_t* nbr, int k,
                       const int32_t* tet_offsets, const int32_t* pair_sites,
                       int pred_mode, orc_cell_header* headers,
                       uint8_t* payload, int64_t payload_capacity,
                       int64_t* stats, int n_threads);

/* ---- per-cell topology of emitted cells: ConvexCellHost::reload_active
 * (src/rpd3d_base/voronoi_defs.cxx:76-106), reload_pc_explicit (:108-188),
 * cal_cell_euler (:190-222) and cal_halfplane_facet_euler (:224-266) for
 * each active bisector plane's neighbour.  One 16-byte header per cell
 *   uint64 offset; float euler; uint8 n_faces, flags, pad[2]
 * and a record at offset:
 *   float facet_euler[nb_p]; uint8 active[nb_p]; int8 lf2active[nb_p];
 *   uint8 active_e[nb_e]; uint8 faces[3 nb_v]; zero padding to 16 bytes.
 * flags: 1 = a vertex's float coordinates are NaN (faces left empty:
 * 255, lf2active -1, n_faces 0), 2 = a face cycle did not close.
 * cells/payload: n_cells emitted cells in orc_clip_cells' format.  Returns
 * the record bytes (offsets follow cell order), or -1 if capacity is too
 * small (out may be NULL to query the size). */
typedef struct {
  uint64_t offset;
  float euler;
  uint8_t n_faces, flags, pad[2];
} orc_topo_header;
size_t orc_topo_bytes(int nb_v, int nb_p, int nb_e);
int64_t orc_cell_topology(int64_t n_cells, const orc_cell_header* cells,
                          const uint8_t* payload, orc_topo_header* headers,
                          uint8_t* out, int64_t capacity);

/* ---- polygon soup of emitted cells: get_one_convex_cell_faces_const
 * (src/IO/IO_CUDA/io_cuda.cxx:21-141) over the cells in order.  points:
 * 3 floats per point (compute_vertex_coordinates); a NaN vertex ends its
 * cell (earlier points stay, no faces).  poly_offsets[n_polys + 1] into
 * indices (global point ids); poly_site / poly_adj_site per polygon.
 * counts[3] receives (points, polygons, indices); with NULL outputs only the
 * counts are computed.  Returns 0, or -1 when a capacity is too small. */
int orc_cell_polygons(int64_t n_cells, const orc_cell_header* cells,
                      const uint8_t* payload, int triangulate, int boundary_only,
                      int max_sf_fid, const double* slice /* NULL or pos[3], normal[3] */,
                      float* points, int64_t max_points,
                      int64_t* poly_offsets, uint32_t* indices, int64_t max_indices,
                      int32_t* poly_site, int32_t* poly_adj_site, int64_t max_polys,
                      int64_t* counts);

/* ---- power neighbours, the stand-in for libmat's regular-triangulation
 * neighbour lists (CGAL, src/rpd3d_base/triangulation.cxx:62-144,
 * :442-558): site j is a neighbour of site i when its float bisector plane
 * is a face of i's power cell inside `region` (lo[3], hi[3]).  The cell is a
 * tet enclosing the region clipped by the clipper above in exact-sign mode
 * (pred_mode 2) with every other site in ascending key order, until the next
 * key exceeds the cell's radius (vertices solved in double) by a margin
 * covering the rounding of the float planes.  Rows of max_nbr ids,
 * ascending, -1 padded; count[i] = neighbours, -1 for an empty cell (a
 * hidden sphere), -2 for a cell beyond the clipper's capacities, -3 for
 * more than max_nbr neighbours.  Returns the number of -2 / -3 sites. */
int orc_power_neighbors(int n_site, const float* site4, const double* region, int max_nbr,
                        int32_t* nbr, int32_t* count, int n_threads);

/* ---- canonical topology hash of each record (0 for cells not emitted):
 * the sum over vertices of splitmix64 (Steele et al. 2014) chained over the
 * sorted face keys (id2 as int32 pairs) of the vertex's three planes and
 * its #adj -- independent of the order of planes and vertices, so cells
 * clipped in different orders compare by their active faces */
void orc_topology_hashes(int64_t n, const orc_cell_header* h, const uint8_t* payload,
                         uint64_t* out);

/* ---- single predicates, exposed for filter tests */
double orc_det4x4_ref(const float* p1, const float* p2, const float* p3,
                      const float* e);
/* returns +1/-1 when the FP32 filter decides, 0 when it cannot */
int orc_filter_sign(const float* p1, const float* p2, const float* p3,
                    const float* e);
/* pred_mode 2 (an extension): the FP64 determinant with its error bound,
 * and the exact sign by floating-point expansions */
double orc_det4x4_bound(const float* p1, const float* p2, const float* p3, const float* e,
                        double* bound);
int orc_det4x4_exact_sign(const float* p1, const float* p2, const float* p3, const float* e);

#ifdef __cplusplus
}
#endif
#endif
