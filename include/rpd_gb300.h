/*
 * rpd_gb300.h -- C ABI of the GB300-native restricted power diagram (RPD)
 * engine (librpd_gb300.so).
 *
 * It replaces the reference's GPU RPD entry point
 *   compute_clipped_voro_diagram_GPU(...)      src/rpd3d/voronoi.h:52-61
 * (host driver src/rpd3d/voronoi.cu:455-795, hot kernel
 *  clipped_voro_cell_test_GPU_param_tet, src/rpd3d/convex_cell.cu:1166-1337)
 * with a context object, plain pointers and sizes, and status codes.  The
 * C++ signature of the reference (returning std::vector<ConvexCellHost>) is
 * kept as a thin shim in rpd_gb300_compat.hpp on top of this ABI.
 *
 * Ownership: the caller owns every input buffer (they are copied into the
 * context's device memory); the context owns its device buffers and one
 * CUDA stream.  Views returned by rpd_get_cells stay valid until the next
 * rpd_compute or rpd_destroy.  No function calls exit(); every failure is a
 * status code, with a message in rpd_last_error().  One context per host
 * thread at a time.
 */
#ifndef RPD_GB300_H
#define RPD_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RPD_GB300_ABI_VERSION 1

/* Opaque handles: a context (one device, one stream) and a batch of meshes.
 * Declared here at file scope so that every prototype below names the same
 * type in C. */
struct rpd_ctx;
struct rpd_batch;

typedef enum rpd_status {
  RPD_OK = 0,
  RPD_ERR_INVALID_ARGUMENT = 1,
  RPD_ERR_CUDA = 2,
  RPD_ERR_OUT_OF_MEMORY = 3,
  RPD_ERR_NOT_READY = 4,  /* compute before mesh / sites / neighbours set */
  RPD_ERR_CAPACITY = 5,   /* a size limit of the call was exceeded */
  RPD_ERR_NO_DEVICE = 6
} rpd_status;

/* How each conflict predicate sign is obtained.  The predicate is the
 * reference's: sign of det4x4 of the vertex's three float planes and the new
 * float plane, evaluated in FP64 (convex_cell.cu:437-500), tie = no
 * conflict. */
typedef enum rpd_predicate_mode {
  RPD_PRED_FP64 = 0,        /* FP64 determinant for every predicate */
  RPD_PRED_FP32_FILTER = 1, /* FP32 cofactor filter with a proven error
                               bound; FP64 determinant only when the filter
                               cannot decide.  Same signs as RPD_PRED_FP64. */
  RPD_PRED_EXACT = 2        /* FP32 filter, then FP64 with its error bound,
                               then the exact sign by floating-point
                               expansions where FP64 cannot certify it: the
                               true sign of the float planes' determinant.
                               Not in the reference: cells can differ from
                               it exactly where its FP64 sign is wrong
                               (counted in rpd_stats.n_exact_flips). */
} rpd_predicate_mode;

/* Where the per-site neighbour lists come from. */
typedef enum rpd_neighbor_source {
  RPD_NEIGH_USER = 0, /* rpd_set_neighbors (e.g. libmat's RT neighbours) */
  RPD_NEIGH_KNN = 1   /* built on the GPU: k smallest power-bisector
                         distances, uniform-grid search */
} rpd_neighbor_source;

/* Clipping order inside a GPU-built list. */
typedef enum rpd_clip_order {
  RPD_ORDER_SITE_ID = 0,  /* ascending site id, as the reference's sorted
                             std::set lists (triangulation.cxx:324-352) */
  RPD_ORDER_DISTANCE = 1  /* ascending bisector distance */
} rpd_clip_order;

typedef struct rpd_config {
  int device;            /* CUDA device ordinal */
  int predicate_mode;    /* rpd_predicate_mode */
  int neighbor_source;   /* rpd_neighbor_source */
  int knn_k;             /* list length for RPD_NEIGH_KNN, 1..128 */
  int clip_order;        /* rpd_clip_order (RPD_NEIGH_KNN only) */
  int compute_geometry;  /* 1: FP64 vertex coordinates and cell volumes */
  int warps_per_block;   /* clip kernel block size in warps, 0 = default */
  int blocks_per_sm;     /* persistent grid: blocks per SM, 0 = default */
  int certify;           /* 1 (RPD_NEIGH_KNN only): clip in ascending bisector
                            distance and stop at the security-radius
                            certificate; cells equal the plain path's up to
                            the order of their records (same topology) */
  int clip_variant;      /* clip kernel register budget: 0 none (occupancy
                            set by registers), 1 = 80 registers (6 blocks of
                            4 warps per SM), 2 = 64 registers (8 blocks) */
  int learned_k;         /* 1 (with certify): per-cell list lengths from the
                            trained k-predictor (rpd_mlp_train); the first
                            pass clips that many list entries and tests the
                            certificate once, cells where it fails are
                            clipped again with the whole list */
  int box_planes;        /* RPD_NEIGH_KNN: nearest bisectors bounding each
                            site's candidate region for the tets of common
                            size (0 = default 44; the few largest tets use
                            at most 12) */
  int topology_hash;     /* 1 (default): canonical topology hash of every
                            cell (rpd_copy_topology_hashes_to_host) */
  int exact_lists;       /* 1 (default; RPD_NEIGH_KNN): a site whose cell
                            its whole list leaves uncertified (sites beyond
                            the list may cut it) gets a longer list -- every
                            site whose key is below the cell's radius bound,
                            at most 512, then 4096 entries -- and those
                            cells are clipped again, for up to three rounds,
                            inside the same rpd_compute.  Lists complete to
                            the radius make every cell exact; cells still
                            uncertified after the rounds keep the flag.
                            0: one pass, cells flagged as they come */
  int reserved[2];
} rpd_config;

/* One record per candidate (tet, site) pair; 32 bytes. */
/* rpd_cell_header.flags: set on an emitted cell of a certified compute
 * (config.certify, GPU-built lists) that was clipped by its site's whole
 * list without the security-radius certificate holding: sites beyond the
 * list may still cut it, so it can be larger than the exact restricted
 * cell.  Lists holding all power neighbours (libmat's triangulation
 * neighbours through rpd_set_neighbors) give exact cells; a longer knn_k
 * flags fewer. */
#define RPD_CELL_UNCERTIFIED 1u

typedef struct rpd_cell_header {
  int32_t tet_id;
  int32_t site_id;
  int32_t status;      /* reference Status value; 4 = success (emitted) */
  uint8_t nb_v, nb_p, nb_e, flags;
  uint64_t offset;     /* payload byte offset (emitted cells) */
  double volume;       /* FP64 cell volume (compute_geometry) */
} rpd_cell_header;

/* Payload of an emitted cell at `offset`, sections 16-byte aligned:
 *   float  plane[nb_p][4]  (a, b, c, d) of a*x+b*y+c*z+d >= 0 (inside)
 *   int32  id2[nb_p][2]    (face id, -1) for tet faces, (min, max) site ids
 *                          for bisectors -- ConvexCellHost::clip_id2_data_trans
 *   uint8  ver[nb_v][4]    (plane, plane, plane, #adjacent cells)
 *   uint8  edge[nb_e][4]   (plane_min, plane_max, #adjacent cells, 0)
 *   uint8  h[nb_p]         #adjacent cells of each face
 *   double xyz[nb_v][3]    FP64 vertex coordinates (compute_geometry) */
size_t rpd_payload_bytes(int nb_v, int nb_p, int nb_e);

typedef struct rpd_stats {
  int64_t n_pairs;            /* candidate (tet, site) pairs clipped */
  int64_t n_cells;            /* emitted cells (status success) */
  int64_t status_counts[10];  /* per reference status value 0..8, [9] other */
  int64_t n_predicates;       /* conflict predicates evaluated */
  int64_t n_escalated;        /* of those, decided by the FP64 determinant */
  int64_t payload_bytes;      /* payload bytes written */
  int32_t tet_k;              /* max pairs of one tet (reference's tet_k) */
  int32_t knn_k;              /* neighbour list length used */
  float ms_total;             /* device time of rpd_compute, CUDA events */
  float ms_knn, ms_pairs, ms_clip, ms_compact;
  float ms_clip_kernel;       /* the clip kernel alone (events around it) */
  int32_t n_launches;         /* kernels launched by this rpd_compute */
  /* candidate search counters: [0] grid cells scanned, [1] cells kept after
   * the grown-cell planes, [2] tets enumerated, [3] tets inside the grown
   * cell (rule evaluated), [4] pairs, [5] site boxes without planes */
  int64_t search[6];
  int64_t n_reclipped;        /* cells whose shortened list (rpd_set_site_k
                                 or learned_k) ran out before the certificate
                                 held, clipped again with the whole list: the
                                 predictor's misses */
  float ms_predict;           /* learned_k: features + inference (in ms_clip) */
  int32_t learned;            /* 1 if the learned list lengths were used */
  int64_t n_fp64_uncertain;   /* RPD_PRED_EXACT: escalated predicates whose
                                 FP64 sign is not certified by the FP64 error
                                 bound, decided by exact arithmetic */
  int64_t n_exact_flips;      /* RPD_PRED_EXACT: of those, exact sign !=
                                 FP64 sign (where the reference errs) */
  float ms_epilogue;          /* coordinates, volumes, hashes (in ms_clip) */
  int64_t n_uncertified;      /* emitted cells flagged RPD_CELL_UNCERTIFIED */
  int64_t n_extended_sites;   /* exact_lists: sites given a longer list
                                 (summed over the rounds) */
  int64_t n_cert_reclipped;   /* exact_lists: cells clipped again with a
                                 longer list (summed over the rounds) */
  float ms_extend;            /* exact_lists: device time of the rounds (in
                                 ms_clip) */
  int32_t n_extend_rounds;    /* rounds that found uncertified cells */
  int32_t ext_longest;        /* longest extended list clipped */
  float ms_extend_lists;      /* exact_lists: of ms_extend, building the
                                 longer lists */
} rpd_stats;

typedef struct rpd_cells_view {
  int64_t n_cells;                 /* emitted cells, (tet, site) ascending */
  const rpd_cell_header* headers;  /* device pointer, n_cells records */
  const uint8_t* payload;          /* device pointer */
  int64_t payload_bytes;
  int64_t n_pairs;                 /* all pairs, including dropped ones */
  const rpd_cell_header* pair_headers; /* device pointer, n_pairs records */
} rpd_cells_view;

const char* rpd_status_string(rpd_status s);
void rpd_config_default(rpd_config* cfg);

rpd_status rpd_create(const rpd_config* cfg, struct rpd_ctx** out);
void rpd_destroy(struct rpd_ctx* ctx);
const char* rpd_last_error(const struct rpd_ctx* ctx);
/* Reads / replaces a context's configuration (same device; the mesh, sites
 * and any trained predictor stay).  The next rpd_compute uses it. */
rpd_status rpd_get_config(const struct rpd_ctx* ctx, rpd_config* cfg);
rpd_status rpd_set_config(struct rpd_ctx* ctx, const rpd_config* cfg);

/* Tet mesh (replaces copy_tet_data + load_num_adjacent_cells_and_ids,
 * voronoi.cu:324-415).  xyz: n_vert x 3 doubles; tets: n_tet x 4 vertex
 * ids, positively oriented; v_adjs: #tets per vertex; e_adj6: #tets per
 * tet edge, edges (0,1)(0,2)(0,3)(1,2)(1,3)(2,3) -- the per-tet form of the
 * reference's dense e_adjs table (io.cxx:264-281); f_adjs, f_ids: per tet
 * face (face i opposite vertex i), as load_tet_adj_info (io.cxx:238-335). */
rpd_status rpd_set_mesh(struct rpd_ctx* ctx, const double* xyz, int n_vert,
                        const int32_t* tets, int n_tet, const int32_t* v_adjs,
                        const uint8_t* e_adj6, const int32_t* f_adjs,
                        const int32_t* f_ids);

/* What rpd_set_mesh derived on the device (for checks and diagnostics):
 * bounding box, total volume, largest tet radius (largest vertex distance
 * to the tet's centroid, FP64), and the two radius classes the candidate
 * search uses -- their tet counts and largest radii. */
typedef struct rpd_mesh_info {
  int32_t n_vert, n_tet;
  double lo[3], hi[3];
  double volume;
  double tet_radius;
  int32_t class_count[2];
  double class_radius[2];
} rpd_mesh_info;
rpd_status rpd_get_mesh_info(const struct rpd_ctx* ctx, rpd_mesh_info* info);

/* Sites: xyzw = n_site x 4 doubles (centre, weight = squared radius);
 * flags: 1 = compute this site's cells (SiteFlag::is_selected,
 * voronoi_common.h:7), 0 = neighbour only.  flags may be NULL (all 1). */
rpd_status rpd_set_sites(struct rpd_ctx* ctx, const double* xyzw, int n_site,
                         const uint32_t* flags);

/* User neighbour lists.  layout 0: row-major n_site x k, -1 padded;
 * layout 1: the reference's site_knn, (k + 1) rows x n_site
 * (triangulation.cxx:324-352).  Each list is clipped in its given order up
 * to its first -1 (convex_cell.cu:1255-1259). */
rpd_status rpd_set_neighbors(struct rpd_ctx* ctx, const int32_t* nbr, int k,
                             int layout);

/* Per-site list lengths for certified clipping (config.certify): site i is
 * clipped with its k_per_site[i] nearest neighbours first, and any of its
 * cells not certified by then is clipped again with the whole list.  NULL
 * clears it.  k_per_site may be a device pointer when on_device is 1. */
rpd_status rpd_set_site_k(struct rpd_ctx* ctx, const int32_t* k_per_site, int on_device);

/* Autotuner: times rpd_compute on the context's current inputs for each
 * candidate launch configuration of the clip kernel -- block size 2, 4 or 8
 * warps, register budgets for 16, 24 or 32 resident warps per SM (the
 * shared-memory budget per SM follows: 5.7 KB per warp) -- and, with
 * config.certify, first-pass list lengths of 16, 32 or all neighbours
 * (k-bucket; cells not certified by their bucket are clipped again whole)
 * and, once a k-predictor is trained or loaded, its per-cell lengths.
 * Keeps the fastest in the context (the cells are the same for every
 * candidate).  repeats >= 1 timed runs per candidate (median). */
typedef struct rpd_tuning {
  int warps_per_block;
  int clip_variant;
  int k_bucket;        /* 0 = whole list */
  int n_candidates;
  float ms_clip_best;  /* clip stage of the chosen configuration */
  float ms_clip_first; /* clip stage of the first candidate (defaults) */
  int learned_k;       /* 1: the k-predictor's lengths won (rpd_config.learned_k set) */
  int knn_k;           /* GPU-built lists with exact_lists: the base list
                          length (64, 96 or 128) of the fastest whole
                          compute -- the cells do not depend on it */
  float ms_total_best; /* the whole compute with the chosen configuration */
} rpd_tuning;
rpd_status rpd_autotune(struct rpd_ctx* ctx, int repeats, rpd_tuning* result);

/* Runs the whole path on the device: neighbour lists (RPD_NEIGH_KNN),
 * candidate pairs (the reference's rule, voronoi.cu:154-193), clipping,
 * compaction.  Blocks until done.  stats may be NULL. */
rpd_status rpd_compute(struct rpd_ctx* ctx, rpd_stats* stats);

rpd_status rpd_get_cells(struct rpd_ctx* ctx, rpd_cells_view* view);

/* Copies the emitted cells to host memory.  Pass NULL buffers to query the
 * sizes first. */
rpd_status rpd_copy_cells_to_host(struct rpd_ctx* ctx, rpd_cell_header* headers,
                                  int64_t max_cells, void* payload,
                                  int64_t payload_capacity, int64_t* n_cells,
                                  int64_t* payload_bytes);

/* The same copies queued on the context's stream without waiting for them
 * (same arguments and checks; sizes are returned at once).  The buffers must
 * be page-locked (rpd_host_alloc) and stay untouched until
 * rpd_synchronize(ctx), or the context's next call that waits on its stream,
 * returns.  Two contexts used in turn overlap one mesh's device->host copy
 * with the next mesh's upload and compute. */
rpd_status rpd_copy_cells_to_host_async(struct rpd_ctx* ctx, rpd_cell_header* headers,
                                        int64_t max_cells, void* payload,
                                        int64_t payload_capacity, int64_t* n_cells,
                                        int64_t* payload_bytes);

/* Waits until everything queued on the context's stream has finished. */
rpd_status rpd_synchronize(struct rpd_ctx* ctx);

/* The headers of every candidate pair of the last rpd_compute (dropped
 * cells included, with their failure status), in (tet, site) order. */
rpd_status rpd_copy_pair_headers_to_host(struct rpd_ctx* ctx, rpd_cell_header* headers,
                                         int64_t capacity, int64_t* n_pairs);

/* Caller-supplied list length of every candidate pair (certify only): the
 * next rpd_compute clips pair q with the first k_per_pair[q] entries of its
 * site's distance-ordered list, tests the certificate once, and clips the
 * cells where it fails again with the whole list.  n_pairs must equal the
 * compute's pair count (pairs are in (tet, site) order, as in
 * rpd_copy_pair_headers_to_host).  NULL clears.  The k-predictor
 * (learned_k) takes precedence. */
rpd_status rpd_set_pair_k(struct rpd_ctx* ctx, const int32_t* k_per_pair, int64_t n_pairs);

/* Canonical topology hash of every pair of the last rpd_compute (0 for
 * dropped cells): the sum over the cell's vertices of a hash of the sorted
 * face keys (clip_id2) of its three planes and its #adjacent cells.  Equal
 * hashes = equal cells up to the order of planes, vertices and edges. */
rpd_status rpd_copy_topology_hashes_to_host(struct rpd_ctx* ctx, uint64_t* hashes,
                                            int64_t capacity, int64_t* n_pairs);

/* ---- per-cell topology of the emitted cells, on the device --------------
 * What libmat's consumers rebuild on the host for every ConvexCellHost
 * (src/rpd3d_base/voronoi_defs.cxx): reload_active (:76-106, active planes
 * and edges), reload_pc_explicit (:108-188, the vertex cycle of every active
 * face and the face -> active face map), cal_cell_euler (:190-222) and
 * cal_halfplane_facet_euler (:224-266, for each active bisector plane's
 * neighbour).  One header per emitted cell, in rpd_get_cells order; record
 * at `offset` (16-byte aligned, zero padded):
 *   float  facet_euler[nb_p]  cal_halfplane_facet_euler(neighbour of plane p)
 *                             for active bisector planes, 0 otherwise
 *   uint8  active[nb_p]       active_clipping_planes: vertices on plane p
 *   int8   lf2active[nb_p]    pc_lf2active_map (-1: inactive)
 *   uint8  active_e[nb_e]     active_edges (0 / 1)
 *   uint8  faces[3 nb_v]      pc_local_active_faces, concatenated in active
 *                             face order; face of plane p has active[p]
 *                             vertex slots
 * flags: RPD_TOPO_VERTEX_NULL when a vertex's float coordinates
 * (compute_vertex_coordinates) are NaN -- the reference then leaves the
 * faces empty, so faces are 255 and lf2active -1; RPD_TOPO_OPEN_FACE when a
 * face's cycle does not close (not possible for a valid cell). */
#define RPD_TOPO_VERTEX_NULL 1
#define RPD_TOPO_OPEN_FACE 2
typedef struct rpd_topo_header {
  uint64_t offset;  /* byte offset of the cell's record */
  float euler;      /* cal_cell_euler (ConvexCellHost::euler is a float) */
  uint8_t n_faces;  /* active faces */
  uint8_t flags;
  uint8_t pad[2];
} rpd_topo_header;
size_t rpd_topo_bytes(int nb_v, int nb_p, int nb_e);

/* Computes the topology of the last rpd_compute's cells (ms may be NULL:
 * device time of the pass). */
rpd_status rpd_compute_topology(struct rpd_ctx* ctx, float* ms);

typedef struct rpd_topo_view {
  int64_t n_cells;
  const rpd_topo_header* headers; /* device pointer */
  const uint8_t* records;         /* device pointer */
  int64_t bytes;
} rpd_topo_view;
rpd_status rpd_get_topology(struct rpd_ctx* ctx, rpd_topo_view* view);
/* NULL buffers: sizes only. */
rpd_status rpd_copy_topology_to_host(struct rpd_ctx* ctx, rpd_topo_header* headers,
                                     int64_t max_cells, void* records, int64_t capacity,
                                     int64_t* n_cells, int64_t* bytes);

/* ---- power cells of the emitted cells ------------------------------------
 * What libmat's get_all_voro_info (src/rpd3d_base/rpd_update.cxx:80-340)
 * gathers for every medial sphere into its PowerCell
 * (src/matbase/medial_sphere.h:145-260), as flat device arrays (cell ids
 * are rpd_get_cells indices, site ids the context's):
 *   site_cells[site_cell_off[s] ..]   cells of site s, ascending (cell_ids)
 *   cell_nbrs[cell_nbr_off[c] ..]     cells of the same site across c's
 *                                     tet faces, ascending (cell_neighbors)
 *   cell_tfids[cell_tfid_off[c] ..]   c's active tet faces, ascending
 *                                     (cell_to_tfids)
 *   facet_keys / facet_cells          (site << 32 | neighbour site) and cell
 *                                     of every active bisector face, sorted
 *                                     by site, neighbour, cell
 *                                     (facet_neigh_to_cells); per site from
 *                                     site_facet_off
 *   edges                             7 int32 per active edge on two
 *                                     bisectors: site, neighbour min, max,
 *                                     cell, its two vertices on both faces,
 *                                     0; sorted by site, neighbours, cell,
 *                                     edge (e_to_cells, edge_2endvertices);
 *                                     per site from site_edge_off
 *   vertex_*                          every vertex with two or more
 *                                     neighbour sites among its planes: cell,
 *                                     vertex slot, the sorted neighbour
 *                                     triple (-1 for a tet face), float
 *                                     position, surface face id or -1
 *                                     (vertex_2id, vertex_2pos); per cell from
 *                                     cell_vertex_off
 *   surface_*                         every active tet face with id <=
 *                                     max_sf_fid: cell, face id, centroid of
 *                                     its vertex cycle (cell_to_surfv2fid);
 *                                     per cell from cell_surface_off
 *   se_covered, ce_covered            with feature edges set
 *                                     (rpd_set_feature_edges), 5 int32 per
 *                                     record: cell, the two vertices (slot
 *                                     order) on both faces of an active tet
 *                                     edge that the map lists as sharp
 *                                     (fe_type 1) or concave (2), fe_line_id,
 *                                     fe_id (se_covered_lvids,
 *                                     ce_covered_lvids); per cell from
 *                                     cell_*_covered_off, sorted, unique
 *   se_line_end, se_line_end_pos      for each of those two vertices (any
 *                                     fe_type) with a bisector among its
 *                                     planes: cell, vertex slot, the first
 *                                     such bisector's neighbour site,
 *                                     fe_line_id, and the float position
 *                                     (se_line_endpos); per cell from
 *                                     cell_se_line_end_off, sorted, unique
 *   cell_cc, facet_cc, edge_cc        update_power_cells' connected
 *                                     components (rpd_update.cxx:454-530)
 *                                     over cell_nbrs: per cell the index of
 *                                     its component among its site's cells
 *                                     (cc_cells), per facet record among the
 *                                     cells of its (site, neighbour) key
 *                                     (facet_cc_cells, components ordered by
 *                                     size, then smallest cell), per edge
 *                                     record among the cells of its (site,
 *                                     neighbour pair) (edge_cc_cells); other
 *                                     components are ordered by smallest
 *                                     cell, as get_CC_given_neighbors finds
 *                                     them.  The *_surf_v2fids lists are the
 *                                     surface records of a component's cells
 *                                     in ascending cell order.
 *   sfg_*                             with a surface mesh set
 *                                     (rpd_set_surface_mesh), libmat's
 *                                     update_sphere_surf_v2fids
 *                                     (rpd_update.cxx:342-405): per site
 *                                     (site_sfg_off) its surface faces, each
 *                                     once with its last surface record
 *                                     (sfg_record), grouped over the face
 *                                     adjacency without crossing a
 *                                     no-cross pair; sorted by group (by
 *                                     smallest face), then face
 *                                     (surf_v2fid_in_groups)
 * Computes the per-cell topology first when needed. */
rpd_status rpd_compute_power_cells(struct rpd_ctx* ctx, int max_sf_fid, float* ms);

/* libmat's SurfaceMesh as update_sphere_surf_v2fids reads it: per
 * triangle the faces across its three edges (facets.adjacent, -1 for none;
 * must be symmetric) and the face pairs across sharp edges that a group does
 * not cross (fe_sf_fs_pairs, n_pairs x 2).  Face ids are the surface face
 * ids of the cells (tet faces numbered first, <= max_sf_fid).  Used by the
 * following rpd_compute_power_cells calls; n_faces = 0 clears it. */
rpd_status rpd_set_surface_mesh(struct rpd_ctx* ctx, const int32_t* facet_adj, int32_t n_faces,
                                const int32_t* no_cross, int64_t n_pairs);

/* libmat's TetMesh::tet_es2fe_map (<tid, lfid_min, lfid_max> -> <fe_type,
 * fe_id, fe_line_id>, src/rpd3d_base/rpd_update.cxx:77-82), one record per
 * key; lf_min < lf_max are local faces (0..3) of tet tet_id.  Of records
 * with the same key the last one counts (a map's last assignment).  Used by
 * the following rpd_compute_power_cells calls; n = 0 clears it. */
typedef struct rpd_feature_edge {
  int32_t tet_id, lf_min, lf_max;
  int32_t fe_type, fe_id, fe_line_id; /* fe_type: 1 sharp (SE), 2 concave (CE) */
} rpd_feature_edge;
rpd_status rpd_set_feature_edges(struct rpd_ctx* ctx, const rpd_feature_edge* edges, int64_t n);

typedef struct rpd_power_cells_view {
  int32_t n_site;
  int64_t n_cells;
  const int64_t* site_cell_off;
  const uint32_t* site_cells;
  const int64_t* cell_nbr_off;
  const int32_t* cell_nbrs;
  const int64_t* cell_tfid_off;
  const int32_t* cell_tfids;
  int64_t n_facets;
  const int64_t* site_facet_off;
  const uint64_t* facet_keys;
  const uint32_t* facet_cells;
  int64_t n_edges;
  const int64_t* site_edge_off;
  const int32_t* edges;
  int64_t n_vertices;
  const int64_t* cell_vertex_off;
  const int32_t* vertex_cell;
  const int32_t* vertex_lvid;
  const int32_t* vertex_ids;  /* 3 per vertex */
  const float* vertex_pos;    /* 3 per vertex */
  const int32_t* vertex_sfid;
  int64_t n_surface;
  const int64_t* cell_surface_off;
  const int32_t* surface_cell;
  const int32_t* surface_fid;
  const float* surface_pos;   /* 3 per face */
  int64_t n_se_covered;
  const int64_t* cell_se_covered_off;
  const int32_t* se_covered;  /* 5 per record */
  int64_t n_ce_covered;
  const int64_t* cell_ce_covered_off;
  const int32_t* ce_covered;  /* 5 per record */
  int64_t n_se_line_end;
  const int64_t* cell_se_line_end_off;
  const int32_t* se_line_end;       /* 4 per record */
  const float* se_line_end_pos;     /* 3 per record */
  const int32_t* cell_cc;     /* n_cells */
  const int32_t* facet_cc;    /* n_facets */
  const int32_t* edge_cc;     /* n_edges */
  int64_t n_sfg;
  const int64_t* site_sfg_off;  /* n_site + 1 */
  const int32_t* sfg_group;
  const int32_t* sfg_fid;
  const int32_t* sfg_record;  /* index into surface_* */
} rpd_power_cells_view;
rpd_status rpd_get_power_cells(struct rpd_ctx* ctx, rpd_power_cells_view* view);

/* Copies `bytes` from a device pointer of one of the views above to host
 * memory, on the context's stream (for callers without CUDA of their own). */
rpd_status rpd_copy_device_to_host(struct rpd_ctx* ctx, void* dst, const void* src, int64_t bytes);

/* ---- incremental update ---------------------------------------------------
 * libmat's RPD3D_GPU::calculate_partial (src/rpd3d_api/rpd_api.cxx:147-316):
 * after rpd_compute (and rpd_set_sites with the same site count, e.g. moved
 * or resized spheres), recomputes the cells of the sites with recompute[i]
 * != 0 -- the changed sites and those whose cells they can change, libmat's
 * spheres_and_1rings -- with the context's current sites, and merges them
 * with the previous cells: cells of the other sites are kept as they were
 * (merge_convex_cells).  The merged cells are the rpd_get_cells /
 * rpd_copy_cells_to_host result, in (tet, site) order; stats and the
 * pair-level outputs (pair headers, pairs, topology hashes) describe the
 * recomputed sites' pairs.  Site flags of rpd_set_sites still apply. */
rpd_status rpd_compute_partial(struct rpd_ctx* ctx, const uint32_t* recompute, rpd_stats* stats);

/* ---- distance to local medial primitives --------------------------------
 * libmat's dist2mat (ClosestDistanceToLocalMat / compute_closest_dist2mat,
 * src/dist2mat/dist2mat.cu:195-310): for every sample point (xyz), the
 * smallest signed distance |p - c| - r to the spheres of its primitives
 * (prims[offsets[s] .. offsets[s] + counts[s]), each three sphere ids:
 * (-1, -1, s) a sphere, (-1, a, b) a cone, (a, b, c) a slab; spheres are
 * (x, y, z, r)) and the index of the closest primitive in its list (the
 * reference's choice among equal minima; -1 for an empty list, whose
 * distance is 1e16).  on_device = 1: every pointer is device memory and the
 * call runs on the context's stream (spheres 16-byte aligned); 0: host
 * memory, copied in and out.  Out-of-range sphere ids or lists are
 * reported (RPD_ERR_INVALID_ARGUMENT) before any distance is computed. */
rpd_status rpd_dist2mat(struct rpd_ctx* ctx, const float* spheres, int n_spheres,
                        const float* samples, int n_samples, const uint32_t* offsets,
                        const uint32_t* counts, const int32_t* prims, int64_t n_prims,
                        float* dist, int32_t* closest, int on_device);

/* ---- polygon soup of the emitted cells, on the device ------------------
 * libmat's Houdini export, get_one_convex_cell_faces_const
 * (src/IO/IO_CUDA/io_cuda.cxx:21-141) over every emitted cell in
 * rpd_get_cells order: the cell's vertices (float, by
 * ConvexCellHost::compute_vertex_coordinates) are appended to one point
 * list -- a NaN vertex ends the cell (the points before it stay, no faces);
 * every active face becomes one polygon over its vertex cycle (point ids
 * global), or with triangulate the fan (c0, cp, cp+1); boundary_only keeps
 * bisector faces and tet faces whose face id is below max_sf_fid.  Each
 * polygon carries its cell's site and the site across the face (-1 for a
 * tet face).  Computes the per-cell topology first when needed. */
rpd_status rpd_compute_polygons(struct rpd_ctx* ctx, int triangulate, int boundary_only,
                                int max_sf_fid, float* ms);

typedef struct rpd_polygon_view {
  int64_t n_points;
  const float* points;          /* device, n_points x 3 */
  int64_t n_polys;
  const int64_t* poly_offsets;  /* device, n_polys + 1 offsets into indices */
  int64_t n_indices;
  const uint32_t* indices;      /* device, point ids */
  const int32_t* poly_site;     /* device, n_polys */
  const int32_t* poly_adj_site; /* device, n_polys */
} rpd_polygon_view;
rpd_status rpd_get_polygons(struct rpd_ctx* ctx, rpd_polygon_view* view);

/* Slicing plane of the following rpd_compute_polygons calls, as
 * save_convex_cells_houdini applies it (src/IO/IO_CUDA/io_cuda.cxx:166-170):
 * a cell whose barycenter -- the float mean of its float vertices,
 * compute_cell_barycenter (io_cuda.cxx:6-17) -- has dot(bary - pos, normal)
 * >= 0 in double (is_slice_by_plane, src/IO/IO_CXX/io.cxx:810-820) is left
 * out, points and faces.  libmat's plane: pos = (xmax / 2.2, 0, 0), normal =
 * (-1, 0, 0).  enable = 0 turns slicing off. */
rpd_status rpd_set_polygon_slice(struct rpd_ctx* ctx, int enable, const double* pos,
                                 const double* normal);

/* The polygon soup of the last rpd_compute_polygons written to `path` as a
 * Houdini binary geometry file, byte for byte what libmat's
 * save_convex_cells_houdini writes through IO::GeometryWriter
 * (src/IO/IO_CUDA/io_utils.cpp:106-231): big-endian, version 5, point
 * attribute P (x, y, z, 1), primitive attribute PrimAttr = the polygon's
 * site, point ids 16-bit up to 65536 points, else 32-bit.  The file image is
 * assembled on the device and written through a pinned staging buffer;
 * *bytes (optional) receives its size.  No points: RPD_ERR_INVALID_ARGUMENT
 * (the reference writer throws). */
rpd_status rpd_write_polygons_bgeo(struct rpd_ctx* ctx, const char* path, int64_t* bytes);
/* NULL buffers: sizes only.  points: 3 floats per point; offsets: n_polys + 1. */
rpd_status rpd_copy_polygons_to_host(struct rpd_ctx* ctx, float* points, int64_t max_points,
                                     int64_t* poly_offsets, uint32_t* indices,
                                     int64_t max_indices, int32_t* poly_site,
                                     int32_t* poly_adj_site, int64_t max_polys,
                                     int64_t* n_points, int64_t* n_polys, int64_t* n_indices);

/* The neighbour lists used by the last rpd_compute (n_site x k, -1 padded),
 * copied to the host.  k_out receives k. */
rpd_status rpd_copy_neighbors_to_host(struct rpd_ctx* ctx, int32_t* nbr,
                                      int64_t capacity, int* k_out);

/* Every site's list as the last rpd_compute clipped its cells with, as a
 * CSR on the host: the extended list of a site that the exact-lists rounds
 * gave one (every site whose key lies below its cells' radius bound, in
 * ascending key; or every site, in id order), else its base list in clip
 * order (ascending key when certified, else as built), holes (-1) dropped.
 * An extended list holds the base list, so the cells of such a site that
 * the base list already certified are its cells too.  offsets: n_site + 1
 * entries; with ids NULL only n_total (the entries) is returned. */
rpd_status rpd_copy_site_lists_to_host(struct rpd_ctx* ctx, int64_t* offsets, int32_t* ids,
                                       int64_t capacity, int64_t* n_total);

/* The candidate pairs of the last rpd_compute as a per-tet CSR (host). */
rpd_status rpd_copy_pairs_to_host(struct rpd_ctx* ctx, int32_t* tet_offsets,
                                  int32_t* pair_sites, int64_t capacity,
                                  int64_t* n_pairs);

/* Compaction of a pair-header array without allocating device memory.
 * No counterpart in the reference: it exists for callers that cannot call
 * cudaMalloc during their run (work recorded into a stream they do not own,
 * applications whose memory pool owns all device memory, code where an
 * allocation would synchronise the device).  It performs the compaction
 * step of rpd_compute: cells_out receives the records of pair_headers whose
 * status is success, in pair order, *n_cells_out their count, and
 * status_counts (optional, 11 entries: statuses 0..8, other, payload full)
 * the status histogram; all pointers are device pointers the caller owns,
 * cells_out holding n_pairs records.  Its only temporary lives in a fixed
 * array inside the library (reserved on each GPU that loads it until exit),
 * so n_pairs is limited to 2^25; larger inputs return RPD_ERR_CAPACITY.  The
 * first call on a device looks up that array's address (call it once before
 * any stream capture); the address is kept per device ordinal, so calls must
 * run in the device's primary context and not after a cudaDeviceReset in
 * the same process.  Calls share the array: calls that overlap on the GPU
 * race and must be serialised by the caller.  A launch that fails returns
 * RPD_ERR_CUDA; an error the caller left pending is neither reported nor
 * cleared.  Asynchronous on `stream` (a cudaStream_t, NULL = default
 * stream). */
rpd_status rpd_compact_cells_noalloc(const rpd_cell_header* pair_headers, int64_t n_pairs,
                                     rpd_cell_header* cells_out, int64_t* n_cells_out,
                                     uint64_t* status_counts, void* stream);

/* ---- Learned list length (k-predictor) ----------------------------------
 * No counterpart in the reference, whose lists have a fixed length.  A
 * 12 -> 64 -> 64 -> 1 MLP (bf16 operands, fp32 accumulation, tensor-core
 * mma) predicts log2 of the number of distance-ordered list entries a cell
 * takes before its security-radius certificate holds.  Parameters are fp32,
 * RPD_MLP_PARAMS of them: W1 [16][64] (feature x hidden), b1 [64], W2
 * [64][64] (in x out), b2 [64], w3 [64], b3.  Features are 16 bf16 values
 * per cell (12 used, 4 zero); bf16 crosses this interface as uint16_t bit
 * patterns. */
#define RPD_MLP_FEATURES 16
#define RPD_MLP_PARAMS 5313

/* Clips the current mesh and sites with the whole distance-ordered lists
 * and the certificate (cells identical to the plain path's), then appends up
 * to max_samples of the emitted cells (evenly strided over the pairs) to the
 * context's training set: features and label log2(max(k*, 1)), k* the list
 * entries the cell took.  Requires certify = 1 and RPD_NEIGH_KNN.  Call it
 * on several meshes and site sets before rpd_mlp_train.  n_total receives
 * the size of the training set. */
rpd_status rpd_mlp_collect(struct rpd_ctx* ctx, int64_t max_samples, int64_t* n_total);
rpd_status rpd_mlp_clear_samples(struct rpd_ctx* ctx);
/* The training set (x: n x RPD_MLP_FEATURES bf16, labels y); NULL buffers
 * query its size. */
rpd_status rpd_mlp_copy_samples(struct rpd_ctx* ctx, uint16_t* x, float* y, int64_t capacity,
                                int64_t* n_samples);

typedef struct rpd_mlp_report {
  int64_t n_train;         /* samples trained on */
  int64_t n_calib;         /* held-out samples that set the margin */
  float loss_first;        /* mean squared error (log2 units), first epoch */
  float loss_last;         /* last epoch */
  float calib_loss;        /* held-out mean squared error */
  float margin;            /* added to the prediction before 2^(.) */
  float calib_miss_rate;   /* held-out cells whose k* exceeds the predicted length */
  float calib_mean_k;      /* mean predicted length over the held-out cells */
  float const_k;           /* one length for all cells with the same miss rate */
  float ms_train;          /* device time of the training loop */
  int32_t steps;           /* optimiser steps */
  int32_t epochs;
  float label_var;         /* variance of the labels (the error of predicting their mean) */
} rpd_mlp_report;

/* Trains the predictor on the GPU (own forward/backward kernels, Adam,
 * mini-batches of `batch` samples, `epochs` passes, learning rate lr) from
 * a fresh initialisation drawn from `seed`.  A random 10% of the samples
 * is held out: the margin is the (1 - miss_target) quantile of their
 * residuals, so about miss_target of the cells are clipped twice. */
rpd_status rpd_mlp_train(struct rpd_ctx* ctx, int epochs, int batch, float lr, float miss_target,
                         uint64_t seed, rpd_mlp_report* report);

/* Switches rpd_config.learned_k of a context (on = 0 or 1; 1 needs
 * certify). */
rpd_status rpd_mlp_enable(struct rpd_ctx* ctx, int on);

/* Saves / loads the parameters (fp32, RPD_MLP_PARAMS) and the margin. */
rpd_status rpd_mlp_get_params(struct rpd_ctx* ctx, float* params, int n_params, float* margin);
rpd_status rpd_mlp_set_params(struct rpd_ctx* ctx, const float* params, int n_params,
                              float margin);

/* The network on caller rows (host buffers, n x RPD_MLP_FEATURES bf16):
 * outputs y, and the gradient of mean((y - target)^2) (grads receives
 * RPD_MLP_PARAMS floats, loss the mean squared error). */
rpd_status rpd_mlp_forward(struct rpd_ctx* ctx, const uint16_t* x, int64_t n, float* y);
rpd_status rpd_mlp_gradient(struct rpd_ctx* ctx, const uint16_t* x, const float* target,
                            int64_t n, float* grads, float* loss);

/* The feature rows of the last rpd_compute's pairs (learned_k, or the
 * cells of the last rpd_mlp_collect), and the list lengths the predictor
 * gave the pairs of the last learned_k compute (pair order). */
rpd_status rpd_mlp_copy_features(struct rpd_ctx* ctx, uint16_t* x, int64_t capacity,
                                 int64_t* n_rows);
rpd_status rpd_mlp_copy_klen(struct rpd_ctx* ctx, int32_t* klen, int64_t capacity,
                             int64_t* n_pairs);

/* ---- Batches of independent meshes ---------------------------------------
 * No counterpart in the reference, which runs one mesh per call.  A batch
 * concatenates many meshes (each with its own sites) into one context; the
 * per-mesh front end (neighbour lists, candidate pairs) is recorded once into
 * a CUDA graph and replayed, and all meshes' cells are clipped by one
 * persistent kernel launch.  Neighbour lists are GPU-built (RPD_NEIGH_KNN);
 * learned_k is not available for batches.  Cells of every mesh equal those
 * of a single-mesh rpd_compute of that mesh. */
struct rpd_batch;
rpd_status rpd_batch_create(const rpd_config* cfg, struct rpd_batch** out);
void rpd_batch_destroy(struct rpd_batch* batch);
const char* rpd_batch_last_error(const struct rpd_batch* batch);
/* Appends a mesh and its sites (same layouts as rpd_set_mesh /
 * rpd_set_sites; tets hold the mesh's own vertex ids).  mesh_index receives
 * the mesh's index in the batch. */
rpd_status rpd_batch_add_mesh(struct rpd_batch* batch, const double* xyz, int n_vert,
                              const int32_t* tets, int n_tet, const int32_t* v_adjs,
                              const uint8_t* e_adj6, const int32_t* f_adjs, const int32_t* f_ids,
                              const double* xyzw, int n_site, const uint32_t* flags,
                              int* mesh_index);
int rpd_batch_size(const struct rpd_batch* batch);
/* 1 (default): record the front end into a CUDA graph and replay it; 0:
 * launch it directly every time. */
rpd_status rpd_batch_set_graph(struct rpd_batch* batch, int use_graph);
/* All meshes; stats are for the whole batch (ms_knn: the front end of all
 * meshes, kNN and candidate search). */
rpd_status rpd_batch_compute(struct rpd_batch* batch, rpd_stats* stats);
/* Autotuner of the batch's clip stage (as rpd_autotune). */
rpd_status rpd_batch_autotune(struct rpd_batch* batch, int repeats, rpd_tuning* result);
/* Range of mesh `mesh` in the compacted cells of the batch's context
 * (rpd_get_cells(rpd_batch_context(batch)) -- there, tet and site ids are
 * the batch's). */
rpd_status rpd_batch_mesh_cells(struct rpd_batch* batch, int mesh, int64_t* first_cell,
                                int64_t* n_cells);
/* The cells of one mesh with the mesh's own tet and site ids (headers and
 * the site pairs of the plane ids) and consecutive payload offsets; NULL
 * buffers query the sizes. */
rpd_status rpd_batch_copy_mesh_cells(struct rpd_batch* batch, int mesh, rpd_cell_header* headers,
                                     int64_t max_cells, void* payload, int64_t payload_capacity,
                                     int64_t* n_cells, int64_t* payload_bytes);
/* The context holding the batch (configuration, statistics views).  Do not
 * call rpd_set_mesh / rpd_set_sites / rpd_compute on it. */
struct rpd_ctx* rpd_batch_context(struct rpd_batch* batch);

/* Page-locked host buffers for fast host<->device copies (cudaMallocHost),
 * every page written once (zeros) before they are returned; NULL on
 * failure. */
void* rpd_host_alloc(size_t bytes);
void rpd_host_free(void* p);

/* Host helper: mesh adjacency counts and face ids with the semantics of
 * load_tet_adj_info (io.cxx:238-335); boundary faces are numbered first in
 * scan order (the surface facets), interior faces from n_boundary_faces up.
 * Returns RPD_ERR_INVALID_ARGUMENT for out-of-range ids or faces shared by
 * more than two tets. */
rpd_status rpd_build_mesh_adjacency(int n_vert, const int32_t* tets, int n_tet,
                                    int32_t* v_adjs, uint8_t* e_adj6,
                                    int32_t* f_adjs, int32_t* f_ids,
                                    int32_t* n_boundary_faces);

#ifdef __cplusplus
}
#endif
#endif
