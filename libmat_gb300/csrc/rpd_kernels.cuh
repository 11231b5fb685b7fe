// rpd_kernels.cuh -- kernel parameter blocks and launchers (host-callable).
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

#include "../../include/rpd_gb300.h"

namespace rpd {

constexpr int kClipMaxThreads = 512;

// kernels launched since the last reset (host counter, one context at a time
// per thread)
void note_launches(int n);
int take_launches();

struct ClipParams {
  const float* vert3f;   // n_vert x 3, float copies of the mesh vertices
  const double* vert3d;  // n_vert x 3
  const int4* tets;
  const int32_t* v_adjs;
  const float4* tet_xyz;  // n_tet x 3: the tet's float vertices, packed
  const uchar4* tet_vadj; // n_tet: #tets of each of the tet's vertices (uint8, as recorded)
  const uint8_t* e_adj6;  // n_tet x 6
  const int32_t* f_adjs;  // n_tet x 4
  const int32_t* f_ids;   // n_tet x 4
  const float4* site4f;   // n_site, (x, y, z, w) float
  const double* site4d;   // n_site x 4
  const float2* vert2;    // n_vert x 3 double-float (hi, lo) vertex coordinates
  const float2* site2;    // n_site x 4 double-float (x, y, z, w)
  const int32_t* nbr;     // n_site x k, -1 padded
  int k;
  const int32_t* pair_tet;
  const int32_t* pair_site;
  long long n_pairs;
  rpd_cell_header* headers;  // n_pairs
  uint8_t* payload;
  unsigned long long* payload_cursor;
  unsigned long long payload_cap;
  unsigned long long* work;      // work-queue counter, zeroed before launch
  unsigned long long* counters;  // [0] predicates, [1] escalated
  unsigned long long* uncertified;  // cells flagged RPD_CELL_UNCERTIFIED, or null
  unsigned long long* exact_counters;  // [0] FP64 sign uncertain, [1] exact != FP64, or null
  int geometry;
  // distance-ordered lists with the security-radius certificate
  const float* keys;             // n_site x k bisector distances (ascending), or null
  const int32_t* site_klen;      // per-site list length, or null (= k)
  const int32_t* pair_klen;      // per-pair list length, or null
  int lazy_cert;                 // 1: one certificate test after the list
  unsigned long long* misses;    // shortened lists whose certificate failed, or null
  int32_t* consumed;             // per pair: list entries taken, or null
  float cert_margin;             // absolute margin of the certificate
  // optional indirection: work item w clips pair pair_index[w]
  const int32_t* pair_index;
  long long n_work;
  unsigned long long* topo_hash;  // n_pairs canonical topology hashes, or null
  // completeness of the lists: every site missing from site s's base list
  // has a key >= nbr_bound[s] (INFINITY: the list holds every site); null =
  // no bound known (no cell is ever flagged uncertified)
  const float* nbr_bound;
  // extended lists: site s clips with row site_row[s] (>= 0) instead of its
  // base row; the row's entries start at ext_off[row], ext_len[row] of them
  // (-1 padded beyond), keys ascending (certified clipping), and every site
  // not in it has a key >= ext_bound[row]
  const int32_t* site_row;       // n_site, or null
  const int32_t* ext_nbr;
  const float* ext_keys;
  const long long* ext_off;
  const int32_t* ext_len;
  const float* ext_bound;
};

// cells flagged RPD_CELL_UNCERTIFIED by the clip kernel, bounded again:
// flag cleared where the certificate holds, else the radius (float bits)
// raised into site_need[site] (optional)
struct RecheckParams {
  rpd_cell_header* headers;  // pair headers
  const int32_t* idx;        // the flagged pairs, *n_dev of them
  const int32_t* n_dev;
  const uint8_t* payload;
  const float4* site4f;
  const int32_t* site_row;   // as ClipParams, or null
  const float* ext_bound;
  const float* nbr_bound;
  float margin;
  unsigned int* site_need;
  int32_t* kept_idx;                // the pairs still flagged, in any order
  unsigned long long* kept_count;   // their number (added to)
};
cudaError_t launch_recheck_cells(const RecheckParams& p, int num_sms, cudaStream_t st);

// coordinates, volume and topology hash of the emitted cells (after the
// clip passes, before compaction)
struct EpilogueParams {
  rpd_cell_header* headers;  // n_pairs; volume written for emitted cells
  long long n_pairs;
  uint8_t* payload;          // xyz sections written
  const float2* face2;            // n_tet x 16: double-float tet face planes
  const float2* site2;
  int geometry;                   // 0: xyz zero, volume 0
  unsigned long long* topo_hash;  // n_pairs, or null
};
cudaError_t launch_cell_epilogue(const EpilogueParams& p, int num_sms, cudaStream_t st);
// double-float (nx, ny, nz, d) of the four face planes of every tet, from FP64
cudaError_t launch_tet_face_planes(const double* vert3d, const int4* tets, int n_tet, float2* out,
                                   cudaStream_t st);

// Sites i of the box, pair and kNN kernels are 0..n_site-1 of one mesh;
// site_base (tet_base) turns them into the indices of the arrays that hold
// every mesh of a batch (0 for a single mesh).  Neighbour ids are global.
struct BoxParams {
  const float4* site4f;   // all sites
  const uint32_t* flags;  // all sites
  int site_base;
  const int32_t* nbr;     // this mesh's rows (stride k); the first k_box entries are used
  int k;
  int k_box;
  int n_site;
  float4 box_lo, box_hi;  // mesh box grown by offset_r
  float offset_r;         // largest distance of a tet vertex to its centroid
  float offset_e;         // bound on the float error of a power distance
  float coord_scale;      // largest coordinate magnitude
  float abs_margin;
  float4* site_box;       // n_site x 2: (lo, status), (hi, 0)
  float4* site_planes;    // n_site x kBoxPlanes: planes of the grown cell
  int32_t* site_nplanes;  // n_site: count (0 = use the box only)
  unsigned long long* counters;
};

constexpr int kBoxPlanes = 48;
// nearest bisectors that bound each site's candidate region for the tets of
// common size (rpd_config.box_planes = 0); measured on the 1M-tet ellipsoid:
// 32 -> 9.07 ms, 40 -> 8.72, 44 -> 8.60, 48 -> 8.65, 56 -> 9.29 ms for the
// pair search
constexpr int kDefaultBoxPlanes = 44;

size_t clip_smem_per_warp();
int clip_blocks_per_sm(int pred_mode, int warps);
int box_blocks_per_sm(int warps);
// variant: 0 = no register cap (warps per block as given), 1 = at most 80
// registers (6 blocks of 4 warps per SM), 2 = at most 64 (8 blocks of 4 warps)
cudaError_t launch_clip_cells(const ClipParams& p, int pred_mode, int certify, int variant,
                              int blocks, int warps, cudaStream_t st);
int clip_blocks_per_sm_cert(int pred_mode, int certify, int warps, int variant);
// indices of the pairs whose header status equals `status`
cudaError_t select_pairs(const rpd_cell_header* h, long long n, int status, int32_t* flag_tmp,
                         int32_t* pos_tmp, int32_t* scan_tmp, int32_t* idx_out,
                         cudaStream_t st);
cudaError_t launch_site_box(const BoxParams& p, int blocks, int warps, cudaStream_t st);

// ---- uniform grids, kNN, candidate pairs, scans (rpd_pairs.cu)
struct Grid {
  float3 lo;
  float inv_cell;  // 1 / cell size
  float cell;
  int nx, ny, nz;
};

// exclusive scan of n int32 counts into out (n + 1 entries, out[n] = total);
// temp must hold scan_temp_ints(n) ints
size_t scan_temp_ints(long long n);
cudaError_t scan_exclusive(const int32_t* in, int32_t* out, long long n, int32_t* temp,
                           cudaStream_t st);

// bins points into grid cells: cell_of[n], cell_start[n_cells + 1],
// cell_items[n] (ascending item id within a cell)
cudaError_t grid_build_sites(const float4* pts, int n, const Grid& g, int32_t* cell_of,
                             int32_t* cell_count, int32_t* cell_start, int32_t* cell_fill,
                             int32_t* cell_items, int32_t* scan_tmp, cudaStream_t st);
// centroid (w = largest vertex distance) of every tet and, optionally, its
// four vertices packed in three float4 and its vertices' tet counts (uint8)
cudaError_t tet_centroids(const float* vert3f, const int4* tets, int n_tet, float4* centroid,
                          cudaStream_t st, float4* tet_xyz = nullptr,
                          const int32_t* v_adjs = nullptr, uchar4* tet_vadj = nullptr);
// bins the tets of radius class `want` (all tets when cls is null) by centroid;
// cell_rmax (optional) gets the largest tet radius (centroid.w) of each cell
cudaError_t grid_build_tets(const float4* centroid, int n_tet, const uint8_t* cls, int want,
                            const Grid& g, int32_t* cell_of, int32_t* cell_count,
                            int32_t* cell_start, int32_t* cell_fill, int32_t* cell_items,
                            int32_t* scan_tmp, cudaStream_t st, float* cell_rmax = nullptr);

// k smallest power-bisector distances per site (ties by id); lists in
// distance order or sorted by id
cudaError_t launch_knn(const float4* site4f, int n_site, const Grid& g,
                       const int32_t* cell_start, const int32_t* cell_items, int k,
                       float w_max, int order_by_id, int32_t* nbr, float* keys,
                       int32_t* nbr_dist, int32_t* status, cudaStream_t st, int id_offset = 0,
                       float* bound_out = nullptr);
// the general form: rows for a subset of the sites, only keys up to a
// per-site bound, longer lists (k <= knn_max_k())
struct KnnArgs {
  const float4* site4f;  // the mesh's sites; subset, rows and grid items index them
  int n_rows;
  Grid g;
  const int32_t* cell_start;
  const int32_t* cell_items;
  int k;                 // row stride and longest list
  float w_max;
  int order_by_id;       // nbr sorted by id (else distance order)
  int32_t* nbr;          // n_rows x k, -1 padded
  float* keys;           // n_rows x k ascending keys (INFINITY padded), or null
  int32_t* nbr_dist;     // n_rows x k in distance order, or null
  int32_t* status;       // per row: 1 = every site of the grid was seen, or null
  int id_offset;         // added to the listed ids
  const int32_t* subset;       // row f lists site subset[f] (null: row f is site f)
  const unsigned int* radius;  // per site, float bits R: only keys <= R * bound_scale +
                               // bound_abs are listed (null: no bound)
  float bound_scale, bound_abs;
  int32_t* len_out;      // per row: entries listed, or null
  float* bound_out;      // per row: every site not listed has a key >= this, or null
  // per site: the ids [x, y) it may list (its mesh's sites in a batch), or
  // null for every site
  const int2* site_range;
  // per site: where the grid holds it, or null (its position).  A batch
  // moves each mesh to a slot of its own in the grid's space; keys use the
  // real positions, and a mesh moves as a whole, so distances within it
  // are kept
  const float4* grid_pos;
};
int knn_max_k();
cudaError_t launch_knn(const KnnArgs& a, cudaStream_t st);

// candidate pairs: per site, tets whose centroid lies in the site's box and
// that pass the reference rule; appends (tet, site) and counts per tet
struct PairParams {
  const float* vert3f;     // all vertices (tets hold global vertex ids)
  const int4* tets;        // this mesh's tets
  const float4* centroid;  // this mesh's tets
  const float4* tet_xyz;   // this mesh's tets: vertices packed in 3 float4
  int tet_base;            // index of this mesh's first tet among all tets
  int site_base;
  Grid tg;
  const int32_t* tcell_start;
  const int32_t* tcell_items;
  const float* tcell_rmax;  // largest tet radius of each tet-grid cell (may be null)
  const float4* site4f;   // all sites
  const uint32_t* flags;  // all sites
  const int32_t* nbr;     // this mesh's rows
  const int32_t* rule_nbr;  // the same lists in another order (rule evaluation), or null
  int k;
  int n_site;
  const float4* site_box;
  const float4* site_planes;   // n_site x kBoxPlanes
  const int32_t* site_nplanes;
  float coord_scale;
  int2* pair_buf;            // (tet, site)
  unsigned long long* pair_cursor;
  long long pair_cap;
  int32_t* tet_count;
  unsigned long long* diag;  // search counters (see rpd_stats::search)
  // the radius the site planes were pushed out by (the tet class's largest
  // tet radius, rounded up): each centroid test takes back what its own
  // tet's radius does not need
  float offset_r;
  // keys of the rule's (distance-ordered) lists, or null; with them a tet
  // whose nearest vertex lies within the key of neighbour r (less the
  // margins) passes the rule for r and every later neighbour at once
  const float* rule_keys;
  float accept_margin;  // absolute rounding of a key (as the certificate's)
  float accept_err;     // bound on the float error of pd_m(v) - pd_i(v)
};
// n_tasks, task_off: n_site and n_site + 1 ints; work: one counter
cudaError_t launch_pairs(const PairParams& p, int32_t* n_tasks, int32_t* task_off,
                         int32_t* scan_tmp, unsigned long long* work, int num_sms,
                         cudaStream_t st);

// scatter the pair buffer into per-tet CSR and sort sites in each tet
cudaError_t pairs_to_csr(const int2* pair_buf, long long n_pairs, int n_tet,
                         const int32_t* tet_offsets, int32_t* tet_fill, int32_t* pair_site,
                         int32_t* pair_tet, int32_t* tet_k_out, cudaStream_t st);

// compaction of emitted cells (status success) in pair order; n_uncert
// (optional) counts the emitted cells flagged RPD_CELL_UNCERTIFIED
cudaError_t compact_cells(const rpd_cell_header* pair_headers, long long n_pairs,
                          int32_t* flag_tmp, int32_t* pos_tmp, int32_t* scan_tmp,
                          rpd_cell_header* out, long long* n_out_dev,
                          unsigned long long* status_hist, cudaStream_t st,
                          unsigned long long* n_uncert = nullptr);
// indices of the pairs whose header carries RPD_CELL_UNCERTIFIED
cudaError_t select_uncertified(const rpd_cell_header* h, long long n, int32_t* flag_tmp,
                               int32_t* pos_tmp, int32_t* scan_tmp, int32_t* idx_out,
                               cudaStream_t st);
// sites with site_need != 0, ascending (idx_out), their count at pos_tmp[n]
cudaError_t select_sites(const unsigned int* site_need, int n, int32_t* flag_tmp,
                         int32_t* pos_tmp, int32_t* scan_tmp, int32_t* idx_out, cudaStream_t st);
// extended rows row0 + f (f < n) of the sites sites[f]: site_row[sites[f]] =
// row0 + f, ext_off[row0 + f] = off0 + f * stride
cudaError_t assign_rows(const int32_t* sites, int n, int row0, long long off0, int stride,
                        int32_t* site_row, long long* ext_off, cudaStream_t st);
// rows row0 + f of the sites sites[f], all on one list of every site
// (written at ext_nbr[off..off + n_site)), bound INFINITY
// (site_range: each row takes only its site's range of the shared list)
cudaError_t complete_rows(const int32_t* sites, int n, int row0, long long off, int n_site,
                          int32_t* site_row, long long* ext_off, int32_t* ext_len,
                          float* ext_bound, int32_t* ext_nbr, cudaStream_t st,
                          const int2* site_range = nullptr);

// batches: first compacted cell of each mesh (n_mesh + 1 entries); record
// sizes; gather of one mesh's records with mesh-local ids
cudaError_t mesh_cell_ranges(const rpd_cell_header* cells, const long long* n_cells,
                             const int32_t* tet_base, int n_mesh, long long* first,
                             cudaStream_t st);
cudaError_t record_sizes(const rpd_cell_header* cells, long long n, unsigned long long* size,
                         cudaStream_t st);
cudaError_t gather_records(const rpd_cell_header* cells, long long n,
                           const unsigned long long* new_off, const uint8_t* payload,
                           int tet_base, int site_base, rpd_cell_header* hout, uint8_t* out,
                           cudaStream_t st);

// per-cell topology (rpd_topo.cu): record sizes in 16-byte units, then the
// records at the scanned offsets (unit_off, 16-byte units)
cudaError_t topo_units(const rpd_cell_header* cells, long long n, int32_t* units, cudaStream_t st);
cudaError_t topo_fill(const rpd_cell_header* cells, long long n, const uint8_t* payload,
                      const int32_t* unit_off, rpd_topo_header* out_h, uint8_t* out, int num_sms,
                      cudaStream_t st);

// polygon soup of the emitted cells (rpd_poly.cu)
struct PolyParams {
  const rpd_cell_header* cells;  // emitted cells
  long long n;
  const uint8_t* payload;
  const rpd_topo_header* topo_h;  // their per-cell topology
  const uint8_t* topo;
  int triangulate, boundary_only, max_sf_fid;
  int slice;               // leave out the cells on the plane's positive side
  double slice_plane[6];   // pos, normal
  int32_t *cnt_points, *cnt_polys, *cnt_indices;        // per cell
  const long long *off_points, *off_polys, *off_indices;  // exclusive scans (n + 1)
  float* points;          // 3 per point
  long long* poly_offsets;  // into indices (n_polys + 1)
  uint32_t* indices;
  int32_t *poly_site, *poly_adj_site;
};
cudaError_t poly_count(const PolyParams& p, cudaStream_t st);
cudaError_t poly_fill(const PolyParams& p, cudaStream_t st);
// the points (16 bytes each) and polygons (13 + 2 or 4 bytes per id) of a
// Houdini binary geometry file, big-endian, at the two section starts
cudaError_t bgeo_fill(const float* points, long long n_points, const long long* poly_offsets,
                      const uint32_t* indices, const int32_t* poly_site, long long n_polys,
                      int wide, uint8_t* points_out, uint8_t* polys_out, int num_sms,
                      cudaStream_t st);
// exclusive scan of n int32 counts into n + 1 int64 (out[n] = total); temp:
// scan64_temp(n) entries
size_t scan64_temp(long long n);
cudaError_t scan64_exclusive(const int32_t* in, long long* out, long long n, long long* temp,
                             cudaStream_t st);

// merge of a partial recompute (rpd_partial.cu): keep[a] = old cell a's site
// not recomputed; slots of the merged (tet, site) order; gather of records
cudaError_t merge_keep(const rpd_cell_header* old_cells, long long n_old, const uint32_t* recomputed,
                       int32_t* keep, cudaStream_t st);
cudaError_t merge_slots(const rpd_cell_header* old_cells, long long n_old, const int32_t* keep,
                        const int32_t* keep_pos, const rpd_cell_header* new_cells, long long n_new,
                        long long n_out, long long* src, int32_t* units, cudaStream_t st);
cudaError_t merge_gather(const long long* src, long long n, const long long* off,
                         const rpd_cell_header* old_cells, const uint8_t* old_payload,
                         const rpd_cell_header* new_cells, const uint8_t* new_payload,
                         rpd_cell_header* out_cells, uint8_t* out_payload, int num_sms,
                         cudaStream_t st);

// stable radix sort of (key, value) pairs by the low `bits` key bits
// (rpd_sort.cu); hist and scan_tmp: radix_hist_ints(n) and
// scan_temp_ints(radix_hist_ints(n)) ints
size_t radix_hist_ints(long long n);
cudaError_t radix_sort_pairs(unsigned long long* keys, uint32_t* vals, long long n, int bits,
                             unsigned long long* keys_tmp, uint32_t* vals_tmp, int32_t* hist,
                             int32_t* scan_tmp, cudaStream_t st);

// power cells of the emitted cells (rpd_powercell.cu)
struct PowerCellParams {
  const rpd_cell_header* cells;
  long long n;
  const uint8_t* payload;
  const rpd_topo_header* topo_h;
  const uint8_t* topo;
  int max_sf_fid;
  int32_t* cnt;           // 8 x n: tet faces, facets, edges, vertices, surface faces,
                          // sharp edges, concave edges, sharp-line endpoints
  const long long* off;   // 8 x (n + 1), their exclusive scans
  // tet faces: fid per cell (ascending), and (site, fid) keys / cell values
  int32_t* tf_fid;
  unsigned long long* tf_key;
  uint32_t* tf_val;
  // facets: (site, neighbour) keys, cell values
  unsigned long long* fa_key;
  uint32_t* fa_val;
  // edges: keys / values for the sorts, fields by record, sorted output (7 per edge)
  unsigned long long* ed_key;
  uint32_t* ed_val;
  int32_t *ed_site, *ed_n0, *ed_n1, *ed_cell, *ed_lv0, *ed_lv1;
  int32_t* ed_out;
  // vertices
  int32_t *vx_cell, *vx_lvid, *vx_ids, *vx_sfid;
  float* vx_pos;
  // surface faces
  int32_t *sf_cell, *sf_fid;
  float* sf_pos;
  // neighbour cells (CSR per cell)
  int32_t *nbr_cnt, *nbr_fill, *nbr;
  const long long* nbr_off;
  // cells by site
  unsigned long long* site_key;
  uint32_t* site_val;
  // feature edges: sorted unique keys (tet << 4 | lf_min << 2 | lf_max) and
  // (fe_type, fe_id, fe_line_id) per key; records 5, 5, 4 int32 + 3 floats
  const unsigned long long* fe_keys;
  const int32_t* fe_vals;
  long long n_fe;
  int32_t *se, *ce, *se_end;
  float* se_end_pos;
};
cudaError_t pc_count(const PowerCellParams& p, cudaStream_t st);
cudaError_t pc_fill(const PowerCellParams& p, cudaStream_t st);
cudaError_t pc_edges_finish(const PowerCellParams& p, long long n_ed, int pass, cudaStream_t st);
// feature-edge counts (fill = 0, into cnt rows 5..7) or records (fill = 1)
cudaError_t pc_feature_edges(const PowerCellParams& p, int fill, cudaStream_t st);

// connected components of the power cells (rpd_cc.cu): per cell, facet
// record and edge record the index of its component in its group
struct CcParams {
  long long n, n_fa, n_ed;
  const long long* nbr_off;  // n + 1: cells across tet faces
  const int32_t* nbrs;
  const unsigned long long* site_key;  // n: site of site_cells[u] (sorted)
  const uint32_t* site_cells;
  const unsigned long long* facet_keys;  // sorted, cells ascending per key
  const uint32_t* facet_cells;
  const int32_t* edges;  // 7 per record, sorted
  // n_total = n + n_fa + n_ed entries each (pos, gstart: n_total + 1)
  int32_t *parent, *root, *rank, *flag, *croot;
  long long *pos, *gid, *gstart;
  int32_t* size;      // n_fa: distinct cells per facet component
  long long* scan_tmp;  // power_cell_components_temp(n_total)
  int32_t *cell_cc, *facet_cc, *edge_cc;
  unsigned int* err;
};
size_t power_cell_components_temp(long long n_total);
cudaError_t power_cell_components(const CcParams& p, cudaStream_t st);

// surface groups of each site (rpd_cc.cu): its surface faces (the last
// record of each) grouped over the surface mesh's face adjacency, not across
// no-cross pairs; output sorted by (site, group, face)
struct SurfaceGroupParams {
  long long n_sf;
  int n_site, site_bits;
  const rpd_cell_header* cells;
  const int32_t *surface_cell, *surface_fid;
  const int32_t* facet_adj;  // 3 per face, -1 for none
  int n_faces;
  const unsigned long long* no_cross;  // sorted (min << 32 | max) face pairs
  long long n_no_cross;
  unsigned long long *keys, *keys_tmp;  // n_sf each
  uint32_t *vals, *vals_tmp;
  int32_t *hist, *hist_tmp;  // radix_hist_ints(n_sf), scan_temp_ints(of that)
  int32_t* flag;             // n_sf
  long long *pos, *scan_tmp;  // n_sf + 1, scan64_temp(n_sf)
  unsigned long long* ekey;   // entries (n_sf at most)
  int32_t *erec, *parent, *root, *rank;
  int32_t *out_group, *out_fid, *out_rec;
  long long* site_off;  // n_site + 1
  unsigned int* err;
};
cudaError_t surface_groups(const SurfaceGroupParams& p, long long* n_entries, cudaStream_t st);
cudaError_t pc_neighbours(const PowerCellParams& p, long long n_tf, int pass, cudaStream_t st);
cudaError_t pc_site_offsets(const unsigned long long* keys, long long n, int n_site, int shift,
                            long long* off, cudaStream_t st);

// distance to local medial primitives (rpd_dist2mat.cu): ids checked first
// (*bad counts offending primitives / samples)
cudaError_t check_dist2mat(const int3* prims, long long n_prims, int n_spheres,
                           const uint32_t* offsets, const uint32_t* counts, int n_samples,
                           unsigned int* bad, cudaStream_t st);
cudaError_t launch_dist2mat(const float3* samples, int n_samples, const float4* spheres,
                            const int3* prims, const uint32_t* offsets, const uint32_t* counts,
                            float* dist, int32_t* closest, cudaStream_t st);

// reference site_knn layout -> row-major lists; validation of ids
cudaError_t neighbors_from_reference(const int32_t* ref, int k, int n_site, int32_t* nbr,
                                     cudaStream_t st);

// ---------------------------------------------------------------------------
// mesh preparation on the device (rpd_prep.cu)
// ---------------------------------------------------------------------------
constexpr int kRadiusBins = 4096;
struct MeshPrepOut {
  unsigned int bad;                    // 1: non-finite vertex, 2: vertex id out of range
  unsigned long long lo_key[3], hi_key[3];  // bounding box (order-preserving keys)
  double volume;
  unsigned long long rmax_key;         // largest tet radius
  int class_count[2];
  unsigned long long class_rmax_key[2];
};
double key_to_double(unsigned long long k);
cudaError_t mesh_prep_init(MeshPrepOut* out, cudaStream_t st);
// copies n bytes from device memory to dst (device-mapped host memory) with
// one block of stores, in stream order
cudaError_t launch_stage_bytes(const void* src, void* dst, size_t n, cudaStream_t st);
// float and double-float vertices, box, id check, FP64 tet radii, volume,
// boundary vertex marks (bmark may be null)
cudaError_t mesh_prep_geometry(const double* xyz, int n_vert, const int4* tets,
                               const int32_t* f_adjs, int n_tet, float* vert3f, float2* vert2,
                               double* rad, uint8_t* bmark, MeshPrepOut* out, cudaStream_t st);
cudaError_t mesh_prep_histogram(const double* rad, int n_tet, double rmax, int32_t* hist,
                                cudaStream_t st);
// class 0: radius <= r0; counts and largest radius per class
cudaError_t mesh_prep_classify(const double* rad, int n_tet, double r0, uint8_t* cls,
                               MeshPrepOut* out, cudaStream_t st);
// marked vertices as float4 (x, y, z, 0), count in *n_bv (device)
cudaError_t boundary_list(const uint8_t* bmark, const float* vert3f, int n_vert, float4* bverts,
                          int32_t* n_bv, cudaStream_t st);

// ---------------------------------------------------------------------------
// learned list length (rpd_mlp.cu)
// ---------------------------------------------------------------------------
constexpr int kMlpFeatures = 16;  // 12 features, zero-padded to the mma's k
constexpr int kMlpHidden = 64;
// fp32 parameters: W1 [16][64], b1 [64], W2 [64][64] (in x out), b2 [64],
// w3 [64], b3 [1]
constexpr int kMlpParams = kMlpFeatures * kMlpHidden + kMlpHidden + kMlpHidden * kMlpHidden +
                           kMlpHidden + kMlpHidden + 1;

struct MlpWeights {
  const uint16_t* W1T;  // bf16 [64][16] (hidden x feature)
  const uint16_t* W2;   // bf16 [64][64] (in x out)
  const uint16_t* W2T;  // bf16 [64][64] (out x in)
  const float* b1;
  const float* b2;
  const float* w3;
  const float* b3;
};
MlpWeights mlp_weights_view(const float* params, const uint16_t* W1T, const uint16_t* W2,
                            const uint16_t* W2T);

struct FeatureParams {
  const int32_t* pair_tet;
  const int32_t* pair_site;
  const int32_t* pair_index;  // row q describes pair pair_index[q], or null
  long long n_pairs;          // rows
  const float4* site4f;
  const float* vert3f;
  const int4* tets;
  const float4* centroid;     // per tet: centroid, w = radius
  const float* keys;          // n_site x k ascending bisector distances
  int k;
  const int32_t* cell_of;     // site -> grid cell of the kNN grid
  const int32_t* cell_count;  // sites per grid cell
  const float* site_bdist;    // distance to the mesh boundary
  float inv_h;                // 1 / mean site spacing
  uint16_t* X;                // rows x 16 bf16 features
  const int32_t* consumed;    // per pair: certifying list length (labels), or null
  float* target;              // rows: log2(max(consumed, 1)), or null
};

cudaError_t launch_boundary_distance(const float4* site4f, int n_site, const float4* bverts,
                                     int n_bv, float* dist, cudaStream_t st);
cudaError_t launch_pair_features(const FeatureParams& p, cudaStream_t st);
// y (optional) and list lengths klen (optional) of rows idx[0..n) (or 0..n)
cudaError_t launch_mlp_predict(const uint16_t* X, const int32_t* idx, long long n,
                               const MlpWeights& w, float margin, int kmin, int kmax,
                               int32_t* klen, float* y, cudaStream_t st);
// grads += scale * d(sum over rows of (y - target)^2)/dparams; loss_sum +=
// the sum of squares; rows are idx[0..n) (or 0..n)
cudaError_t launch_mlp_grad(const uint16_t* X, const float* target, const int32_t* idx,
                            long long n, float scale, const MlpWeights& w, float* grads,
                            float* loss_sum, cudaStream_t st);
cudaError_t launch_mlp_adam(float* params, float* grads, float* m, float* v, int step, float lr,
                            uint16_t* W1T, uint16_t* W2, uint16_t* W2T, cudaStream_t st);
cudaError_t launch_mlp_sync_operands(const float* params, uint16_t* W1T, uint16_t* W2,
                                     uint16_t* W2T, cudaStream_t st);

}  // namespace rpd
