"""Python host bindings of librpd_gb300.so (ctypes over the C ABI of
include/rpd_gb300.h).

The library is the product; this module only marshals numpy arrays.  It
raises if the library is missing or cannot be loaded -- there is no CPU
fallback anywhere in the package.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "librpd_gb300.so")

PRED_FP64 = 0
PRED_FP32_FILTER = 1
PRED_EXACT = 2
NEIGH_USER = 0
NEIGH_KNN = 1
ORDER_SITE_ID = 0
ORDER_DISTANCE = 1

STATUS_NAMES = ["triangle_overflow", "vertex_overflow", "inconsistent_boundary",
                "security_radius_not_reached", "success", "needs_exact_predicates",
                "no_intersection", "edge_overflow", "needs_perturb", "other"]
SUCCESS = 4
CELL_UNCERTIFIED = 1  # rpd_cell_header.flags: RPD_CELL_UNCERTIFIED

HEADER_DTYPE = np.dtype([
    ("tet_id", "<i4"), ("site_id", "<i4"), ("status", "<i4"),
    ("nb_v", "u1"), ("nb_p", "u1"), ("nb_e", "u1"), ("flags", "u1"),
    ("offset", "<u8"), ("volume", "<f8"),
])

# rpd_topo_header (per-cell topology, rpd_compute_topology), 16 bytes
TOPO_DTYPE = np.dtype([
    ("offset", "<u8"), ("euler", "<f4"), ("n_faces", "u1"), ("flags", "u1"),
    ("pad", "u1", (2,)),
])
TOPO_VERTEX_NULL = 1
TOPO_OPEN_FACE = 2

# every symbol declared in include/rpd_gb300.h
EXPORTS = [
    "rpd_status_string", "rpd_config_default", "rpd_payload_bytes", "rpd_create",
    "rpd_destroy", "rpd_last_error", "rpd_set_mesh", "rpd_set_sites", "rpd_set_neighbors",
    "rpd_compute", "rpd_get_cells", "rpd_copy_cells_to_host", "rpd_copy_cells_to_host_async",
    "rpd_synchronize", "rpd_copy_neighbors_to_host",
    "rpd_copy_pairs_to_host", "rpd_copy_pair_headers_to_host", "rpd_build_mesh_adjacency",
    "rpd_copy_site_lists_to_host",
    "rpd_host_alloc", "rpd_host_free", "rpd_compact_cells_noalloc", "rpd_set_site_k",
    "rpd_copy_topology_hashes_to_host", "rpd_autotune",
    "rpd_mlp_collect", "rpd_mlp_clear_samples", "rpd_mlp_train", "rpd_mlp_enable",
    "rpd_mlp_get_params", "rpd_mlp_set_params", "rpd_mlp_forward", "rpd_mlp_gradient",
    "rpd_mlp_copy_features", "rpd_mlp_copy_klen", "rpd_mlp_copy_samples", "rpd_set_pair_k",
    "rpd_get_config", "rpd_set_config", "rpd_get_mesh_info",
    "rpd_topo_bytes", "rpd_compute_topology", "rpd_get_topology", "rpd_copy_topology_to_host",
    "rpd_compute_polygons", "rpd_get_polygons", "rpd_copy_polygons_to_host", "rpd_dist2mat",
    "rpd_compute_partial", "rpd_compute_power_cells", "rpd_get_power_cells",
    "rpd_set_feature_edges", "rpd_copy_device_to_host", "rpd_set_polygon_slice",
    "rpd_write_polygons_bgeo", "rpd_set_surface_mesh",
    "rpd_batch_create", "rpd_batch_destroy", "rpd_batch_last_error", "rpd_batch_add_mesh",
    "rpd_batch_size", "rpd_batch_set_graph", "rpd_batch_compute", "rpd_batch_autotune",
    "rpd_batch_mesh_cells", "rpd_batch_copy_mesh_cells", "rpd_batch_context",
]

MLP_FEATURES = 16
MLP_PARAMS = 5313


class Config(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("predicate_mode", ctypes.c_int),
                ("neighbor_source", ctypes.c_int), ("knn_k", ctypes.c_int),
                ("clip_order", ctypes.c_int), ("compute_geometry", ctypes.c_int),
                ("warps_per_block", ctypes.c_int), ("blocks_per_sm", ctypes.c_int),
                ("certify", ctypes.c_int), ("clip_variant", ctypes.c_int),
                ("learned_k", ctypes.c_int), ("box_planes", ctypes.c_int),
                ("topology_hash", ctypes.c_int), ("exact_lists", ctypes.c_int),
                ("reserved", ctypes.c_int * 2)]


class MeshInfo(ctypes.Structure):
    _fields_ = [("n_vert", ctypes.c_int32), ("n_tet", ctypes.c_int32),
                ("lo", ctypes.c_double * 3), ("hi", ctypes.c_double * 3),
                ("volume", ctypes.c_double), ("tet_radius", ctypes.c_double),
                ("class_count", ctypes.c_int32 * 2), ("class_radius", ctypes.c_double * 2)]


class PowerCellsView(ctypes.Structure):
    _fields_ = [("n_site", ctypes.c_int32), ("n_cells", ctypes.c_int64)] + [
        (f, ctypes.c_void_p) for f in ("site_cell_off", "site_cells", "cell_nbr_off", "cell_nbrs",
                                       "cell_tfid_off", "cell_tfids")] + [
        ("n_facets", ctypes.c_int64)] + [
        (f, ctypes.c_void_p) for f in ("site_facet_off", "facet_keys", "facet_cells")] + [
        ("n_edges", ctypes.c_int64)] + [(f, ctypes.c_void_p) for f in ("site_edge_off", "edges")] + [
        ("n_vertices", ctypes.c_int64)] + [
        (f, ctypes.c_void_p) for f in ("cell_vertex_off", "vertex_cell", "vertex_lvid", "vertex_ids",
                                       "vertex_pos", "vertex_sfid")] + [
        ("n_surface", ctypes.c_int64)] + [
        (f, ctypes.c_void_p) for f in ("cell_surface_off", "surface_cell", "surface_fid",
                                       "surface_pos")] + [
        ("n_se_covered", ctypes.c_int64)] + [
        (f, ctypes.c_void_p) for f in ("cell_se_covered_off", "se_covered")] + [
        ("n_ce_covered", ctypes.c_int64)] + [
        (f, ctypes.c_void_p) for f in ("cell_ce_covered_off", "ce_covered")] + [
        ("n_se_line_end", ctypes.c_int64)] + [
        (f, ctypes.c_void_p) for f in ("cell_se_line_end_off", "se_line_end", "se_line_end_pos",
                                       "cell_cc", "facet_cc", "edge_cc")] + [
        ("n_sfg", ctypes.c_int64)] + [
        (f, ctypes.c_void_p) for f in ("site_sfg_off", "sfg_group", "sfg_fid", "sfg_record")]


class Stats(ctypes.Structure):
    _fields_ = [("n_pairs", ctypes.c_int64), ("n_cells", ctypes.c_int64),
                ("status_counts", ctypes.c_int64 * 10), ("n_predicates", ctypes.c_int64),
                ("n_escalated", ctypes.c_int64), ("payload_bytes", ctypes.c_int64),
                ("tet_k", ctypes.c_int32), ("knn_k", ctypes.c_int32),
                ("ms_total", ctypes.c_float), ("ms_knn", ctypes.c_float),
                ("ms_pairs", ctypes.c_float), ("ms_clip", ctypes.c_float),
                ("ms_compact", ctypes.c_float), ("ms_clip_kernel", ctypes.c_float),
                ("n_launches", ctypes.c_int32), ("search", ctypes.c_int64 * 6),
                ("n_reclipped", ctypes.c_int64), ("ms_predict", ctypes.c_float),
                ("learned", ctypes.c_int32), ("n_fp64_uncertain", ctypes.c_int64),
                ("n_exact_flips", ctypes.c_int64), ("ms_epilogue", ctypes.c_float),
                ("n_uncertified", ctypes.c_int64), ("n_extended_sites", ctypes.c_int64),
                ("n_cert_reclipped", ctypes.c_int64), ("ms_extend", ctypes.c_float),
                ("n_extend_rounds", ctypes.c_int32), ("ext_longest", ctypes.c_int32),
                ("ms_extend_lists", ctypes.c_float)]

    def as_dict(self):
        d = {f: getattr(self, f) for f, _ in self._fields_ if f not in ("status_counts", "search")}
        d["search"] = [int(x) for x in self.search]
        d["status_counts"] = {STATUS_NAMES[i]: int(self.status_counts[i]) for i in range(10)}
        return d


class Tuning(ctypes.Structure):
    _fields_ = [("warps_per_block", ctypes.c_int), ("clip_variant", ctypes.c_int),
                ("k_bucket", ctypes.c_int), ("n_candidates", ctypes.c_int),
                ("ms_clip_best", ctypes.c_float), ("ms_clip_first", ctypes.c_float),
                ("learned_k", ctypes.c_int), ("knn_k", ctypes.c_int),
                ("ms_total_best", ctypes.c_float)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class MlpReport(ctypes.Structure):
    _fields_ = [("n_train", ctypes.c_int64), ("n_calib", ctypes.c_int64),
                ("loss_first", ctypes.c_float), ("loss_last", ctypes.c_float),
                ("calib_loss", ctypes.c_float), ("margin", ctypes.c_float),
                ("calib_miss_rate", ctypes.c_float), ("calib_mean_k", ctypes.c_float),
                ("const_k", ctypes.c_float), ("ms_train", ctypes.c_float),
                ("steps", ctypes.c_int32), ("epochs", ctypes.c_int32),
                ("label_var", ctypes.c_float)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class CellsView(ctypes.Structure):
    _fields_ = [("n_cells", ctypes.c_int64), ("headers", ctypes.c_void_p),
                ("payload", ctypes.c_void_p), ("payload_bytes", ctypes.c_int64),
                ("n_pairs", ctypes.c_int64), ("pair_headers", ctypes.c_void_p)]


_lib = None


def load(path=LIB_PATH):
    """Loads librpd_gb300.so; raises if it was not built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError("librpd_gb300.so not built (run __graft_entry__.build())")
    L = ctypes.CDLL(path)
    vp, i32, i64, c = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes
    L.rpd_status_string.restype = c.c_char_p
    L.rpd_status_string.argtypes = [i32]
    L.rpd_config_default.restype = None
    L.rpd_config_default.argtypes = [c.POINTER(Config)]
    L.rpd_payload_bytes.restype = c.c_size_t
    L.rpd_payload_bytes.argtypes = [i32, i32, i32]
    L.rpd_create.restype = i32
    L.rpd_create.argtypes = [c.POINTER(Config), c.POINTER(vp)]
    L.rpd_destroy.restype = None
    L.rpd_destroy.argtypes = [vp]
    L.rpd_last_error.restype = c.c_char_p
    L.rpd_last_error.argtypes = [vp]
    L.rpd_set_mesh.restype = i32
    L.rpd_set_mesh.argtypes = [vp, vp, i32, vp, i32, vp, vp, vp, vp]
    L.rpd_set_sites.restype = i32
    L.rpd_set_sites.argtypes = [vp, vp, i32, vp]
    L.rpd_set_neighbors.restype = i32
    L.rpd_set_neighbors.argtypes = [vp, vp, i32, i32]
    L.rpd_compute.restype = i32
    L.rpd_compute.argtypes = [vp, c.POINTER(Stats)]
    L.rpd_get_cells.restype = i32
    L.rpd_get_cells.argtypes = [vp, c.POINTER(CellsView)]
    L.rpd_copy_cells_to_host.restype = i32
    L.rpd_copy_cells_to_host.argtypes = [vp, vp, i64, vp, i64, c.POINTER(i64), c.POINTER(i64)]
    L.rpd_copy_cells_to_host_async.restype = i32
    L.rpd_copy_cells_to_host_async.argtypes = [vp, vp, i64, vp, i64, c.POINTER(i64),
                                               c.POINTER(i64)]
    L.rpd_synchronize.restype = i32
    L.rpd_synchronize.argtypes = [vp]
    L.rpd_copy_neighbors_to_host.restype = i32
    L.rpd_copy_neighbors_to_host.argtypes = [vp, vp, i64, c.POINTER(i32)]
    L.rpd_copy_site_lists_to_host.restype = i32
    L.rpd_copy_site_lists_to_host.argtypes = [vp, vp, vp, i64, c.POINTER(i64)]
    L.rpd_copy_pairs_to_host.restype = i32
    L.rpd_copy_pairs_to_host.argtypes = [vp, vp, vp, i64, c.POINTER(i64)]
    L.rpd_copy_pair_headers_to_host.restype = i32
    L.rpd_copy_pair_headers_to_host.argtypes = [vp, vp, i64, c.POINTER(i64)]
    L.rpd_compact_cells_noalloc.restype = i32
    L.rpd_compact_cells_noalloc.argtypes = [vp, i64, vp, vp, vp, vp]
    L.rpd_autotune.restype = i32
    L.rpd_autotune.argtypes = [vp, i32, c.POINTER(Tuning)]
    L.rpd_set_site_k.restype = i32
    L.rpd_set_site_k.argtypes = [vp, vp, i32]
    L.rpd_copy_topology_hashes_to_host.restype = i32
    L.rpd_copy_topology_hashes_to_host.argtypes = [vp, vp, i64, c.POINTER(i64)]
    L.rpd_mlp_collect.restype = i32
    L.rpd_mlp_collect.argtypes = [vp, i64, c.POINTER(i64)]
    L.rpd_mlp_clear_samples.restype = i32
    L.rpd_mlp_clear_samples.argtypes = [vp]
    L.rpd_mlp_train.restype = i32
    L.rpd_mlp_train.argtypes = [vp, i32, i32, c.c_float, c.c_float, c.c_uint64,
                                c.POINTER(MlpReport)]
    L.rpd_mlp_enable.restype = i32
    L.rpd_mlp_enable.argtypes = [vp, i32]
    L.rpd_mlp_get_params.restype = i32
    L.rpd_mlp_get_params.argtypes = [vp, vp, i32, c.POINTER(c.c_float)]
    L.rpd_mlp_set_params.restype = i32
    L.rpd_mlp_set_params.argtypes = [vp, vp, i32, c.c_float]
    L.rpd_mlp_forward.restype = i32
    L.rpd_mlp_forward.argtypes = [vp, vp, i64, vp]
    L.rpd_mlp_gradient.restype = i32
    L.rpd_mlp_gradient.argtypes = [vp, vp, vp, i64, vp, c.POINTER(c.c_float)]
    L.rpd_mlp_copy_features.restype = i32
    L.rpd_mlp_copy_features.argtypes = [vp, vp, i64, c.POINTER(i64)]
    L.rpd_get_config.restype = i32
    L.rpd_get_config.argtypes = [vp, c.POINTER(Config)]
    L.rpd_set_config.restype = i32
    L.rpd_set_config.argtypes = [vp, c.POINTER(Config)]
    L.rpd_get_mesh_info.restype = i32
    L.rpd_get_mesh_info.argtypes = [vp, c.POINTER(MeshInfo)]
    L.rpd_topo_bytes.restype = c.c_size_t
    L.rpd_topo_bytes.argtypes = [i32, i32, i32]
    L.rpd_compute_topology.restype = i32
    L.rpd_compute_topology.argtypes = [vp, c.POINTER(c.c_float)]
    L.rpd_get_topology.restype = i32
    L.rpd_get_topology.argtypes = [vp, vp]
    L.rpd_copy_topology_to_host.restype = i32
    L.rpd_copy_topology_to_host.argtypes = [vp, vp, i64, vp, i64, c.POINTER(i64), c.POINTER(i64)]
    L.rpd_compute_power_cells.restype = i32
    L.rpd_compute_power_cells.argtypes = [vp, i32, c.POINTER(c.c_float)]
    L.rpd_get_power_cells.restype = i32
    L.rpd_get_power_cells.argtypes = [vp, c.POINTER(PowerCellsView)]
    L.rpd_set_feature_edges.restype = i32
    L.rpd_set_feature_edges.argtypes = [vp, vp, i64]
    L.rpd_set_surface_mesh.restype = i32
    L.rpd_set_surface_mesh.argtypes = [vp, vp, i32, vp, i64]
    L.rpd_set_polygon_slice.restype = i32
    L.rpd_set_polygon_slice.argtypes = [vp, i32, vp, vp]
    L.rpd_write_polygons_bgeo.restype = i32
    L.rpd_write_polygons_bgeo.argtypes = [vp, c.c_char_p, c.POINTER(i64)]
    L.rpd_copy_device_to_host.restype = i32
    L.rpd_copy_device_to_host.argtypes = [vp, vp, vp, i64]
    L.rpd_compute_partial.restype = i32
    L.rpd_compute_partial.argtypes = [vp, vp, c.POINTER(Stats)]
    L.rpd_dist2mat.restype = i32
    L.rpd_dist2mat.argtypes = [vp, vp, i32, vp, i32, vp, vp, vp, i64, vp, vp, i32]
    L.rpd_compute_polygons.restype = i32
    L.rpd_compute_polygons.argtypes = [vp, i32, i32, i32, c.POINTER(c.c_float)]
    L.rpd_get_polygons.restype = i32
    L.rpd_get_polygons.argtypes = [vp, vp]
    L.rpd_copy_polygons_to_host.restype = i32
    L.rpd_copy_polygons_to_host.argtypes = [vp, vp, i64, vp, vp, i64, vp, vp, i64,
                                            c.POINTER(i64), c.POINTER(i64), c.POINTER(i64)]
    L.rpd_batch_create.restype = i32
    L.rpd_batch_create.argtypes = [c.POINTER(Config), c.POINTER(vp)]
    L.rpd_batch_destroy.restype = None
    L.rpd_batch_destroy.argtypes = [vp]
    L.rpd_batch_last_error.restype = c.c_char_p
    L.rpd_batch_last_error.argtypes = [vp]
    L.rpd_batch_add_mesh.restype = i32
    L.rpd_batch_add_mesh.argtypes = [vp, vp, i32, vp, i32, vp, vp, vp, vp, vp, i32, vp,
                                     c.POINTER(i32)]
    L.rpd_batch_size.restype = i32
    L.rpd_batch_size.argtypes = [vp]
    L.rpd_batch_set_graph.restype = i32
    L.rpd_batch_set_graph.argtypes = [vp, i32]
    L.rpd_batch_compute.restype = i32
    L.rpd_batch_compute.argtypes = [vp, c.POINTER(Stats)]
    L.rpd_batch_autotune.restype = i32
    L.rpd_batch_autotune.argtypes = [vp, i32, c.POINTER(Tuning)]
    L.rpd_batch_mesh_cells.restype = i32
    L.rpd_batch_mesh_cells.argtypes = [vp, i32, c.POINTER(i64), c.POINTER(i64)]
    L.rpd_batch_copy_mesh_cells.restype = i32
    L.rpd_batch_copy_mesh_cells.argtypes = [vp, i32, vp, i64, vp, i64, c.POINTER(i64),
                                            c.POINTER(i64)]
    L.rpd_batch_context.restype = vp
    L.rpd_batch_context.argtypes = [vp]
    L.rpd_set_pair_k.restype = i32
    L.rpd_set_pair_k.argtypes = [vp, vp, i64]
    L.rpd_mlp_copy_samples.restype = i32
    L.rpd_mlp_copy_samples.argtypes = [vp, vp, vp, i64, c.POINTER(i64)]
    L.rpd_mlp_copy_klen.restype = i32
    L.rpd_mlp_copy_klen.argtypes = [vp, vp, i64, c.POINTER(i64)]
    L.rpd_host_alloc.restype = vp
    L.rpd_host_alloc.argtypes = [c.c_size_t]
    L.rpd_host_free.restype = None
    L.rpd_host_free.argtypes = [vp]
    L.rpd_build_mesh_adjacency.restype = i32
    L.rpd_build_mesh_adjacency.argtypes = [i32, vp, i32, vp, vp, vp, vp, vp]
    _lib = L
    return L


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


class RPDError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s: %s" % (status, msg))
        self.status = status


def mesh_adjacency(n_vert, tets):
    """v_adjs, e_adj6, f_adjs, f_ids, n_boundary_faces (load_tet_adj_info)."""
    L = load()
    tets = np.ascontiguousarray(tets, np.int32)
    n_tet = tets.shape[0]
    v = np.zeros(n_vert, np.int32)
    e6 = np.zeros((n_tet, 6), np.uint8)
    fa = np.zeros((n_tet, 4), np.int32)
    fi = np.zeros((n_tet, 4), np.int32)
    nb = np.zeros(1, np.int32)
    s = L.rpd_build_mesh_adjacency(n_vert, _p(tets), n_tet, _p(v), _p(e6), _p(fa), _p(fi), _p(nb))
    if s != 0:
        raise RPDError(s, "rpd_build_mesh_adjacency failed")
    return dict(v_adjs=v, e_adj6=e6, f_adjs=fa, f_ids=fi, n_boundary_faces=int(nb[0]))


def payload_bytes(nb_v, nb_p, nb_e):
    return int(load().rpd_payload_bytes(int(nb_v), int(nb_p), int(nb_e)))


class RPD:
    """One engine context (one GPU, one stream)."""

    def __init__(self, device=0, predicate_mode=PRED_FP32_FILTER, neighbor_source=NEIGH_KNN,
                 knn_k=64, clip_order=ORDER_SITE_ID, compute_geometry=True,
                 warps_per_block=0, blocks_per_sm=0, certify=False, clip_variant=0,
                 learned_k=False, box_planes=0, topology_hash=True, exact_lists=True):
        L = load()
        cfg = Config()
        L.rpd_config_default(ctypes.byref(cfg))
        cfg.device = device
        cfg.predicate_mode = predicate_mode
        cfg.neighbor_source = neighbor_source
        cfg.knn_k = knn_k
        cfg.clip_order = clip_order
        cfg.compute_geometry = 1 if compute_geometry else 0
        cfg.warps_per_block = warps_per_block
        cfg.blocks_per_sm = blocks_per_sm
        cfg.certify = 1 if certify else 0
        cfg.clip_variant = clip_variant
        cfg.learned_k = 1 if learned_k else 0
        cfg.box_planes = box_planes
        cfg.topology_hash = 1 if topology_hash else 0
        cfg.exact_lists = 1 if exact_lists else 0
        h = ctypes.c_void_p()
        s = L.rpd_create(ctypes.byref(cfg), ctypes.byref(h))
        if s != 0:
            raise RPDError(s, L.rpd_status_string(s).decode())
        self._L = L
        self._h = h
        self._keep = []

    def close(self):
        if self._h:
            self._L.rpd_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, s):
        if s != 0:
            raise RPDError(s, self._L.rpd_last_error(self._h).decode())

    def set_mesh(self, vert3d, tets, v_adjs, e_adj6, f_adjs, f_ids):
        v = np.ascontiguousarray(vert3d, np.float64)
        t = np.ascontiguousarray(tets, np.int32)
        self._check(self._L.rpd_set_mesh(
            self._h, _p(v), v.shape[0], _p(t), t.shape[0],
            _p(np.ascontiguousarray(v_adjs, np.int32)),
            _p(np.ascontiguousarray(e_adj6, np.uint8)),
            _p(np.ascontiguousarray(f_adjs, np.int32)),
            _p(np.ascontiguousarray(f_ids, np.int32))))

    def set_sites(self, xyzw, flags=None):
        s = np.ascontiguousarray(xyzw, np.float64)
        f = None if flags is None else np.ascontiguousarray(flags, np.uint32)
        self._check(self._L.rpd_set_sites(self._h, _p(s), s.shape[0], _p(f)))

    def set_neighbors(self, nbr, layout=0):
        n = np.ascontiguousarray(nbr, np.int32)
        k = n.shape[1] if layout == 0 else n.shape[0] - 1
        self._check(self._L.rpd_set_neighbors(self._h, _p(n), k, layout))

    def set_site_k(self, k_per_site):
        """Per-site list lengths for certified clipping (None clears)."""
        if k_per_site is None:
            self._check(self._L.rpd_set_site_k(self._h, None, 0))
            return
        a = np.ascontiguousarray(k_per_site, np.int32)
        self._check(self._L.rpd_set_site_k(self._h, _p(a), 0))

    def config(self):
        cfg = Config()
        self._check(self._L.rpd_get_config(self._h, ctypes.byref(cfg)))
        return cfg

    def mesh_info(self):
        """What set_mesh derived on the device: dict with lo, hi, volume,
        tet_radius, class_count, class_radius."""
        m = MeshInfo()
        self._check(self._L.rpd_get_mesh_info(self._h, ctypes.byref(m)))
        return dict(n_vert=m.n_vert, n_tet=m.n_tet, lo=list(m.lo), hi=list(m.hi),
                    volume=m.volume, tet_radius=m.tet_radius,
                    class_count=list(m.class_count), class_radius=list(m.class_radius))

    def set_config(self, cfg):
        """Replaces the whole configuration (a Config from config())."""
        self._check(self._L.rpd_set_config(self._h, ctypes.byref(cfg)))

    def configure(self, **fields):
        """Changes configuration fields (e.g. topology_hash=0, clip_variant=2)."""
        cfg = self.config()
        for k, v in fields.items():
            if not hasattr(cfg, k):
                raise KeyError(k)
            setattr(cfg, k, int(v))
        self._check(self._L.rpd_set_config(self._h, ctypes.byref(cfg)))

    def set_pair_k(self, k_per_pair):
        """Per-pair list lengths for the next certified compute (None clears)."""
        if k_per_pair is None:
            self._check(self._L.rpd_set_pair_k(self._h, None, 0))
            return
        a = np.ascontiguousarray(k_per_pair, np.int32)
        self._check(self._L.rpd_set_pair_k(self._h, _p(a), a.shape[0]))

    def autotune(self, repeats=2):
        """Picks the fastest clip launch configuration on the current inputs."""
        t = Tuning()
        self._check(self._L.rpd_autotune(self._h, repeats, ctypes.byref(t)))
        return t

    def topology_hashes(self):
        n = ctypes.c_int64()
        self._check(self._L.rpd_copy_topology_hashes_to_host(self._h, None, 0, ctypes.byref(n)))
        out = np.zeros(n.value, np.uint64)
        self._check(self._L.rpd_copy_topology_hashes_to_host(self._h, _p(out), out.shape[0],
                                                             ctypes.byref(n)))
        return out

    # ---- learned list length
    def mlp_collect(self, max_samples):
        """Appends up to max_samples labelled cells of the current inputs to
        the training set; returns its size."""
        n = ctypes.c_int64()
        self._check(self._L.rpd_mlp_collect(self._h, int(max_samples), ctypes.byref(n)))
        return n.value

    def mlp_clear_samples(self):
        self._check(self._L.rpd_mlp_clear_samples(self._h))

    def mlp_samples(self):
        """The training set: (features (n, 16) bf16 bits, labels)."""
        n = ctypes.c_int64()
        self._check(self._L.rpd_mlp_copy_samples(self._h, None, None, 0, ctypes.byref(n)))
        x = np.zeros((n.value, MLP_FEATURES), np.uint16)
        y = np.zeros(n.value, np.float32)
        self._check(self._L.rpd_mlp_copy_samples(self._h, _p(x), _p(y), n.value, ctypes.byref(n)))
        return x, y

    def mlp_train(self, epochs=20, batch=512, lr=2e-3, miss_target=0.02, seed=0):
        r = MlpReport()
        self._check(self._L.rpd_mlp_train(self._h, epochs, batch, lr, miss_target, seed,
                                          ctypes.byref(r)))
        return r

    def mlp_enable(self, on=True):
        """Per-cell list lengths from the k-predictor (misses re-clipped)."""
        self._check(self._L.rpd_mlp_enable(self._h, 1 if on else 0))

    def mlp_params(self):
        out = np.zeros(MLP_PARAMS, np.float32)
        m = ctypes.c_float()
        self._check(self._L.rpd_mlp_get_params(self._h, _p(out), MLP_PARAMS, ctypes.byref(m)))
        return out, m.value

    def mlp_set_params(self, params, margin=0.0):
        a = np.ascontiguousarray(params, np.float32)
        self._check(self._L.rpd_mlp_set_params(self._h, _p(a), a.shape[0], margin))

    def mlp_forward(self, x_bf16):
        x = np.ascontiguousarray(x_bf16, np.uint16)
        y = np.zeros(x.shape[0], np.float32)
        self._check(self._L.rpd_mlp_forward(self._h, _p(x), x.shape[0], _p(y)))
        return y

    def mlp_gradient(self, x_bf16, target):
        x = np.ascontiguousarray(x_bf16, np.uint16)
        t = np.ascontiguousarray(target, np.float32)
        g = np.zeros(MLP_PARAMS, np.float32)
        loss = ctypes.c_float()
        self._check(self._L.rpd_mlp_gradient(self._h, _p(x), _p(t), x.shape[0], _p(g),
                                             ctypes.byref(loss)))
        return g, loss.value

    def mlp_features(self):
        n = ctypes.c_int64()
        self._check(self._L.rpd_mlp_copy_features(self._h, None, 0, ctypes.byref(n)))
        out = np.zeros((n.value, MLP_FEATURES), np.uint16)
        self._check(self._L.rpd_mlp_copy_features(self._h, _p(out), n.value, ctypes.byref(n)))
        return out

    def mlp_klen(self):
        n = ctypes.c_int64()
        self._check(self._L.rpd_mlp_copy_klen(self._h, None, 0, ctypes.byref(n)))
        out = np.zeros(n.value, np.int32)
        self._check(self._L.rpd_mlp_copy_klen(self._h, _p(out), n.value, ctypes.byref(n)))
        return out

    def compute(self):
        st = Stats()
        self._check(self._L.rpd_compute(self._h, ctypes.byref(st)))
        return st

    def view(self):
        v = CellsView()
        self._check(self._L.rpd_get_cells(self._h, ctypes.byref(v)))
        return v

    def cells(self, headers_out=None, payload_out=None):
        """Emitted cells copied to the host: (headers, payload)."""
        n = ctypes.c_int64()
        b = ctypes.c_int64()
        self._check(self._L.rpd_copy_cells_to_host(self._h, None, 0, None, 0,
                                                   ctypes.byref(n), ctypes.byref(b)))
        h = headers_out if headers_out is not None else np.zeros(n.value, HEADER_DTYPE)
        p = payload_out if payload_out is not None else np.zeros(max(b.value, 1), np.uint8)
        self._check(self._L.rpd_copy_cells_to_host(self._h, _p(h), h.shape[0], _p(p), p.nbytes,
                                                   ctypes.byref(n), ctypes.byref(b)))
        return h[:n.value], p[:b.value]

    def cells_async(self, headers_out, payload_out):
        """Queues the copy of the emitted cells into page-locked arrays
        (PinnedArray) and returns their (headers, payload) views at once;
        they hold the cells after synchronize()."""
        n = ctypes.c_int64()
        b = ctypes.c_int64()
        self._check(self._L.rpd_copy_cells_to_host_async(
            self._h, _p(headers_out), headers_out.shape[0], _p(payload_out), payload_out.nbytes,
            ctypes.byref(n), ctypes.byref(b)))
        return headers_out[:n.value], payload_out[:b.value]

    def synchronize(self):
        self._check(self._L.rpd_synchronize(self._h))

    def compute_topology(self):
        """Per-cell topology of the emitted cells on the device (active
        planes and edges, face cycles, Euler numbers); returns its device
        time in ms."""
        ms = ctypes.c_float()
        self._check(self._L.rpd_compute_topology(self._h, ctypes.byref(ms)))
        return ms.value

    def topology(self):
        """The per-cell topology copied to the host: (TOPO_DTYPE headers,
        record bytes), one header per emitted cell in cells() order."""
        n = ctypes.c_int64()
        b = ctypes.c_int64()
        self._check(self._L.rpd_copy_topology_to_host(self._h, None, 0, None, 0,
                                                      ctypes.byref(n), ctypes.byref(b)))
        h = np.zeros(max(n.value, 1), TOPO_DTYPE)
        r = np.zeros(max(b.value, 16), np.uint8)
        self._check(self._L.rpd_copy_topology_to_host(self._h, _p(h), h.shape[0], _p(r), r.nbytes,
                                                      ctypes.byref(n), ctypes.byref(b)))
        return h[:n.value], r[:b.value]

    def compute_power_cells(self, max_sf_fid=-1):
        """The power cells of the emitted cells on the device (libmat's
        get_all_voro_info); returns the device time in ms."""
        ms = ctypes.c_float()
        self._check(self._L.rpd_compute_power_cells(self._h, int(max_sf_fid), ctypes.byref(ms)))
        return ms.value

    def set_feature_edges(self, records):
        """libmat's TetMesh::tet_es2fe_map as (m, 6) int records (tet, lf_min,
        lf_max, fe_type, fe_id, fe_line_id), in insertion order; None or an
        empty array clears it."""
        r = np.ascontiguousarray(np.zeros((0, 6)) if records is None else records,
                                 np.int32).reshape(-1, 6)
        self._check(self._L.rpd_set_feature_edges(self._h, _p(r), r.shape[0]))

    def set_surface_mesh(self, facet_adj, no_cross=None):
        """libmat's SurfaceMesh for the surface groups: (n_faces, 3) face
        adjacency (-1 for none) and (m, 2) no-cross face pairs; None clears."""
        a = np.ascontiguousarray(np.zeros((0, 3)) if facet_adj is None else facet_adj, np.int32)
        b = np.ascontiguousarray(np.zeros((0, 2)) if no_cross is None else no_cross, np.int32)
        self._check(self._L.rpd_set_surface_mesh(self._h, _p(a), a.reshape(-1, 3).shape[0], _p(b),
                                                 b.reshape(-1, 2).shape[0]))

    def _d2h(self, ptr, dtype, count):
        out = np.zeros(max(int(count), 1), dtype)
        if count > 0:
            self._check(self._L.rpd_copy_device_to_host(self._h, _p(out), ptr, out.nbytes))
        return out[:int(count)]

    def power_cells(self):
        """The power cells copied to the host: dict of numpy arrays named as
        the fields of rpd_power_cells_view."""
        v = PowerCellsView()
        self._check(self._L.rpd_get_power_cells(self._h, ctypes.byref(v)))
        ns, n = v.n_site, v.n_cells
        d = {}
        d["site_cell_off"] = self._d2h(v.site_cell_off, np.int64, ns + 1)
        d["site_cells"] = self._d2h(v.site_cells, np.uint32, n)
        d["cell_nbr_off"] = self._d2h(v.cell_nbr_off, np.int64, n + 1)
        d["cell_nbrs"] = self._d2h(v.cell_nbrs, np.int32, d["cell_nbr_off"][-1])
        d["cell_tfid_off"] = self._d2h(v.cell_tfid_off, np.int64, n + 1)
        d["cell_tfids"] = self._d2h(v.cell_tfids, np.int32, d["cell_tfid_off"][-1])
        d["site_facet_off"] = self._d2h(v.site_facet_off, np.int64, ns + 1)
        d["facet_keys"] = self._d2h(v.facet_keys, np.uint64, v.n_facets)
        d["facet_cells"] = self._d2h(v.facet_cells, np.uint32, v.n_facets)
        d["site_edge_off"] = self._d2h(v.site_edge_off, np.int64, ns + 1)
        d["edges"] = self._d2h(v.edges, np.int32, 7 * v.n_edges).reshape(-1, 7)
        d["cell_vertex_off"] = self._d2h(v.cell_vertex_off, np.int64, n + 1)
        d["vertex_cell"] = self._d2h(v.vertex_cell, np.int32, v.n_vertices)
        d["vertex_lvid"] = self._d2h(v.vertex_lvid, np.int32, v.n_vertices)
        d["vertex_ids"] = self._d2h(v.vertex_ids, np.int32, 3 * v.n_vertices).reshape(-1, 3)
        d["vertex_pos"] = self._d2h(v.vertex_pos, np.float32, 3 * v.n_vertices).reshape(-1, 3)
        d["vertex_sfid"] = self._d2h(v.vertex_sfid, np.int32, v.n_vertices)
        d["cell_surface_off"] = self._d2h(v.cell_surface_off, np.int64, n + 1)
        d["surface_cell"] = self._d2h(v.surface_cell, np.int32, v.n_surface)
        d["surface_fid"] = self._d2h(v.surface_fid, np.int32, v.n_surface)
        d["surface_pos"] = self._d2h(v.surface_pos, np.float32, 3 * v.n_surface).reshape(-1, 3)
        for name in ("se_covered", "ce_covered"):
            m = getattr(v, "n_" + name)
            d["cell_%s_off" % name] = self._d2h(getattr(v, "cell_%s_off" % name), np.int64, n + 1)
            d[name] = self._d2h(getattr(v, name), np.int32, 5 * m).reshape(-1, 5)
        m = v.n_se_line_end
        d["cell_se_line_end_off"] = self._d2h(v.cell_se_line_end_off, np.int64, n + 1)
        d["se_line_end"] = self._d2h(v.se_line_end, np.int32, 4 * m).reshape(-1, 4)
        d["se_line_end_pos"] = self._d2h(v.se_line_end_pos, np.float32, 3 * m).reshape(-1, 3)
        d["cell_cc"] = self._d2h(v.cell_cc, np.int32, n)
        d["facet_cc"] = self._d2h(v.facet_cc, np.int32, v.n_facets)
        d["edge_cc"] = self._d2h(v.edge_cc, np.int32, v.n_edges)
        d["site_sfg_off"] = self._d2h(v.site_sfg_off, np.int64, ns + 1)
        for f in ("sfg_group", "sfg_fid", "sfg_record"):
            d[f] = self._d2h(getattr(v, f), np.int32, v.n_sfg)
        return d

    def compute_partial(self, recompute):
        """Recomputes the cells of the sites with recompute[i] != 0 and
        merges them with the previous cells (libmat's calculate_partial);
        returns the partial compute's stats."""
        fl = np.ascontiguousarray(np.asarray(recompute) != 0, np.uint32)
        st = Stats()
        self._check(self._L.rpd_compute_partial(self._h, _p(fl), ctypes.byref(st)))
        return st

    def dist2mat(self, spheres, samples, offsets, counts, prims):
        """libmat's dist2mat on the device: per sample, the smallest signed
        distance to its medial primitives and the closest one's index in its
        list.  spheres (n, 4) float32 (x, y, z, r); samples (m, 3); offsets,
        counts (m,) uint32; prims (k, 3) int32.  Returns (dist, closest)."""
        sph = np.ascontiguousarray(spheres, np.float32)
        smp = np.ascontiguousarray(samples, np.float32)
        off = np.ascontiguousarray(offsets, np.uint32)
        cnt = np.ascontiguousarray(counts, np.uint32)
        prm = np.ascontiguousarray(prims, np.int32)
        m = smp.shape[0]
        dist = np.zeros(m, np.float32)
        closest = np.zeros(m, np.int32)
        self._check(self._L.rpd_dist2mat(self._h, _p(sph), sph.shape[0], _p(smp), m, _p(off),
                                         _p(cnt), _p(prm), prm.shape[0], _p(dist), _p(closest), 0))
        return dist, closest

    def compute_polygons(self, triangulate=False, boundary_only=False, max_sf_fid=0):
        """Polygon soup of the emitted cells on the device (libmat's Houdini
        export); returns its device time in ms."""
        ms = ctypes.c_float()
        self._check(self._L.rpd_compute_polygons(self._h, int(triangulate), int(boundary_only),
                                                 int(max_sf_fid), ctypes.byref(ms)))
        return ms.value

    def set_polygon_slice(self, pos=None, normal=None):
        """Slicing plane of the following compute_polygons calls (libmat's
        is_slice_by_plane, as save_convex_cells_houdini applies it); None
        turns it off."""
        if pos is None:
            self._check(self._L.rpd_set_polygon_slice(self._h, 0, None, None))
            return
        a = np.ascontiguousarray(pos, np.float64)
        b = np.ascontiguousarray(normal, np.float64)
        self._check(self._L.rpd_set_polygon_slice(self._h, 1, _p(a), _p(b)))

    def write_polygons_bgeo(self, path):
        """Writes the last polygon soup as a Houdini binary geometry file
        (libmat's save_convex_cells_houdini format); returns its size."""
        n = ctypes.c_int64()
        self._check(self._L.rpd_write_polygons_bgeo(self._h, str(path).encode(), ctypes.byref(n)))
        return n.value

    def polygons(self):
        """The polygon soup copied to the host: dict(points (n, 3) float32,
        poly_offsets, indices, poly_site, poly_adj_site)."""
        a, b, d = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        self._check(self._L.rpd_copy_polygons_to_host(self._h, None, 0, None, None, 0, None, None,
                                                      0, ctypes.byref(a), ctypes.byref(b),
                                                      ctypes.byref(d)))
        npt, npoly, nidx = a.value, b.value, d.value
        pts = np.zeros((max(npt, 1), 3), np.float32)
        offs = np.zeros(npoly + 1, np.int64)
        idx = np.zeros(max(nidx, 1), np.uint32)
        site = np.zeros(max(npoly, 1), np.int32)
        adj = np.zeros(max(npoly, 1), np.int32)
        self._check(self._L.rpd_copy_polygons_to_host(
            self._h, _p(pts), npt, _p(offs), _p(idx), nidx, _p(site), _p(adj), npoly,
            ctypes.byref(a), ctypes.byref(b), ctypes.byref(d)))
        return dict(points=pts[:npt], poly_offsets=offs, indices=idx[:nidx],
                    poly_site=site[:npoly], poly_adj_site=adj[:npoly])

    def pair_headers(self):
        """Headers of all candidate pairs (dropped ones included)."""
        n = ctypes.c_int64()
        self._check(self._L.rpd_copy_pair_headers_to_host(self._h, None, 0, ctypes.byref(n)))
        out = np.zeros(n.value, HEADER_DTYPE)
        self._check(self._L.rpd_copy_pair_headers_to_host(self._h, _p(out), out.shape[0],
                                                          ctypes.byref(n)))
        return out

    def neighbors(self):
        k = ctypes.c_int()
        self._check(self._L.rpd_copy_neighbors_to_host(self._h, None, 0, ctypes.byref(k)))
        return k.value

    def neighbor_lists(self, n_site):
        k = self.neighbors()
        out = np.zeros((n_site, k), np.int32)
        kk = ctypes.c_int()
        self._check(self._L.rpd_copy_neighbors_to_host(self._h, _p(out), out.size, ctypes.byref(kk)))
        return out

    def site_lists(self, n_site):
        """Every site's list as the last compute clipped its cells with (CSR:
        offsets [n_site + 1] int64, ids)."""
        n = ctypes.c_int64()
        self._check(self._L.rpd_copy_site_lists_to_host(self._h, None, None, 0, ctypes.byref(n)))
        offs = np.zeros(n_site + 1, np.int64)
        ids = np.zeros(max(n.value, 1), np.int32)
        self._check(self._L.rpd_copy_site_lists_to_host(self._h, _p(offs), _p(ids), ids.size,
                                                        ctypes.byref(n)))
        return offs, ids[:n.value]

    def site_lists_padded(self, n_site):
        """The same lists as an [n_site, longest] matrix, -1 padded (the
        oracle's list layout)."""
        offs, ids = self.site_lists(n_site)
        lens = np.diff(offs)
        k = max(int(lens.max()) if n_site else 1, 1)
        out = np.full((n_site, k), -1, np.int32)
        rows = np.repeat(np.arange(n_site), lens)
        cols = np.arange(ids.size) - np.repeat(offs[:-1], lens)
        out[rows, cols] = ids
        return out

    def pairs(self, n_tet):
        n = ctypes.c_int64()
        self._check(self._L.rpd_copy_pairs_to_host(self._h, None, None, 0, ctypes.byref(n)))
        offs = np.zeros(n_tet + 1, np.int32)
        sites = np.zeros(max(n.value, 1), np.int32)
        self._check(self._L.rpd_copy_pairs_to_host(self._h, _p(offs), _p(sites), sites.size,
                                                   ctypes.byref(n)))
        return offs, sites[:n.value]


class Batch:
    """Many independent meshes clipped together (rpd_batch_*)."""

    def __init__(self, device=0, predicate_mode=PRED_FP32_FILTER, knn_k=64,
                 clip_order=ORDER_SITE_ID, compute_geometry=True, certify=False, clip_variant=0,
                 topology_hash=True, use_graph=True, exact_lists=True):
        L = load()
        cfg = Config()
        L.rpd_config_default(ctypes.byref(cfg))
        cfg.device = device
        cfg.predicate_mode = predicate_mode
        cfg.neighbor_source = NEIGH_KNN
        cfg.knn_k = knn_k
        cfg.clip_order = clip_order
        cfg.compute_geometry = 1 if compute_geometry else 0
        cfg.certify = 1 if certify else 0
        cfg.clip_variant = clip_variant
        cfg.topology_hash = 1 if topology_hash else 0
        cfg.exact_lists = 1 if exact_lists else 0
        h = ctypes.c_void_p()
        s = L.rpd_batch_create(ctypes.byref(cfg), ctypes.byref(h))
        if s != 0:
            raise RPDError(s, L.rpd_status_string(s).decode())
        self._L = L
        self._h = h
        self._L.rpd_batch_set_graph(h, 1 if use_graph else 0)
        self.meshes = []

    def close(self):
        if self._h:
            self._L.rpd_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, s):
        if s != 0:
            raise RPDError(s, self._L.rpd_batch_last_error(self._h).decode())

    def add_mesh(self, vert3d, tets, v_adjs, e_adj6, f_adjs, f_ids, sites, flags=None):
        v = np.ascontiguousarray(vert3d, np.float64)
        t = np.ascontiguousarray(tets, np.int32)
        s = np.ascontiguousarray(sites, np.float64)
        f = None if flags is None else np.ascontiguousarray(flags, np.uint32)
        idx = ctypes.c_int()
        self._check(self._L.rpd_batch_add_mesh(
            self._h, _p(v), v.shape[0], _p(t), t.shape[0],
            _p(np.ascontiguousarray(v_adjs, np.int32)), _p(np.ascontiguousarray(e_adj6, np.uint8)),
            _p(np.ascontiguousarray(f_adjs, np.int32)), _p(np.ascontiguousarray(f_ids, np.int32)),
            _p(s), s.shape[0], _p(f), ctypes.byref(idx)))
        self.meshes.append((t.shape[0], s.shape[0]))
        return idx.value

    def compute(self):
        st = Stats()
        self._check(self._L.rpd_batch_compute(self._h, ctypes.byref(st)))
        return st

    def autotune(self, repeats=1):
        t = Tuning()
        self._check(self._L.rpd_batch_autotune(self._h, repeats, ctypes.byref(t)))
        return t

    def mesh_cells(self, mesh):
        """(headers, payload) of one mesh with its own tet / site ids."""
        n = ctypes.c_int64()
        b = ctypes.c_int64()
        self._check(self._L.rpd_batch_copy_mesh_cells(self._h, mesh, None, 0, None, 0,
                                                      ctypes.byref(n), ctypes.byref(b)))
        h = np.zeros(max(n.value, 1), HEADER_DTYPE)
        p = np.zeros(max(b.value, 1), np.uint8)
        self._check(self._L.rpd_batch_copy_mesh_cells(self._h, mesh, _p(h), h.shape[0], _p(p),
                                                      p.nbytes, ctypes.byref(n), ctypes.byref(b)))
        return h[:n.value], p[:b.value]

    def _ctx(self):
        return ctypes.c_void_p(self._L.rpd_batch_context(self._h))

    def topology_hashes(self):
        """Topology hashes of all pairs of all meshes (batch order)."""
        c = self._ctx()
        n = ctypes.c_int64()
        self._check(self._L.rpd_copy_topology_hashes_to_host(c, None, 0, ctypes.byref(n)))
        out = np.zeros(max(n.value, 1), np.uint64)
        self._check(self._L.rpd_copy_topology_hashes_to_host(c, _p(out), out.shape[0],
                                                             ctypes.byref(n)))
        return out[:n.value]

    def pair_headers(self):
        """Headers of all pairs of all meshes (batch tet / site ids)."""
        c = self._ctx()
        n = ctypes.c_int64()
        self._check(self._L.rpd_copy_pair_headers_to_host(c, None, 0, ctypes.byref(n)))
        out = np.zeros(max(n.value, 1), HEADER_DTYPE)
        self._check(self._L.rpd_copy_pair_headers_to_host(c, _p(out), out.shape[0],
                                                          ctypes.byref(n)))
        return out[:n.value]

    def configure(self, **fields):
        c = self._ctx()
        cfg = Config()
        self._check(self._L.rpd_get_config(c, ctypes.byref(cfg)))
        for k, v in fields.items():
            setattr(cfg, k, int(v))
        self._check(self._L.rpd_set_config(c, ctypes.byref(cfg)))

    def mesh_range(self, mesh):
        f = ctypes.c_int64()
        n = ctypes.c_int64()
        self._check(self._L.rpd_batch_mesh_cells(self._h, mesh, ctypes.byref(f), ctypes.byref(n)))
        return f.value, n.value


class PinnedArray:
    """A numpy array in page-locked host memory (rpd_host_alloc)."""

    def __init__(self, shape, dtype):
        self._L = load()
        dt = np.dtype(dtype)
        n = int(np.prod(shape)) * dt.itemsize
        self._ptr = self._L.rpd_host_alloc(max(n, 1))
        if not self._ptr:
            raise MemoryError("rpd_host_alloc(%d) failed" % n)
        buf = (ctypes.c_uint8 * max(n, 1)).from_address(self._ptr)
        self.array = np.frombuffer(buf, dtype=dt, count=int(np.prod(shape))).reshape(shape)

    def free(self):
        if self._ptr:
            self.array = None
            self._L.rpd_host_free(self._ptr)
            self._ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass
