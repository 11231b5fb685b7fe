"""ctypes bindings of the oracle (test infrastructure only).

Only tests/, the smoke check and bench.py's CPU-baseline leg import this
module.  It wraps liboracle.so (the CPU restatement of libmat's RPD path) and,
where the reference sources were present at build time, _ref/libref.so (the
reference's own clipping kernel compiled for the CPU).
"""
import ctypes
import os

import numpy as np

from . import build as _build

HERE = os.path.dirname(os.path.abspath(__file__))

HEADER_DTYPE = np.dtype([
    ("tet_id", "<i4"), ("site_id", "<i4"), ("status", "<i4"),
    ("nb_v", "u1"), ("nb_p", "u1"), ("nb_e", "u1"), ("flags", "u1"),
    ("offset", "<u8"), ("volume", "<f8"),
])
assert HEADER_DTYPE.itemsize == 32

SUCCESS = 4

# per-cell topology header (orc_topo_header / rpd_topo_header), 16 bytes
TOPO_DTYPE = np.dtype([
    ("offset", "<u8"), ("euler", "<f4"), ("n_faces", "u1"), ("flags", "u1"),
    ("pad", "u1", (2,)),
])
assert TOPO_DTYPE.itemsize == 16

_lib = None
_ref = None
_reftopo = None


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def lib():
    global _lib
    if _lib is None:
        path = _build.build_oracle()
        L = ctypes.CDLL(path)
        vp, i32, i64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64
        L.orc_payload_bytes.restype = ctypes.c_size_t
        L.orc_payload_bytes.argtypes = [i32, i32, i32]
        L.orc_mesh_adjacency.restype = i32
        L.orc_mesh_adjacency.argtypes = [i32, i32, vp, vp, vp, vp, vp, vp]
        L.orc_dense_e_adjs_size.restype = i64
        L.orc_dense_e_adjs_size.argtypes = [i32]
        L.orc_dense_e_adjs.restype = None
        L.orc_dense_e_adjs.argtypes = [i32, i32, vp, vp, vp]
        L.orc_knn.restype = None
        L.orc_knn.argtypes = [i32, vp, i32, vp, vp, i32]
        L.orc_candidate_pairs.restype = i64
        L.orc_candidate_pairs.argtypes = [i32, vp, i32, vp, i32, vp, vp, vp,
                                          i32, vp, vp, i64, i32]
        L.orc_clip_cells.restype = i64
        L.orc_clip_cells.argtypes = [i32, vp, vp, i32, vp, vp, vp, vp, vp, i32,
                                     vp, vp, vp, i32, vp, vp, i32, vp, vp, i64,
                                     vp, i32]
        L.orc_det4x4_ref.restype = ctypes.c_double
        L.orc_det4x4_ref.argtypes = [vp, vp, vp, vp]
        L.orc_filter_sign.restype = i32
        L.orc_filter_sign.argtypes = [vp, vp, vp, vp]
        L.orc_det4x4_bound.restype = ctypes.c_double
        L.orc_det4x4_bound.argtypes = [vp, vp, vp, vp, vp]
        L.orc_det4x4_exact_sign.restype = i32
        L.orc_det4x4_exact_sign.argtypes = [vp, vp, vp, vp]
        L.orc_bisector_key.restype = ctypes.c_float
        L.orc_bisector_key.argtypes = [vp, vp]
        L.orc_topo_bytes.restype = ctypes.c_size_t
        L.orc_topo_bytes.argtypes = [i32, i32, i32]
        L.orc_cell_topology.restype = i64
        L.orc_cell_topology.argtypes = [i64, vp, vp, vp, vp, i64]
        L.orc_topology_hashes.restype = None
        L.orc_topology_hashes.argtypes = [i64, vp, vp, vp]
        L.orc_power_neighbors.restype = i32
        L.orc_power_neighbors.argtypes = [i32, vp, vp, i32, vp, vp, i32]
        L.orc_cell_polygons.restype = i32
        L.orc_cell_polygons.argtypes = [i64, vp, vp, i32, i32, i32, vp, vp, i64, vp, vp, i64,
                                        vp, vp, i64, vp]
        _lib = L
    return _lib


def ref_lib():
    """The reference's own clipper on the CPU, or None when unavailable."""
    global _ref
    if _ref is None:
        path = _build.build_ref()
        if path is None:
            return None
        L = ctypes.CDLL(path)
        vp, i32, i64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64
        L.ref_clip_cells.restype = i64
        L.ref_clip_cells.argtypes = [i32, vp, i32, vp, vp, vp, vp, vp, i32, vp,
                                     vp, vp, vp, i32, vp, i32, vp, vp, vp, i64,
                                     i32]
        _ref = L
    return _ref


_refd2m = None


def ref_dist2mat(spheres, samples, offsets, counts, prims):
    """The reference's own dist2mat distance functions (src/dist2mat/
    dist2mat.cu:5-193, compiled for the CPU) with the kernel's selection
    rule: (dist float32, closest int32) per sample, or None where the
    reference sources (or nvcc) are absent."""
    global _refd2m
    if _refd2m is None:
        path = _build.build_ref_dist2mat()
        if path is None:
            return None
        L = ctypes.CDLL(path)
        vp, i32 = ctypes.c_void_p, ctypes.c_int
        L.refd2m_eval.restype = None
        L.refd2m_eval.argtypes = [i32, vp, vp, vp, vp, vp, vp, vp]
        _refd2m = L
    smp = np.ascontiguousarray(samples, np.float32).reshape(-1, 3)
    sph = np.ascontiguousarray(spheres, np.float32).reshape(-1, 4)
    pr = np.ascontiguousarray(prims, np.int32).reshape(-1, 3)
    off = np.ascontiguousarray(offsets, np.uint32)
    cnt = np.ascontiguousarray(counts, np.uint32)
    dist = np.empty(smp.shape[0], np.float32)
    closest = np.empty(smp.shape[0], np.int32)
    _refd2m.refd2m_eval(smp.shape[0], _p(smp), _p(sph), _p(pr), _p(off), _p(cnt), _p(dist),
                        _p(closest))
    return dist, closest


def ref_topo_lib():
    """The reference's own ConvexCellHost topology on the CPU, or None."""
    global _reftopo
    if _reftopo is None:
        path = _build.build_ref_topo()
        if path is None:
            return None
        L = ctypes.CDLL(path)
        vp, i32, i64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64
        L.ref_cell_topology.restype = i64
        L.ref_cell_topology.argtypes = [i64, vp, vp, vp, vp, i64, i32]
        _reftopo = L
    return _reftopo


def nthreads():
    return max(1, os.cpu_count() or 1)


def payload_bytes(nb_v, nb_p, nb_e):
    return int(lib().orc_payload_bytes(int(nb_v), int(nb_p), int(nb_e)))


def mesh_adjacency(n_vert, tets):
    tets = np.ascontiguousarray(tets, dtype=np.int32)
    n_tet = tets.shape[0]
    v_adjs = np.zeros(n_vert, np.int32)
    e_adj6 = np.zeros((n_tet, 6), np.uint8)
    f_adjs = np.zeros((n_tet, 4), np.int32)
    f_ids = np.zeros((n_tet, 4), np.int32)
    nb = np.zeros(1, np.int32)
    rc = lib().orc_mesh_adjacency(n_vert, n_tet, _p(tets), _p(v_adjs), _p(e_adj6),
                                  _p(f_adjs), _p(f_ids), _p(nb))
    if rc != 0:
        raise ValueError("mesh adjacency failed (%d)" % rc)
    return dict(v_adjs=v_adjs, e_adj6=e_adj6, f_adjs=f_adjs, f_ids=f_ids,
                n_boundary_faces=int(nb[0]))


def dense_e_adjs(n_vert, tets, e_adj6):
    tets = np.ascontiguousarray(tets, dtype=np.int32)
    n = int(lib().orc_dense_e_adjs_size(n_vert))
    out = np.empty(n, np.int32)
    lib().orc_dense_e_adjs(n_vert, tets.shape[0], _p(tets),
                           _p(np.ascontiguousarray(e_adj6, np.uint8)), _p(out))
    return out


def knn(site4f, k, n_threads=None):
    site4f = np.ascontiguousarray(site4f, dtype=np.float32)
    n = site4f.shape[0]
    nbr = np.empty((n, k), np.int32)
    keys = np.empty((n, k), np.float32)
    lib().orc_knn(n, _p(site4f), k, _p(nbr), _p(keys), n_threads or nthreads())
    return nbr, keys


def topology_hashes(headers, payload):
    """Canonical topology hash of every record (0 where not emitted)."""
    headers = np.ascontiguousarray(headers)
    payload = np.ascontiguousarray(payload, np.uint8)
    out = np.zeros(len(headers), np.uint64)
    lib().orc_topology_hashes(len(headers), _p(headers), _p(payload), _p(out))
    return out


def power_neighbors(site4f, lo, hi, max_nbr=96, n_threads=None):
    """Power neighbours of every site inside the box [lo, hi] -- the stand-in
    for libmat's regular-triangulation lists (exact signs, ascending keys
    until no unseen site can cut the cell).  Returns (nbr [n, max_nbr] ids
    ascending, -1 padded; count [n]: neighbours, -1 hidden, -2 / -3 the
    clipper's capacity or max_nbr exceeded)."""
    site4f = np.ascontiguousarray(site4f, np.float32)
    n = site4f.shape[0]
    region = np.ascontiguousarray(np.concatenate([np.asarray(lo, np.float64).ravel(),
                                                  np.asarray(hi, np.float64).ravel()]))
    nbr = np.empty((n, max_nbr), np.int32)
    count = np.empty(n, np.int32)
    lib().orc_power_neighbors(n, _p(site4f), _p(region), max_nbr, _p(nbr), _p(count),
                              n_threads or nthreads())
    return nbr, count


def candidate_pairs(vert3f, tets, site4f, flags, nbr, n_threads=None):
    vert3f = np.ascontiguousarray(vert3f, np.float32)
    tets = np.ascontiguousarray(tets, np.int32)
    site4f = np.ascontiguousarray(site4f, np.float32)
    flags = np.ascontiguousarray(flags, np.uint32)
    nbr = np.ascontiguousarray(nbr, np.int32)
    n_tet = tets.shape[0]
    offs = np.zeros(n_tet + 1, np.int32)
    cap = max(16, 64 * n_tet)
    while True:
        sites = np.empty(cap, np.int32)
        n = lib().orc_candidate_pairs(vert3f.shape[0], _p(vert3f), n_tet, _p(tets),
                                      site4f.shape[0], _p(site4f), _p(flags),
                                      _p(nbr), nbr.shape[1], _p(offs), _p(sites),
                                      cap, n_threads or nthreads())
        if n >= 0:
            return offs, sites[:n].copy()
        cap = int(offs[-1]) + 16


def clip_cells(mesh, sites, nbr, offs, pair_sites, pred_mode=0, n_threads=None):
    """mesh: dict(vert3d, tets, v_adjs, e_adj6, f_adjs, f_ids);
    sites: float64 [n, 4] (x, y, z, w).  Returns (headers, payload, stats)."""
    vert3d = np.ascontiguousarray(mesh["vert3d"], np.float64)
    vert3f = vert3d.astype(np.float32)
    site4d = np.ascontiguousarray(sites, np.float64)
    site4f = site4d.astype(np.float32)
    tets = np.ascontiguousarray(mesh["tets"], np.int32)
    nbr = np.ascontiguousarray(nbr, np.int32)
    offs = np.ascontiguousarray(offs, np.int32)
    pair_sites = np.ascontiguousarray(pair_sites, np.int32)
    n_pairs = int(offs[-1])
    headers = np.zeros(max(n_pairs, 1), HEADER_DTYPE)
    stats = np.zeros(4, np.int64)
    cap = max(4096, 1024 * n_pairs)
    for _ in range(3):
        payload = np.zeros(cap, np.uint8)
        used = lib().orc_clip_cells(
            vert3d.shape[0], _p(vert3f), _p(vert3d), tets.shape[0], _p(tets),
            _p(np.ascontiguousarray(mesh["v_adjs"], np.int32)),
            _p(np.ascontiguousarray(mesh["e_adj6"], np.uint8)),
            _p(np.ascontiguousarray(mesh["f_adjs"], np.int32)),
            _p(np.ascontiguousarray(mesh["f_ids"], np.int32)),
            site4d.shape[0], _p(site4f), _p(site4d), _p(nbr), nbr.shape[1],
            _p(offs), _p(pair_sites), pred_mode, _p(headers), _p(payload), cap,
            _p(stats), n_threads or nthreads())
        if used >= 0:
            return headers[:n_pairs], payload[:used], stats
        last = headers[n_pairs - 1]
        cap = int(last["offset"]) + payload_bytes(last["nb_v"], last["nb_p"], last["nb_e"]) + 16
    raise RuntimeError("oracle payload sizing failed")


def ref_clip_cells(mesh, sites, flags, nbr, offs, pair_sites, n_threads=None):
    """Runs the reference's own kernel code (CPU build) on the same pairs.
    Returns (headers, payload, thread_ids) or None without the reference."""
    L = ref_lib()
    if L is None:
        return None
    vert3f = np.ascontiguousarray(mesh["vert3d"], np.float64).astype(np.float32)
    tets = np.ascontiguousarray(mesh["tets"], np.int32)
    n_vert, n_tet = vert3f.shape[0], tets.shape[0]
    site4f = np.ascontiguousarray(sites, np.float64).astype(np.float32)
    n_site = site4f.shape[0]
    vert_soa = np.ascontiguousarray(vert3f.T)
    idx_soa = np.ascontiguousarray(tets.T)
    site_soa = np.ascontiguousarray(site4f[:, :3].T)
    site_w = np.ascontiguousarray(site4f[:, 3])
    k = nbr.shape[1]
    site_knn = np.full((k + 1, n_site), -1, np.int32)
    site_knn[:k] = np.asarray(nbr, np.int32).T
    counts = np.diff(offs)
    tet_k = int(counts.max()) if n_tet else 0
    tet_knn = np.full((max(tet_k, 1), n_tet), -1, np.int32)
    for t in range(n_tet):
        c = counts[t]
        tet_knn[:c, t] = pair_sites[offs[t]:offs[t + 1]]
    e_adjs = dense_e_adjs(n_vert, tets, mesh["e_adj6"])
    n_pairs = int(offs[-1])
    headers = np.zeros(max(n_pairs, 1), HEADER_DTYPE)
    tids = np.zeros(max(n_pairs, 1), np.int32)
    cap = max(4096, 1024 * n_pairs)
    payload = np.zeros(cap, np.uint8)
    used = L.ref_clip_cells(
        n_vert, _p(vert_soa), n_tet, _p(idx_soa),
        _p(np.ascontiguousarray(mesh["v_adjs"], np.int32)), _p(e_adjs),
        _p(np.ascontiguousarray(mesh["f_adjs"], np.int32)),
        _p(np.ascontiguousarray(mesh["f_ids"], np.int32)), n_site, _p(site_soa),
        _p(site_w), _p(np.ascontiguousarray(flags, np.uint32)), _p(site_knn), k,
        _p(tet_knn), tet_k, _p(headers), _p(tids), _p(payload), cap,
        n_threads or nthreads())
    if used < 0:
        raise RuntimeError("reference payload capacity too small")
    return headers[:n_pairs], payload[:used], tids[:n_pairs]


def det4x4_ref(p1, p2, p3, e):
    a = [np.ascontiguousarray(x, np.float32) for x in (p1, p2, p3, e)]
    return float(lib().orc_det4x4_ref(*[_p(x) for x in a]))


def filter_sign(p1, p2, p3, e):
    a = [np.ascontiguousarray(x, np.float32) for x in (p1, p2, p3, e)]
    return int(lib().orc_filter_sign(*[_p(x) for x in a]))


def det4x4_bound(p1, p2, p3, e):
    a = [np.ascontiguousarray(x, np.float32) for x in (p1, p2, p3, e)]
    b = np.zeros(1, np.float64)
    d = float(lib().orc_det4x4_bound(*[_p(x) for x in a], _p(b)))
    return d, float(b[0])


def det4x4_exact_sign(p1, p2, p3, e):
    a = [np.ascontiguousarray(x, np.float32) for x in (p1, p2, p3, e)]
    return int(lib().orc_det4x4_exact_sign(*[_p(x) for x in a]))


def _emitted(headers, payload):
    """The emitted cells (status success) of a pair-header array."""
    h = np.ascontiguousarray(headers[headers["status"] == SUCCESS])
    return h, np.ascontiguousarray(payload, np.uint8)


def cell_topology(cells, payload):
    """Per-cell topology of emitted cells (oracle restatement of
    ConvexCellHost::reload_active / reload_pc_explicit / cal_cell_euler /
    cal_halfplane_facet_euler).  cells: HEADER_DTYPE records of emitted
    cells, in output order.  Returns (TOPO_DTYPE headers, record bytes)."""
    h, payload = _emitted(cells, payload)
    n = h.shape[0]
    th = np.zeros(max(n, 1), TOPO_DTYPE)
    size = int(lib().orc_cell_topology(n, _p(h), _p(payload), _p(th), None, 0))
    out = np.zeros(max(size, 16), np.uint8)
    used = lib().orc_cell_topology(n, _p(h), _p(payload), _p(th), _p(out), out.size)
    if used < 0:
        raise RuntimeError("oracle topology sizing failed")
    return th[:n], out[:used]


def ref_cell_topology(cells, payload, n_threads=None):
    """The same computed by the reference's own voronoi_defs.cxx, or None
    without the reference sources."""
    L = ref_topo_lib()
    if L is None:
        return None
    h, payload = _emitted(cells, payload)
    n = h.shape[0]
    th = np.zeros(max(n, 1), TOPO_DTYPE)
    size = sum(topo_bytes(c["nb_v"], c["nb_p"], c["nb_e"]) for c in h)
    out = np.zeros(max(size, 16), np.uint8)
    used = L.ref_cell_topology(n, _p(h), _p(payload), _p(th), _p(out), out.size,
                               n_threads or nthreads())
    if used < 0:
        raise RuntimeError("reference topology capacity too small")
    return th[:n], out[:used]


_refpc = None

# the arrays of ref_pc_get, in its order: (name, dtype, columns)
REF_PC_ARRAYS = [("site_cells", np.int32, 1), ("nbr_cell", np.int32, 1), ("nbr", np.int32, 1),
                 ("tfid_cell", np.int32, 1), ("tfid", np.int32, 1), ("facet_keys", np.int64, 1),
                 ("facet_cells", np.int32, 1), ("facet_cc", np.int32, 1), ("cell_cc", np.int32, 1),
                 ("edges", np.int32, 7), ("edge_cc", np.int32, 1), ("vertex_cell", np.int32, 1),
                 ("vertex_lvid", np.int32, 1), ("vertex_ids", np.int32, 3),
                 ("vertex_pos", np.float32, 3), ("vertex_sfid", np.int32, 1),
                 ("surface_cell", np.int32, 1), ("surface_fid", np.int32, 1),
                 ("surface_pos", np.float32, 3), ("sfg", np.int32, 4), ("se_covered", np.int32, 5),
                 ("ce_covered", np.int32, 5), ("se_line_end", np.int32, 4),
                 ("se_line_end_pos", np.float32, 3)]


def ref_power_cells(cells, payload, n_site, max_sf_fid, feature_edges=None, surface=None):
    """libmat's own get_all_voro_info and the per-sphere component updates
    (src/rpd3d_base/rpd_update.cxx:1-521 compiled for the CPU,
    ref_powercell_driver.cpp) on the emitted cells of `cells`, as the arrays
    of powercell_oracle.power_cells (same arguments), plus "n_failed"
    (spheres whose construction threw) and "n_mismatch" (maps that disagree
    with each other); None without the reference sources."""
    global _refpc
    if _refpc is None:
        path = _build.build_ref_powercell()
        if path is None:
            return None
        L = ctypes.CDLL(path)
        vp, i32, i64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64
        L.ref_pc_run.restype = vp
        L.ref_pc_run.argtypes = [i64, vp, vp, i32, i32, i64, vp, i32, vp, i64, vp]
        L.ref_pc_get.restype = i64
        L.ref_pc_get.argtypes = [vp, i32, vp, i64]
        L.ref_pc_free.restype = None
        L.ref_pc_free.argtypes = [vp]
        _refpc = L
    L = _refpc
    h = np.ascontiguousarray(cells)
    payload = np.ascontiguousarray(payload, np.uint8)
    fe = np.ascontiguousarray(np.zeros((0, 6)) if feature_edges is None else feature_edges,
                              np.int32).reshape(-1, 6)
    if surface is not None:
        adj = np.ascontiguousarray(surface[0], np.int32).reshape(-1, 3)
        nc = np.ascontiguousarray(surface[1], np.int32).reshape(-1, 2)
    else:
        adj, nc = None, np.zeros((0, 2), np.int32)
    handle = L.ref_pc_run(h.shape[0], _p(h), _p(payload), int(n_site), int(max_sf_fid),
                          fe.shape[0], _p(fe), 0 if adj is None else adj.shape[0],
                          None if adj is None else _p(adj), nc.shape[0], _p(nc))
    try:
        raw = {}
        for i, (name, dt, cols) in enumerate(REF_PC_ARRAYS):
            n = L.ref_pc_get(handle, i, None, 0)
            a = np.zeros(max(n, 1), dt)
            L.ref_pc_get(handle, i, _p(a), a.size)
            raw[name] = a[:n].reshape(-1, cols) if cols > 1 else a[:n]
        n_failed = int(L.ref_pc_get(handle, 24, None, 0))
        n_mismatch = int(L.ref_pc_get(handle, 25, None, 0))
    finally:
        L.ref_pc_free(handle)
    n = int((h["status"] == SUCCESS).sum())
    site = h[h["status"] == SUCCESS]["site_id"].astype(np.int64)

    def csr(rows, vals, count, dtype):
        rows = np.asarray(rows, np.int64)
        off = np.searchsorted(rows, np.arange(count + 1)).astype(np.int64)
        return off, np.asarray(vals, dtype)

    out = {}
    out["site_cell_off"] = np.searchsorted(site[raw["site_cells"]] if n else np.zeros(0, np.int64),
                                           np.arange(n_site + 1)).astype(np.int64)
    out["site_cells"] = raw["site_cells"].astype(np.uint32)
    out["cell_nbr_off"], out["cell_nbrs"] = csr(raw["nbr_cell"], raw["nbr"], n, np.int32)
    out["cell_tfid_off"], out["cell_tfids"] = csr(raw["tfid_cell"], raw["tfid"], n, np.int32)
    out["facet_keys"] = raw["facet_keys"].astype(np.uint64)
    out["facet_cells"] = raw["facet_cells"].astype(np.uint32)
    out["cell_cc"] = raw["cell_cc"]
    out["facet_cc"] = raw["facet_cc"]
    out["edge_cc"] = raw["edge_cc"]
    out["site_facet_off"] = np.searchsorted(raw["facet_keys"] >> 32,
                                            np.arange(n_site + 1)).astype(np.int64)
    out["edges"] = raw["edges"].reshape(-1, 7)
    out["site_edge_off"] = np.searchsorted(out["edges"][:, 0], np.arange(n_site + 1)).astype(np.int64)
    for k in ("vertex_cell", "vertex_lvid", "vertex_sfid"):
        out[k] = raw[k]
    out["vertex_ids"] = raw["vertex_ids"].reshape(-1, 3)
    out["vertex_pos"] = raw["vertex_pos"].reshape(-1, 3)
    out["cell_vertex_off"] = np.searchsorted(raw["vertex_cell"], np.arange(n + 1)).astype(np.int64)
    out["surface_cell"] = raw["surface_cell"]
    out["surface_fid"] = raw["surface_fid"]
    out["surface_pos"] = raw["surface_pos"].reshape(-1, 3)
    out["cell_surface_off"] = np.searchsorted(raw["surface_cell"], np.arange(n + 1)).astype(np.int64)
    sfg = raw["sfg"].reshape(-1, 4)
    out["site_sfg_off"] = np.searchsorted(sfg[:, 0], np.arange(n_site + 1)).astype(np.int64)
    out["sfg_group"], out["sfg_fid"], out["sfg_record"] = sfg[:, 1], sfg[:, 2], sfg[:, 3]
    for name in ("se_covered", "ce_covered"):
        rows = raw[name].reshape(-1, 5)
        out["cell_%s_off" % name] = np.searchsorted(rows[:, 0], np.arange(n + 1)).astype(np.int64)
        out[name] = rows
    out["se_line_end"] = raw["se_line_end"].reshape(-1, 4)
    out["se_line_end_pos"] = raw["se_line_end_pos"].reshape(-1, 3)
    out["cell_se_line_end_off"] = np.searchsorted(out["se_line_end"][:, 0],
                                                  np.arange(n + 1)).astype(np.int64)
    out["n_failed"] = n_failed
    out["n_mismatch"] = n_mismatch
    return out


def topo_bytes(nb_v, nb_p, nb_e):
    return int(lib().orc_topo_bytes(int(nb_v), int(nb_p), int(nb_e)))


def cell_polygons(cells, payload, triangulate=False, boundary_only=False, max_sf_fid=0,
                  slice_plane=None):
    """Polygon soup of emitted cells (oracle restatement of
    get_one_convex_cell_faces_const; with slice_plane = (pos, normal), the
    cells save_convex_cells_houdini slices away are left out).  Returns
    dict(points (n, 3) float32, poly_offsets, indices, poly_site,
    poly_adj_site)."""
    h, payload = _emitted(cells, payload)
    n = h.shape[0]
    counts = np.zeros(3, np.int64)
    sl = None if slice_plane is None else np.ascontiguousarray(
        np.concatenate([np.asarray(slice_plane[0], np.float64), np.asarray(slice_plane[1], np.float64)]))
    args = (n, _p(h), _p(payload), int(triangulate), int(boundary_only), int(max_sf_fid),
            None if sl is None else _p(sl))
    if lib().orc_cell_polygons(*args, None, 0, None, None, 0, None, None, 0, _p(counts)) != 0:
        raise RuntimeError("oracle polygon count failed")
    npt, npoly, nidx = (int(x) for x in counts)
    pts = np.zeros((max(npt, 1), 3), np.float32)
    offs = np.zeros(npoly + 1, np.int64)
    idx = np.zeros(max(nidx, 1), np.uint32)
    site = np.zeros(max(npoly, 1), np.int32)
    adj = np.zeros(max(npoly, 1), np.int32)
    if lib().orc_cell_polygons(*args, _p(pts), npt, _p(offs), _p(idx), nidx, _p(site), _p(adj),
                               npoly, _p(counts)) != 0:
        raise RuntimeError("oracle polygon fill failed")
    return dict(points=pts[:npt], poly_offsets=offs, indices=idx[:nidx], poly_site=site[:npoly],
                poly_adj_site=adj[:npoly])
