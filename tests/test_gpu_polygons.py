"""Polygon soup on the device (rpd_compute_polygons, libmat's Houdini export
get_one_convex_cell_faces_const, src/IO/IO_CUDA/io_cuda.cxx:21-141) against
the oracle on the same cells: points (float bits), polygon offsets, point
ids and sites, in every mode."""
import numpy as np
import pytest

from libmat_gb300 import rpd
from libmat_gb300 import workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu

MODES = [(False, False), (True, False), (False, True), (True, True)]


def _same(a, b):
    for k in ("points", "poly_offsets", "indices", "poly_site", "poly_adj_site"):
        assert a[k].shape == b[k].shape, k
        assert np.array_equal(a[k].view(np.uint8), b[k].view(np.uint8)), k


def test_golden_polygons_match_oracle(golden_cases):
    for name, c in golden_cases.items():
        nb = int((c["f_adjs"] == 1).sum())  # boundary faces are numbered first
        with rpd.RPD(predicate_mode=rpd.PRED_FP32_FILTER, neighbor_source=rpd.NEIGH_USER) as r:
            r.set_mesh(c["vert3d"], c["tets"], c["v_adjs"], c["e_adj6"], c["f_adjs"], c["f_ids"])
            r.set_sites(c["sites"], c["flags"])
            r.set_neighbors(c["nbr"])
            r.compute()
            h, p = r.cells()
            for tri, bo in MODES:
                r.compute_polygons(triangulate=tri, boundary_only=bo, max_sf_fid=nb)
                _same(r.polygons(), O.cell_polygons(h, p, tri, bo, nb))


def test_polygons_match_oracle_48k():
    cfg = W.config_small_cube()
    adj = rpd.mesh_adjacency(cfg["vert3d"].shape[0], cfg["tets"])
    nb = int((adj["f_adjs"] == 1).sum())
    with rpd.RPD(predicate_mode=rpd.PRED_FP32_FILTER, neighbor_source=rpd.NEIGH_KNN, knn_k=64,
                 certify=True) as r:
        r.set_mesh(cfg["vert3d"], cfg["tets"], adj["v_adjs"], adj["e_adj6"], adj["f_adjs"],
                   adj["f_ids"])
        r.set_sites(cfg["sites"], cfg["flags"])
        r.compute()
        h, p = r.cells()
        ms = r.compute_polygons()  # computes the topology first
        got = r.polygons()
        r.compute_polygons(triangulate=True, boundary_only=True, max_sf_fid=nb)
        got_tb = r.polygons()
    assert ms > 0
    _same(got, O.cell_polygons(h, p))
    _same(got_tb, O.cell_polygons(h, p, True, True, nb))
    assert got["points"].shape[0] == int(h["nb_v"].astype(np.int64).sum())
