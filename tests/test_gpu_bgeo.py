"""Houdini export on the device: the sliced polygon soup against the oracle,
and the file rpd_write_polygons_bgeo writes against the oracle's writer
(itself pinned byte for byte to libmat's GeometryWriter)."""
import numpy as np
import pytest

from libmat_gb300 import rpd
from libmat_gb300 import workloads as W
from oracle import bgeo_oracle as B
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _run_golden(c, slice_plane, path):
    with rpd.RPD(predicate_mode=rpd.PRED_FP32_FILTER, neighbor_source=rpd.NEIGH_USER) as r:
        r.set_mesh(c["vert3d"], c["tets"], c["v_adjs"], c["e_adj6"], c["f_adjs"], c["f_ids"])
        r.set_sites(c["sites"], c["flags"])
        r.set_neighbors(c["nbr"])
        r.compute()
        h, p = r.cells()
        if slice_plane is not None:
            r.set_polygon_slice(*slice_plane)
        r.compute_polygons()
        soup = r.polygons()
        n = r.write_polygons_bgeo(path)
    return h, p, soup, n


@pytest.mark.parametrize("sliced", [False, True])
def test_golden_bgeo(golden_cases, tmp_path, sliced):
    for name, c in golden_cases.items():
        plane = ((0.2, 0.0, 0.0), (-1.0, 0.0, 0.0)) if sliced else None
        path = tmp_path / (name + ".bgeo")
        h, p, soup, n = _run_golden(c, plane, path)
        ref = O.cell_polygons(h, p, slice_plane=plane)
        for k in ref:
            assert np.array_equal(soup[k], ref[k]), (name, k)
        want = B.bgeo_bytes(ref["points"], ref["poly_offsets"], ref["indices"], ref["poly_site"])
        got = path.read_bytes()
        assert n == len(got) == len(want) and got == want, name


def test_wide_ids_and_slice_off(tmp_path):
    """More than 65536 points (32-bit ids in the file); a plane that keeps
    part of the cells; slicing turned off again."""
    cfg = W.config_small_cube(n=10, n_site=300, seed=9)
    adj = rpd.mesh_adjacency(cfg["vert3d"].shape[0], cfg["tets"])
    with rpd.RPD(predicate_mode=rpd.PRED_FP32_FILTER, neighbor_source=rpd.NEIGH_KNN, knn_k=64,
                 certify=True) as r:
        r.set_mesh(cfg["vert3d"], cfg["tets"], adj["v_adjs"], adj["e_adj6"], adj["f_adjs"],
                   adj["f_ids"])
        r.set_sites(cfg["sites"], cfg["flags"])
        r.compute()
        h, p = r.cells()
        r.compute_polygons()
        full = r.polygons()
        r.write_polygons_bgeo(tmp_path / "full.bgeo")
        plane = (cfg["vert3d"].mean(axis=0), np.array([0.3, -1.0, 0.2]))
        r.set_polygon_slice(*plane)
        r.compute_polygons()
        part = r.polygons()
        r.write_polygons_bgeo(tmp_path / "part.bgeo")
        with pytest.raises(rpd.RPDError):
            r.set_polygon_slice((np.nan, 0, 0), (1, 0, 0))
        r.set_polygon_slice(None)
        r.compute_polygons()
        again = r.polygons()
    assert full["points"].shape[0] > 65536
    assert 0 < part["points"].shape[0] < full["points"].shape[0]
    for k in full:
        assert np.array_equal(full[k], again[k]), k
    for soup, name, plane_ in ((full, "full", None), (part, "part", plane)):
        ref = O.cell_polygons(h, p, slice_plane=plane_)
        for k in ref:
            assert np.array_equal(soup[k], ref[k]), (name, k)
        want = B.bgeo_bytes(ref["points"], ref["poly_offsets"], ref["indices"], ref["poly_site"])
        assert (tmp_path / (name + ".bgeo")).read_bytes() == want, name
