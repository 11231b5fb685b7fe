"""Power cells on the device (rpd_compute_power_cells, libmat's
get_all_voro_info) against the oracle's restatement on the same cells:
every array equal, floats bit for bit."""
import numpy as np
import pytest

from libmat_gb300 import rpd
from libmat_gb300 import workloads as W
from oracle import powercell_oracle as P
from tests.helpers import feature_edge_records, surface_mesh

pytestmark = pytest.mark.gpu


def _same(got, ref):
    for k, v in ref.items():
        g = got[k]
        assert g.shape == v.shape, (k, g.shape, v.shape)
        assert np.array_equal(g.view(np.uint8), v.astype(g.dtype).view(np.uint8)), k


@pytest.mark.parametrize("features", [False, True])
def test_golden_power_cells(golden_cases, features):
    for name, c in golden_cases.items():
        nb = int((c["f_adjs"] == 1).sum())
        fe = feature_edge_records(c["tets"].shape[0], seed=3) if features else None
        with rpd.RPD(predicate_mode=rpd.PRED_FP32_FILTER, neighbor_source=rpd.NEIGH_USER) as r:
            r.set_mesh(c["vert3d"], c["tets"], c["v_adjs"], c["e_adj6"], c["f_adjs"], c["f_ids"])
            r.set_sites(c["sites"], c["flags"])
            r.set_neighbors(c["nbr"])
            r.compute()
            h, p = r.cells()
            r.set_feature_edges(fe)
            r.compute_power_cells(nb - 1)
            got = r.power_cells()
        ref = P.power_cells(h, p, c["sites"].shape[0], nb - 1, fe)
        _same(got, ref)
        if features and name in ("cube_k64", "random_full"):
            assert len(ref["se_covered"]) and len(ref["ce_covered"]) and len(ref["se_line_end"])


def test_power_cells_match_oracle_knn():
    cfg = W.config_small_cube(n=10, n_site=300, seed=9)
    adj = rpd.mesh_adjacency(cfg["vert3d"].shape[0], cfg["tets"])
    nb = int((adj["f_adjs"] == 1).sum())
    with rpd.RPD(predicate_mode=rpd.PRED_FP32_FILTER, neighbor_source=rpd.NEIGH_KNN, knn_k=64,
                 certify=True) as r:
        r.set_mesh(cfg["vert3d"], cfg["tets"], adj["v_adjs"], adj["e_adj6"], adj["f_adjs"],
                   adj["f_ids"])
        r.set_sites(cfg["sites"], cfg["flags"])
        r.compute()
        h, p = r.cells()
        fe = feature_edge_records(cfg["tets"].shape[0], seed=11, frac=0.5)
        r.set_feature_edges(fe)
        ms = r.compute_power_cells(nb - 1)
        got = r.power_cells()
        # bad local faces are refused; an empty map clears the records
        for bad in ((0, 2, 1), (0, 0, 4), (-1, 0, 1)):
            with pytest.raises(rpd.RPDError):
                r.set_feature_edges(np.array([list(bad) + [1, 0, 0]], np.int32))
        r.set_feature_edges(None)
        r.compute_power_cells(nb - 1)
        cleared = r.power_cells()
    assert ms > 0
    _same(got, P.power_cells(h, p, cfg["sites"].shape[0], nb - 1, fe))
    assert len(got["se_covered"]) > 0 and len(cleared["se_covered"]) == 0
    assert cleared["cell_se_line_end_off"][-1] == 0
    # every interior tet face inside one power cell joins two of its cells
    assert got["cell_nbr_off"][-1] > 0


def test_components_on_a_non_convex_domain():
    """The slotted cube splits power cells, facets and edges into several
    components; every array, the component indices included, equals the
    oracle's on the device's own cells."""
    cfg = W.config_slotted_cube()
    adj = rpd.mesh_adjacency(cfg["vert3d"].shape[0], cfg["tets"])
    nb = int((adj["f_adjs"] == 1).sum())
    with rpd.RPD(predicate_mode=rpd.PRED_FP32_FILTER, neighbor_source=rpd.NEIGH_KNN, knn_k=64,
                 certify=True) as r:
        r.set_mesh(cfg["vert3d"], cfg["tets"], adj["v_adjs"], adj["e_adj6"], adj["f_adjs"],
                   adj["f_ids"])
        r.set_sites(cfg["sites"], cfg["flags"])
        r.compute()
        h, p = r.cells()
        sadj, pairs = surface_mesh(cfg["vert3d"], cfg["tets"], adj["f_adjs"], adj["f_ids"])
        bad = sadj.copy()  # face 0 names a face that does not name it back
        bad[0, 0] = next(g for g in range(1, sadj.shape[0]) if 0 not in sadj[g])
        for a, b in ((bad, pairs), (sadj, pairs + sadj.shape[0])):
            with pytest.raises(rpd.RPDError):
                r.set_surface_mesh(a, b)
        r.set_surface_mesh(sadj, pairs)
        r.compute_power_cells(nb - 1)
        got = r.power_cells()
    _same(got, P.power_cells(h, p, cfg["sites"].shape[0], nb - 1, surface=(sadj, pairs)))
    assert got["cell_cc"].max() >= 1 and got["facet_cc"].max() >= 1 and got["edge_cc"].max() >= 1
    assert got["sfg_group"].max() >= 1
