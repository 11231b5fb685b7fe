"""Power cells on the device (rpd_compute_power_cells, libmat's
get_all_voro_info) against the oracle's restatement on the same cells:
every array equal, floats bit for bit."""
import numpy as np
import pytest

from libmat_gb300 import rpd
from libmat_gb300 import workloads as W
from oracle import powercell_oracle as P

pytestmark = pytest.mark.gpu


def _same(got, ref):
    for k, v in ref.items():
        g = got[k]
        assert g.shape == v.shape, (k, g.shape, v.shape)
        assert np.array_equal(g.view(np.uint8), v.astype(g.dtype).view(np.uint8)), k


def test_golden_power_cells(golden_cases):
    for name, c in golden_cases.items():
        nb = int((c["f_adjs"] == 1).sum())
        with rpd.RPD(predicate_mode=rpd.PRED_FP32_FILTER, neighbor_source=rpd.NEIGH_USER) as r:
            r.set_mesh(c["vert3d"], c["tets"], c["v_adjs"], c["e_adj6"], c["f_adjs"], c["f_ids"])
            r.set_sites(c["sites"], c["flags"])
            r.set_neighbors(c["nbr"])
            r.compute()
            h, p = r.cells()
            r.compute_power_cells(nb - 1)
            got = r.power_cells()
        _same(got, P.power_cells(h, p, c["sites"].shape[0], nb - 1))


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
        ms = r.compute_power_cells(nb - 1)
        got = r.power_cells()
    assert ms > 0
    _same(got, P.power_cells(h, p, cfg["sites"].shape[0], nb - 1))
    # every interior tet face inside one power cell joins two of its cells
    assert got["cell_nbr_off"][-1] > 0
