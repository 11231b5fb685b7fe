"""Per-cell topology on the device (rpd_compute_topology) against the
reference's own ConvexCellHost code (golden fixtures made by
src/rpd3d_base/voronoi_defs.cxx on the reference's cells) and against the
oracle on larger workloads: headers and records bit for bit."""
import numpy as np
import pytest

from libmat_gb300 import rpd
from libmat_gb300 import workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _same(th, rec, oh, orec):
    assert th.shape == oh.shape
    assert np.array_equal(th.view(np.uint8).reshape(-1, 16), oh.view(np.uint8).reshape(-1, 16))
    assert np.array_equal(rec, orec)


def test_golden_topology_bit_exact(golden_cases):
    for name, c in golden_cases.items():
        with rpd.RPD(predicate_mode=rpd.PRED_FP32_FILTER, neighbor_source=rpd.NEIGH_USER) as r:
            r.set_mesh(c["vert3d"], c["tets"], c["v_adjs"], c["e_adj6"], c["f_adjs"], c["f_ids"])
            r.set_sites(c["sites"], c["flags"])
            r.set_neighbors(c["nbr"])
            r.compute()
            ms = r.compute_topology()
            th, rec = r.topology()
        assert ms >= 0.0
        gh = c["topo_headers"].reshape(-1).view(O.TOPO_DTYPE)
        _same(th, rec, gh, c["topo_records"])


@pytest.mark.parametrize("which", ["small", "ellipsoid"])
def test_topology_matches_oracle(which):
    if which == "small":
        cfg = W.config_small_cube()  # 48,000 tets, 2,000 sites
    else:
        cfg = W.config_ellipsoid(target_tets=200_000, n_site=10_000, seed=4)
    adj = rpd.mesh_adjacency(cfg["vert3d"].shape[0], cfg["tets"])
    with rpd.RPD(predicate_mode=rpd.PRED_FP32_FILTER, neighbor_source=rpd.NEIGH_KNN, knn_k=64,
                 certify=True) as r:
        r.set_mesh(cfg["vert3d"], cfg["tets"], adj["v_adjs"], adj["e_adj6"], adj["f_adjs"],
                   adj["f_ids"])
        r.set_sites(cfg["sites"], cfg["flags"])
        st = r.compute()
        h, p = r.cells()
        r.compute_topology()
        th, rec = r.topology()
        # a second compute invalidates the topology until it is recomputed
        r.compute()
        with pytest.raises(rpd.RPDError):
            r.topology()
    assert th.shape[0] == st.n_cells > 0
    oh, orec = O.cell_topology(h, p)
    _same(th, rec, oh, orec)
    assert np.all(th["flags"] == 0)
    # per site: sum of cell Euler numbers - #cells (libmat's power-cell
    # Euler check) is 1 for nearly every site
    eul = np.bincount(h["site_id"], weights=th["euler"].astype(np.float64))
    cnt = np.bincount(h["site_id"])
    has = cnt > 0
    assert np.mean(np.abs(eul[has] - cnt[has] - 1.0) < 1e-3) > 0.9
