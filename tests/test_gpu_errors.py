"""Input validation done on the device (rpd_set_mesh): bad vertex ids and
non-finite coordinates are reported as errors, and the context stays usable."""
import numpy as np
import pytest

from libmat_gb300 import rpd
from libmat_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def test_set_mesh_rejects_bad_input_and_recovers():
    cfg = W.config_small_cube(n=4, n_site=60, seed=7)
    adj = rpd.mesh_adjacency(cfg["vert3d"].shape[0], cfg["tets"])
    args = (adj["v_adjs"], adj["e_adj6"], adj["f_adjs"], adj["f_ids"])
    with rpd.RPD(knn_k=32) as r:
        bad = cfg["tets"].copy()
        bad[5, 2] = cfg["vert3d"].shape[0]  # one past the last vertex
        with pytest.raises(rpd.RPDError, match="out of range"):
            r.set_mesh(cfg["vert3d"], bad, *args)
        v = cfg["vert3d"].copy()
        v[3, 1] = np.nan
        with pytest.raises(rpd.RPDError, match="non-finite"):
            r.set_mesh(v, cfg["tets"], *args)
        with pytest.raises(rpd.RPDError):
            r.compute()  # no valid mesh loaded
        r.set_mesh(cfg["vert3d"], cfg["tets"], *args)
        r.set_sites(cfg["sites"], cfg["flags"])
        st = r.compute()
        assert st.n_cells > 0
        # the cells tile the mesh: volumes sum to the mesh volume
        h, _ = r.cells()
        assert abs(h["volume"].sum() - 1000.0 ** 3) < 1e-3 * 1000.0 ** 3
