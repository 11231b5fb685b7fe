"""Incremental update (rpd_compute_partial, libmat's calculate_partial,
src/rpd3d_api/rpd_api.cxx:147-316): after some sites move, recomputing the
changed sites and every site whose neighbour list holds one of them, and
merging with the previous cells, gives exactly the cells of a full
recompute."""
import numpy as np
import pytest

from libmat_gb300 import rpd
from libmat_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _engine(cfg, adj):
    # one pass: the recomputed set below is derived from the 64-entry lists
    r = rpd.RPD(predicate_mode=rpd.PRED_FP32_FILTER, neighbor_source=rpd.NEIGH_KNN, knn_k=64,
                certify=True, topology_hash=False, exact_lists=False)
    r.set_mesh(cfg["vert3d"], cfg["tets"], adj["v_adjs"], adj["e_adj6"], adj["f_adjs"], adj["f_ids"])
    return r


def _record(p, h, q):
    return p[int(h["offset"][q]):int(h["offset"][q]) + rpd.payload_bytes(h["nb_v"][q], h["nb_p"][q],
                                                                         h["nb_e"][q])]


@pytest.mark.parametrize("n_moved", [1, 25])
def test_partial_update_equals_full_recompute(n_moved):
    cfg = W.config_ellipsoid(target_tets=60_000, n_site=3000, seed=23)
    adj = rpd.mesh_adjacency(cfg["vert3d"].shape[0], cfg["tets"])
    ns = cfg["sites"].shape[0]
    rng = np.random.default_rng(n_moved)
    s0 = cfg["sites"]
    s1 = s0.copy()
    moved = rng.choice(ns, n_moved, replace=False)
    spacing = 1000.0 / ns ** (1.0 / 3.0)
    s1[moved, :3] += rng.normal(0.0, 0.3 * spacing, (n_moved, 3))
    with _engine(cfg, adj) as full:
        full.set_sites(s1, cfg["flags"])
        full.compute()
        n1 = full.neighbor_lists(ns)
        hf, pf = full.cells()
    with _engine(cfg, adj) as r:
        with pytest.raises(rpd.RPDError):
            r.compute_partial(np.ones(ns))  # no previous cells
        r.set_sites(s0, cfg["flags"])
        r.compute()
        n0 = r.neighbor_lists(ns)
        # the sites whose cells can change: the moved ones, their neighbours
        # before and after, and the sites that list a moved one
        hit = np.zeros(ns, bool)
        hit[moved] = True
        for lists in (n0, n1):
            hit[lists[moved][lists[moved] >= 0]] = True
            hit |= np.isin(lists, moved).any(axis=1)
        r.set_sites(s1, cfg["flags"])
        st = r.compute_partial(hit)
        hm, pm = r.cells()
    assert st.n_cells < len(hf)  # only the recomputed sites were clipped
    assert len(hm) == len(hf)
    for f in ("tet_id", "site_id", "status", "nb_v", "nb_p", "nb_e", "volume"):
        assert np.array_equal(hm[f], hf[f]), f
    for q in range(len(hf)):
        assert np.array_equal(_record(pm, hm, q), _record(pf, hf, q))
