"""The headline workload at full size -- a 1,040,957-tet ellipsoid with
50,000 weighted sites and k = 64 neighbours -- checked through properties
that do not depend on the size (the oracle takes hours there):

* the fast path (FP32-filter predicates, GPU kNN lists in ascending bisector
  distance, the security-radius certificate) and the plain FP64 path (whole
  lists in site-id order: the reference's algorithm) see the same candidate
  pairs, emit the same cells, and every emitted cell has the same canonical
  topology (vertex face-key triples and adjacency counts) in both;
* no emitted cell stays uncertified: the sites whose cells their 64-entry
  lists leave uncertified get longer lists inside the same compute
  (rpd_config.exact_lists), and every tet is partitioned by its cells (their
  volumes add up to the tet's).  Without the rounds, 10 % of the cells are
  flagged and the volumes over-cover some tets."""
import numpy as np
import pytest

from libmat_gb300 import rpd
from libmat_gb300 import workloads as W
from tests.helpers import tet_volumes

pytestmark = pytest.mark.gpu
NO_INTERSECTION = rpd.STATUS_NAMES.index("no_intersection")


@pytest.fixture(scope="module")
def full_size():
    cfg = W.config_ellipsoid()
    adj = rpd.mesh_adjacency(cfg["vert3d"].shape[0], cfg["tets"])
    out = {}
    for name, pred, cert in (("fast", rpd.PRED_FP32_FILTER, True), ("plain", rpd.PRED_FP64, False)):
        with rpd.RPD(predicate_mode=pred, neighbor_source=rpd.NEIGH_KNN, knn_k=64,
                     clip_order=rpd.ORDER_SITE_ID, certify=cert, topology_hash=True) as r:
            r.set_mesh(cfg["vert3d"], cfg["tets"], adj["v_adjs"], adj["e_adj6"], adj["f_adjs"],
                       adj["f_ids"])
            r.set_sites(cfg["sites"], cfg["flags"])
            st = r.compute()
            out[name] = dict(ph=r.pair_headers(), hash=r.topology_hashes(), stats=st)
    return cfg, out


def test_fast_path_equals_plain_fp64(full_size):
    cfg, out = full_size
    f, p = out["fast"], out["plain"]
    assert cfg["tets"].shape[0] == 1_040_957 and cfg["sites"].shape[0] == 50_000
    assert np.array_equal(f["ph"]["tet_id"], p["ph"]["tet_id"])
    assert np.array_equal(f["ph"]["site_id"], p["ph"]["site_id"])
    assert np.array_equal(f["ph"]["status"], p["ph"]["status"])
    ok = f["ph"]["status"] == rpd.SUCCESS
    assert ok.sum() > 3_000_000
    assert np.array_equal(f["hash"][ok], p["hash"][ok])
    # only emptied pairs besides the cells: no capacity or certificate drops
    assert set(np.unique(f["ph"]["status"]).tolist()) <= {rpd.SUCCESS, NO_INTERSECTION}


def test_every_cell_certified_and_every_tet_partitioned(full_size):
    cfg, out = full_size
    vt = tet_volumes(cfg["vert3d"], cfg["tets"].astype(np.int64))
    t = cfg["tets"].astype(np.int64)
    v = cfg["vert3d"]
    L = np.max([np.linalg.norm(v[t[:, a]] - v[t[:, b]], axis=1)
                for a, b in ((0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3))], axis=0)
    for name in ("fast", "plain"):
        st = out[name]["stats"]
        assert st.n_uncertified == 0, name
        assert st.n_extended_sites > 0 and st.n_cert_reclipped > 0, name
        ph = out[name]["ph"]
        ok = ph["status"] == rpd.SUCCESS
        assert not np.any(ph["flags"][ok] & rpd.CELL_UNCERTIFIED), name
        per_tet = np.bincount(ph["tet_id"][ok], weights=ph["volume"][ok], minlength=vt.shape[0])
        err = np.abs(per_tet - vt)
        # cell volumes are FP32 sums about a point of the cell: their error
        # scales with the tet's size cubed (L its longest edge), not with its
        # volume, which is tiny for slivers
        bound = 1e-4 * vt + 1e-4 * L ** 3
        assert np.all(err <= bound), (name, np.nonzero(err > bound)[0][:5])
        assert np.median(err / vt) < 1e-5, name


def test_one_pass_leaves_cells_uncertified():
    """Without the rounds the 64-entry lists leave cells uncertified (the
    rounds above are not vacuous)."""
    cfg = W.config_ellipsoid()
    adj = rpd.mesh_adjacency(cfg["vert3d"].shape[0], cfg["tets"])
    with rpd.RPD(neighbor_source=rpd.NEIGH_KNN, knn_k=64, certify=True, exact_lists=False) as r:
        r.set_mesh(cfg["vert3d"], cfg["tets"], adj["v_adjs"], adj["e_adj6"], adj["f_adjs"],
                   adj["f_ids"])
        r.set_sites(cfg["sites"], cfg["flags"])
        st = r.compute()
    assert st.n_uncertified > 100_000
    assert st.n_extend_rounds == 0
