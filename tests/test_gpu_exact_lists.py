"""Exact cells from GPU-built lists (rpd_config.exact_lists).

libmat clips every site with its regular triangulation's power neighbours
(src/rpd3d_base/triangulation.cxx:442-558, used at
src/rpd3d_api/rpd_api.cxx:67-69), so its cells are the exact restricted power
diagram.  The GPU lists hold the k smallest bisector keys; a cell that its
whole list leaves uncertified gets its site a longer list (every key up to
the cell's radius bound) and is clipped again.  Checked here against the
oracle's power neighbours (the stand-in for the triangulation: exact signs,
ascending keys until no unseen site can cut the cell), clipped by the same
engine as libmat's own lists would be:

* no emitted cell stays uncertified, and short lists (k = 16) make the
  rounds do real work;
* the emitted (tet, site) cells and their canonical topology equal those of
  the power-neighbour lists, which the reference's algorithm clips in
  site-id order with FP64 predicates;
* the plain FP64 path (site-id order, no early stop) extends the same way
  and gives the same cells;
* every tet is partitioned by its cells (volumes)."""
import numpy as np
import pytest

from libmat_gb300 import rpd
from libmat_gb300 import workloads as W
from oracle import oracle as O
from tests.helpers import tet_volumes

pytestmark = pytest.mark.gpu


def run(cfg, **kw):
    adj = rpd.mesh_adjacency(cfg["vert3d"].shape[0], cfg["tets"])
    nbr = kw.pop("user_lists", None)
    flags = kw.pop("flags", cfg["flags"])
    src = rpd.NEIGH_USER if nbr is not None else rpd.NEIGH_KNN
    with rpd.RPD(neighbor_source=src, topology_hash=True, **kw) as r:
        r.set_mesh(cfg["vert3d"], cfg["tets"], adj["v_adjs"], adj["e_adj6"], adj["f_adjs"],
                   adj["f_ids"])
        r.set_sites(cfg["sites"], flags)
        if nbr is not None:
            r.set_neighbors(nbr)
        st = r.compute()
        ph = r.pair_headers()
        hs = r.topology_hashes()
    ok = ph["status"] == rpd.SUCCESS
    key = ph["tet_id"][ok].astype(np.int64) << 32 | ph["site_id"][ok].astype(np.int64)
    order = np.argsort(key)
    return dict(stats=st, key=key[order], hash=hs[ok][order], vol=ph["volume"][ok][order],
                tet=ph["tet_id"][ok][order], ph=ph)


def power_lists(cfg):
    s4 = cfg["sites"].astype(np.float32)
    v = cfg["vert3d"]
    nbr, cnt = O.power_neighbors(s4, v.min(0), v.max(0), max_nbr=96)
    assert (cnt >= -1).all(), "oracle capacity"
    k = max(int(cnt.max()), 1)
    flags = cfg["flags"].copy()
    flags[cnt < 0] = 0  # hidden spheres: no cells (libmat's is_rt_valid)
    return np.ascontiguousarray(nbr[:, :k]), flags, int((cnt < 0).sum())


CASES = {
    "ellipsoid": lambda: W.config_ellipsoid(target_tets=60000, n_site=3000, seed=31),
    "cube": lambda: W.config_small_cube(n=12, n_site=900, seed=32),
}


@pytest.fixture(scope="module", params=sorted(CASES))
def case(request):
    cfg = CASES[request.param]()
    nbr, flags, n_hidden = power_lists(cfg)
    ref = run(cfg, user_lists=nbr, flags=flags, predicate_mode=rpd.PRED_FP64)
    return request.param, cfg, ref, n_hidden


def test_short_lists_leave_uncertified_cells_without_rounds(case):
    _, cfg, _, _ = case
    one = run(cfg, knn_k=16, certify=True, exact_lists=False)
    assert one["stats"].n_uncertified > 0
    assert one["stats"].n_extend_rounds == 0


@pytest.mark.parametrize("k", [16, 64])
def test_certified_rounds_give_the_power_neighbour_cells(case, k):
    name, cfg, ref, _ = case
    got = run(cfg, knn_k=k, certify=True, exact_lists=True)
    st = got["stats"]
    assert st.n_uncertified == 0, name
    if k == 16:
        assert st.n_extended_sites > 0 and st.n_cert_reclipped > 0
    assert np.array_equal(got["key"], ref["key"]), (name, k)
    assert np.array_equal(got["hash"], ref["hash"]), (name, k)


def test_plain_fp64_rounds_give_the_same_cells(case):
    name, cfg, ref, _ = case
    got = run(cfg, knn_k=16, certify=False, exact_lists=True, predicate_mode=rpd.PRED_FP64)
    assert got["stats"].n_uncertified == 0
    assert got["stats"].n_extended_sites > 0
    assert np.array_equal(got["key"], ref["key"]), name
    assert np.array_equal(got["hash"], ref["hash"]), name


def test_every_tet_is_partitioned(case):
    name, cfg, _, _ = case
    got = run(cfg, knn_k=16, certify=True, exact_lists=True)
    vt = tet_volumes(cfg["vert3d"], cfg["tets"].astype(np.int64))
    per_tet = np.bincount(got["tet"], weights=got["vol"], minlength=vt.shape[0])
    t = cfg["tets"].astype(np.int64)
    v = cfg["vert3d"]
    L = np.max([np.linalg.norm(v[t[:, a]] - v[t[:, b]], axis=1)
                for a, b in ((0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3))], axis=0)
    err = np.abs(per_tet - vt)
    assert np.all(err <= 1e-4 * vt + 1e-4 * L ** 3), (name, np.nonzero(err > 1e-4 * vt + 1e-4 * L ** 3)[0][:5])


def test_hidden_spheres_get_no_cells(case):
    name, cfg, _, n_hidden = case
    s4 = cfg["sites"].astype(np.float32)
    v = cfg["vert3d"]
    _, cnt = O.power_neighbors(s4, v.min(0), v.max(0), max_nbr=96)
    hidden = np.flatnonzero(cnt == -1)
    got = run(cfg, knn_k=8, certify=True, exact_lists=True)
    sites = (got["key"] & 0xffffffff).astype(np.int64)
    assert not np.isin(sites, hidden).any(), name
    assert len(hidden) == n_hidden
