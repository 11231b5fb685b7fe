"""Batches of independent meshes (rpd_batch_*): one persistent clip launch
for all meshes, the per-mesh front end replayed from a CUDA graph.  Every
mesh's cells must equal those of a single-mesh run of that mesh, bit for
bit (topology bytes, FP64 coordinates, volumes)."""
import numpy as np
import pytest

from libmat_gb300 import rpd
from libmat_gb300 import workloads as W
from tests.helpers import compare_cells, topology_hash, xyz_of

pytestmark = pytest.mark.gpu


def meshes():
    out = [W.config_small_cube(n=6, n_site=150, seed=41),
           W.config_ellipsoid(target_tets=20000, n_site=1000, seed=42),
           W.config_small_cube(n=8, n_site=300, seed=43)]
    for cfg in out:
        cfg["adj"] = rpd.mesh_adjacency(cfg["vert3d"].shape[0], cfg["tets"])
    return out


def single(cfg, **kw):
    # the batch clips with the GPU lists as built (one pass, uncertified
    # cells flagged): the single-mesh run the same way
    a = cfg["adj"]
    kw.setdefault("exact_lists", False)
    with rpd.RPD(neighbor_source=rpd.NEIGH_KNN, knn_k=64, **kw) as r:
        r.set_mesh(cfg["vert3d"], cfg["tets"], a["v_adjs"], a["e_adj6"], a["f_adjs"], a["f_ids"])
        r.set_sites(cfg["sites"], cfg["flags"])
        st = r.compute()
        h, p = r.cells()
    return st, h, p


def same_cells(h1, p1, h2, p2):
    if len(h1) != len(h2) or compare_cells(h1, p1, h2, p2) != 0:
        return False
    if not np.array_equal(h1["volume"], h2["volume"]):
        return False
    for q in range(0, len(h1), max(1, len(h1) // 200)):
        a = xyz_of(p1, h1["offset"][q], h1["nb_v"][q], h1["nb_p"][q], h1["nb_e"][q])
        b = xyz_of(p2, h2["offset"][q], h2["nb_v"][q], h2["nb_p"][q], h2["nb_e"][q])
        if not np.array_equal(a, b):
            return False
    return True


@pytest.mark.parametrize("certify", [False, True])
def test_batch_equals_single_mesh_runs(certify):
    ms = meshes()
    kw = dict(predicate_mode=rpd.PRED_FP32_FILTER, certify=certify)
    with rpd.Batch(exact_lists=False, **kw) as b:
        for cfg in ms:
            a = cfg["adj"]
            b.add_mesh(cfg["vert3d"], cfg["tets"], a["v_adjs"], a["e_adj6"], a["f_adjs"],
                       a["f_ids"], cfg["sites"], cfg["flags"])
        st = b.compute()
        got = [b.mesh_cells(m) for m in range(len(ms))]
        st2 = b.compute()  # replay of the recorded front end
        again = [b.mesh_cells(m) for m in range(len(ms))]
    total = 0
    for m, cfg in enumerate(ms):
        sst, h, p = single(cfg, **kw)
        gh, gp = got[m]
        assert same_cells(h, p, gh, gp), m
        assert same_cells(gh, gp, *again[m]), m
        total += sst.n_cells
    assert st.n_cells == total == st2.n_cells


def canonical(h, p):
    """(tet << 32 | site, canonical topology hash) of emitted cells, sorted;
    the hash is computed here from the records, whose plane ids are the
    mesh's own (rpd_batch_copy_mesh_cells maps them back)."""
    key = (h["tet_id"].astype(np.int64) << 32) | h["site_id"].astype(np.int64)
    hs = np.array([topology_hash(p, h["offset"][q], h["nb_v"][q], h["nb_p"][q], h["nb_e"][q])
                   for q in range(len(h))], np.uint64)
    order = np.argsort(key)
    return key[order], hs[order]


def test_exact_batch_equals_exact_single_mesh_runs():
    """Exact lists in a batch: the rounds search one grid of every site of
    the batch, each site restricted to its own mesh's sites.  With short
    base lists the rounds do real work; every mesh's cells then equal (by
    (tet, site) and canonical topology) those of an exact single-mesh run."""
    ms = meshes()
    kw = dict(predicate_mode=rpd.PRED_FP32_FILTER, certify=True, knn_k=16)
    with rpd.Batch(exact_lists=True, **kw) as b:
        for cfg in ms:
            a = cfg["adj"]
            b.add_mesh(cfg["vert3d"], cfg["tets"], a["v_adjs"], a["e_adj6"], a["f_adjs"],
                       a["f_ids"], cfg["sites"], cfg["flags"])
        st = b.compute()
        got = [canonical(*b.mesh_cells(m)) for m in range(len(ms))]
    assert st.n_uncertified == 0
    assert st.n_extended_sites > 0 and st.n_cert_reclipped > 0
    for m, cfg in enumerate(ms):
        a = cfg["adj"]
        with rpd.RPD(neighbor_source=rpd.NEIGH_KNN, exact_lists=True, **kw) as r:
            r.set_mesh(cfg["vert3d"], cfg["tets"], a["v_adjs"], a["e_adj6"], a["f_adjs"],
                       a["f_ids"])
            r.set_sites(cfg["sites"], cfg["flags"])
            sst = r.compute()
            want = canonical(*r.cells())
        assert sst.n_uncertified == 0
        assert np.array_equal(got[m][0], want[0]), m
        assert np.array_equal(got[m][1], want[1]), m


def test_batch_without_graph_and_tuned():
    ms = meshes()
    with rpd.Batch(use_graph=False) as b:
        for cfg in ms:
            a = cfg["adj"]
            b.add_mesh(cfg["vert3d"], cfg["tets"], a["v_adjs"], a["e_adj6"], a["f_adjs"],
                       a["f_ids"], cfg["sites"], cfg["flags"])
        b.compute()
        ref = [b.mesh_cells(m) for m in range(len(ms))]
    with rpd.Batch(certify=True) as b:
        for cfg in ms:
            a = cfg["adj"]
            b.add_mesh(cfg["vert3d"], cfg["tets"], a["v_adjs"], a["e_adj6"], a["f_adjs"],
                       a["f_ids"], cfg["sites"], cfg["flags"])
        t = b.autotune(repeats=1)
        assert t.n_candidates >= 6
        b.compute()
        for m in range(len(ms)):
            h, p = b.mesh_cells(m)
            rh, rp = ref[m]
            # certified order: same statuses, same canonical cells
            assert len(h) == len(rh)
            assert np.array_equal(h["tet_id"], rh["tet_id"]) and np.array_equal(h["site_id"], rh["site_id"])
