"""Certified clipping: neighbours in ascending bisector distance, stop at the
security-radius certificate.  Its cells must have exactly the topology of the
plain path (whole list in site-id order, FP64 predicates) -- compared through
the canonical topology hash -- and per-site shortened lists must be repaired
by the re-clip pass."""
import numpy as np
import pytest

from libmat_gb300 import rpd
from libmat_gb300 import workloads as W
from tests.helpers import SUCCESS, topology_hash

pytestmark = pytest.mark.gpu


def engine(cfg, **kw):
    adj = rpd.mesh_adjacency(cfg["vert3d"].shape[0], cfg["tets"])
    r = rpd.RPD(neighbor_source=rpd.NEIGH_KNN, **kw)
    r.set_mesh(cfg["vert3d"], cfg["tets"], adj["v_adjs"], adj["e_adj6"], adj["f_adjs"], adj["f_ids"])
    r.set_sites(cfg["sites"], cfg["flags"])
    return r


def test_topology_hash_definition():
    cfg = W.config_small_cube(n=6, n_site=150, seed=21)
    with engine(cfg, knn_k=40) as r:
        r.compute()
        ph = r.pair_headers()
        _, p = r.cells()
        hs = r.topology_hashes()
    ok = np.flatnonzero(ph["status"] == SUCCESS)
    assert np.all(hs[ph["status"] != SUCCESS] == 0)
    for q in ok[:: max(1, len(ok) // 300)]:
        assert int(hs[q]) == topology_hash(p, ph["offset"][q], ph["nb_v"][q], ph["nb_p"][q],
                                           ph["nb_e"][q])


@pytest.mark.parametrize("cfg_name", ["cube", "ellipsoid"])
def test_certified_equals_plain_topology(cfg_name):
    cfg = (W.config_small_cube(n=12, n_site=800, seed=22) if cfg_name == "cube"
           else W.config_ellipsoid(target_tets=60000, n_site=3000, seed=23))
    with engine(cfg, knn_k=64, predicate_mode=rpd.PRED_FP64) as r:
        sp = r.compute()
        hp = r.pair_headers()
        tp = r.topology_hashes()
    with engine(cfg, knn_k=64, predicate_mode=rpd.PRED_FP32_FILTER, certify=True) as r:
        sf = r.compute()
        hf = r.pair_headers()
        tf = r.topology_hashes()
    assert sp.n_pairs == sf.n_pairs
    assert np.array_equal(hp["status"], hf["status"])
    assert np.array_equal(tp, tf)
    # distance order + certificate evaluates far fewer predicates
    assert sf.n_predicates < 0.7 * sp.n_predicates


def test_short_lists_are_reclipped():
    cfg = W.config_small_cube(n=12, n_site=800, seed=24)
    with engine(cfg, knn_k=64, certify=True) as r:
        r.compute()
        t_full = r.topology_hashes()
        h_full = r.pair_headers()
        r.set_site_k(np.full(800, 6, np.int32))
        st = r.compute()
        t_short = r.topology_hashes()
        h_short = r.pair_headers()
    assert st.n_reclipped > 0
    assert np.array_equal(h_full["status"], h_short["status"])
    assert np.array_equal(t_full, t_short)


def _emitted(r):
    """(tet << 32 | site, topology hash) of the emitted cells, sorted."""
    ph = r.pair_headers()
    ok = ph["status"] == rpd.SUCCESS
    key = ph["tet_id"][ok].astype(np.int64) << 32 | ph["site_id"][ok].astype(np.int64)
    order = np.argsort(key)
    return key[order], r.topology_hashes()[ok][order]


def test_autotune_keeps_cells():
    """The tuned configuration (block shape, register budget, first-pass and
    base list lengths) emits the same cells.  The base list length changes
    which (tet, site) pairs the candidate rule keeps, so the comparison is
    over the emitted cells."""
    cfg = W.config_small_cube(n=12, n_site=800, seed=25)
    with engine(cfg, knn_k=64, certify=True) as r:
        r.compute()
        base_key, base_hash = _emitted(r)
        t = r.autotune(repeats=1)
        assert t.n_candidates >= 6
        assert t.warps_per_block in (2, 4, 8) and t.clip_variant in (0, 1, 2)
        assert t.k_bucket in (0, 16, 32)
        st = r.compute()
        assert st.n_uncertified == 0
        key, hsh = _emitted(r)
        assert np.array_equal(key, base_key)
        assert np.array_equal(hsh, base_hash)


def test_longest_lists_and_no_geometry():
    """k = 128 (the longest GPU-built list) with the certificate against the
    plain path, and the clipping without the FP64 geometry pass: the same
    cells."""
    cfg = W.config_ellipsoid(target_tets=30000, n_site=2000, seed=25)
    with engine(cfg, knn_k=128, predicate_mode=rpd.PRED_FP64) as r:
        r.compute()
        hp = r.pair_headers()
        tp = r.topology_hashes()
    with engine(cfg, knn_k=128, predicate_mode=rpd.PRED_FP32_FILTER, certify=True) as r:
        r.compute()
        hf = r.pair_headers()
        tf = r.topology_hashes()
        r.configure(compute_geometry=0)
        r.compute()
        hg = r.pair_headers()
        tg = r.topology_hashes()
    assert np.array_equal(hp["status"], hf["status"]) and np.array_equal(tp, tf)
    assert np.array_equal(hg["status"], hf["status"]) and np.array_equal(tg, tf)
    assert np.all(hg["volume"] == 0.0)
