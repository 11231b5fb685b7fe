"""Parity of the CUDA path (through the C ABI) with the reference's own
kernel code (golden fixtures) and with the oracle.  Bit-exact for statuses,
counts, planes, plane ids, vertices and edges; FP64 geometry within 1e-9
relative."""
import numpy as np
import pytest

from libmat_gb300 import rpd
from libmat_gb300 import workloads as W
from oracle import oracle as O
from tests.helpers import (SUCCESS, compare_cells, mesh_of, ref_headers, tet_volumes,
                           xyz_of)

pytestmark = pytest.mark.gpu


def run_user(case, pred, geometry=True):
    with rpd.RPD(predicate_mode=pred, neighbor_source=rpd.NEIGH_USER,
                 compute_geometry=geometry) as r:
        r.set_mesh(case["vert3d"], case["tets"], case["v_adjs"], case["e_adj6"],
                   case["f_adjs"], case["f_ids"])
        r.set_sites(case["sites"], case["flags"])
        r.set_neighbors(case["nbr"])
        st = r.compute()
        ph = r.pair_headers()
        h, p = r.cells()
        offs, ps = r.pairs(case["tets"].shape[0])
    return st, ph, h, p, offs, ps


@pytest.mark.parametrize("pred", [rpd.PRED_FP64, rpd.PRED_FP32_FILTER])
def test_golden_cells_bit_exact(golden_cases, pred):
    for name, c in golden_cases.items():
        st, ph, h, p, offs, ps = run_user(c, pred)
        assert np.array_equal(offs, c["tet_offsets"]), name
        assert np.array_equal(ps, c["pair_sites"]), name
        rh = ref_headers(c)
        assert compare_cells(ph, p, rh, c["ref_payload"]) == 0, name
        # compact view = the emitted subset in pair order
        ok = rh["status"] == SUCCESS
        assert len(h) == ok.sum() == st.n_cells
        assert np.array_equal(h["tet_id"], rh["tet_id"][ok])
        assert np.array_equal(h["site_id"], rh["site_id"][ok])
        # the reference's thread ids: tet * tet_k + slot
        assert st.tet_k == int(np.diff(c["tet_offsets"]).max())


def test_filter_escalates_rarely_and_changes_nothing(golden_cases):
    c = golden_cases["cube_k64"]
    st0, ph0, h0, p0, _, _ = run_user(c, rpd.PRED_FP64)
    st1, ph1, h1, p1, _, _ = run_user(c, rpd.PRED_FP32_FILTER)
    assert compare_cells(ph0, p0, ph1, p1) == 0
    assert st1.n_escalated < 0.01 * st1.n_predicates
    assert st0.n_escalated == 0


def test_geometry_matches_oracle(golden_cases):
    for name in ("random_full", "cube_k64"):
        c = golden_cases[name]
        st, ph, h, p, offs, ps = run_user(c, rpd.PRED_FP32_FILTER)
        oh, op, _ = O.clip_cells(mesh_of(c), c["sites"], c["nbr"], offs, ps)
        ok = np.flatnonzero(ph["status"] == SUCCESS)
        # vertices: FP64-accurate (double-float Cramer in the seed frame);
        # volumes: the reference's six-tets-per-vertex decomposition in FP32
        # (the reference computes cell volumes in FP32 too)
        # (errors measured against each cell's parent tet, the quantity the
        # cell volumes partition)
        tv = tet_volumes(c["vert3d"], c["tets"])[ph["tet_id"][ok]]
        err = np.abs(ph["volume"][ok] - oh["volume"][ok])
        assert np.all(err <= 1e-4 * np.abs(oh["volume"][ok]) + 1e-6 * tv), name
        worst = 0.0
        for q in ok[:: max(1, len(ok) // 500)]:
            a = xyz_of(p, ph["offset"][q], ph["nb_v"][q], ph["nb_p"][q], ph["nb_e"][q])
            b = xyz_of(op, oh["offset"][q], oh["nb_v"][q], oh["nb_p"][q], oh["nb_e"][q])
            worst = max(worst, float(np.abs(a - b).max()) / 1000.0)
        assert worst < 1e-9, name


def test_volume_partition_complete_lists(golden_cases):
    c = golden_cases["random_full"]
    st, ph, h, p, offs, ps = run_user(c, rpd.PRED_FP32_FILTER)
    per_tet = np.bincount(h["tet_id"], weights=h["volume"], minlength=c["tets"].shape[0])
    assert np.allclose(per_tet, tet_volumes(c["vert3d"], c["tets"]), rtol=1e-6)


@pytest.mark.parametrize("k", [32, 64, 128])
@pytest.mark.parametrize("order", [rpd.ORDER_DISTANCE, rpd.ORDER_SITE_ID])
def test_knn_matches_oracle(order, k):
    for cfg in (W.config_small_cube(n=6, n_site=300, seed=4),
                W.config_ellipsoid(target_tets=20000, n_site=3000, seed=9)):
        s4f = cfg["sites"].astype(np.float32)
        with rpd.RPD(neighbor_source=rpd.NEIGH_KNN, knn_k=k, clip_order=order) as r:
            adj = rpd.mesh_adjacency(cfg["vert3d"].shape[0], cfg["tets"])
            r.set_mesh(cfg["vert3d"], cfg["tets"], adj["v_adjs"], adj["e_adj6"],
                       adj["f_adjs"], adj["f_ids"])
            r.set_sites(cfg["sites"], cfg["flags"])
            r.compute()
            got = r.neighbor_lists(s4f.shape[0])
        ref, _ = O.knn(s4f, k)
        if order == rpd.ORDER_SITE_ID:
            ref = np.sort(ref, axis=1)
        assert np.array_equal(got, ref)


def test_candidate_pairs_match_reference_rule():
    cfg = W.config_small_cube(n=10, n_site=400, seed=8)
    s4f = cfg["sites"].astype(np.float32)
    adj = rpd.mesh_adjacency(cfg["vert3d"].shape[0], cfg["tets"])
    with rpd.RPD(neighbor_source=rpd.NEIGH_KNN, knn_k=64) as r:
        r.set_mesh(cfg["vert3d"], cfg["tets"], adj["v_adjs"], adj["e_adj6"], adj["f_adjs"],
                   adj["f_ids"])
        r.set_sites(cfg["sites"], cfg["flags"])
        r.compute()
        nbr = r.neighbor_lists(s4f.shape[0])
        offs, ps = r.pairs(cfg["tets"].shape[0])
    ro, rp = O.candidate_pairs(cfg["vert3d"].astype(np.float32), cfg["tets"], s4f,
                               cfg["flags"], nbr)
    assert np.array_equal(offs, ro) and np.array_equal(ps, rp)


def test_small_config_end_to_end_matches_oracle():
    """The 'Plain RPD, small' configuration: 20^3 x 6 tets, 2,000 sites,
    k = 64, FP64 predicates; every pair bit-exact against the oracle."""
    cfg = W.config_small_cube()
    s4f = cfg["sites"].astype(np.float32)
    adj = rpd.mesh_adjacency(cfg["vert3d"].shape[0], cfg["tets"])
    mesh = dict(vert3d=cfg["vert3d"], tets=cfg["tets"], **{k: adj[k] for k in
                ("v_adjs", "e_adj6", "f_adjs", "f_ids")})
    # the reference's algorithm on the GPU's 64-entry lists, one pass
    with rpd.RPD(predicate_mode=rpd.PRED_FP64, neighbor_source=rpd.NEIGH_KNN, knn_k=64,
                 exact_lists=False) as r:
        r.set_mesh(cfg["vert3d"], cfg["tets"], adj["v_adjs"], adj["e_adj6"], adj["f_adjs"],
                   adj["f_ids"])
        r.set_sites(cfg["sites"], cfg["flags"])
        st = r.compute()
        nbr = r.neighbor_lists(s4f.shape[0])
        offs, ps = r.pairs(cfg["tets"].shape[0])
        ph = r.pair_headers()
        h, p = r.cells()
    oh, op, _ = O.clip_cells(mesh, cfg["sites"], nbr, offs, ps)
    assert compare_cells(ph, p, oh, op) == 0
    assert st.n_cells == (oh["status"] == SUCCESS).sum()
