"""The oracle (CPU restatement of libmat's RPD path) pinned against the
reference itself: golden fixtures made by the reference's own clipping
kernel, a live cross-check when the reference sources are present, and
known-answer / property tests."""
import numpy as np
import pytest

from libmat_gb300 import workloads as W
from oracle import oracle as O
from tests.helpers import SUCCESS, compare_cells, mesh_of, ref_headers, tet_volumes


def test_oracle_matches_golden(golden_cases):
    assert len(golden_cases) >= 6
    for name, c in golden_cases.items():
        h, p, _ = O.clip_cells(mesh_of(c), c["sites"], c["nbr"], c["tet_offsets"],
                               c["pair_sites"])
        bad = compare_cells(h, p, ref_headers(c), c["ref_payload"])
        assert bad == 0, name


def test_filter_mode_identical_to_fp64(golden_cases):
    for name, c in golden_cases.items():
        h0, p0, s0 = O.clip_cells(mesh_of(c), c["sites"], c["nbr"], c["tet_offsets"],
                                  c["pair_sites"], pred_mode=0)
        h1, p1, s1 = O.clip_cells(mesh_of(c), c["sites"], c["nbr"], c["tet_offsets"],
                                  c["pair_sites"], pred_mode=1)
        assert compare_cells(h0, p0, h1, p1) == 0, name
        assert s1[0] == s0[0] and s1[1] < s1[0]


def test_candidate_pairs_and_adjacency_match_golden(golden_cases):
    for name, c in golden_cases.items():
        adj = O.mesh_adjacency(c["vert3d"].shape[0], c["tets"])
        for f in ("v_adjs", "e_adj6", "f_adjs", "f_ids"):
            assert np.array_equal(adj[f], c[f]), (name, f)
        offs, ps = O.candidate_pairs(c["vert3d"].astype(np.float32), c["tets"],
                                     c["sites"].astype(np.float32), c["flags"], c["nbr"])
        assert np.array_equal(offs, c["tet_offsets"]) and np.array_equal(ps, c["pair_sites"])


def test_live_reference_cross_check():
    if O.ref_lib() is None:
        pytest.skip("reference sources not present")
    for seed in range(3):
        c = W.random_small(n_cube=3, n_site=25, seed=100 + seed)
        adj = O.mesh_adjacency(c["vert3d"].shape[0], c["tets"])
        mesh = dict(vert3d=c["vert3d"], tets=c["tets"], **{k: adj[k] for k in
                    ("v_adjs", "e_adj6", "f_adjs", "f_ids")})
        nbr, _ = O.knn(c["sites"].astype(np.float32), 20)
        for order in (np.sort(nbr, axis=1), nbr):
            offs, ps = O.candidate_pairs(c["vert3d"].astype(np.float32), c["tets"],
                                         c["sites"].astype(np.float32), c["flags"], order)
            h, p, _ = O.clip_cells(mesh, c["sites"], order, offs, ps)
            hr, pr, _ = O.ref_clip_cells(mesh, c["sites"], c["flags"], order, offs, ps)
            assert compare_cells(h, p, hr, pr) == 0


def test_cube_adjacency_known_answers():
    n = 3
    vert, tets = W.cube_grid_mesh(n)
    adj = O.mesh_adjacency(vert.shape[0], tets)
    assert adj["n_boundary_faces"] == 12 * n * n
    assert (adj["f_adjs"] == 1).sum() == 12 * n * n
    assert adj["v_adjs"].sum() == 4 * tets.shape[0]
    # each interior face id appears exactly twice, boundary ids once
    ids, cnt = np.unique(adj["f_ids"], return_counts=True)
    assert np.all(cnt[ids < adj["n_boundary_faces"]] == 1)
    assert np.all(cnt[ids >= adj["n_boundary_faces"]] == 2)
    # corner vertex (0,0,0) of a Kuhn grid belongs to 1 tet... 6 tets share
    # the main diagonal of each cube
    assert adj["v_adjs"][0] == 1 or adj["v_adjs"][0] == 6


def test_one_site_gives_the_tet_itself():
    vert, tets = W.cube_grid_mesh(1)
    vert = vert * 1000
    sites = np.array([[500.0, 500.0, 500.0, 100.0]])
    adj = O.mesh_adjacency(vert.shape[0], tets)
    mesh = dict(vert3d=vert, tets=tets, **{k: adj[k] for k in ("v_adjs", "e_adj6", "f_adjs", "f_ids")})
    nbr = np.full((1, 1), -1, np.int32)
    offs, ps = O.candidate_pairs(vert.astype(np.float32), tets, sites.astype(np.float32),
                                 np.ones(1, np.uint32), nbr)
    assert list(ps) == [0] * 6
    h, p, _ = O.clip_cells(mesh, sites, nbr, offs, ps)
    assert np.all(h["status"] == SUCCESS) and np.all(h["nb_v"] == 4) and np.all(h["nb_p"] == 4)
    assert np.allclose(h["volume"], tet_volumes(vert, tets), rtol=1e-14)


def test_two_equal_sites_split_along_bisector():
    vert, tets = W.cube_grid_mesh(2)
    vert = vert * 1000
    sites = np.array([[300.0, 500.0, 500.0, 400.0], [700.0, 500.0, 500.0, 400.0]])
    adj = O.mesh_adjacency(vert.shape[0], tets)
    mesh = dict(vert3d=vert, tets=tets, **{k: adj[k] for k in ("v_adjs", "e_adj6", "f_adjs", "f_ids")})
    nbr = np.array([[1], [0]], np.int32)
    offs, ps = O.candidate_pairs(vert.astype(np.float32), tets, sites.astype(np.float32),
                                 np.ones(2, np.uint32), nbr)
    h, p, _ = O.clip_cells(mesh, sites, nbr, offs, ps)
    ok = h["status"] == SUCCESS
    vol = np.bincount(h["site_id"][ok], weights=h["volume"][ok], minlength=2)
    assert np.allclose(vol, [5e8, 5e8], rtol=1e-12)


def test_volume_partition_with_complete_lists():
    c = W.config_small_cube(n=5, n_site=60, seed=3)
    adj = O.mesh_adjacency(c["vert3d"].shape[0], c["tets"])
    mesh = dict(vert3d=c["vert3d"], tets=c["tets"], **{k: adj[k] for k in ("v_adjs", "e_adj6", "f_adjs", "f_ids")})
    nbr, _ = O.knn(c["sites"].astype(np.float32), 59)
    offs, ps = O.candidate_pairs(c["vert3d"].astype(np.float32), c["tets"],
                                 c["sites"].astype(np.float32), c["flags"], nbr)
    h, p, _ = O.clip_cells(mesh, c["sites"], nbr, offs, ps)
    ok = h["status"] == SUCCESS
    per_tet = np.bincount(h["tet_id"][ok], weights=h["volume"][ok], minlength=c["tets"].shape[0])
    assert np.allclose(per_tet, tet_volumes(c["vert3d"], c["tets"]), rtol=1e-9)


def test_filter_is_sound_on_near_degenerate_planes():
    """Whenever the FP32 filter decides, its sign equals the reference's FP64
    determinant sign, including on planes built to be nearly coplanar."""
    rng = np.random.default_rng(11)
    decided = 0
    for it in range(20000):
        p = rng.normal(size=(3, 4)).astype(np.float32) * np.float32(10 ** rng.uniform(-2, 6))
        # e close to a combination of the three planes: near-zero determinant
        w = rng.normal(size=3)
        e = (w @ p.astype(np.float64) + rng.normal(size=4) * 10 ** rng.uniform(-12, 0)).astype(np.float32)
        s = O.filter_sign(p[0], p[1], p[2], e)
        if s != 0:
            decided += 1
            d = O.det4x4_ref(p[0], p[1], p[2], e)
            assert (d > 0) == (s > 0)
    assert decided > 1000


def test_topology_hash_matches_the_python_definition():
    """The oracle's canonical topology hash (used by the benchmark's parity
    check) equals the definition in tests/helpers.py, which the engine's
    hashes are tested against."""
    from tests.helpers import topology_hash

    cfg = W.config_small_cube(n=6, n_site=150, seed=3)
    adj = O.mesh_adjacency(cfg["vert3d"].shape[0], cfg["tets"])
    nbr, _ = O.knn(cfg["sites"].astype(np.float32), 32)
    nbr = np.sort(nbr, axis=1)
    offs, ps = O.candidate_pairs(cfg["vert3d"].astype(np.float32), cfg["tets"],
                                 cfg["sites"].astype(np.float32), cfg["flags"], nbr)
    mesh = dict(vert3d=cfg["vert3d"], tets=cfg["tets"],
                **{k: adj[k] for k in ("v_adjs", "e_adj6", "f_adjs", "f_ids")})
    h, p, _ = O.clip_cells(mesh, cfg["sites"], nbr, offs, ps)
    hs = O.topology_hashes(h, p)
    ok = np.flatnonzero(h["status"] == O.SUCCESS)
    assert len(ok) > 1000
    for q in ok[::7]:
        assert int(hs[q]) == topology_hash(p, h["offset"][q], h["nb_v"][q], h["nb_p"][q],
                                           h["nb_e"][q])
    assert np.all(hs[h["status"] != O.SUCCESS] == 0)
