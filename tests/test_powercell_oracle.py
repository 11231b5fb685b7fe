"""The power-cell oracle (libmat's get_all_voro_info, restated on the
per-cell topology that is pinned to the reference's own voronoi_defs.cxx):
structural properties on the reference's golden cells."""
import numpy as np

from oracle import powercell_oracle as P
from tests.helpers import SUCCESS, ref_headers


def test_power_cell_structure(golden_cases):
    for name in ("cube_k64", "random_full", "dups_flags_holes"):
        c = golden_cases[name]
        h = ref_headers(c)
        cells = h[h["status"] == SUCCESS]
        ns = c["sites"].shape[0]
        nb = int((c["f_adjs"] == 1).sum())  # boundary faces are numbered first
        pc = P.power_cells(h, c["ref_payload"], ns, nb - 1)
        site = cells["site_id"].astype(np.int64)
        # every cell once, under its site
        assert sorted(pc["site_cells"].tolist()) == list(range(len(cells)))
        for s in range(ns):
            a, b = pc["site_cell_off"][s], pc["site_cell_off"][s + 1]
            assert np.all(site[pc["site_cells"][a:b]] == s)
        # neighbours: same site, symmetric, sharing a tet face
        for q in range(len(cells)):
            for r in pc["cell_nbrs"][pc["cell_nbr_off"][q]:pc["cell_nbr_off"][q + 1]]:
                assert site[r] == site[q]
                assert q in pc["cell_nbrs"][pc["cell_nbr_off"][r]:pc["cell_nbr_off"][r + 1]]
                fq = set(pc["cell_tfids"][pc["cell_tfid_off"][q]:pc["cell_tfid_off"][q + 1]])
                fr = set(pc["cell_tfids"][pc["cell_tfid_off"][r]:pc["cell_tfid_off"][r + 1]])
                assert fq & fr
        # facets and edges grouped by site, keys sorted
        assert np.all(np.diff(pc["facet_keys"].astype(np.float64)) >= 0)
        assert np.all(site[pc["facet_cells"]] == (pc["facet_keys"] >> np.uint64(32)).astype(np.int64))
        e = pc["edges"]
        if len(e):
            assert np.all(site[e[:, 3]] == e[:, 0]) and np.all(e[:, 1] < e[:, 2])
            assert np.all(e[:, 4] < e[:, 5])
        # vertex triples sorted, -1 only first
        v = pc["vertex_ids"]
        assert np.all(np.diff(v, axis=1) > 0)
        assert len(pc["surface_cell"]) > 0 and np.all(pc["surface_fid"] < nb)


def test_feature_edge_records(golden_cases):
    """se/ce records and sharp-line endpoints against a second derivation:
    the edge's vertices from the dual triangles (both tet faces among the
    vertex's planes) instead of the face cycles."""
    from tests.helpers import feature_edge_records, float_vertices, cell_planes_ver
    for name in ("cube_k64", "random_full"):
        c = golden_cases[name]
        h = ref_headers(c)
        cells = h[h["status"] == SUCCESS]
        n_tet = c["tets"].shape[0]
        recs = feature_edge_records(n_tet, seed=5)
        fe = {(int(r[0]), int(r[1]), int(r[2])): (int(r[3]), int(r[4]), int(r[5])) for r in recs}
        nb = int((c["f_adjs"] == 1).sum())
        pc = P.power_cells(h, c["ref_payload"], c["sites"].shape[0], nb - 1, recs)
        plain = P.power_cells(h, c["ref_payload"], c["sites"].shape[0], nb - 1)
        fe_keys = ("se_covered", "ce_covered", "se_line_end")
        for k in plain:  # the other arrays do not depend on the feature edges
            if not any(x in k for x in fe_keys):
                assert np.array_equal(plain[k], pc[k]), k
        want = {1: set(), 2: set()}
        ends = {}
        for q in range(len(cells)):
            pl, ver = cell_planes_ver(c["ref_payload"], cells["offset"][q], cells["nb_v"][q],
                                      cells["nb_p"][q])
            xyz = float_vertices(pl, ver)
            o = int(cells["offset"][q])
            n_p = int(cells["nb_p"][q])
            id2 = c["ref_payload"][o + 16 * n_p:o + 24 * n_p].view(np.int32).reshape(-1, 2)
            for a, b in [(a, b) for a in range(4) for b in range(a + 1, 4)]:
                info = fe.get((int(cells["tet_id"][q]), a, b))
                if info is None:
                    continue
                on = [v for v in range(len(ver)) if a in ver[v][:3] and b in ver[v][:3]]
                if len(on) < 2:  # no edge of the cell on this tet edge
                    continue
                lv = sorted(on)[:2]
                if info[0] in want:
                    want[info[0]].add((q, lv[0], lv[1], info[2], info[1]))
                for v in lv:
                    for i in range(3):
                        hp = id2[ver[v][i]]
                        if hp[1] != -1:
                            s = int(cells["site_id"][q])
                            ends[(q, v, int(hp[1]) if int(hp[0]) == s else int(hp[0]), info[2])] = xyz[v]
                            break
        for t, key in ((1, "se_covered"), (2, "ce_covered")):
            assert set(map(tuple, pc[key].tolist())) == want[t], (name, key)
            off = pc["cell_%s_off" % key]
            assert off[-1] == len(pc[key]) and np.all(np.diff(off) >= 0)
        got = {tuple(k): p for k, p in zip(pc["se_line_end"].tolist(), pc["se_line_end_pos"])}
        assert set(got) == set(ends), name
        for k in got:
            assert np.array_equal(got[k], ends[k]), (name, k)
        assert len(want[1]) > 0 and len(want[2]) > 0 and len(ends) > 0


def _check_groups(labels, members, adj, by_size):
    """labels[i] of members[i] (cells of one group): the connected
    components of the group under adj, numbered by smallest cell, or by
    size then smallest cell."""
    from scipy.sparse import coo_matrix
    from scipy.sparse.csgraph import connected_components
    cells = sorted(set(members))
    pos = {c: i for i, c in enumerate(cells)}
    r, c = [], []
    for a in cells:
        for b in adj.get(a, ()):
            if b in pos:
                r.append(pos[a])
                c.append(pos[b])
    m = coo_matrix((np.ones(len(r)), (r, c)), shape=(len(cells), len(cells)))
    _, comp = connected_components(m, directed=False)
    lab = {}
    for cell, l in zip(members, labels):
        assert lab.setdefault(cell, l) == l
    # same partition
    for a in cells:
        for b in cells:
            assert (comp[pos[a]] == comp[pos[b]]) == (lab[a] == lab[b])
    groups = {}
    for cell in cells:
        groups.setdefault(lab[cell], []).append(cell)
    order = sorted(groups.values(), key=lambda g: (len(g), g[0]) if by_size else g[0])
    assert [lab[g[0]] for g in order] == list(range(len(groups)))


def slotted_cells():
    """Cells of the slotted cube (a non-convex domain) by the oracle's own
    pipeline: kNN lists, the candidate rule, clipping."""
    from libmat_gb300 import workloads as W
    from oracle import oracle as O
    cfg = W.config_slotted_cube()
    adj = O.mesh_adjacency(cfg["vert3d"].shape[0], cfg["tets"])
    mesh = dict(vert3d=cfg["vert3d"], tets=cfg["tets"],
                **{k: adj[k] for k in ("v_adjs", "e_adj6", "f_adjs", "f_ids")})
    s4f = cfg["sites"].astype(np.float32)
    nbr, _ = O.knn(s4f, 64)
    offs, ps = O.candidate_pairs(cfg["vert3d"].astype(np.float32), cfg["tets"], s4f, cfg["flags"], nbr)
    h, p, _ = O.clip_cells(mesh, cfg["sites"], nbr, offs, ps)
    return cfg, adj, h, p


def test_power_cell_components(golden_cases):
    cfg, madj, hs, ps = slotted_cells()
    cases = [(name, ref_headers(golden_cases[name]), golden_cases[name]["ref_payload"],
              golden_cases[name]["sites"].shape[0], int((golden_cases[name]["f_adjs"] == 1).sum()))
             for name in ("cube_k64", "random_full", "dups_flags_holes", "overflow")]
    cases.append(("slotted", hs, ps, cfg["sites"].shape[0], madj["n_boundary_faces"]))
    split = 0
    for name, h, payload, ns, nb in cases:
        pc = P.power_cells(h, payload, ns, nb - 1)
        n = len(pc["cell_cc"])
        adj = {q: set(pc["cell_nbrs"][pc["cell_nbr_off"][q]:pc["cell_nbr_off"][q + 1]].tolist())
               for q in range(n)}
        for s in range(ns):
            cs = pc["site_cells"][pc["site_cell_off"][s]:pc["site_cell_off"][s + 1]].tolist()
            if cs:
                _check_groups(pc["cell_cc"][cs].tolist(), cs, adj, False)
        keys = pc["facet_keys"]
        for k in np.unique(keys):
            rows = np.nonzero(keys == k)[0]
            _check_groups(pc["facet_cc"][rows].tolist(), pc["facet_cells"][rows].tolist(), adj, True)
        e = pc["edges"]
        if len(e):
            _, first = np.unique(e[:, :3], axis=0, return_inverse=True)
            for g in np.unique(first):
                rows = np.nonzero(first == g)[0]
                _check_groups(pc["edge_cc"][rows].tolist(), e[rows, 3].tolist(), adj, False)
        if name == "slotted":
            split = min(pc["cell_cc"].max(), pc["facet_cc"].max(), pc["edge_cc"].max())
    assert split >= 1  # the non-convex domain splits cells, facets and edges


def test_surface_groups():
    """update_sphere_surf_v2fids: per site, its surface faces once (with the
    last record of the face), in groups that are the components of the face
    adjacency without the sharp pairs, ordered by smallest face."""
    from tests.helpers import surface_mesh
    cfg, madj, h, p = slotted_cells()
    adj, pairs = surface_mesh(cfg["vert3d"], cfg["tets"], madj["f_adjs"], madj["f_ids"])
    assert len(pairs) > 0
    ns, nb = cfg["sites"].shape[0], madj["n_boundary_faces"]
    pc = P.power_cells(h, p, ns, nb - 1, surface=(adj, pairs))
    sharp = {(min(a, b), max(a, b)) for a, b in pairs.tolist()}
    nbrs = {f: {int(g) for g in adj[f] if g >= 0 and (min(f, g), max(f, g)) not in sharp}
            for f in range(adj.shape[0])}
    site_of_rec = h[h["status"] == SUCCESS]["site_id"][pc["surface_cell"]]
    split = 0
    for s in range(ns):
        a, b = pc["site_sfg_off"][s], pc["site_sfg_off"][s + 1]
        fids = pc["sfg_fid"][a:b].tolist()
        recs = np.nonzero(site_of_rec == s)[0]
        assert sorted(fids) == sorted(set(pc["surface_fid"][recs].tolist()))
        for f, r in zip(fids, pc["sfg_record"][a:b]):  # the last record of the face
            assert r == recs[pc["surface_fid"][recs] == f].max()
        if fids:
            _check_groups(pc["sfg_group"][a:b].tolist(), fids, nbrs, False)
            split = max(split, int(pc["sfg_group"][a:b].max()))
        g = pc["sfg_group"][a:b]
        assert np.all(np.diff(g) >= 0)  # grouped, faces ascending in a group
    assert split >= 1


def test_power_cells_without_cells(golden_cases):
    """No emitted cell (every status other than success): all record arrays
    empty, every offset array zeros, with and without the optional maps."""
    from tests.helpers import feature_edge_records
    c = golden_cases["cube_k64"]
    h = ref_headers(c).copy()
    h["status"] = 6  # no_intersection
    ns = c["sites"].shape[0]
    adj = -np.ones((4, 3), np.int32)
    pc = P.power_cells(h, c["ref_payload"], ns, 0, feature_edge_records(c["tets"].shape[0], 1),
                       surface=(adj, np.zeros((0, 2), np.int32)))
    for k, v in pc.items():
        if k.endswith("_off"):
            assert not np.any(v), k
        else:
            assert len(v) == 0, k
