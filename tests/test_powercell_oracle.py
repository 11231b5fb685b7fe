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
