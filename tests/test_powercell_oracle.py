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
