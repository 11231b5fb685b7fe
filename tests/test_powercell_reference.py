"""The power-cell oracle against libmat's own code: get_all_voro_info,
update_sphere_surf_v2fids and the per-sphere component updates
(src/rpd3d_base/rpd_update.cxx:1-521), compiled for the CPU behind
oracle/ref_powercell_driver.cpp and run per sphere in update_power_cells'
order (:568-638).  Every array of oracle/powercell_oracle.py's power cells --
cells per site, cell neighbours, tet faces, facets, edges, vertices with
their float positions, surface records, surface groups, feature-edge records,
sharp-line endpoints and the component labels -- equals the reference's,
positions bit for bit.  Skipped where the reference sources are absent."""
import numpy as np
import pytest

from oracle import oracle as O
from oracle import powercell_oracle as P
from tests.helpers import feature_edge_records, ref_headers, surface_mesh


def _same(a, b, name):
    assert b["n_failed"] == 0, name
    assert b["n_mismatch"] == 0, name
    for k in a:
        assert a[k].dtype == b[k].dtype and a[k].shape == b[k].shape, (name, k)
        assert np.array_equal(a[k], b[k]), (name, k)


@pytest.mark.parametrize("with_fe", [False, True])
def test_golden_power_cells_match_reference(golden_cases, with_fe):
    if O.ref_power_cells(ref_headers(golden_cases["cube_k64"])[:0],
                         golden_cases["cube_k64"]["ref_payload"], 1, 0) is None:
        pytest.skip("reference sources not present")
    n_rows = 0
    for name, c in sorted(golden_cases.items()):
        h = ref_headers(c)
        ns = c["sites"].shape[0]
        nb = int((c["f_adjs"] == 1).sum())
        fe = feature_edge_records(c["tets"].shape[0], seed=5) if with_fe else None
        a = P.power_cells(h, c["ref_payload"], ns, nb - 1, fe)
        b = O.ref_power_cells(h, c["ref_payload"], ns, nb - 1, fe)
        _same(a, b, name)
        n_rows += len(a["facet_keys"]) + len(a["edges"]) + len(a["vertex_cell"])
        if with_fe:
            n_rows += len(a["se_covered"]) + len(a["ce_covered"])
    assert n_rows > 10000


def test_slotted_cube_power_cells_match_reference():
    """A non-convex domain: cells, facets and edges split into several
    components, surface groups split at the slot's sharp edges."""
    from tests.test_powercell_oracle import slotted_cells
    cfg, madj, h, p = slotted_cells()
    if O.ref_power_cells(h[:0], p, 1, 0) is None:
        pytest.skip("reference sources not present")
    adj, pairs = surface_mesh(cfg["vert3d"], cfg["tets"], madj["f_adjs"], madj["f_ids"])
    ns, nb = cfg["sites"].shape[0], madj["n_boundary_faces"]
    fe = feature_edge_records(cfg["tets"].shape[0], seed=7)
    a = P.power_cells(h, p, ns, nb - 1, fe, surface=(adj, pairs))
    b = O.ref_power_cells(h, p, ns, nb - 1, fe, surface=(adj, pairs))
    _same(a, b, "slotted")
    assert min(a["cell_cc"].max(), a["facet_cc"].max(), a["edge_cc"].max()) >= 1
    assert a["sfg_group"].max() >= 1
    assert len(a["se_covered"]) > 0 and len(a["se_line_end"]) > 0
