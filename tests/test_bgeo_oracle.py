"""The Houdini export's oracle: the file writer against libmat's own
GeometryWriter (compiled from the reference's sources when present), and
the slicing plane against an independent barycenter computation."""
import numpy as np
import pytest

from oracle import bgeo_oracle as B
from oracle import oracle as O
from tests.helpers import SUCCESS, ref_headers, float_vertices, cell_planes_ver


def _random_soup(n_pts, n_polys, seed):
    rng = np.random.default_rng(seed)
    pts = rng.normal(size=(n_pts, 3)).astype(np.float32)
    sizes = rng.integers(3, 9, size=n_polys)
    off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    idx = rng.integers(0, n_pts, size=int(off[-1])).astype(np.uint32)
    idx[:min(len(idx), 1)] = n_pts - 1  # the largest id appears
    site = rng.integers(-1, 1 << 20, size=n_polys).astype(np.int32)
    return pts, off, idx, site


@pytest.mark.parametrize("n_pts", [5, 65536, 65537])
def test_writer_matches_reference(tmp_path, n_pts):
    # 65536 points: the last with 16-bit ids; 65537: 32-bit ids
    soup = _random_soup(n_pts, 300, seed=n_pts)
    ref = B.ref_bgeo_bytes(*soup, tmp_path)
    if ref is None:
        pytest.skip("reference sources not present")
    assert B.bgeo_bytes(*soup) == ref


def test_writer_on_cells_matches_reference(tmp_path, golden_cases):
    c = golden_cases["cube_k64"]
    h = ref_headers(c)
    s = O.cell_polygons(h, c["ref_payload"], slice_plane=((0.2, 0.0, 0.0), (-1.0, 0.0, 0.0)))
    ref = B.ref_bgeo_bytes(s["points"], s["poly_offsets"], s["indices"], s["poly_site"], tmp_path)
    if ref is None:
        pytest.skip("reference sources not present")
    assert B.bgeo_bytes(s["points"], s["poly_offsets"], s["indices"], s["poly_site"]) == ref


def test_slice_plane(golden_cases):
    """The sliced soup is the soup of the cells whose barycenter (float sum
    of the float vertices in order, / nb_v) lies on the kept side."""
    for name in ("cube_k64", "random_full"):
        c = golden_cases[name]
        h = ref_headers(c)
        cells = h[h["status"] == SUCCESS]
        pos, nrm = np.array([0.1, -0.05, 0.02]), np.array([-0.6, 0.3, 0.74])
        keep = np.zeros(len(cells), bool)
        for q in range(len(cells)):
            pl, ver = cell_planes_ver(c["ref_payload"], cells["offset"][q], cells["nb_v"][q],
                                      cells["nb_p"][q])
            xyz = float_vertices(pl, ver)
            b = np.zeros(3, np.float32)
            for v in xyz:
                b = (v + b).astype(np.float32)
            b = (b / np.float32(len(xyz))).astype(np.float32)
            d = b.astype(np.float64) - pos
            keep[q] = not (d[0] * nrm[0] + d[1] * nrm[1] + d[2] * nrm[2] >= 0)
        assert 0 < keep.sum() < len(cells)
        got = O.cell_polygons(h, c["ref_payload"], slice_plane=(pos, nrm))
        want = O.cell_polygons(cells[keep], c["ref_payload"])
        for k in want:
            assert np.array_equal(got[k], want[k]), (name, k)


@pytest.mark.parametrize("mode", ["triangles", "boundary"])
def test_writer_on_other_soups_matches_reference(tmp_path, golden_cases, mode):
    c = golden_cases["random_full"]
    h = ref_headers(c)
    nb = int((c["f_adjs"] == 1).sum())
    s = O.cell_polygons(h, c["ref_payload"], triangulate=mode == "triangles",
                        boundary_only=mode == "boundary", max_sf_fid=nb - 1)
    ref = B.ref_bgeo_bytes(s["points"], s["poly_offsets"], s["indices"], s["poly_site"], tmp_path)
    if ref is None:
        pytest.skip("reference sources not present")
    assert B.bgeo_bytes(s["points"], s["poly_offsets"], s["indices"], s["poly_site"]) == ref


def test_no_points_is_refused(tmp_path):
    """The reference writer throws on a geometry without points; the oracle
    raises (and rpd_write_polygons_bgeo returns an error)."""
    empty = (np.zeros((0, 3), np.float32), np.zeros(1, np.int64), np.zeros(0, np.uint32),
             np.zeros(0, np.int32))
    with pytest.raises(ValueError):
        B.bgeo_bytes(*empty)
    try:
        ref = B.ref_bgeo_bytes(*empty, tmp_path)
    except RuntimeError:
        return  # the reference refused too
    if ref is None:
        pytest.skip("reference sources not present")
    raise AssertionError("the reference wrote a file without points")
