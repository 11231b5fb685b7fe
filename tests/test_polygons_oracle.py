"""Polygon soup (libmat's Houdini export, get_one_convex_cell_faces_const,
src/IO/IO_CUDA/io_cuda.cxx:21-141): the oracle's restatement against the
reference's own face cycles (golden topology fixtures made by
src/rpd3d_base/voronoi_defs.cxx, the same walk) and the reference's float
vertex formula."""
import numpy as np

from oracle import oracle as O
from tests.helpers import SUCCESS, cell_planes_ver, float_vertices, ref_headers


def test_polygons_are_the_reference_face_cycles(golden_cases):
    for name, c in golden_cases.items():
        h = ref_headers(c)
        cells = h[h["status"] == SUCCESS]
        poly = O.cell_polygons(h, c["ref_payload"])
        th = c["topo_headers"].reshape(-1).view(O.TOPO_DTYPE)
        rec = c["topo_records"]
        row, pi, pts = 0, 0, []
        for q in range(cells.shape[0]):
            nv, np_, ne = int(cells["nb_v"][q]), int(cells["nb_p"][q]), int(cells["nb_e"][q])
            pl, ver = cell_planes_ver(c["ref_payload"], cells["offset"][q], nv, np_)
            pts.append(float_vertices(pl, ver))
            o = int(th["offset"][q])
            act = rec[o + 4 * np_:o + 5 * np_]
            faces = rec[o + 6 * np_ + ne:o + 6 * np_ + ne + 3 * nv]
            pos = 0
            for p in range(np_):
                if act[p] == 0:
                    continue
                a, b = poly["poly_offsets"][pi], poly["poly_offsets"][pi + 1]
                assert np.array_equal(poly["indices"][a:b] - row, faces[pos:pos + act[p]]), name
                pos += act[p]
                pi += 1
            row += nv
        assert pi == len(poly["poly_site"]), name
        assert np.array_equal(poly["points"], np.concatenate(pts)), name


def test_triangles_and_boundary_filter(golden_cases):
    c = golden_cases["cube_k64"]
    h = ref_headers(c)
    full = O.cell_polygons(h, c["ref_payload"])
    lens = np.diff(full["poly_offsets"])
    tri = O.cell_polygons(h, c["ref_payload"], triangulate=True)
    assert len(tri["poly_site"]) == int((lens - 2).sum())
    assert np.all(np.diff(tri["poly_offsets"]) == 3)
    # fans: every triangle's first point is its polygon's first point
    first = np.repeat(full["indices"][full["poly_offsets"][:-1]], lens - 2)
    assert np.array_equal(tri["indices"][0::3], first)
    assert np.array_equal(tri["poly_site"], np.repeat(full["poly_site"], lens - 2))
    # boundary only: bisector faces plus tet faces with face id below the bound
    nb = int((c["f_adjs"] == 1).sum())  # boundary faces are numbered first
    bnd = O.cell_polygons(h, c["ref_payload"], boundary_only=True, max_sf_fid=nb)
    keep = (full["poly_adj_site"] != -1)
    assert len(bnd["poly_site"]) > keep.sum()
    assert len(bnd["poly_site"]) < len(full["poly_site"])
    assert np.array_equal(bnd["points"], full["points"])
