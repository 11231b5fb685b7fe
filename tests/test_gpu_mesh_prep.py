"""Mesh preparation done on the device by rpd_set_mesh (bounding box,
volume, FP64 tet radii, radius classes) against numpy on the same mesh.

The reference derives the same quantities on the host (the bounding box and
grid set-up of src/rpd3d/voronoi.cu:324-415); the radius classes are this
implementation's split of the candidate search and only have to cover every
tet with its class's largest radius exact."""
import numpy as np
import pytest

from libmat_gb300 import rpd
from libmat_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _radii(vert, tets):
    p = vert[tets]                      # n x 4 x 3
    cen = p.mean(axis=1, keepdims=True)
    return np.sqrt(((p - cen) ** 2).sum(axis=2)).max(axis=1)


def _volume(vert, tets):
    a, b, c, d = (vert[tets[:, i]] for i in range(4))
    return np.abs(np.einsum("ij,ij->i", np.cross(b - a, c - a), d - a)).sum() / 6.0


@pytest.mark.parametrize("which", ["ellipsoid", "cube", "rotated"])
def test_mesh_info_matches_numpy(which):
    if which == "ellipsoid":
        cfg = W.config_ellipsoid(target_tets=60_000, n_site=500, seed=4)
    elif which == "cube":
        cfg = W.config_small_cube(n=12, n_site=200, seed=4)
    else:
        cfg = W.batch_mesh(7)
    vert, tets = cfg["vert3d"], cfg["tets"]
    adj = rpd.mesh_adjacency(vert.shape[0], tets)
    with rpd.RPD(knn_k=32) as r:
        r.set_mesh(vert, tets, adj["v_adjs"], adj["e_adj6"], adj["f_adjs"], adj["f_ids"])
        info = r.mesh_info()
    assert info["n_vert"] == vert.shape[0] and info["n_tet"] == tets.shape[0]
    assert np.array_equal(np.array(info["lo"]), vert.min(axis=0))
    assert np.array_equal(np.array(info["hi"]), vert.max(axis=0))
    # block partial sums are added in any order: 1e-12 relative
    vol = _volume(vert, tets)
    assert abs(info["volume"] - vol) <= 1e-12 * vol
    rad = _radii(vert, tets)
    assert abs(info["tet_radius"] - rad.max()) <= 1e-12 * rad.max()
    cc, cr = info["class_count"], info["class_radius"]
    assert cc[0] + cc[1] == tets.shape[0]
    # the small-radius class holds at least 99.5% of the tets
    assert cc[0] >= int(np.ceil(0.995 * tets.shape[0]))
    # each class's radius is the largest radius of its tets
    assert np.sum(rad <= cr[0] * (1 + 1e-12)) == cc[0]
    if cc[1]:
        assert abs(cr[1] - rad.max()) <= 1e-12 * rad.max()
        assert cr[1] > cr[0]
