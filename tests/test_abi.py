"""The C ABI library: it builds, loads and exports every symbol declared in
include/rpd_gb300.h; host-side helpers work without a GPU."""
import re

import numpy as np

from libmat_gb300 import rpd
from libmat_gb300 import workloads as W
from oracle import oracle as O
from tests.conftest import ROOT


def declared_symbols():
    src = open(ROOT + "/include/rpd_gb300.h").read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(rpd_[a-z0-9_]+)\s*\(", src)))


def test_exports_every_declared_symbol():
    L = rpd.load()
    names = declared_symbols()
    assert len(names) >= 15
    for n in names:
        assert hasattr(L, n), n
    assert sorted(rpd.EXPORTS) == names


def test_payload_layout_matches_oracle():
    for nv, np_, ne in [(4, 4, 6), (13, 9, 21), (95, 63, 152), (1, 1, 1)]:
        assert rpd.payload_bytes(nv, np_, ne) == O.payload_bytes(nv, np_, ne)


def test_mesh_adjacency_matches_oracle():
    for cfg in (W.cube_grid_mesh(4), W.ellipsoid_mesh(3000, seed=3)):
        vert, tets = cfg
        a = rpd.mesh_adjacency(vert.shape[0], tets)
        b = O.mesh_adjacency(vert.shape[0], tets)
        for k in ("v_adjs", "e_adj6", "f_adjs", "f_ids", "n_boundary_faces"):
            assert np.array_equal(a[k], b[k]), k


def test_invalid_mesh_rejected():
    import pytest

    with pytest.raises(rpd.RPDError):
        rpd.mesh_adjacency(3, np.array([[0, 1, 2, 5]], np.int32))
