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


def test_header_is_plain_c(tmp_path):
    """include/rpd_gb300.h compiles as C99 (a cgo / FFI binding reads it as
    C), and the structs the ctypes mirror reads have the same size and field
    offsets in C."""
    import ctypes
    import os
    import subprocess
    mirrors = {"rpd_config": rpd.Config, "rpd_mesh_info": rpd.MeshInfo,
               "rpd_power_cells_view": rpd.PowerCellsView, "rpd_stats": rpd.Stats,
               "rpd_tuning": rpd.Tuning, "rpd_mlp_report": rpd.MlpReport,
               "rpd_cells_view": rpd.CellsView}
    fields = {c: (cls, [f[0] for f in cls._fields_]) for c, cls in mirrors.items()}
    lines = ['#include "rpd_gb300.h"', "#include <stddef.h>", "#include <stdio.h>",
             "int main(void) {"]
    for cname, (_, names) in fields.items():
        lines.append('  printf("%%zu\\n", sizeof(%s));' % cname)
        for f in names:
            lines.append('  printf("%%zu\\n", offsetof(%s, %s));' % (cname, f))
    lines += ['  printf("%u\\n", RPD_CELL_UNCERTIFIED);',
              '  printf("%zu\\n", sizeof(rpd_feature_edge));', "  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I" + os.path.join(ROOT, "include"),
                        str(src), "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True,
                                          check=True).stdout.split()]
    want = []
    for _, (cls, names) in fields.items():
        want.append(ctypes.sizeof(cls))
        want += [getattr(cls, f).offset for f in names]
    want += [rpd.CELL_UNCERTIFIED, 24]
    assert out == want
