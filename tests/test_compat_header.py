"""The header-only shim include/rpd_gb300_compat.hpp compiles against libmat's
own ConvexCellHost (src/rpd3d_base/voronoi_defs.h) -- the type it fills,
topology members included -- when the reference sources are present."""
import os
import subprocess

import pytest

from oracle.build import REF_ROOT
from tests.conftest import ROOT

TU = r"""
#include "voronoi_defs.h"
#include "rpd_gb300_compat.hpp"
// instantiate the entry point with the reference's own types
auto* entry = &compute_clipped_voro_diagram_GPU;
"""


def test_compat_shim_compiles_against_reference_types(tmp_path):
    inc = os.path.join(REF_ROOT, "src", "rpd3d_base")
    if not os.path.exists(os.path.join(inc, "voronoi_defs.h")):
        pytest.skip("reference sources not present")
    src = tmp_path / "tu.cpp"
    src.write_text(TU)
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-I" + os.path.join(REF_ROOT, "include"),
                        "-I" + inc, "-I" + os.path.join(ROOT, "include"), str(src)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
