"""Generates the per-cell topology fixtures tests/golden/<case>_topo.npz.

For each golden case it takes the reference's own cells stored in
<case>.npz (made by make_golden.py) and runs libmat's own host-side cell
topology on them -- ConvexCellHost::reload_active, reload_pc_explicit,
cal_cell_euler and cal_halfplane_facet_euler from
src/rpd3d_base/voronoi_defs.cxx, compiled for the CPU by oracle/build.py into
oracle/_ref/libreftopo.so -- and stores the topology headers and records of
the emitted cells.  Needs the reference sources, so it runs in the
development container only; the .npz files travel with the tests.

    python tests/golden/make_golden_topology.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def main():
    for f in sorted(os.listdir(OUT)):
        if not f.endswith(".npz") or f.endswith("_topo.npz"):
            continue
        case = dict(np.load(os.path.join(OUT, f)))
        h = case["ref_headers"].reshape(-1).view(O.HEADER_DTYPE)
        r = O.ref_cell_topology(h, case["ref_payload"])
        if r is None:
            raise SystemExit("reference sources not found")
        th, rec = r
        name = f[:-4] + "_topo.npz"
        np.savez_compressed(os.path.join(OUT, name), topo_headers=th.view(np.uint8).reshape(-1, 16),
                            topo_records=rec)
        print(name, th.shape[0], "cells", rec.size, "bytes")


if __name__ == "__main__":
    main()
