"""Generates tests/golden/dist2mat_ref.npz from the reference itself: libmat's
own dist2mat distance functions (src/dist2mat/dist2mat.cu:5-193, compiled for
the CPU by oracle/build.py into oracle/_ref/librefd2m.so, with the kernel's
per-sample selection rule) on seeded inputs.  Needs the reference sources,
so it runs in the development container only; the .npz it writes is
committed and travels with the tests.

    python tests/golden/make_golden_dist2mat.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from tests.helpers import dist2mat_workload  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))

# (name, seed, radius levels): random radii, and few distinct radii so that
# the equal-radius branches of the cone and slab formulas are taken
CASES = [("random", 5, 0), ("levels", 6, 3)]


def main():
    out = {}
    for name, seed, levels in CASES:
        sph, smp, offs, cnts, prims = dist2mat_workload(seed, n_smp=300, radius_levels=levels)
        res = O.ref_dist2mat(sph, smp, offs, cnts, prims)
        if res is None:
            raise SystemExit("the reference sources (or nvcc) are not available")
        d, c = res
        for k, v in dict(spheres=sph, samples=smp, offsets=offs, counts=cnts, prims=prims,
                         dist=d, closest=c).items():
            out["%s_%s" % (name, k)] = v
    np.savez_compressed(os.path.join(OUT, "dist2mat_ref.npz"), **out)
    print("wrote", os.path.join(OUT, "dist2mat_ref.npz"))


if __name__ == "__main__":
    main()
