"""The dist2mat oracle pinned to the reference: libmat's own distance
functions (src/dist2mat/dist2mat.cu:5-193), compiled for the CPU from its
sources, with the selection rule of ClosestDistanceToLocalMat (:195-270).
The oracle's float32 evaluation (one rounding per operation, the
reference's double literals widened where its source widens them) must
equal them bit for bit -- distances and closest indices -- on random inputs
and on inputs whose spheres take few radii (the equal-radius branches), and
on the committed golden vectors made by the reference build (which the GPU
test holds the device to as well)."""
import os

import numpy as np
import pytest

from oracle import dist2mat_oracle as D
from oracle import oracle as O
from tests.helpers import dist2mat_workload

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "dist2mat_ref.npz")


def golden_cases():
    g = np.load(GOLDEN)
    names = sorted({k.split("_")[0] for k in g.files})
    return [(n, {k[len(n) + 1:]: g[k] for k in g.files if k.startswith(n + "_")}) for n in names]


@pytest.mark.parametrize("seed,levels", [(0, 0), (1, 0), (2, 4), (3, 2)])
def test_float32_oracle_equals_reference_build(seed, levels):
    sph, smp, offs, cnts, prims = dist2mat_workload(seed, radius_levels=levels)
    ref = O.ref_dist2mat(sph, smp, offs, cnts, prims)
    if ref is None:
        pytest.skip("reference sources not available")
    rd, ri = ref
    fd, fi, _ = D.dist2mat(sph, smp, offs, cnts, prims, dtype=np.float32)
    assert np.array_equal(rd, fd.astype(np.float32))
    assert np.array_equal(ri, fi.astype(np.int32))


def test_float32_oracle_equals_golden_vectors():
    for name, c in golden_cases():
        fd, fi, _ = D.dist2mat(c["spheres"], c["samples"], c["offsets"], c["counts"], c["prims"],
                               dtype=np.float32)
        assert np.array_equal(c["dist"], fd.astype(np.float32)), name
        assert np.array_equal(c["closest"], fi.astype(np.int32)), name
        assert (c["counts"] == 0).any() and (c["counts"] > 32).any()  # empty and multi-lane lists
