"""libmat's dist2mat on the device (rpd_dist2mat) against the float64
oracle of ClosestDistanceToLocalMat (src/dist2mat/dist2mat.cu): distances
within float tolerance, the closest primitive wherever the minimum is not a
near tie, the reference's index rule, empty lists, and rejected ids."""
import numpy as np
import pytest

from libmat_gb300 import rpd
from oracle import dist2mat_oracle as D
from tests.helpers import dist2mat_workload as workload

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed", [0, 1])
def test_dist2mat_matches_oracle(seed):
    sph, smp, offs, cnts, prims = workload(seed)
    with rpd.RPD() as r:
        dist, closest = r.dist2mat(sph, smp, offs, cnts, prims)
    od, oi, all_d = D.dist2mat(sph, smp, offs, cnts, prims)               # float64
    fd, fi, _ = D.dist2mat(sph, smp, offs, cnts, prims, dtype=np.float32)  # device arithmetic
    empty = cnts == 0
    assert np.all(dist[empty] == 1e16) and np.all(closest[empty] == -1)
    ne = ~empty
    # the same float32 expressions, one rounding per operation (the oracle
    # pinned to the reference's own functions): bit for bit, and the same
    # primitive
    f32 = fd.astype(np.float32)
    assert np.array_equal(dist[ne], f32[ne])
    assert np.array_equal(closest[ne], fi[ne])
    # against float64: within float error except where the float closed form
    # cancels (ill-conditioned slabs; the reference's float kernel shares
    # it -- the worst of these two workloads is 1.0e-2 in a unit cube)
    own = np.abs(fd - od)
    assert np.mean(own[ne] < 2e-5) > 0.98 and np.max(own[ne]) < 5e-2
    well = ne & (own < 1e-5)
    assert well[ne].mean() > 0.95
    for s in np.flatnonzero(well):
        d = np.sort(all_d[s])
        if len(d) == 1 or d[1] - d[0] > 1e-4:  # no near tie: the same primitive
            assert closest[s] == oi[s]


def test_index_rule_and_errors():
    sph = np.array([[0.0, 0, 0, 0.1], [1.0, 0, 0, 0.1]], np.float32)
    prims = np.array([[-1, -1, 0]] * 40, np.int32)
    prims[1:32] = [-1, -1, 1]
    prims[34:] = [-1, -1, 1]
    with rpd.RPD() as r:
        d, i = r.dist2mat(sph, np.zeros((2, 3), np.float32), np.array([0, 0], np.uint32),
                          np.array([40, 0], np.uint32), prims)
        assert d[0] == np.float32(-0.1) and i[0] == 33 and d[1] == 1e16 and i[1] == -1
        bad = prims.copy()
        bad[5] = [-1, -1, 2]  # sphere id out of range
        with pytest.raises(rpd.RPDError, match="out of range"):
            r.dist2mat(sph, np.zeros((1, 3), np.float32), np.array([0], np.uint32),
                       np.array([40], np.uint32), bad)
        with pytest.raises(rpd.RPDError, match="out of range"):
            r.dist2mat(sph, np.zeros((1, 3), np.float32), np.array([10], np.uint32),
                       np.array([40], np.uint32), prims)  # list past the end
        d2, i2 = r.dist2mat(sph, np.zeros((1, 3), np.float32), np.array([0], np.uint32),
                            np.array([40], np.uint32), prims)  # still usable
        assert i2[0] == 33


def test_device_pointers_match_host():
    torch = pytest.importorskip("torch")
    import ctypes

    sph, smp, offs, cnts, prims = workload(3, n_smp=200)
    with rpd.RPD() as r:
        dist_h, cl_h = r.dist2mat(sph, smp, offs, cnts, prims)
        dev = {k: torch.from_numpy(v).cuda() for k, v in
               dict(sph=sph, smp=smp, offs=offs.view(np.int32), cnts=cnts.view(np.int32),
                    prims=prims).items()}
        dist = torch.zeros(len(smp), dtype=torch.float32, device="cuda")
        cl = torch.zeros(len(smp), dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        vp = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
        st = r._L.rpd_dist2mat(r._h, vp(dev["sph"]), len(sph), vp(dev["smp"]), len(smp),
                               vp(dev["offs"]), vp(dev["cnts"]), vp(dev["prims"]), len(prims),
                               vp(dist), vp(cl), 1)
        assert st == 0
    assert np.array_equal(dist.cpu().numpy(), dist_h) and np.array_equal(cl.cpu().numpy(), cl_h)


def test_dist2mat_equals_reference_golden_vectors():
    """The device against the reference's own distance functions (golden
    vectors made by the reference compiled for the CPU,
    tests/golden/make_golden_dist2mat.py): bit for bit."""
    import os

    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                             "dist2mat_ref.npz"))
    for name in sorted({k.split("_")[0] for k in g.files}):
        c = {k[len(name) + 1:]: g[k] for k in g.files if k.startswith(name + "_")}
        with rpd.RPD() as r:
            dist, closest = r.dist2mat(c["spheres"], c["samples"], c["offsets"], c["counts"],
                                       c["prims"])
        assert np.array_equal(dist, c["dist"]), name
        assert np.array_equal(closest, c["closest"]), name
