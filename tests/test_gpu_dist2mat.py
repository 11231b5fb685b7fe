"""libmat's dist2mat on the device (rpd_dist2mat) against the float64
oracle of ClosestDistanceToLocalMat (src/dist2mat/dist2mat.cu): distances
within float tolerance, the closest primitive wherever the minimum is not a
near tie, the reference's index rule, empty lists, and rejected ids."""
import numpy as np
import pytest

from libmat_gb300 import rpd
from oracle import dist2mat_oracle as D

pytestmark = pytest.mark.gpu


def workload(seed, n_sph=300, n_smp=400, max_prims=80):
    """Random medial spheres in the unit cube, samples near them, per sample
    a list of spheres, cones and slabs over nearby spheres (no sphere of a
    primitive inside another)."""
    rng = np.random.default_rng(seed)
    c = rng.uniform(0, 1, (n_sph, 3))
    r = rng.uniform(0.01, 0.05, n_sph)
    sph = np.c_[c, r].astype(np.float32)
    smp = (c[rng.integers(0, n_sph, n_smp)] + rng.normal(0, 0.05, (n_smp, 3))).astype(np.float32)
    offs, cnts, prims = [], [], []
    for s in range(n_smp):
        near = np.argsort(np.linalg.norm(c - smp[s], axis=1))[:12]
        n = int(rng.integers(0, max_prims + 1)) if s % 17 else 0
        offs.append(len(prims))
        cnts.append(n)
        for _ in range(n):
            kind = rng.integers(0, 3)
            while True:
                a, b, cc = rng.choice(near, 3, replace=False)
                ok = all(abs(r[u] - r[v]) < 0.9 * np.linalg.norm(c[u] - c[v])
                         for u, v in ((a, b), (a, cc), (b, cc)))
                if ok:
                    break
            prims.append([-1, -1, a] if kind == 0 else ([-1, a, b] if kind == 1 else [a, b, cc]))
    return sph, smp, np.array(offs, np.uint32), np.array(cnts, np.uint32), np.array(prims, np.int32)


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
    # the same float32 expressions, one rounding per operation: bit for bit
    # on nearly every sample (a few slabs that cancel differ in the last
    # bits), and the same primitive
    f32 = fd.astype(np.float32)
    assert np.mean(dist[ne] == f32[ne]) > 0.99
    assert np.all(np.abs(dist[ne] - f32[ne]) <= 2e-5 * np.maximum(np.abs(f32[ne]), 1e-2))
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
