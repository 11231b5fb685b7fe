"""The dist2mat oracle (libmat's ClosestDistanceToLocalMat,
src/dist2mat/dist2mat.cu) in float64: its closed-form cone and slab distances
against an independent convex minimisation, known answers, and the
reference's choice among equal minima."""
import numpy as np

from oracle import dist2mat_oracle as D


def _sphere(rng):
    return np.r_[rng.uniform(0, 1, 3), rng.uniform(0.02, 0.12)]


def test_closed_forms_are_the_minimum():
    rng = np.random.default_rng(0)
    n = 0
    while n < 150:
        m1, m2, m3 = _sphere(rng), _sphere(rng), _sphere(rng)
        # medial primitives: no sphere inside another
        if not all(abs(a[3] - b[3]) < 0.9 * np.linalg.norm(a[:3] - b[:3])
                   for a, b in ((m1, m2), (m1, m3), (m2, m3))):
            continue
        p = rng.uniform(-0.2, 1.2, 3)
        assert abs(D.cone_d(p, m1, m2) - D.numeric_cone_d(p, m1, m2)) < 1e-9
        assert abs(D.slab_d(p, m1, m2, m3) - D.numeric_slab_d(p, m1, m2, m3)) < 1e-8
        n += 1


def test_known_answers():
    s1 = np.array([0.0, 0.0, 0.0, 0.2])
    s2 = np.array([1.0, 0.0, 0.0, 0.2])
    s3 = np.array([0.0, 1.0, 0.0, 0.2])
    assert D.sphere_d(np.zeros(3), s1) == -0.2
    # equal radii: a tube around the segment / a thickened triangle
    assert abs(D.cone_d(np.array([0.5, 0.7, 0.0]), s1, s2) - 0.5) < 1e-12
    assert abs(D.slab_d(np.array([0.25, 0.25, 0.9]), s1, s2, s3) - 0.7) < 1e-12
    # beyond the end the nearest sphere counts
    assert abs(D.cone_d(np.array([2.0, 0.0, 0.0]), s1, s2) - 0.8) < 1e-12


def test_index_choice_among_equal_minima():
    sph = np.array([[0.0, 0, 0, 0.1], [1.0, 0, 0, 0.1]])
    # primitives 0 and 33 (lanes 0 and 1) and 32 (lane 0 again) all at the
    # same distance: lane 0 keeps its first (0), lane 1 its 33; the last
    # lane with the minimum wins
    prims = np.array([[-1, -1, 0]] * 40)
    prims[1:32] = [-1, -1, 1]
    prims[34:] = [-1, -1, 1]
    d, i, _ = D.dist2mat(sph, np.zeros((1, 3)), np.array([0]), np.array([40]), prims)
    assert d[0] == -0.1 and i[0] == 33
    d, i, _ = D.dist2mat(sph, np.zeros((1, 3)), np.array([0]), np.array([0]), prims)
    assert d[0] == 1e16 and i[0] == -1
