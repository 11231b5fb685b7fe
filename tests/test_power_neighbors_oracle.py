"""The oracle's power-neighbour lists (the stand-in for libmat's CGAL regular
triangulation, src/rpd3d_base/triangulation.cxx:62-144, :442-558) against an
independent construction of the same triangulation: the lower convex hull of
the sites lifted to (x, y, z, |x|^2 - w) (scipy's Qhull), whose edges join
exactly the power neighbours.  With the region far larger than the sites'
spread every face of every cell lies inside it, so the two must agree; known
answers (a lattice, a hidden sphere, two sites) pin the edge cases."""
import itertools

import numpy as np
import pytest

from oracle import oracle as O


def lifted_hull_neighbours(s4):
    spatial = pytest.importorskip("scipy.spatial")
    x = s4[:, :3].astype(np.float64)
    lift = np.c_[x, (x * x).sum(1) - s4[:, 3].astype(np.float64)]
    hull = spatial.ConvexHull(lift)
    nb = [set() for _ in range(len(s4))]
    on_hull = set()
    for simplex, eq in zip(hull.simplices, hull.equations):
        if eq[3] >= 0:  # upper hull
            continue
        for a, b in itertools.combinations(simplex, 2):
            nb[a].add(int(b))
            nb[b].add(int(a))
        on_hull.update(int(v) for v in simplex)
    return nb, on_hull


def test_random_sites_match_the_lifted_hull():
    spatial = pytest.importorskip("scipy.spatial")
    rng = np.random.default_rng(5)
    n = 300
    xyz = rng.uniform(100, 900, size=(n, 3))
    r = rng.uniform(5, 110, size=n)
    s4 = np.c_[xyz, r * r].astype(np.float32)
    nbr, cnt = O.power_neighbors(s4, [-1e5] * 3, [1e5] * 3, max_nbr=128)
    hull_nb, on_hull = lifted_hull_neighbours(s4)
    # sites on the convex hull of the centres have unbounded cells, whose
    # faces can reach beyond any region: for them the region's neighbours
    # are a subset of the triangulation's
    outer = set(spatial.ConvexHull(s4[:, :3].astype(np.float64)).vertices.tolist())
    n_inner = 0
    for i in range(n):
        if i not in on_hull:
            assert cnt[i] == -1, i  # hidden: not a vertex of the triangulation
            continue
        assert cnt[i] >= 0, i
        got = set(nbr[i, :cnt[i]].tolist())
        if i in outer:
            assert got <= hull_nb[i], i
        else:
            assert got == hull_nb[i], i
            n_inner += 1
        assert np.all(np.diff(nbr[i, :cnt[i]]) > 0)
        assert np.all(nbr[i, cnt[i]:] == -1)
    assert n_inner > 150
    assert (cnt == -1).sum() > 0  # the radii hide some spheres


def test_lattice_cells_are_cubes():
    g = np.stack(np.meshgrid(*[np.arange(5.0)] * 3, indexing="ij"), -1).reshape(-1, 3)
    s4 = np.c_[100 + 100 * g, np.full(len(g), 25.0)].astype(np.float32)
    nbr, cnt = O.power_neighbors(s4, [0] * 3, [600] * 3)
    for i, p in enumerate(g):
        want = sum(1 for a in range(3) for d in (-1, 1) if 0 <= p[a] + d <= 4)
        assert cnt[i] == want, (i, cnt[i])
        for j in nbr[i, :cnt[i]]:
            assert np.abs(g[j] - p).sum() == 1


def test_hidden_sphere_and_pair():
    big = np.array([[0, 0, 0], [100, 0, 0], [0, 100, 0], [0, 0, 100]], np.float64)
    c = big.mean(0)
    s4 = np.r_[np.c_[big, np.full(4, 90.0 ** 2)], [[*c, 1.0]]].astype(np.float32)
    nbr, cnt = O.power_neighbors(s4, [-200] * 3, [300] * 3)
    assert cnt[4] == -1  # dominated everywhere by the four heavy spheres
    assert all(4 not in nbr[i, :cnt[i]] for i in range(4))
    two = np.array([[0, 0, 0, 0], [10, 0, 0, 0]], np.float32)
    nbr, cnt = O.power_neighbors(two, [-50] * 3, [50] * 3)
    assert cnt.tolist() == [1, 1] and nbr[0, 0] == 1 and nbr[1, 0] == 0
