"""Seeded synthetic RPD workloads (tet meshes + weighted sites).

libmat normalises every mesh to [0, 1000]^3 (src/IO/IO_CXX/io.cxx:157-185,
scale_max = 1000 in src/inputs/params.h:15) and its clipper relies on that
scale (e.g. the 0.1 volume floor, src/rpd3d/convex_cell.cu:1040-1043).  The
generators below build meshes and sites in unit coordinates and return them
already mapped to that frame: v' = 1000 (v - min) / maxside, radii scaled by
1000 / maxside, weights w = r'^2.  Coordinates are float64; the float copies
used by the reference-faithful arithmetic are plain casts.
"""
import numpy as np

SCALE = 1000.0


def _orient_positive(vert, tets):
    """Swaps two vertices of every negatively oriented tet so that the face
    planes built by tri2plane point inwards (include/common_cuda.h:248-254)."""
    a, b, c, d = (vert[tets[:, i]] for i in range(4))
    vol = np.einsum("ij,ij->i", np.cross(b - a, c - a), d - a)
    neg = vol < 0
    t = tets.copy()
    t[neg, 0], t[neg, 1] = tets[neg, 1], tets[neg, 0]
    return t, np.abs(vol) / 6.0


def cube_grid_mesh(n):
    """Unit cube split into n^3 cubes of 6 tets each (Kuhn subdivision along
    the main diagonal).  Returns (vert float64 [(n+1)^3, 3], tets int32)."""
    g = np.arange(n + 1, dtype=np.float64) / n
    z, y, x = np.meshgrid(g, g, g, indexing="ij")
    vert = np.stack([x.ravel(), y.ravel(), z.ravel()], axis=1)

    def vid(i, j, k):
        return i + (n + 1) * (j + (n + 1) * k)

    i, j, k = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    i, j, k = i.ravel(), j.ravel(), k.ravel()
    e = [(1, 0, 0), (0, 1, 0), (0, 0, 1)]
    tets = []
    for perm in [(0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)]:
        p0 = (i, j, k)
        s1 = tuple(p0[a] + e[perm[0]][a] for a in range(3))
        s2 = tuple(s1[a] + e[perm[1]][a] for a in range(3))
        p3 = (i + 1, j + 1, k + 1)
        tets.append(np.stack([vid(*p0), vid(*s1), vid(*s2), vid(*p3)], axis=1))
    tets = np.stack(tets, axis=1).reshape(-1, 4).astype(np.int32)
    tets, _ = _orient_positive(vert, tets)
    return vert, tets


def ellipsoid_mesh(target_tets, axes=(1.0, 0.6, 0.4), jitter=0.2, seed=0):
    """Jittered-grid Delaunay tetrahedralisation of an ellipsoid (scipy Qhull).
    The spacing is chosen so the mesh has about target_tets tets (Delaunay of
    a jittered grid gives ~6.5 tets per point).  Near-flat hull slivers are
    removed.  Tets are positively oriented and sorted for a deterministic
    order."""
    from scipy.spatial import Delaunay

    rng = np.random.default_rng(seed)
    a, b, c = axes
    vol = 4.0 / 3.0 * np.pi * a * b * c
    n_pts = target_tets / 6.5
    h = (vol / n_pts) ** (1.0 / 3.0)
    gx = np.arange(-a, a + h, h)
    gy = np.arange(-b, b + h, h)
    gz = np.arange(-c, c + h, h)
    X, Y, Z = np.meshgrid(gx, gy, gz, indexing="ij")
    p = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
    p = p + rng.uniform(-jitter * h, jitter * h, size=p.shape)
    inside = (p[:, 0] / a) ** 2 + (p[:, 1] / b) ** 2 + (p[:, 2] / c) ** 2 <= 1.0
    p = p[inside]
    tri = Delaunay(p)
    tets = tri.simplices.astype(np.int64)
    tets, tv = _orient_positive(p, tets)
    keep = tv > 1e-3 * h ** 3
    tets = tets[keep]
    used = np.unique(tets)
    remap = np.full(p.shape[0], -1, np.int64)
    remap[used] = np.arange(used.size)
    p = p[used]
    tets = remap[tets]
    # canonical order: sorted rows, then lexicographic
    st = np.sort(tets, axis=1)
    order = np.lexsort((st[:, 3], st[:, 2], st[:, 1], st[:, 0]))
    tets = tets[order].astype(np.int32)
    return p, tets


def _normalise(vert, site_xyz, site_r):
    lo = vert.min(axis=0)
    maxside = float((vert.max(axis=0) - lo).max())
    s = SCALE / maxside
    v = (vert - lo) * s
    x = (site_xyz - lo) * s
    r = site_r * s
    return v, x, r


def _pack_sites(xyz, r):
    return np.concatenate([xyz, (r * r)[:, None]], axis=1)


def config_small_cube(n=20, n_site=2000, seed=1):
    """The 'Plain RPD, small' workload: unit cube n^3 x 6 tets, sites with
    centres U[0.05, 0.95]^3 and radii U[0.01, 0.05], w = r^2 (scaled x1000)."""
    rng = np.random.default_rng(seed)
    vert, tets = cube_grid_mesh(n)
    xyz = rng.uniform(0.05, 0.95, size=(n_site, 3))
    r = rng.uniform(0.01, 0.05, size=n_site)
    v, x, rr = _normalise(vert, xyz, r)
    return dict(vert3d=v, tets=tets, sites=_pack_sites(x, rr),
                flags=np.ones(n_site, np.uint32))


def config_slotted_cube(n=10, n_site=80, n_slot_sites=12, seed=4):
    """A non-convex domain: the n^3 x 6-tet unit cube without the tets of a
    one-cube-wide slot (x in [0.4, 0.5], y < 0.8, all z), so that power
    cells of the sites placed in the slot reach both walls and fall into
    several connected pieces.  Unused vertices are dropped."""
    rng = np.random.default_rng(seed)
    vert, tets = cube_grid_mesh(n)
    c = vert[tets].mean(axis=1)
    keep = ~((c[:, 0] > 0.4) & (c[:, 0] < 0.5) & (c[:, 1] < 0.8))
    tets = tets[keep]
    used = np.unique(tets)
    remap = np.full(vert.shape[0], -1, np.int64)
    remap[used] = np.arange(used.shape[0])
    vert, tets = vert[used], remap[tets].astype(np.int32)
    xyz = rng.uniform(0.05, 0.95, size=(n_site, 3))
    slot = np.stack([np.full(n_slot_sites, 0.45), rng.uniform(0.05, 0.7, n_slot_sites),
                     rng.uniform(0.05, 0.95, n_slot_sites)], axis=1)
    xyz = np.concatenate([xyz, slot])
    r = rng.uniform(0.01, 0.05, size=xyz.shape[0])
    v, x, rr = _normalise(vert, xyz, r)
    return dict(vert3d=v, tets=tets, sites=_pack_sites(x, rr),
                flags=np.ones(xyz.shape[0], np.uint32))


def config_ellipsoid(target_tets=1_000_000, n_site=50_000, seed=2,
                     axes=(1.0, 0.6, 0.4)):
    """The 'plain vs FP32-filtered at scale' workload: jittered-grid Delaunay
    ellipsoid (semi-axes 1.0/0.6/0.4), 70% of the sites near the surface
    (inward offset |N(0, 0.02)|) and 30% uniform inside, radii
    lognormal(ln 0.01, 0.5)."""
    rng = np.random.default_rng(seed)
    vert, tets = ellipsoid_mesh(target_tets, axes=axes, seed=seed)
    a, b, c = axes
    n_surf = int(round(0.7 * n_site))
    n_in = n_site - n_surf
    u = rng.normal(size=(n_surf, 3))
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    ps = u * np.array([a, b, c])
    nrm = ps / np.array([a * a, b * b, c * c])
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    ps = ps - np.abs(rng.normal(0.0, 0.02, size=(n_surf, 1))) * nrm
    pin = []
    while sum(len(q) for q in pin) < n_in:
        q = rng.uniform(-1, 1, size=(2 * n_in, 3)) * np.array([a, b, c])
        q = q[(q[:, 0] / a) ** 2 + (q[:, 1] / b) ** 2 + (q[:, 2] / c) ** 2 <= 1.0]
        pin.append(q)
    pin = np.concatenate(pin)[:n_in]
    xyz = np.concatenate([ps, pin])
    perm = rng.permutation(n_site)
    xyz = xyz[perm]
    r = rng.lognormal(np.log(0.01), 0.5, size=n_site)
    v, x, rr = _normalise(vert, xyz, r)
    return dict(vert3d=v, tets=tets, sites=_pack_sites(x, rr),
                flags=np.ones(n_site, np.uint32))


def config_lattice(n=100, m=50, radius=0.01, perturb_frac=0.05, sigma=1e-12,
                   seed=5):
    """Near-degenerate stress: lattice cube with n grid points per axis
    ((n-1)^3 cubes x 6 tets), m^3 sites on a lattice with equal radii, a
    fraction perturbed by N(0, sigma)."""
    rng = np.random.default_rng(seed)
    vert, tets = cube_grid_mesh(n - 1)
    g = (np.arange(m) + 0.5) / m
    z, y, x = np.meshgrid(g, g, g, indexing="ij")
    xyz = np.stack([x.ravel(), y.ravel(), z.ravel()], axis=1)
    k = int(round(perturb_frac * xyz.shape[0]))
    idx = rng.choice(xyz.shape[0], size=k, replace=False)
    xyz[idx] += rng.normal(0.0, sigma, size=(k, 3))
    r = np.full(xyz.shape[0], radius)
    v, x, rr = _normalise(vert, xyz, r)
    return dict(vert3d=v, tets=tets, sites=_pack_sites(x, rr),
                flags=np.ones(xyz.shape[0], np.uint32))


def random_small(n_cube=4, n_site=40, seed=0, r_range=(0.01, 0.08)):
    """Small random case for parity tests."""
    rng = np.random.default_rng(seed)
    vert, tets = cube_grid_mesh(n_cube)
    xyz = rng.uniform(0.0, 1.0, size=(n_site, 3))
    r = rng.uniform(r_range[0], r_range[1], size=n_site)
    v, x, rr = _normalise(vert, xyz, r)
    return dict(vert3d=v, tets=tets, sites=_pack_sites(x, rr),
                flags=np.ones(n_site, np.uint32))


def _random_rotation(rng):
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def batch_mesh(i, seed=3, tet_range=(2_000, 200_000), site_range=(100, 20_000),
               r_range=(0.005, 0.04)):
    """Mesh i of the 'batched uneven' workload: a unit cube or an ellipsoid
    (semi-axes 1.0/0.6/0.4), randomly rotated and scaled, with log-uniform
    tet and site counts, sites uniform in the volume, radii uniform; seeded
    by (seed, i).  Rotation and scale are applied before the mesh is mapped
    to [0, 1000]^3 (so they change its shape in that frame, not its size)."""
    rng = np.random.default_rng([seed, i])
    n_tet = int(np.exp(rng.uniform(np.log(tet_range[0]), np.log(tet_range[1]))))
    n_site = int(np.exp(rng.uniform(np.log(site_range[0]), np.log(site_range[1]))))
    cube = rng.uniform() < 0.5
    if cube:
        n = max(2, int(round((n_tet / 6.0) ** (1.0 / 3.0))))
        vert, tets = cube_grid_mesh(n)
        xyz = rng.uniform(0.0, 1.0, size=(n_site, 3))
    else:
        axes = np.array([1.0, 0.6, 0.4])
        vert, tets = ellipsoid_mesh(max(n_tet, 500), axes=tuple(axes), seed=int(rng.integers(1 << 30)))
        pts = []
        while sum(len(q) for q in pts) < n_site:
            q = rng.uniform(-1, 1, size=(2 * n_site, 3)) * axes
            q = q[((q / axes) ** 2).sum(axis=1) <= 1.0]
            pts.append(q)
        xyz = np.concatenate(pts)[:n_site]
    R = _random_rotation(rng) * rng.uniform(0.5, 2.0)
    vert = vert @ R.T
    xyz = xyz @ R.T
    r = rng.uniform(r_range[0], r_range[1], size=n_site) * np.abs(np.linalg.det(R)) ** (1.0 / 3.0)
    if np.linalg.det(R) < 0:  # keep tets positively oriented
        tets = tets[:, [1, 0, 2, 3]].copy()
    v, x, rr = _normalise(vert, xyz, r)
    return dict(vert3d=v, tets=tets.astype(np.int32), sites=_pack_sites(x, rr),
                flags=np.ones(n_site, np.uint32), kind="cube" if cube else "ellipsoid")


def config_batch(n_mesh=256, seed=3, **kw):
    """The 'batched uneven' workload: n_mesh independent meshes (batch_mesh)."""
    return [batch_mesh(i, seed=seed, **kw) for i in range(n_mesh)]
