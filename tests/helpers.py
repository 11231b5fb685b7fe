"""Shared helpers for the tests: golden-case unpacking and cell comparison."""
import numpy as np

from oracle import oracle as O

SUCCESS = 4


def mesh_of(case):
    return dict(vert3d=case["vert3d"], tets=case["tets"], v_adjs=case["v_adjs"],
                e_adj6=case["e_adj6"], f_adjs=case["f_adjs"], f_ids=case["f_ids"])


def ref_headers(case):
    return case["ref_headers"].reshape(-1).view(O.HEADER_DTYPE)


def section_sizes(nb_v, nb_p, nb_e):
    a = lambda x: (x + 15) // 16 * 16  # noqa: E731
    return dict(plane=16 * nb_p, id2=a(8 * nb_p), ver=a(4 * nb_v), edge=a(4 * nb_e),
                h=a(nb_p), xyz=a(24 * nb_v))


def topo_bytes(payload, off, nb_v, nb_p, nb_e):
    s = section_sizes(int(nb_v), int(nb_p), int(nb_e))
    n = s["plane"] + s["id2"] + s["ver"] + s["edge"] + s["h"]
    return payload[int(off):int(off) + n]


def xyz_of(payload, off, nb_v, nb_p, nb_e):
    s = section_sizes(int(nb_v), int(nb_p), int(nb_e))
    start = int(off) + s["plane"] + s["id2"] + s["ver"] + s["edge"] + s["h"]
    return payload[start:start + 24 * int(nb_v)].view(np.float64).reshape(-1, 3)


def compare_cells(h1, p1, h2, p2):
    """Bit-exact comparison of two packed cell sets over the same pairs:
    statuses, counts and the topology/plane bytes of every emitted cell.
    Returns the number of differing pairs."""
    assert len(h1) == len(h2)
    bad = 0
    for f in ("tet_id", "site_id", "status", "nb_v", "nb_p", "nb_e"):
        bad += int((h1[f] != h2[f]).sum())
    if bad:
        return bad
    ok = np.flatnonzero(h1["status"] == SUCCESS)
    for q in ok:
        a = topo_bytes(p1, h1["offset"][q], h1["nb_v"][q], h1["nb_p"][q], h1["nb_e"][q])
        b = topo_bytes(p2, h2["offset"][q], h2["nb_v"][q], h2["nb_p"][q], h2["nb_e"][q])
        if not np.array_equal(a, b):
            bad += 1
    return bad


def tet_volumes(vert, tets):
    a = vert[tets[:, 0]]
    return np.abs(np.einsum("ij,ij->i", np.cross(vert[tets[:, 1]] - a, vert[tets[:, 2]] - a),
                            vert[tets[:, 3]] - a)) / 6.0


M64 = (1 << 64) - 1


def mix64(z):
    z = (z + 0x9E3779B97F4A7C15) & M64
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M64
    return z ^ (z >> 31)


def topology_hash(payload, off, nb_v, nb_p, nb_e):
    """Order-independent hash of a cell's topology: sum over vertices of a
    hash of the sorted face keys of its three planes and its #adj (the
    definition the engine's rpd_copy_topology_hashes_to_host uses)."""
    s = section_sizes(int(nb_v), int(nb_p), int(nb_e))
    off = int(off)
    id2 = payload[off + s["plane"]:off + s["plane"] + 8 * int(nb_p)].view(np.int32).reshape(-1, 2)
    ver = payload[off + s["plane"] + s["id2"]:][:4 * int(nb_v)].reshape(-1, 4)
    keys = [((int(a) & 0xFFFFFFFF) << 32) | (int(b) & 0xFFFFFFFF) for a, b in id2]
    h = 0
    for t in ver:
        a, b, d = sorted((keys[t[0]], keys[t[1]], keys[t[2]]))
        hv = mix64(a)
        hv = mix64(hv ^ b)
        hv = mix64(hv ^ d)
        hv = mix64(hv ^ int(t[3]))
        h = (h + hv) & M64
    return h


def _det3(a11, a12, a13, a21, a22, a23, a31, a32, a33):
    # include/common_cxx.h:128-135, one float32 rounding per operation
    d1 = a22 * a33 - a23 * a32
    d2 = a12 * a33 - a13 * a32
    d3 = a12 * a23 - a13 * a22
    return a11 * d1 - a21 * d2 + a31 * d3


def float_vertices(pl, ver):
    """compute_vertex_coordinates of every vertex (float32, perspective
    divide), voronoi_defs.cxx:33-74.  pl: (n_p, 4) float32 planes; ver:
    (n_v, 4) uint8 dual triangles."""
    a, b, c = (pl[ver[:, i].astype(np.int64)].astype(np.float32) for i in range(3))
    x = -_det3(a[:, 3], a[:, 1], a[:, 2], b[:, 3], b[:, 1], b[:, 2], c[:, 3], c[:, 1], c[:, 2])
    y = -_det3(a[:, 0], a[:, 3], a[:, 2], b[:, 0], b[:, 3], b[:, 2], c[:, 0], c[:, 3], c[:, 2])
    z = -_det3(a[:, 0], a[:, 1], a[:, 3], b[:, 0], b[:, 1], b[:, 3], c[:, 0], c[:, 1], c[:, 3])
    w = _det3(a[:, 0], a[:, 1], a[:, 2], b[:, 0], b[:, 1], b[:, 2], c[:, 0], c[:, 1], c[:, 2])
    return np.stack([x / w, y / w, z / w], axis=1).astype(np.float32)


def cell_planes_ver(payload, off, nb_v, nb_p):
    """(planes (n_p, 4) float32, ver (n_v, 4) uint8) of one packed cell."""
    s = section_sizes(int(nb_v), int(nb_p), 0)
    o = int(off)
    pl = payload[o:o + 16 * int(nb_p)].view(np.float32).reshape(-1, 4)
    ver = payload[o + s["plane"] + s["id2"]:][:4 * int(nb_v)].reshape(-1, 4)
    return pl, ver


TET_FACE_PAIRS = [(a, b) for a in range(4) for b in range(a + 1, 4)]


def feature_edge_records(n_tet, seed, frac=0.3):
    """Seeded stand-in for TetMesh::tet_es2fe_map: (m, 6) int32 records (tet,
    lf_min, lf_max, fe_type, fe_id, fe_line_id) on about frac of the tets,
    types sharp (1), concave (2) and unknown (-1), in shuffled order, then a
    tenth of the keys again with other values (the later record counts)."""
    rng = np.random.default_rng(seed)
    recs = []
    for t in rng.choice(n_tet, size=max(1, int(frac * n_tet)), replace=False):
        for j in rng.choice(6, size=int(rng.integers(1, 4)), replace=False):
            a, b = TET_FACE_PAIRS[j]
            recs.append((t, a, b, rng.choice([1, 2, -1]), rng.integers(0, 1000), rng.integers(0, 50)))
    recs = np.array(recs, np.int64)
    recs = recs[rng.permutation(len(recs))]
    again = recs[rng.choice(len(recs), size=len(recs) // 10, replace=False)].copy()
    again[:, 3] = rng.choice([1, 2], size=len(again))
    again[:, 4] += 1000
    return np.concatenate([recs, again]).astype(np.int32)


FACE_LV = [(2, 1, 3), (0, 2, 3), (1, 0, 3), (0, 1, 2)]  # tet face f leaves out vertex f


def surface_mesh(vert, tets, f_adjs, f_ids):
    """libmat's SurfaceMesh inputs of the surface groups, from a tet mesh:
    its boundary triangles (face ids 0 .. nb - 1, numbered first), per face
    the faces across its three edges (-1 for none), and the pairs across a
    sharp edge (normals more than ~8 degrees apart) as the no-cross pairs."""
    f_adjs, f_ids = np.asarray(f_adjs), np.asarray(f_ids)
    nb = int((f_adjs == 1).sum())
    tri = np.zeros((nb, 3), np.int64)
    for t, f in zip(*np.nonzero(f_adjs == 1)):
        tri[f_ids[t, f]] = np.asarray(tets)[t, list(FACE_LV[f])]
    edge_faces = {}
    for fid in range(nb):
        for le in range(3):
            a, b = int(tri[fid, le]), int(tri[fid, (le + 1) % 3])
            edge_faces.setdefault((min(a, b), max(a, b)), []).append(fid)
    adj = -np.ones((nb, 3), np.int32)
    for fid in range(nb):
        for le in range(3):
            a, b = int(tri[fid, le]), int(tri[fid, (le + 1) % 3])
            others = [x for x in edge_faces[(min(a, b), max(a, b))] if x != fid]
            if len(others) == 1:
                adj[fid, le] = others[0]
    p = np.asarray(vert)[tri]
    nrm = np.cross(p[:, 1] - p[:, 0], p[:, 2] - p[:, 0])
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    pairs = [(f, int(g)) for f in range(nb) for g in adj[f]
             if g > f and abs(float(nrm[f] @ nrm[g])) < 0.99]
    return adj, np.array(pairs, np.int32).reshape(-1, 2)


def dist2mat_workload(seed, n_sph=300, n_smp=400, max_prims=80, radius_levels=0):
    """dist2mat inputs: random medial spheres in the unit cube, samples near
    them, per sample a list of spheres, cones and slabs over nearby spheres
    (no sphere of a primitive inside another)."""
    rng = np.random.default_rng(seed)
    c = rng.uniform(0, 1, (n_sph, 3))
    r = rng.uniform(0.01, 0.05, n_sph)
    if radius_levels:  # few distinct radii: the slab's and cone's equal-radius branches
        r = np.round(r * radius_levels / 0.05) * (0.05 / radius_levels)
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
