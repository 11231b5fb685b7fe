"""Generates the golden fixtures of tests/golden/ from the reference itself.

Each case runs libmat's own clipping kernel (src/rpd3d/convex_cell.cu,
compiled for the CPU by oracle/build.py into oracle/_ref/) on seeded inputs
and stores inputs, candidate pairs and the reference's cells.  Needs the
reference sources, so it runs in the development container only; the .npz
files it writes are committed and travel with the tests.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from libmat_gb300 import workloads as W  # noqa: E402
from oracle import oracle as O  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def sites_from(xyz, r, scale=1.0):
    return np.concatenate([xyz * scale, ((r * scale) ** 2)[:, None]], axis=1)


def cases():
    # 1. small random cube, complete neighbour lists
    c = W.random_small(n_cube=4, n_site=40, seed=0)
    yield "random_full", c, 39, "id"
    # 2. the small plain config shape at reduced size, k = 64 nearest
    c = W.config_small_cube(n=8, n_site=200, seed=1)
    yield "cube_k64", c, 64, "id"
    # 3. same, lists in distance order (clip order differs from id order)
    yield "cube_k64_distorder", c, 64, "dist"
    # 4. lattice sites with equal radii: cospherical ties, det == 0 cases
    vert, tets = W.cube_grid_mesh(4)
    g = (np.arange(4) + 0.5) / 4
    z, y, x = np.meshgrid(g, g, g, indexing="ij")
    xyz = np.stack([x.ravel(), y.ravel(), z.ravel()], 1)
    c = dict(vert3d=vert * 1000, tets=tets,
             sites=sites_from(xyz, np.full(64, 0.02), 1000.0),
             flags=np.ones(64, np.uint32))
    yield "lattice_ties", c, 63, "id"
    # 5. one big cube (6 tets) with many sites: plane/vertex/edge overflow
    rng = np.random.default_rng(5)
    vert, tets = W.cube_grid_mesh(1)
    xyz = rng.uniform(0, 1, size=(400, 3))
    r = rng.uniform(0.0, 0.02, size=400)
    c = dict(vert3d=vert * 1000, tets=tets, sites=sites_from(xyz, r, 1000.0),
             flags=np.ones(400, np.uint32))
    yield "overflow", c, 200, "id"
    # 6. duplicated sites (identical planes), some sites not flagged,
    #    and -1 holes inside neighbour lists
    rng = np.random.default_rng(6)
    vert, tets = W.cube_grid_mesh(3)
    xyz = rng.uniform(0.05, 0.95, size=(30, 3))
    r = rng.uniform(0.01, 0.06, size=30)
    xyz = np.concatenate([xyz, xyz[:5]])
    r = np.concatenate([r, r[:5]])
    flags = np.ones(35, np.uint32)
    flags[rng.choice(35, 6, replace=False)] = 0
    c = dict(vert3d=vert * 1000, tets=tets, sites=sites_from(xyz, r, 1000.0),
             flags=flags)
    yield "dups_flags_holes", c, 34, "holes"


def make(name, c, k, order):
    adj = O.mesh_adjacency(c["vert3d"].shape[0], c["tets"])
    s4f = c["sites"].astype(np.float32)
    nbr, _ = O.knn(s4f, k)
    if order == "id":
        nbr = np.sort(nbr, axis=1)
    elif order == "holes":
        nbr = np.sort(nbr, axis=1)
        rng = np.random.default_rng(7)
        for i in range(0, nbr.shape[0], 3):
            nbr[i, rng.integers(k // 2, k)] = -1
    offs, ps = O.candidate_pairs(c["vert3d"].astype(np.float32), c["tets"], s4f,
                                 c["flags"], nbr)
    mesh = dict(vert3d=c["vert3d"], tets=c["tets"],
                **{x: adj[x] for x in ("v_adjs", "e_adj6", "f_adjs", "f_ids")})
    h, p, tids = O.ref_clip_cells(mesh, c["sites"], c["flags"], nbr, offs, ps)
    np.savez_compressed(
        os.path.join(OUT, name + ".npz"),
        vert3d=c["vert3d"], tets=c["tets"], sites=c["sites"], flags=c["flags"],
        nbr=nbr, v_adjs=adj["v_adjs"], e_adj6=adj["e_adj6"],
        f_adjs=adj["f_adjs"], f_ids=adj["f_ids"], tet_offsets=offs,
        pair_sites=ps, ref_headers=h.view(np.uint8).reshape(-1, 32),
        ref_payload=p, ref_thread_ids=tids)
    print(name, "pairs", len(ps), "statuses", np.bincount(h["status"] + 1))


if __name__ == "__main__":
    if O.ref_lib() is None:
        raise SystemExit("reference sources not present")
    for args in cases():
        make(*args)
