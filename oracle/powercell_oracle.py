"""Oracle of libmat's get_all_voro_info (test infrastructure only).

Restates src/rpd3d_base/rpd_update.cxx:80-340 with Python dicts and sets,
one power cell (site) at a time over its convex cells in ascending cell id,
on the packed cell records and their per-cell topology (oracle.cell_topology),
then flattens the maps in the device view's order (rpd_power_cells_view):
per site ascending, then key, then cell.  Positions and face centroids are
float32, one rounding per operation: compute_vertex_coordinates
(src/rpd3d_base/voronoi_defs.cxx:33-74, include/common_cxx.h:128-135) and
get_cell_v2surffid's running float sum and division (rpd_update.cxx:20-42).
The feature-edge records follow rpd_update.cxx:206-254 with
convert_e_lfids_to_lvids (:44-67), the map TetMesh::tet_es2fe_map given as
records (tet, lf_min, lf_max, fe_type, fe_id, fe_line_id) in insertion
order (a later record with the same key replaces an earlier one).
"""
import numpy as np

from . import oracle as O

F = np.float32


def _det2(a11, a12, a21, a22):
    return F(a11 * a22) - F(a12 * a21)


def _det3(a11, a12, a13, a21, a22, a23, a31, a32, a33):
    return F(F(a11 * _det2(a22, a23, a32, a33)) - F(a21 * _det2(a12, a13, a32, a33))) + \
        F(a31 * _det2(a12, a13, a22, a23))


def _vertex(pl, t):
    a, b, c = pl[t[0]], pl[t[1]], pl[t[2]]
    x = -_det3(a[3], a[1], a[2], b[3], b[1], b[2], c[3], c[1], c[2])
    y = -_det3(a[0], a[3], a[2], b[0], b[3], b[2], c[0], c[3], c[2])
    z = -_det3(a[0], a[1], a[3], b[0], b[1], b[3], c[0], c[1], c[3])
    w = _det3(a[0], a[1], a[2], b[0], b[1], b[2], c[0], c[1], c[2])
    with np.errstate(all="ignore"):
        return F(x / w), F(y / w), F(z / w)


def _cell(h, payload, th, rec):
    a = lambda x: (x + 15) // 16 * 16  # noqa: E731
    nv, np_, ne = int(h["nb_v"]), int(h["nb_p"]), int(h["nb_e"])
    o = int(h["offset"])
    pl = payload[o:o + 16 * np_].view(np.float32).reshape(-1, 4)
    o2 = o + 16 * np_
    id2 = payload[o2:o2 + 8 * np_].view(np.int32).reshape(-1, 2)
    o3 = o2 + a(8 * np_)
    ver = payload[o3:o3 + 4 * nv].reshape(-1, 4)
    o4 = o3 + a(4 * nv)
    edge = payload[o4:o4 + 4 * ne].reshape(-1, 4)
    t = int(th["offset"])
    act = rec[t + 4 * np_:t + 5 * np_]
    acte = rec[t + 6 * np_:t + 6 * np_ + ne]
    faces = rec[t + 6 * np_ + ne:t + 6 * np_ + ne + 3 * nv]
    face = {}
    pos = 0
    for p in range(np_):
        if act[p]:
            face[p] = [int(x) for x in faces[pos:pos + act[p]]]
            pos += act[p]
    return dict(nv=nv, np=np_, ne=ne, pl=pl, id2=id2, ver=ver, edge=edge, act=act, acte=acte,
                face=face, null=bool(th["flags"] & 1))


SE, CE = 1, 2  # EdgeType (src/inputs/input_types.h:13-17)


def _cc(to_visit, neighbors):
    """get_CC_given_neighbors (include/common_cxx.h:447-488): breadth-first
    from the smallest unvisited id, neighbours in ascending order, only
    those in to_visit; returns the components (sets) in discovery order."""
    from collections import deque
    inside, visited, left, out = set(to_visit), set(), set(to_visit), []
    while left:
        queue, one = deque([min(left)]), set()
        while queue:
            c = queue.popleft()
            if c in visited:
                continue
            visited.add(c)
            left.discard(c)
            one.add(c)
            for nb in sorted(neighbors.get(c, ())):
                if nb in inside:
                    queue.append(nb)
        out.append(one)
    return out


def power_cells(cells, payload, n_site, max_sf_fid, feature_edges=None, surface=None):
    """cells: emitted cells (HEADER_DTYPE, output order); feature_edges:
    (m, 6) int records or None; surface: (facet_adj (n_faces, 3), no_cross
    pairs (m, 2)) or None.  Returns the arrays of rpd_power_cells_view."""
    fe = {}
    if feature_edges is not None:
        for r in np.asarray(feature_edges, np.int64).reshape(-1, 6):
            fe[(int(r[0]), int(r[1]), int(r[2]))] = (int(r[3]), int(r[4]), int(r[5]))
    h = np.ascontiguousarray(cells[cells["status"] == O.SUCCESS])
    th, rec = O.cell_topology(h, payload)
    n = h.shape[0]
    by_site = [[] for _ in range(n_site)]
    for q in range(n):
        by_site[int(h["site_id"][q])].append(q)
    nbrs = [set() for _ in range(n)]
    tfids = [set() for _ in range(n)]
    facets, edges, verts, surf = [], [], {}, {}
    se_cov, ce_cov, se_end = [set() for _ in range(n)], [set() for _ in range(n)], {}
    cell_cc, facet_cc, edge_cc = np.zeros(n, np.int32), {}, {}
    for s in range(n_site):
        facet_neigh_to_cells, tfid_to_cells, edge_2endvertices = {}, {}, {}
        for q in by_site[s]:  # ascending cell id
            c = _cell(h[q], payload, th[q], rec)
            pl, id2, ver = c["pl"], c["id2"], c["ver"]
            for p in range(c["np"]):
                if c["act"][p] <= 0:
                    continue
                hx, hy = int(id2[p][0]), int(id2[p][1])
                if hy != -1:
                    facet_neigh_to_cells.setdefault(hy if hx == s else hx, set()).add(q)
                else:
                    if hx <= max_sf_fid and not c["null"]:
                        cx = cy = cz = F(0.0)
                        for lv in c["face"][p]:
                            x, y, z = _vertex(pl, ver[lv])
                            cx, cy, cz = F(cx + x), F(cy + y), F(cz + z)
                        k = F(len(c["face"][p]))
                        surf.setdefault(q, []).append((hx, (F(cx / k), F(cy / k), F(cz / k))))
                    tfid_to_cells.setdefault(hx, set()).add(q)
                    tfids[q].add(hx)
            for vid in range(c["nv"]):
                seeds, sfid = set(), -1
                for i in range(3):
                    hx, hy = (int(x) for x in id2[ver[vid][i]])
                    if hy != -1:
                        seeds.add(hy if hx == s else hx)
                    elif hx <= max_sf_fid:
                        sfid = hx
                if len(seeds) < 2:
                    continue
                if len(seeds) == 2:
                    seeds.add(-1)
                verts[(q, vid)] = (sorted(seeds), _vertex(pl, ver[vid]), sfid)
            for e in range(c["ne"]):
                if c["acte"][e] <= 0:
                    continue
                ex, ey = int(c["edge"][e][0]), int(c["edge"][e][1])
                h1, h2 = id2[ex], id2[ey]
                if h1[1] == -1 and h2[1] == -1:  # an edge of the tet
                    lf = (min(ex, ey), max(ex, ey))
                    info = fe.get((int(h["tet_id"][q]), lf[0], lf[1]))
                    if info is None:
                        continue
                    # the two smallest vertices on both faces' cycles
                    common = sorted(set(c["face"][lf[0]]) & set(c["face"][lf[1]]))
                    lv = (common + [-1, -1])[:2]
                    covered = (q, lv[0], lv[1], info[2], info[1])
                    if info[0] == SE:
                        se_cov[q].add(covered)
                    elif info[0] == CE:
                        ce_cov[q].add(covered)
                    for lvid in lv:
                        if lvid < 0:
                            continue
                        for i in range(3):
                            hp = id2[ver[lvid][i]]
                            if hp[1] == -1:
                                continue
                            nb = int(hp[1]) if int(hp[0]) == s else int(hp[0])
                            se_end[(q, lvid, nb, info[2])] = _vertex(pl, ver[lvid])
                            break
                if h1[1] == -1 or h2[1] == -1:
                    continue
                n1 = int(h1[1]) if int(h1[0]) == s else int(h1[0])
                n2 = int(h2[1]) if int(h2[0]) == s else int(h2[0])
                key = tuple(sorted((n1, n2)))
                ends = sorted(set(c["face"][ex]) & set(c["face"][ey]))
                edge_2endvertices.setdefault(key, []).append((q, ends[0], ends[1]))
        for fid, cs in tfid_to_cells.items():
            if len(cs) == 2:
                c1, c2 = sorted(cs)
                nbrs[c1].add(c2)
                nbrs[c2].add(c1)
        # update_pc_cc_info, update_pc_facet_cc_info (components sorted by
        # size, stably: libstdc++'s std::sort on at most 16 elements),
        # update_pc_edge_cc_info (rpd_update.cxx:454-530)
        site_nbrs = {q: nbrs[q] for q in by_site[s]}
        for j, comp in enumerate(_cc(by_site[s], site_nbrs)):
            for q in comp:
                cell_cc[q] = j
        for neigh, cs in facet_neigh_to_cells.items():
            for j, comp in enumerate(sorted(_cc(cs, site_nbrs), key=len)):
                for q in comp:
                    facet_cc[(s, neigh, q)] = j
        for key, rows in edge_2endvertices.items():
            for j, comp in enumerate(_cc({q for q, _, _ in rows}, site_nbrs)):
                for q in comp:
                    edge_cc[(s, key, q)] = j
        for neigh in sorted(facet_neigh_to_cells):
            for q in sorted(facet_neigh_to_cells[neigh]):
                facets.append(((s << 32) | neigh, q))
        for key in sorted(edge_2endvertices):
            for q, a, b in edge_2endvertices[key]:
                edges.append((s, key[0], key[1], q, a, b, 0))
    out = {}
    out["site_cell_off"] = np.cumsum([0] + [len(x) for x in by_site]).astype(np.int64)
    out["site_cells"] = np.array([q for x in by_site for q in x], np.uint32)
    out["cell_nbr_off"] = np.cumsum([0] + [len(x) for x in nbrs]).astype(np.int64)
    out["cell_nbrs"] = np.array([c for x in nbrs for c in sorted(x)], np.int32)
    out["cell_tfid_off"] = np.cumsum([0] + [len(x) for x in tfids]).astype(np.int64)
    out["cell_tfids"] = np.array([f for x in tfids for f in sorted(x)], np.int32)
    out["facet_keys"] = np.array([k for k, _ in facets], np.uint64)
    out["facet_cells"] = np.array([q for _, q in facets], np.uint32)
    out["cell_cc"] = cell_cc
    out["facet_cc"] = np.array([facet_cc[(k >> 32, k & 0xffffffff, q)] for k, q in facets], np.int32)
    out["edge_cc"] = np.array([edge_cc[(e[0], (e[1], e[2]), e[3])] for e in edges], np.int32)
    fs = np.array([k >> 32 for k, _ in facets], np.int64)
    out["site_facet_off"] = np.searchsorted(fs, np.arange(n_site + 1)).astype(np.int64)
    out["edges"] = np.array(edges, np.int32).reshape(-1, 7)
    out["site_edge_off"] = np.searchsorted(out["edges"][:, 0], np.arange(n_site + 1)).astype(np.int64)
    vk = sorted(verts)
    out["vertex_cell"] = np.array([q for q, _ in vk], np.int32)
    out["vertex_lvid"] = np.array([v for _, v in vk], np.int32)
    out["vertex_ids"] = np.array([verts[k][0] for k in vk], np.int32).reshape(-1, 3)
    out["vertex_pos"] = np.array([verts[k][1] for k in vk], np.float32).reshape(-1, 3)
    out["vertex_sfid"] = np.array([verts[k][2] for k in vk], np.int32)
    out["cell_vertex_off"] = np.searchsorted(out["vertex_cell"], np.arange(n + 1)).astype(np.int64)
    sk = sorted(surf)
    out["surface_cell"] = np.array([q for q in sk for _ in surf[q]], np.int32)
    out["surface_fid"] = np.array([f for q in sk for f, _ in surf[q]], np.int32)
    out["surface_pos"] = np.array([p for q in sk for _, p in surf[q]], np.float32).reshape(-1, 3)
    out["cell_surface_off"] = np.searchsorted(out["surface_cell"], np.arange(n + 1)).astype(np.int64)
    # update_sphere_surf_v2fids (rpd_update.cxx:342-405): per sphere its
    # surface faces (the last record of each face, cells ascending), grouped
    # over the surface mesh's face adjacency without crossing sharp edges
    rec_at, k = {}, 0
    for q in sk:
        for j in range(len(surf[q])):
            rec_at[(q, j)] = k
            k += 1
    sfg = []
    if surface is not None:
        fadj = np.asarray(surface[0]).reshape(-1, 3)
        no_cross = {(min(int(a), int(b)), max(int(a), int(b))) for a, b in np.asarray(surface[1]).reshape(-1, 2)}
        for s_ in range(n_site):
            fid2rec = {}
            for q in by_site[s_]:
                for j, (fid, _) in enumerate(surf.get(q, [])):
                    fid2rec[fid] = rec_at[(q, j)]
            fids = set(fid2rec)
            nb = {}
            for f in sorted(fids):
                if f >= fadj.shape[0]:
                    continue
                for nf in fadj[f]:
                    nf = int(nf)
                    if nf < 0 or (min(f, nf), max(f, nf)) in no_cross or nf not in fids:
                        continue
                    nb.setdefault(f, set()).add(nf)
            for j, comp in enumerate(_cc(fids, nb)):
                for f in sorted(comp):
                    sfg.append((s_, j, f, fid2rec[f]))
    sfg = np.array(sfg, np.int64).reshape(-1, 4)
    out["site_sfg_off"] = np.searchsorted(sfg[:, 0], np.arange(n_site + 1)).astype(np.int64)
    out["sfg_group"] = sfg[:, 1].astype(np.int32)
    out["sfg_fid"] = sfg[:, 2].astype(np.int32)
    out["sfg_record"] = sfg[:, 3].astype(np.int32)
    for name, cov in (("se_covered", se_cov), ("ce_covered", ce_cov)):
        out["cell_%s_off" % name] = np.cumsum([0] + [len(x) for x in cov]).astype(np.int64)
        out[name] = np.array([r for x in cov for r in sorted(x)], np.int32).reshape(-1, 5)
    ek = sorted(se_end)
    out["se_line_end"] = np.array(ek, np.int32).reshape(-1, 4)
    out["se_line_end_pos"] = np.array([se_end[k] for k in ek], np.float32).reshape(-1, 3)
    out["cell_se_line_end_off"] = np.searchsorted(out["se_line_end"][:, 0],
                                                  np.arange(n + 1)).astype(np.int64)
    return out
