"""rpd_copy_cells_to_host_async + rpd_synchronize: the queued copy lands the
same cells as the blocking copy, and two contexts used in turn (one's copy
in flight while the other uploads and computes) give every step's cells."""
import numpy as np
import pytest

from libmat_gb300 import rpd
from libmat_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def same_cells(h1, p1, h2, p2):
    """Equal cells of two computes: headers but the payload offset (taken
    from an atomic cursor), and each cell's record bytes."""
    if h1.shape != h2.shape:
        return False
    for f in h1.dtype.names:
        if f != "offset" and not np.array_equal(h1[f], h2[f]):
            return False
    for q in range(h1.shape[0]):
        n = rpd.payload_bytes(int(h1["nb_v"][q]), int(h1["nb_p"][q]), int(h1["nb_e"][q]))
        a = p1[int(h1["offset"][q]):int(h1["offset"][q]) + n]
        b = p2[int(h2["offset"][q]):int(h2["offset"][q]) + n]
        if not np.array_equal(a, b):
            return False
    return True


def engine(cfg):
    adj = rpd.mesh_adjacency(cfg["vert3d"].shape[0], cfg["tets"])
    r = rpd.RPD(certify=True)
    r.set_mesh(cfg["vert3d"], cfg["tets"], adj["v_adjs"], adj["e_adj6"], adj["f_adjs"],
               adj["f_ids"])
    r.set_sites(cfg["sites"], cfg["flags"])
    return r, adj


def test_async_copy_equals_blocking_copy():
    cfg = W.config_ellipsoid(target_tets=30000, n_site=1500, seed=61)
    r, _ = engine(cfg)
    with r:
        st = r.compute()
        h0, p0 = r.cells()
        hb = rpd.PinnedArray((st.n_cells + 16,), rpd.HEADER_DTYPE)
        pb = rpd.PinnedArray((st.payload_bytes + 64,), np.uint8)
        h1, p1 = r.cells_async(hb.array, pb.array)
        r.synchronize()
        assert h1.shape == h0.shape and p1.shape == p0.shape
        assert np.array_equal(h1, h0) and np.array_equal(p1, p0)
        with pytest.raises(rpd.RPDError):  # same capacity checks as the blocking copy
            r.cells_async(hb.array[:1], pb.array)
        hb.free()
        pb.free()


def test_two_contexts_in_turn():
    cfgs = [W.config_ellipsoid(target_tets=20000, n_site=1000 + 100 * i, seed=70 + i)
            for i in range(4)]
    want = []
    for cfg in cfgs:
        r, _ = engine(cfg)
        with r:
            r.compute()
            h, p = r.cells()
            want.append((h.copy(), p.copy()))
    ctx = [rpd.RPD(certify=True), rpd.RPD(certify=True)]
    bufs = [(rpd.PinnedArray((200000,), rpd.HEADER_DTYPE),
             rpd.PinnedArray((64 << 20,), np.uint8)) for _ in range(2)]
    got = [None] * len(cfgs)
    pending = [None, None]
    for i, cfg in enumerate(cfgs):
        r = ctx[i % 2]
        hb, pb = bufs[i % 2]
        if pending[i % 2] is not None:  # the previous copy on this context
            j, hv, pv = pending[i % 2]
            r.synchronize()
            got[j] = (hv.copy(), pv.copy())
        adj = rpd.mesh_adjacency(cfg["vert3d"].shape[0], cfg["tets"])
        r.set_mesh(cfg["vert3d"], cfg["tets"], adj["v_adjs"], adj["e_adj6"], adj["f_adjs"],
                   adj["f_ids"])
        r.set_sites(cfg["sites"], cfg["flags"])
        r.compute()
        hv, pv = r.cells_async(hb.array, pb.array)
        pending[i % 2] = (i, hv, pv)
    for k in range(2):
        j, hv, pv = pending[k]
        ctx[k].synchronize()
        got[j] = (hv.copy(), pv.copy())
    for (h, p), (hw, pw) in zip(got, want):
        assert same_cells(h, p, hw, pw)
    for r in ctx:
        r.close()
    for hb, pb in bufs:
        hb.free()
        pb.free()
