"""The allocation-free compaction entry point, rpd_compact_cells_noalloc.

Callers that cannot allocate device memory while they run (work recorded
into a stream they do not own, a memory pool that owns the whole device,
code where cudaMalloc would synchronise) use this entry point with their own
buffers; its temporary lives in a fixed array inside the library.  Checked
through the C ABI against the compaction inside rpd_compute, on two calls in
a row (the second call reuses the array the first one left behind).  Kept in
a file of its own that pytest collects last.
"""
import ctypes

import numpy as np
import pytest

from libmat_gb300 import rpd
from libmat_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def test_noalloc_compaction_matches_rpd_compute():
    torch = pytest.importorskip("torch")
    L = rpd.load()
    cfg = W.config_small_cube(n=10, n_site=500, seed=12)
    adj = rpd.mesh_adjacency(cfg["vert3d"].shape[0], cfg["tets"])
    with rpd.RPD(neighbor_source=rpd.NEIGH_KNN, knn_k=48) as r:
        r.set_mesh(cfg["vert3d"], cfg["tets"], adj["v_adjs"], adj["e_adj6"], adj["f_adjs"],
                   adj["f_ids"])
        r.set_sites(cfg["sites"], cfg["flags"])
        st = r.compute()
        want, _ = r.cells()
        want_status = np.array(st.status_counts[:10], np.int64)
        view = r.view()
        n_pairs = int(view.n_pairs)
        assert n_pairs > 1000 and len(want) > 0
        # the caller's own device buffers (allocated before the calls)
        out = torch.zeros(n_pairs * 32, dtype=torch.uint8, device="cuda")
        n_out = torch.zeros(1, dtype=torch.int64, device="cuda")
        hist = torch.zeros(11, dtype=torch.int64, device="cuda")
        stream = torch.cuda.current_stream().cuda_stream
        for call in range(2):
            out.fill_(0xAB)
            torch.cuda.synchronize()
            s = L.rpd_compact_cells_noalloc(ctypes.c_void_p(view.pair_headers), n_pairs,
                                            ctypes.c_void_p(out.data_ptr()),
                                            ctypes.c_void_p(n_out.data_ptr()),
                                            ctypes.c_void_p(hist.data_ptr()),
                                            ctypes.c_void_p(stream))
            assert s == 0, "call %d returned %d" % (call, s)
            torch.cuda.synchronize()
            n = int(n_out.item())
            assert n == len(want), call
            got = out[: n * 32].cpu().numpy().view(rpd.HEADER_DTYPE)
            assert got.tobytes() == want.tobytes(), call
            assert np.array_equal(hist.cpu().numpy()[:10], want_status), call
            assert int(hist[10].item()) == 0, call  # no payload-full cells, as rpd_compute
        # without the status histogram: the same compacted records
        out.fill_(0xAB)
        torch.cuda.synchronize()
        s = L.rpd_compact_cells_noalloc(ctypes.c_void_p(view.pair_headers), n_pairs,
                                        ctypes.c_void_p(out.data_ptr()),
                                        ctypes.c_void_p(n_out.data_ptr()), None,
                                        ctypes.c_void_p(stream))
        assert s == 0
        torch.cuda.synchronize()
        assert int(n_out.item()) == len(want)
        assert out[: len(want) * 32].cpu().numpy().tobytes() == want.tobytes()
        # no pairs: no cells, an all-zero histogram (the array still holds the
        # previous call's counts)
        n_out.fill_(-1)
        hist.fill_(7)
        s = L.rpd_compact_cells_noalloc(None, 0, None, ctypes.c_void_p(n_out.data_ptr()),
                                        ctypes.c_void_p(hist.data_ptr()), ctypes.c_void_p(stream))
        assert s == 0
        torch.cuda.synchronize()
        assert int(n_out.item()) == 0
        assert not hist.cpu().numpy().any()
        # beyond the fixed array: rejected before any launch
        s = L.rpd_compact_cells_noalloc(ctypes.c_void_p(view.pair_headers), (1 << 25) + 1,
                                        ctypes.c_void_p(out.data_ptr()),
                                        ctypes.c_void_p(n_out.data_ptr()), None,
                                        ctypes.c_void_p(stream))
        assert s == 5  # RPD_ERR_CAPACITY
