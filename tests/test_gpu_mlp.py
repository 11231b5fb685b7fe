"""The learned list length on the GPU: the bf16 tensor-core forward and
gradient kernels against the CPU oracle, training, and certified clipping
with predicted list lengths (cells identical to the plain path's, misses
re-clipped, and what the network gains over one list length for all)."""
import numpy as np
import pytest

from libmat_gb300 import rpd
from libmat_gb300 import workloads as W
from oracle import mlp_oracle as M
from tests.test_mlp_oracle import random_params

pytestmark = pytest.mark.gpu


def engine(cfg, **kw):
    adj = rpd.mesh_adjacency(cfg["vert3d"].shape[0], cfg["tets"])
    r = rpd.RPD(neighbor_source=rpd.NEIGH_KNN, **kw)
    r.set_mesh(cfg["vert3d"], cfg["tets"], adj["v_adjs"], adj["e_adj6"], adj["f_adjs"], adj["f_ids"])
    r.set_sites(cfg["sites"], cfg["flags"])
    return r


def random_rows(rng, n):
    X = rng.normal(0, 1.5, (n, 16))
    X[:, 12:] = 0.0
    bits = M.bf16_bits(X)
    return bits, M.bf16_value(bits)


@pytest.mark.parametrize("n", [16, 1000, 4099])
def test_forward_matches_oracle(n):
    rng = np.random.default_rng(n)
    p = random_params(rng).astype(np.float32)
    bits, X = random_rows(rng, n)
    with rpd.RPD(certify=True) as r:
        r.mlp_set_params(p)
        y = r.mlp_forward(bits)
    want, _ = M.forward(p.astype(np.float64), X, rounding=True)
    # fp32 accumulation on the tensor cores vs float64, same bf16 roundings
    assert np.max(np.abs(y - want)) <= 2e-3 * (1 + np.max(np.abs(want)))


@pytest.mark.parametrize("n", [64, 1000])
def test_gradient_matches_oracle(n):
    rng = np.random.default_rng(100 + n)
    p = random_params(rng).astype(np.float32)
    bits, X = random_rows(rng, n)
    t = rng.normal(3, 1, n).astype(np.float32)
    with rpd.RPD(certify=True) as r:
        r.mlp_set_params(p)
        g, loss = r.mlp_gradient(bits, t)
    want_loss, want = M.loss_and_grad(p.astype(np.float64), X, t.astype(np.float64), rounding=True)
    assert abs(loss - want_loss) <= 1e-4 * want_loss + 1e-6
    gb, wb = M.blocks(g.astype(np.float64)), M.blocks(want)
    for name in wb:
        err = np.linalg.norm(gb[name] - wb[name])
        assert err <= 3e-3 * np.linalg.norm(wb[name]) + 1e-7, (name, err)


def _train(r_cfgs, samples_per_mesh, epochs=15, miss=0.02, seed=0):
    """Collects labelled cells of each training input, trains, returns the
    parameters, margin and report."""
    with engine(r_cfgs[0], knn_k=64, certify=True) as r:
        for i, cfg in enumerate(r_cfgs):
            if i > 0:
                adj = rpd.mesh_adjacency(cfg["vert3d"].shape[0], cfg["tets"])
                r.set_mesh(cfg["vert3d"], cfg["tets"], adj["v_adjs"], adj["e_adj6"],
                           adj["f_adjs"], adj["f_ids"])
                r.set_sites(cfg["sites"], cfg["flags"])
            n = r.mlp_collect(samples_per_mesh)
        rep = r.mlp_train(epochs=epochs, batch=256, lr=2e-3, miss_target=miss, seed=seed)
        p, m = r.mlp_params()
    return p, m, rep, n


@pytest.fixture(scope="module")
def trained():
    train = [W.config_ellipsoid(target_tets=40000, n_site=2000, seed=s) for s in (31, 32)]
    return _train(train, 30000)


def test_training_learns(trained):
    p, m, rep, n = trained
    assert n >= 40000 and rep.n_train + rep.n_calib == n
    assert np.all(np.isfinite(p))
    assert rep.loss_last < rep.loss_first
    # well below the error of predicting the mean label, on held-out cells
    assert rep.calib_loss < 0.75 * rep.label_var
    # the held-out miss rate is the requested one (quantile margin)
    assert rep.calib_miss_rate <= 0.03
    # what the network gains: at the same miss rate, shorter lists than the
    # one length that serves every cell
    assert rep.calib_mean_k < 0.8 * rep.const_k


def test_learned_lengths_keep_plain_cells(trained):
    p, m, rep, _ = trained
    cfg = W.config_ellipsoid(target_tets=40000, n_site=2000, seed=33)  # unseen seed
    with engine(cfg, knn_k=64, predicate_mode=rpd.PRED_FP64) as r:
        sp = r.compute()
        hp = r.pair_headers()
        tp = r.topology_hashes()
    with engine(cfg, knn_k=64, certify=True, learned_k=True) as r:
        r.mlp_set_params(p, m)
        sl = r.compute()
        hl = r.pair_headers()
        tl = r.topology_hashes()
        klen = r.mlp_klen()
        feats = r.mlp_features()
    assert sl.learned == 1
    assert sp.n_pairs == sl.n_pairs == klen.shape[0] == feats.shape[0]
    assert np.array_equal(hp["status"], hl["status"])
    assert np.array_equal(tp, tl)
    assert np.all(klen >= 1) and np.all(klen <= 64)
    assert np.all(feats[:, 12:] == 0)
    # misses on an unseen mesh stay near the calibrated rate
    assert sl.n_reclipped <= 0.08 * sl.n_pairs
    assert klen.mean() < rep.const_k


def test_learned_requires_predictor():
    cfg = W.config_small_cube(n=6, n_site=150, seed=34)
    with engine(cfg, knn_k=40, certify=True, learned_k=True) as r:
        with pytest.raises(rpd.RPDError):
            r.compute()
        r.mlp_enable(False)
        r.compute()


def test_repass_counts_with_and_without_the_network(trained):
    """Both re-passes, with the network and without it, on one unseen mesh
    with exact lists: the network's misses (cells whose predicted length did
    not certify, clipped again with the whole list) are its only extra
    re-pass; the cells left uncertified by their whole base list -- and so
    the exact-lists re-clip -- are the same set either way, as are the
    emitted cells."""
    p, m, _, _ = trained
    cfg = W.config_ellipsoid(target_tets=40000, n_site=2000, seed=35)
    runs = {}
    for net in (False, True):
        with engine(cfg, knn_k=32, certify=True, learned_k=net, exact_lists=True) as r:
            if net:
                r.mlp_set_params(p, m)
            st = r.compute()
            runs[net] = (st, r.pair_headers(), r.topology_hashes())
    (s0, h0, t0), (s1, h1, t1) = runs[False], runs[True]
    assert s0.learned == 0 and s1.learned == 1
    assert s0.n_uncertified == 0 and s1.n_uncertified == 0
    # without the network there is no first-pass re-clip
    assert s0.n_reclipped == 0
    assert 0 < s1.n_reclipped <= 0.08 * s1.n_pairs
    # the exact-lists re-pass does real work at k = 32 and is the same
    assert s0.n_cert_reclipped > 0
    assert s1.n_cert_reclipped == s0.n_cert_reclipped
    assert s1.n_extended_sites == s0.n_extended_sites
    assert np.array_equal(h0["status"], h1["status"])
    assert np.array_equal(t0, t1)
