"""The k-predictor's CPU oracle: its float64 analytic gradient against
central finite differences, and its bf16 rounding against torch's."""
import numpy as np
import torch

from oracle import mlp_oracle as M


def random_params(rng, scale=1.0):
    W1 = rng.normal(0, scale * np.sqrt(2 / 12), (16, 64))
    W1[12:] = 0.0
    W2 = rng.normal(0, scale * np.sqrt(2 / 64), (64, 64))
    return M.pack(W1, rng.normal(0, 0.1, 64), W2, rng.normal(0, 0.1, 64),
                  rng.normal(0, 0.2, 64), 2.5)


def test_bf16_rounding_matches_torch():
    rng = np.random.default_rng(0)
    x = np.concatenate([rng.normal(0, 1, 20000), rng.normal(0, 1e-3, 2000),
                        [1.0, 1 + 2 ** -8, 1 + 3 * 2 ** -8, -1 - 2 ** -8, 0.0]]).astype(np.float32)
    want = torch.from_numpy(x).to(torch.bfloat16).float().numpy().astype(np.float64)
    assert np.array_equal(M.bf16_round(x), want)
    assert M.bf16_round(np.float32(1 + 2 ** -8)) == 1.0            # tie to even
    assert M.bf16_round(np.float32(1 + 3 * 2 ** -8)) == 1 + 2 ** -6
    bits = M.bf16_bits(x)
    assert np.array_equal(M.bf16_value(bits), want)


def test_analytic_gradient_matches_finite_differences():
    rng = np.random.default_rng(1)
    p = random_params(rng)
    X = rng.normal(0, 1, (40, 16))
    X[:, 12:] = 0.0
    t = rng.normal(3, 1, 40)
    _, g = M.loss_and_grad(p, X, t, rounding=False)
    # a sample of every block
    offs = {"W1": 0, "b1": 1024, "W2": 1088, "b2": 5184, "w3": 5248, "b3": 5312}
    idx = []
    for name, o in offs.items():
        size = {"W1": 768, "b1": 64, "W2": 4096, "b2": 64, "w3": 64, "b3": 1}[name]
        idx += list(o + rng.choice(size, min(size, 12), replace=False))
    fd = M.finite_difference(p, X, t, idx)
    assert np.allclose(g[idx], fd, rtol=1e-5, atol=1e-8)


def test_rounded_gradient_close_to_float64():
    """bf16 operands change the gradient by bf16-sized amounts only."""
    rng = np.random.default_rng(2)
    p = random_params(rng)
    X = M.bf16_round(rng.normal(0, 1, (256, 16)))
    t = rng.normal(3, 1, 256)
    _, g64 = M.loss_and_grad(p, X, t, rounding=False)
    _, g16 = M.loss_and_grad(p, X, t, rounding=True)
    for name, a in M.blocks(g64).items():
        b = M.blocks(g16)[name]
        assert np.linalg.norm(a - b) <= 0.05 * np.linalg.norm(a) + 1e-9, name
