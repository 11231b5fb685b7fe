"""CPU oracle of the k-predictor MLP (test infrastructure only).

float64 restatement of the network the engine trains on the GPU
(libmat_gb300/csrc/rpd_mlp.cu): 16 bf16 inputs -> 64 -> 64 -> 1, ReLU,
squared error.  With ``rounding=True`` it rounds to bf16 at the points where
the GPU kernels feed the tensor cores (inputs, the two weight matrices, the
hidden activation h1, and the back-propagated dz2 / dz1), everything else in
float64; with ``rounding=False`` it is the plain float64 network, whose
analytic gradient the tests check against central finite differences.

The reference has no learned component; nothing here follows a reference
file.

Parameter layout (fp32 vector of 5313): W1 [16][64] (feature x hidden),
b1 [64], W2 [64][64] (in x out), b2 [64], w3 [64], b3.
"""
import numpy as np

NF, NH = 16, 64
N_PARAMS = NF * NH + NH + NH * NH + NH + NH + 1


def bf16_round(x):
    """Round to the nearest bf16 (ties to even) through float32, as
    __float2bfloat16_rn does for finite values."""
    f = np.asarray(x, np.float32)
    b = f.view(np.uint32).astype(np.uint64)
    r = ((b + 0x7FFF + ((b >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def bf16_bits(x):
    """bf16 bit patterns (uint16) of float values."""
    f = np.asarray(bf16_round(x), np.float32)
    return (f.view(np.uint32) >> 16).astype(np.uint16)


def bf16_value(bits):
    """float64 values of bf16 bit patterns."""
    b = np.asarray(bits, np.uint16).astype(np.uint32) << 16
    return b.view(np.float32).astype(np.float64)


def unpack(params):
    p = np.asarray(params, np.float64)
    assert p.shape == (N_PARAMS,)
    o = 0
    W1 = p[o:o + NF * NH].reshape(NF, NH); o += NF * NH
    b1 = p[o:o + NH]; o += NH
    W2 = p[o:o + NH * NH].reshape(NH, NH); o += NH * NH
    b2 = p[o:o + NH]; o += NH
    w3 = p[o:o + NH]; o += NH
    b3 = p[o]
    return W1, b1, W2, b2, w3, b3


def pack(W1, b1, W2, b2, w3, b3):
    return np.concatenate([np.ravel(W1), b1, np.ravel(W2), b2, w3, [b3]]).astype(np.float64)


def _rnd(x, rounding):
    return bf16_round(x) if rounding else np.asarray(x, np.float64)


def forward(params, X, rounding=True):
    """X: (n, 16) float64 values (already bf16 when rounding).  Returns y and
    the intermediates."""
    W1, b1, W2, b2, w3, b3 = unpack(params)
    W1r, W2r = _rnd(W1, rounding), _rnd(W2, rounding)
    Xr = _rnd(X, rounding)
    z1 = Xr @ W1r + b1
    h1 = _rnd(np.maximum(z1, 0.0), rounding)
    z2 = h1 @ W2r + b2
    a2 = np.maximum(z2, 0.0)
    y = a2 @ w3 + b3
    return y, dict(X=Xr, z1=z1, h1=h1, z2=z2, a2=a2, W1r=W1r, W2r=W2r)


def loss_and_grad(params, X, target, rounding=True):
    """Mean squared error over the rows and its gradient (parameter layout)."""
    W1, b1, W2, b2, w3, b3 = unpack(params)
    y, c = forward(params, X, rounding)
    n = X.shape[0]
    d = y - np.asarray(target, np.float64)
    loss = float(np.mean(d * d))
    dy = 2.0 * d / n
    gb3 = dy.sum()
    gw3 = c["a2"].T @ dy
    dz2 = np.outer(dy, w3) * (c["z2"] > 0)
    gb2 = dz2.sum(0)
    dz2r = _rnd(dz2, rounding)
    gW2 = c["h1"].T @ dz2r
    dh1 = dz2r @ c["W2r"].T
    dz1 = dh1 * (c["z1"] > 0)
    gb1 = dz1.sum(0)
    gW1 = c["X"].T @ _rnd(dz1, rounding)
    return loss, pack(gW1, gb1, gW2, gb2, gw3, gb3)


def finite_difference(params, X, target, idx, eps=1e-6):
    """Central differences of the float64 loss for parameter indices idx."""
    p = np.asarray(params, np.float64).copy()
    out = []
    for i in idx:
        old = p[i]
        p[i] = old + eps
        lp, _ = loss_and_grad(p, X, target, rounding=False)
        p[i] = old - eps
        lm, _ = loss_and_grad(p, X, target, rounding=False)
        p[i] = old
        out.append((lp - lm) / (2 * eps))
    return np.array(out)


def blocks(vec):
    """Named parameter blocks of a parameter-layout vector."""
    W1, b1, W2, b2, w3, b3 = unpack(vec)
    return {"W1": W1, "b1": b1, "W2": W2, "b2": b2, "w3": w3, "b3": np.array([b3])}
