"""CPU oracle of the learned analysis form's network (test infrastructure
only: the tests compare the CUDA training and inference kernels against it;
the product never calls it).

The network of umd-letkf_gb300/csrc/lgpu_mlp.cu restated in float64 numpy:
three dense layers din -> H -> H -> dout, GELU (erf form) between them,
parameters and the input rounded to BF16 (round to nearest even), hidden
activations rounded to BF16 after GELU, loss = mean squared error over rows
and outputs.  The gradient treats the BF16 roundings as identities (the
straight-through convention the training kernels follow).  The network has
no counterpart in the reference (UMD-LETKF solves every column exactly).
"""
import numpy as np
from scipy.special import erf


def bf16(x):
    """Round float32 values to BF16 (nearest, ties to even), as float32."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    u = (u + 0x7FFF + lsb) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).reshape(x.shape)


def split(params, din, hidden, dout):
    shapes = [(hidden, din), (hidden,), (hidden, hidden), (hidden,), (dout, hidden), (dout,)]
    out, o = [], 0
    for s in shapes:
        n = int(np.prod(s))
        out.append(params[o:o + n].reshape(s))
        o += n
    assert o == params.size
    return out


def gelu(z):
    return 0.5 * z * (1.0 + erf(z / np.sqrt(2.0)))


def gelu_grad(z):
    return 0.5 * (1.0 + erf(z / np.sqrt(2.0))) + z * np.exp(-0.5 * z * z) / np.sqrt(2.0 * np.pi)


def forward(params, x, hidden, dout, rounding=True):
    din = x.shape[1]
    r = bf16 if rounding else (lambda a: np.asarray(a, np.float32))
    W1, b1, W2, b2, W3, b3 = [r(p).astype(np.float64) for p in split(np.asarray(params, np.float32), din, hidden, dout)]
    X = r(x).astype(np.float64)
    Z1 = X @ W1.T + b1
    H1 = r(gelu(Z1).astype(np.float32)).astype(np.float64) if rounding else gelu(Z1)
    Z2 = H1 @ W2.T + b2
    H2 = r(gelu(Z2).astype(np.float32)).astype(np.float64) if rounding else gelu(Z2)
    Y = H2 @ W3.T + b3
    return dict(X=X, W1=W1, W2=W2, W3=W3, Z1=Z1, H1=H1, Z2=Z2, H2=H2, Y=Y)


def loss_grad(params, x, t, hidden, dout, rounding=True):
    f = forward(params, x, hidden, dout, rounding)
    rows = x.shape[0]
    d = f["Y"] - np.asarray(t, np.float64)
    loss = float(np.mean(d * d))
    dY = 2.0 * d / (rows * dout)
    gW3 = dY.T @ f["H2"]
    gb3 = dY.sum(0)
    dZ2 = (dY @ f["W3"]) * gelu_grad(f["Z2"])
    gW2 = dZ2.T @ f["H1"]
    gb2 = dZ2.sum(0)
    dZ1 = (dZ2 @ f["W2"]) * gelu_grad(f["Z1"])
    gW1 = dZ1.T @ f["X"]
    gb1 = dZ1.sum(0)
    grad = np.concatenate([g.ravel() for g in (gW1, gb1, gW2, gb2, gW3, gb3)])
    return loss, grad, f["Y"]
