"""CPU: the network oracle (oracle/mlp_oracle.py) pinned by finite
differences of its own loss (BF16 rounding off: the roundings are steps) and
its BF16 rounding against numpy's round-to-nearest-even reference values."""
import numpy as np

from oracle import mlp_oracle as M


def test_bf16_rounding_known_values():
    x = np.array([1.0, 1.00390625, 1.005859375, -2.5, 3.0e38, 1e-40, 0.0], np.float32)
    # 1 + 2^-8 is a tie between 1 and 1 + 2^-7: even -> 1; 1.005859375 rounds up
    want = np.array([1.0, 1.0, 1.0078125, -2.5, 2.9980e38, 1e-40, 0.0], np.float32)
    got = M.bf16(x)
    assert got[0] == 1.0 and got[1] == 1.0 and got[2] == np.float32(1.0078125) and got[3] == -2.5
    assert abs(got[4] - want[4]) / want[4] < 4e-3
    assert got[6] == 0.0


def test_oracle_gradient_finite_differences():
    rng = np.random.default_rng(3)
    din, hidden, dout, rows = 7, 16, 5, 11
    n = hidden * din + hidden + hidden * hidden + hidden + dout * hidden + dout
    p = (rng.standard_normal(n) * 0.3).astype(np.float64)
    x = rng.standard_normal((rows, din))
    t = rng.standard_normal((rows, dout))

    def loss(q):
        f = M.forward(q.astype(np.float32), x.astype(np.float32), hidden, dout, rounding=False)
        return float(np.mean((f["Y"] - t) ** 2))

    _, g, _ = M.loss_grad(p.astype(np.float32), x.astype(np.float32), t, hidden, dout, rounding=False)
    idx = rng.choice(n, size=40, replace=False)
    p32 = p.astype(np.float32).astype(np.float64)
    for i in idx:
        h = 1e-3
        a, b = p32.copy(), p32.copy()
        a[i] += h
        b[i] -= h
        fd = (loss(a) - loss(b)) / (2 * h)
        assert abs(fd - g[i]) <= 2e-3 * max(1.0, abs(fd)) + 1e-5, (i, fd, g[i])
