"""GPU: the eigensolve + transform stage (k_eig, through lgpu_debug_transform)
on crafted Gram matrices against float64 numpy: random SPD cases over a
range of conditioning, no observations (G = 0), rank-one and rank-two
updates with very large weights (many co-located observations), fewer
observations than members.

Bar: the float64 eigendecomposition of the float32 packed input is the
target; the allowed relative error is the larger of 2e-5, four times the
error of float32 LAPACK (numpy's eigh on the float32 matrix, the precision
of the reference's REAL eigensolver) on the same input, and 2*eps32*kappa:
a backward-stable float32 eigensolver perturbs the eigenvalues by about
eps32*|A|, which moves sqrt((k-1)/lambda) of the smallest eigenvalues by
about eps32*kappa/2 relative (kappa = condition number of G + (k-1)I); the
rank-one cases with 131073 co-located observations reach kappa ~ 2e5."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def pack(G, b):
    k = G.shape[0]
    iu = np.triu_indices(k)
    return np.concatenate([G[iu], b]).astype(np.float32)


def transform64(G, b):
    k = G.shape[0]
    A = G.astype(np.float64) + (k - 1) * np.eye(k)
    lam, V = np.linalg.eigh(A)
    W = (V * np.sqrt((k - 1) / lam)) @ V.T
    wbar = (V / lam) @ (V.T @ b.astype(np.float64))
    return W + wbar[:, None]


def transform32(G, b):
    k = G.shape[0]
    A = (G + (k - 1) * np.eye(k)).astype(np.float32)
    lam, V = np.linalg.eigh(A)
    W = (V * np.sqrt(np.float32(k - 1) / lam)) @ V.T
    wbar = (V / lam) @ (V.T @ b.astype(np.float32))
    return W + wbar[:, None]


def cases(k, rng):
    out = []
    for n, scale in ((3 * k, 1.0), (10 * k, 10.0), (200, 100.0), (k // 2, 1.0)):
        Y = rng.standard_normal((k, n))
        Y -= Y.mean(0)
        w = rng.random(n) * scale
        out.append(((Y * w) @ Y.T, (Y * w) @ rng.standard_normal(n)))
    out.append((np.zeros((k, k)), np.zeros(k)))                     # no observations
    y = rng.standard_normal(k)
    y -= y.mean()
    out.append((131073.0 * np.outer(y, y), 131073.0 * y * 0.7))       # co-located observations
    y2 = rng.standard_normal(k)
    y2 -= y2.mean()
    out.append((131073.0 * (np.outer(y, y) + np.outer(y2, y2)), 131073.0 * (0.3 * y - 0.2 * y2)))
    return out


# every width of the register-resident first stage (k rounded up to 8: one
# warp up to 48, a team of ceil(k / 32) warps above) and both replay teams
@pytest.mark.parametrize("k", [5, 12, 20, 28, 33, 40, 47, 56, 64, 65, 77, 88, 96, 100, 105, 117, 128])
def test_transform_against_float64(k):
    from letkf_gb300 import Solver
    rng = np.random.default_rng(k)
    cs = cases(k, rng)
    packed = np.stack([pack(G, b) for G, b in cs])
    with Solver(0) as s:
        T = s.debug_transform(packed)
    bad = []
    for ci, ((G, b), t) in enumerate(zip(cs, T)):
        # the float32 packed input is the reference's input
        Gi = np.zeros((k, k))
        iu = np.triu_indices(k)
        Gi[iu] = pack(G, b)[: len(iu[0])]
        Gi = Gi + np.triu(Gi, 1).T
        bi = pack(G, b)[len(iu[0]):]
        ref = transform64(Gi, bi)
        assert np.all(np.isfinite(t))
        scale = max(1.0, np.abs(ref).max())
        err = np.abs(t - ref).max() / scale
        err32 = np.abs(transform32(Gi, bi) - ref).max() / scale
        lam = np.linalg.eigvalsh(Gi + (k - 1) * np.eye(k))
        tol = max(2e-5, 4.0 * err32, 2.0 * 5.96e-8 * lam[-1] / lam[0])
        if not err < tol:
            bad.append((ci, err, err32, tol))
    assert not bad, (k, bad)
