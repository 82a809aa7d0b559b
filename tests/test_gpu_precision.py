"""GPU: precision modes of the eigensolve stage (lgpu_set_precision).

Bars (written here):
  - FP64 mode, crafted Gram blocks (test_gpu_eig's cases): the transform
    within 1e-6 relative (max norm, scaled by max(1, |T|)) of float64 numpy
    on the same float32 input -- the FP32 storage of T is the only rounding
    left -- and, on the cases where the FP32 solve errs by more than 1e-5
    (the co-located rank-one and rank-two blocks), at least 4x closer than
    the FP32 solve;
  - FP32_RESOLVE flagging: a unit with two equal relevant eigenvalues is
    flagged and re-solved in FP64 (count in the timings' fp64_units); a unit
    with separated eigenvalues, and a unit with fewer observations than
    members (whose (k-1) floor is exactly degenerate), is not; re-solved
    units reach the FP64 bar, the others are bit-identical to FP32 mode;
  - whole analyses in both modes: the parity bars of the FP32 path against
    the FP32 and FP64 oracles; FP32_RESOLVE with no flagged unit is
    bit-identical to FP32 mode.
"""
import numpy as np
import pytest

from conftest import workload
from helpers import compare, gpu_run, oracle_for, workload_cfg
from test_gpu_eig import cases, pack, transform64

pytestmark = pytest.mark.gpu


def _unpack(p, k):
    iu = np.triu_indices(k)
    G = np.zeros((k, k))
    G[iu] = p[: len(iu[0])]
    return G + np.triu(G, 1).T, p[len(iu[0]):].astype(np.float64)


def _err(t, ref):
    return np.abs(t - ref).max() / max(1.0, np.abs(ref).max())


def _transform(packed, mode, gap=1e-6):
    from letkf_gb300 import Solver
    with Solver(0) as s:
        s.set_precision(mode, gap)
        T = s.debug_transform(packed)
        return T, s.timings()


@pytest.mark.parametrize("k", [5, 20, 40, 64, 100, 128])
def test_fp64_transform(k):
    rng = np.random.default_rng(100 + k)
    cs = cases(k, rng)
    packed = np.stack([pack(G, b) for G, b in cs])
    T64, tim = _transform(packed, "fp64")
    T32, _ = _transform(packed, "fp32")
    assert tim["fp64_units"] == len(cs) and tim["precision"] == 2
    for p, t64, t32 in zip(packed, T64, T32):
        ref = transform64(*_unpack(p, k))
        e64, e32 = _err(t64, ref), _err(t32, ref)
        assert e64 <= 1e-6, (k, e64)
        if e32 > 1e-5:
            assert 4 * e64 <= e32, (k, e64, e32)


def _spectral(k, g, rng):
    Q, _ = np.linalg.qr(rng.standard_normal((k, k)))
    return (Q * g) @ Q.T, rng.standard_normal(k) * 3.0


@pytest.mark.parametrize("k", [20, 40, 100])
def test_resolve_flags_degenerate_units(k):
    rng = np.random.default_rng(200 + k)
    blocks, expect = [], []
    for rep in range(6):
        # separated relevant eigenvalues (relative gaps >= 1e-3)
        g = np.linspace(0.5, 400.0, k) + rng.uniform(0, 0.1, k)
        blocks.append(_spectral(k, g, rng)); expect.append(False)
        # fewer observations than members: rank 4, the (k-1) floor repeated k-4 times
        g = np.zeros(k); g[:4] = [300.0, 120.0, 40.0, 9.0]
        blocks.append(_spectral(k, g, rng)); expect.append(False)
        # two equal relevant eigenvalues
        g = np.linspace(0.5, 400.0, k); g[k // 2] = g[k // 2 + 1]
        blocks.append(_spectral(k, g, rng)); expect.append(True)
        # equal pair inside a low-rank spectrum
        g = np.zeros(k); g[:5] = [250.0, 80.0, 80.0, 20.0, 3.0]
        blocks.append(_spectral(k, g, rng)); expect.append(True)
    packed = np.stack([pack(G, b) for G, b in blocks])
    T32, _ = _transform(packed, "fp32")
    Tr, tim = _transform(packed, "fp32_resolve", 1e-4)
    T64, _ = _transform(packed, "fp64")
    assert tim["precision"] == 1
    assert tim["fp64_units"] == sum(expect), (tim["fp64_units"], sum(expect))
    for i, (p, flagged) in enumerate(zip(packed, expect)):
        if flagged:
            assert np.array_equal(Tr[i], T64[i]), i
            assert _err(Tr[i], transform64(*_unpack(p, k))) <= 1e-6
        else:
            assert np.array_equal(Tr[i], T32[i]), i


def _analysis(name, precision):
    cfg = workload_cfg(name)
    prob = workload(cfg["gen"]["workload"], **{k: v for k, v in cfg["gen"].items() if k != "workload"})
    gpu = gpu_run(prob, cfg["localization"], cfg["solver"], variant="plain", precision=precision)
    return cfg, prob, gpu


@pytest.mark.parametrize("name", ["c1", "c2small"])
def test_analysis_precision_modes(name):
    cfg, prob, g32 = _analysis(name, "fp32")
    _, _, gres = _analysis(name, "fp32_resolve")
    _, _, g64 = _analysis(name, "fp64")
    assert g64["timings"]["fp64_units"] == g64["timings"]["units"]
    assert g64["timings"]["fp64_ms"] > 0
    if gres["timings"]["fp64_units"] == 0:
        assert np.array_equal(gres["state"], g32["state"])
        assert np.array_equal(gres["mean"], g32["mean"])
    active = np.nonzero(prob.mask == 0)[0]
    rng = np.random.default_rng(5)
    cols = np.sort(rng.choice(active, size=min(400, len(active)), replace=False))
    o = oracle_for(prob, cfg["localization"], cfg["solver"])
    ref64 = o.run(64, cols=cols)
    pr = ref64["state"] - ref64["mean"][:, :, None]
    pn = np.sqrt(np.sum(pr.astype(np.float64) ** 2, axis=(0, 2)))
    ok = pn > 1e-6 * max(pn.max(), 1e-30)
    errs = {}
    for label, g in (("fp32", g32), ("fp32_resolve", gres), ("fp64", g64)):
        cmp = compare(prob, g, ref64, cols)
        assert np.all(cmp["pert"][ok] <= 1e-5), (label, cmp["pert"].max())
        assert np.all(cmp["mean"] <= 1e-5), (label, cmp["mean"].max())
        errs[label] = float(cmp["pert"][ok].max())
    # the FP64 eigensolve leaves the FP32 Gram as the error source: no worse
    # than the FP32 solve beyond rounding of the stored result
    assert errs["fp64"] <= errs["fp32"] * 1.25 + 1e-7, errs
    o.close()


@pytest.mark.parametrize("mode,gap", [("fp32_resolve", 1e-4), ("fp64", 1e-6)])
def test_precision_with_bound_state(mode, gap):
    """A bound state runs the eigensolve in 8 column chunks: the FP64 re-solve
    of each chunk takes the units flagged since the previous chunk (a device
    count); the result equals the unbound run's bit for bit."""
    from letkf_gb300 import Solver
    cfg = workload_cfg("c4small")
    p = workload(cfg["gen"]["workload"], **{k: v for k, v in cfg["gen"].items() if k != "workload"})

    def solver():
        s = Solver(0)
        s.set_variant("batched")
        s.set_precision(mode, gap)
        s.solver_init(cfg["solver"])
        s.loc_init(cfg["localization"], p.vars, p.lev_depth)
        s.set_grid(p.lat, p.lon, p.mask)
        return s

    s = solver()
    try:
        s.set_state(p.state, p.mean, p.sprd, p.vars)
        s.set_obs(p.olat, p.olon, p.oz, p.otime, p.oval, p.oerr, p.oobsid, p.oplatid, p.hx, p.hx_mean)
        s.run()
        ref, tref = s.get_state(), s.timings()
    finally:
        s.close()
    arrs = [a.copy() for a in (p.state, p.mean, p.sprd)]
    s = solver()
    try:
        s.bind_state(arrs[0], arrs[1], arrs[2], p.vars)
        s.set_obs(p.olat, p.olon, p.oz, p.otime, p.oval, p.oerr, p.oobsid, p.oplatid, p.hx, p.hx_mean)
        s.run()
        tb = s.timings()
    finally:
        s.close()
    assert tb["fp64_units"] == tref["fp64_units"] and tb["fp64_units"] > 0
    for got, want in zip(arrs, ref):
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), mode
