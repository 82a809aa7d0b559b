"""GPU: the benchmark workloads at their full sizes, through properties that
do not depend on size and the oracle on samples of their columns.

  c2     720x360x40, k = 40, 440,000 observations (the headline workload)
  c3     720x360x40, k = 32, 500,000 clustered observations
  c3k64  the same with k = 64
  c4     1440x720x50, k = 100, 1,000,000 clustered observations

For each, the batched (tensor-core) form:
  - every analysis slab's perturbations sum to zero over the members
    (the recentering of src/letkf_solver.F90:299-303) to FP32 rounding;
    spreads are finite and non-negative; masked columns keep the background;
  - 48 sampled columns -- 40 at random and the 8 with the most kept local
    observations: observation lists bit-exact against the oracle on 16 of
    them (the 4 densest among them), and the analysis against the FP64
    oracle within 1e-5 relative L2 over the sample (perturbations and mean),
    the error per variable and level printed;
  - c2: the reference's own FP32 arithmetic on the same columns printed for
    context (the Gram with single-precision BLAS and the eigensolve with
    LAPACK ssyev, src/letkf_core.F90:92-141, here numpy float32 matmul and
    scipy's ssyev driver), and the plain form against the batched form on
    every column;
  - c4: the FP32 eigensolve with FP64 re-solves of flagged units
    (lgpu_set_precision FP32_RESOLVE): units are flagged, the columns whose
    analysis the re-solve changed are checked against the FP64 oracle, every
    other column is bit-identical to the FP32 mode.
"""
import numpy as np
import pytest

from helpers import oracle_for, rel_l2, workload_cfg

pytestmark = pytest.mark.gpu

PERT_TOL = 1e-5
MEAN_TOL = 1e-5


def _generate(name):
    from letkf_gb300 import synth
    cfg = workload_cfg(name)
    gen = dict(cfg["gen"])
    w = gen.pop("workload")
    return synth.generate(w, **gen), cfg


def _solver(prob, cfg, variant="batched", precision="fp32"):
    from letkf_gb300 import Solver
    s = Solver(0)
    s.set_variant(variant)
    s.set_precision(precision)
    s.solver_init(cfg["solver"])
    s.loc_init(cfg["localization"], prob.vars, prob.lev_depth)
    s.set_problem(prob)
    s.run()
    return s


def _pert(x, m):
    return x.astype(np.float64) - m.astype(np.float64)[:, :, None]


def _slab_report(name, prob, e):
    out = []
    for v in prob.vars:
        i0, n = v["grid_s_idx"], v["levels"]
        ev = e[i0:i0 + n]
        out.append("%s max %.2e (lev %d) median %.2e" % (v["name"], ev.max(), int(np.argmax(ev)) + 1,
                                                          float(np.median(ev))))
    print("%s per-slab perturbation error vs FP64: %s" % (name, "; ".join(out)))


CHUNK = 4096   # columns per step of the whole-grid checks (C4 holds 41.5 GB per state copy)


def _column_hash(x):
    """A 64-bit fingerprint of every column's bits (chunked; wrapping uint64)."""
    w = np.random.default_rng(3).integers(1, 2 ** 63, size=x.shape[1] * x.shape[2], dtype=np.uint64) | np.uint64(1)
    out = np.empty(x.shape[0], np.uint64)
    for c0 in range(0, x.shape[0], CHUNK):
        v = x[c0:c0 + CHUNK].reshape(-1, w.size).view(np.uint32).astype(np.uint64)
        out[c0:c0 + CHUNK] = (v * w).sum(axis=1)
    return out


def _check(name, prob, cfg, s, x, m, sp):
    act = np.nonzero(prob.mask == 0)[0]
    mc = np.nonzero(prob.mask)[0]
    assert np.all(np.isfinite(m)) and np.all(sp[act] >= 0.0)
    worst = 0.0
    for i0 in range(0, len(act), CHUNK):
        c = act[i0:i0 + CHUNK]
        xc = x[c]
        assert np.all(np.isfinite(xc))
        pert = _pert(xc, m[c])
        scale = np.maximum(np.abs(xc).max(axis=2), 1e-6)
        worst = max(worst, float(np.max(np.abs(pert.sum(axis=2)) / scale)))
    assert worst < 1e-4, (name, worst)
    for i0 in range(0, len(mc), CHUNK):
        c = mc[i0:i0 + CHUNK]
        assert np.array_equal(x[c], prob.state[c]) and np.array_equal(m[c], prob.mean[c])
    kept = s.get_diag()["lg_obscount"].sum(axis=0)
    rng = np.random.default_rng(11)
    dense = act[np.argsort(kept[act])[-8:]]
    cols = np.unique(np.concatenate([rng.choice(act, size=40, replace=False), dense]))
    list_cols = np.unique(np.concatenate([cols[:12], dense[-4:]]))
    lists = {int(c): s.obslist(int(c), 0) for c in list_cols}
    o = oracle_for(prob, cfg["localization"], cfg["solver"])
    try:
        r64 = o.run(64, cols=cols)
        for c, (gi, gr, gn) in lists.items():
            oi, orr, on = o.obslist(c, 0)
            assert gn == on and np.array_equal(gi, oi), (name, c)
    finally:
        o.close()
    p64 = _pert(r64["state"], r64["mean"])
    e = rel_l2(_pert(x[cols], m[cols]), p64)
    em = rel_l2(m[cols], r64["mean"])
    _slab_report(name, prob, rel_l2(_pert(x[cols], m[cols]), p64, axis=(0, 2)))
    print("%s: perturbations vs FP64 %.3g, mean %.3g, densest sampled column %d kept observations"
          % (name, e, em, int(kept[dense[-1]])))
    assert e <= PERT_TOL, (name, e)
    assert em <= MEAN_TOL, (name, em)
    return cols, lists, p64, r64


def _reference_fp32(prob, lists, p64, r64, cols):
    """The reference's FP32 core solve (sgemm + ssyev) on the listed columns."""
    sla = pytest.importorskip("scipy.linalg")
    k = prob.k
    pr32, mr32, sel = [], [], []
    for c, (gi, gr, gn) in lists.items():
        Y = prob.hx[gi].astype(np.float32)
        rinv = (Y / prob.oerr[gi][:, None].astype(np.float32)) * gr[:, None].astype(np.float32)
        dep = (prob.oval[gi] - prob.hx_mean[gi]).astype(np.float32)
        A = rinv.T @ Y + np.float32(k - 1) * np.eye(k, dtype=np.float32)
        lam, V = sla.eigh(A, driver="ev")
        Pa = (V / lam) @ V.T
        wbar = (Pa @ rinv.T) @ dep
        T = (V * np.sqrt(np.float32(k - 1) / lam)) @ V.T + wbar[:, None]
        xa = prob.state[c].astype(np.float32) @ T + prob.mean[c][:, None]
        mn = xa.mean(axis=1, dtype=np.float32)
        pr32.append(xa - mn[:, None])
        mr32.append(mn)
        sel.append(int(np.searchsorted(cols, c)))
    return rel_l2(np.array(pr32), p64[sel]), rel_l2(np.array(mr32), r64["mean"][sel])


def test_c2_full_size():
    prob, cfg = _generate("c2")
    s = _solver(prob, cfg)
    try:
        x, m, sp = s.get_state()
        cols, lists, p64, r64 = _check("c2", prob, cfg, s, x, m, sp)
    finally:
        s.close()
    e_ref, em_ref = _reference_fp32(prob, lists, p64, r64, cols)
    print("c2: the reference's FP32 arithmetic on the listed columns: perturbations %.3g, mean %.3g" % (e_ref, em_ref))
    # the plain form on every column
    p = _solver(prob, cfg, variant="plain")
    try:
        xp, mp, _ = p.get_state()
    finally:
        p.close()
    act = np.nonzero(prob.mask == 0)[0]
    e_bp = rel_l2(_pert(x[act], m[act]), _pert(xp[act], mp[act]))
    em_bp = rel_l2(m[act], mp[act])
    print("c2 batched vs plain, all columns: perturbations %.3g, mean %.3g" % (e_bp, em_bp))
    assert e_bp <= 2 * PERT_TOL and em_bp <= MEAN_TOL


@pytest.mark.parametrize("name", ["c3", "c3k64"])
def test_c3_full_size(name):
    prob, cfg = _generate(name)
    s = _solver(prob, cfg)
    try:
        x, m, sp = s.get_state()
        _check(name, prob, cfg, s, x, m, sp)
    finally:
        s.close()


def test_c4_full_size_with_fp64_resolve():
    prob, cfg = _generate("c4")
    s = _solver(prob, cfg)
    try:
        x, m, sp = s.get_state()
        _check("c4", prob, cfg, s, x, m, sp)
        hx, hm = _column_hash(x), m.copy()
        del x, sp
        s.set_precision("fp32_resolve", 1e-6)
        s.run()
        t = s.timings()
        xr, mr, _ = s.get_state()
    finally:
        s.close()
    assert t["fp64_units"] > 0, t
    changed = np.nonzero((_column_hash(xr) != hx) | np.any(mr != hm, axis=1))[0]
    print("c4 FP32_RESOLVE: %d units re-solved in FP64, %d columns changed" % (t["fp64_units"], len(changed)))
    # every other column is bit-identical to the FP32 mode (equal fingerprints and means)
    assert 0 < len(changed) <= t["fp64_units"]
    sel = changed[:: max(1, len(changed) // 12)][:12]
    o = oracle_for(prob, cfg["localization"], cfg["solver"])
    try:
        r64 = o.run(64, cols=sel)
    finally:
        o.close()
    e = rel_l2(_pert(xr[sel], mr[sel]), _pert(r64["state"], r64["mean"]))
    em = rel_l2(mr[sel], r64["mean"])
    print("c4 re-solved columns vs FP64: perturbations %.3g, mean %.3g" % (e, em))
    assert e <= PERT_TOL and em <= MEAN_TOL
