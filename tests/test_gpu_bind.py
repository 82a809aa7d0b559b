"""GPU: in-place state (lgpu_bind_state), the reference's letkf_solver_run
semantics (src/letkf_solver.F90:283-330 overwrites state_ij, state_mean_ij,
state_sprd_ij with the analysis).  Two cycles through bound arrays -- pageable
numpy arrays and page-locked ones -- must give the same bits as
lgpu_set_state + lgpu_solver_run + lgpu_get_state, the second cycle starting
from the first one's analysis."""
import numpy as np
import pytest

from conftest import workload
from helpers import workload_cfg

pytestmark = pytest.mark.gpu


def _solver(cfg, p):
    from letkf_gb300 import Solver
    s = Solver(0)
    # one Gram form for both solvers: AUTO decides by timing, and the two
    # forms agree to rounding, not bit for bit
    s.set_variant("batched")
    s.solver_init(cfg["solver"])
    s.loc_init(cfg["localization"], p.vars, p.lev_depth)
    s.set_grid(p.lat, p.lon, p.mask)
    return s


def _set_obs(s, p):
    s.set_obs(p.olat, p.olon, p.oz, p.otime, p.oval, p.oerr, p.oobsid, p.oplatid, p.hx, p.hx_mean)


@pytest.mark.parametrize("name,pinned", [("c1", False), ("ocean", True), ("c2small", True)])
def test_bound_state_matches_set_get(name, pinned):
    from letkf_gb300 import PinnedArray
    cfg = workload_cfg(name)
    p = workload(cfg["gen"]["workload"], **{k: v for k, v in cfg["gen"].items() if k != "workload"})
    ref = []
    s = _solver(cfg, p)
    try:
        x, m, sp = p.state, p.mean, p.sprd
        for _ in range(2):
            s.set_state(x, m, sp, p.vars)
            _set_obs(s, p)
            s.run()
            x, m, sp = s.get_state()
            ref.append((x, m, sp))
    finally:
        s.close()
    pins = []
    if pinned:
        pins = [PinnedArray(a.shape) for a in (p.state, p.mean, p.sprd)]
        arrs = [q.array for q in pins]
    else:
        arrs = [np.empty_like(a) for a in (p.state, p.mean, p.sprd)]
    for a, src in zip(arrs, (p.state, p.mean, p.sprd)):
        a[...] = src
    s = _solver(cfg, p)
    try:
        s.bind_state(arrs[0], arrs[1], arrs[2], p.vars)
        _set_obs(s, p)
        for cyc in range(2):
            s.run()
            for got, want in zip(arrs, ref[cyc]):
                assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (name, cyc)
        # the device copy is the same analysis
        x, m, sp = s.get_state()
        assert np.array_equal(x, arrs[0]) and np.array_equal(m, arrs[1]) and np.array_equal(sp, arrs[2])
    finally:
        s.close()
        for q in pins:
            q.free()
