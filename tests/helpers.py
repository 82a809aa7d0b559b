"""Shared helpers for the parity tests: run the GPU library and the oracle on
the same workload and compare per variable and level."""
import numpy as np

from letkf_gb300 import Solver, normalize_loc, normalize_solver
from letkf_gb300.workloads import WORKLOADS


def gpu_run(prob, localization, solver=None, variables=None, keep_open=False, variant="auto", precision="fp32"):
    s = Solver(0)
    s.set_variant(variant)
    s.set_precision(precision)
    s.solver_init(solver)
    s.loc_init(localization, variables if variables is not None else prob.vars, prob.lev_depth)
    s.set_problem(prob, variables)
    s.run()
    x, m, sp = s.get_state()
    out = dict(state=x, mean=m, sprd=sp, diag=s.get_diag(), timings=s.timings())
    if keep_open:
        out["solver"] = s
    else:
        s.close()
    return out


def oracle_for(prob, localization, solver=None, variables=None):
    from oracle import oracle as O
    inf = normalize_solver(solver)
    return O.Oracle(prob, normalize_loc(localization, prob.vars), rtps=inf["rtps"], rtpp=inf["rtpp"],
                    mul=inf["mul"], variables=variables)


def rel_l2(a, b, axis=None):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    num = np.sqrt(np.sum((a - b) ** 2, axis=axis))
    den = np.sqrt(np.sum(b ** 2, axis=axis))
    return num / np.maximum(den, 1e-30)


def compare(prob, gpu, ref, cols, variables=None):
    """Per-slab (variable, level) relative L2 errors over the listed columns:
    analysis perturbations, analysis mean, mean increment."""
    xg = gpu["state"][cols].astype(np.float64)
    mg = gpu["mean"][cols].astype(np.float64)
    pg = xg - mg[:, :, None]
    xr = ref["state"].astype(np.float64)
    mr = ref["mean"].astype(np.float64)
    pr = xr - mr[:, :, None]
    mb = prob.mean[cols].astype(np.float64)
    out = dict(pert=rel_l2(pg, pr, axis=(0, 2)), mean=rel_l2(mg, mr, axis=0),
               inc=np.sqrt(np.sum((mg - mr) ** 2, 0)) / np.maximum(np.sqrt(np.sum((mr - mb) ** 2, 0)), 1e-12),
               inc_norm=np.sqrt(np.sum((mr - mb) ** 2, 0)),
               sprd=rel_l2(gpu["sprd"][cols], ref["sprd"], axis=0))
    out["pert_all"] = rel_l2(pg, pr)
    out["mean_all"] = rel_l2(mg, mr)
    return out


def workload_cfg(name):
    return WORKLOADS[name]
