"""Seeded synthetic LETKF workloads (ctypes binding of synth/lgsynth.c).

A Problem holds the arrays the reference's letkf_solver_run reads from its
module globals after pre-processing (background perturbations / mean /
spread, QC-compacted observations, hx perturbations and mean), with the
reference's layouts: state[ij, slab, member], hx[obs, member].
"""
import ctypes
import os
from dataclasses import dataclass, field

import numpy as np

from ._build import synth_lib_path

W_C1, W_C2, W_C3, W_C4, W_SIMPLE3D, W_OCEAN = 1, 2, 3, 4, 5, 6
WORKLOADS = {"c1": W_C1, "c2": W_C2, "c3": W_C3, "c4": W_C4, "simple3d": W_SIMPLE3D, "ocean": W_OCEAN}

FP = ctypes.POINTER(ctypes.c_float)
IP = ctypes.POINTER(ctypes.c_int)


class _Var(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char * 16), ("grid_s_idx", ctypes.c_int), ("levels", ctypes.c_int),
                ("ana_inc_max", ctypes.c_float), ("ana_bounds", ctypes.c_float * 2)]


class _Opt(ctypes.Structure):
    _fields_ = [("workload", ctypes.c_int), ("seed", ctypes.c_uint64), ("nx", ctypes.c_int),
                ("ny", ctypes.c_int), ("nz", ctypes.c_int), ("k", ctypes.c_int),
                ("n_profiles", ctypes.c_int), ("n_swaths", ctypes.c_int), ("swath_len", ctypes.c_int),
                ("n_obs", ctypes.c_int), ("n_clusters", ctypes.c_int), ("cluster_sigma_m", ctypes.c_float),
                ("nthreads", ctypes.c_int)]


class _Prob(ctypes.Structure):
    _fields_ = ([(n, ctypes.c_int) for n in ("nx", "ny", "nz", "ncol", "k", "ns", "nvars", "nobs")] +
                [("vars", _Var * 8), ("lev_depth", FP), ("lat", FP), ("lon", FP), ("mask", IP),
                 ("state", FP), ("mean", FP), ("sprd", FP), ("truth", FP)] +
                [(n, FP) for n in ("olat", "olon", "oz", "otime", "oval", "oerr")] +
                [(n, IP) for n in ("oobsid", "oplatid", "oqc")] + [("hx", FP), ("hx_mean", FP)])


@dataclass
class Problem:
    nx: int
    ny: int
    nz: int
    k: int
    ns: int
    vars: list
    lev_depth: np.ndarray
    lat: np.ndarray
    lon: np.ndarray
    mask: np.ndarray
    state: np.ndarray
    mean: np.ndarray
    sprd: np.ndarray
    truth: np.ndarray
    olat: np.ndarray
    olon: np.ndarray
    oz: np.ndarray
    otime: np.ndarray
    oval: np.ndarray
    oerr: np.ndarray
    oobsid: np.ndarray
    oplatid: np.ndarray
    hx: np.ndarray
    hx_mean: np.ndarray
    name: str = ""
    meta: dict = field(default_factory=dict)

    @property
    def ncol(self):
        return self.lat.shape[0]

    @property
    def nobs(self):
        return self.olat.shape[0]

    def var(self, name):
        for v in self.vars:
            if v["name"] == name:
                return v
        raise KeyError(name)


_lib = None


def _L():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(synth_lib_path())
        _lib.lgs_generate.argtypes = [ctypes.POINTER(_Opt), ctypes.POINTER(_Prob)]
        _lib.lgs_free.argtypes = [ctypes.POINTER(_Prob)]
        _lib.lgs_forecast.argtypes = [ctypes.POINTER(_Prob), ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                      ctypes.c_int]
        _lib.lgs_observe.argtypes = [ctypes.POINTER(_Opt), ctypes.POINTER(_Prob), ctypes.c_uint64]
        _lib.lgs_free_obs.argtypes = [ctypes.POINTER(_Prob)]
    return _lib


def _view(prob):
    """A _Prob over the Problem's own grid / state arrays (no copies)."""
    p = _Prob()
    p.nx, p.ny, p.nz, p.ncol, p.k, p.ns = prob.nx, prob.ny, prob.nz, prob.ncol, prob.k, prob.ns
    p.nvars = len(prob.vars)
    for i, v in enumerate(prob.vars):
        p.vars[i].name = v["name"].encode()[:15]
        p.vars[i].grid_s_idx = v["grid_s_idx"]
        p.vars[i].levels = v["levels"]
        p.vars[i].ana_inc_max = v["ana_inc_max"]
        p.vars[i].ana_bounds[0], p.vars[i].ana_bounds[1] = v["ana_bounds"]
    for name in ("lev_depth", "lat", "lon", "state", "mean", "sprd", "truth"):
        a = getattr(prob, name)
        assert a.dtype == np.float32 and a.flags.c_contiguous
        setattr(p, name, a.ctypes.data_as(FP))
    assert prob.mask.dtype == np.int32 and prob.mask.flags.c_contiguous
    p.mask = prob.mask.ctypes.data_as(IP)
    return p


def forecast(prob, u=0.5, kappa=1.0e3, dt=21600.0, nthreads=0):
    """One forecast step of a cycling experiment, in place: members and truth
    advected by a zonal jet u (m/s) over dt (s) and diffused with kappa
    (m^2/s); background mean / perturbations / spread recomputed."""
    p = _view(prob)
    rc = _L().lgs_forecast(ctypes.byref(p), float(u), float(kappa), float(dt), int(nthreads))
    if rc != 0:
        raise RuntimeError("lgs_forecast failed (%d)" % rc)
    return prob


def observe(prob, seed, n_obs=0, n_clusters=0, cluster_sigma_m=0.0, centre_seed=1003):
    """A copy of prob with new clustered observations of its current
    background and truth: the C3/C4 network with cluster centres from
    `centre_seed` (persistent from cycle to cycle), positions and errors
    drawn with `seed`."""
    from dataclasses import replace
    p = _view(prob)
    o = _Opt()
    o.seed = int(seed)
    o.n_obs = int(n_obs)
    o.n_clusters = int(n_clusters)
    o.cluster_sigma_m = float(cluster_sigma_m)
    rc = _L().lgs_observe(ctypes.byref(o), ctypes.byref(p), int(centre_seed))
    try:
        if rc != 0:
            raise RuntimeError("lgs_observe failed (%d)" % rc)
        n, k = p.nobs, prob.k

        def arr(ptr, shape, dt=np.float32):
            m = int(np.prod(shape))
            if m == 0:
                return np.zeros(shape, dt)
            return np.ctypeslib.as_array(ptr, (m,)).astype(dt, copy=True).reshape(shape)

        return replace(prob, olat=arr(p.olat, (n,)), olon=arr(p.olon, (n,)), oz=arr(p.oz, (n,)),
                       otime=arr(p.otime, (n,)), oval=arr(p.oval, (n,)), oerr=arr(p.oerr, (n,)),
                       oobsid=arr(p.oobsid, (n,), np.int32), oplatid=arr(p.oplatid, (n,), np.int32),
                       hx=arr(p.hx, (n, k)), hx_mean=arr(p.hx_mean, (n,)))
    finally:
        _L().lgs_free_obs(ctypes.byref(p))


def generate(workload, seed=0, nthreads=0, **overrides):
    """Generate a workload ('c1', 'c2', 'c3', 'c4', 'simple3d', 'ocean').
    Keyword overrides: nx, ny, nz, k, n_profiles, n_swaths, swath_len, n_obs,
    n_clusters, cluster_sigma_m."""
    w = WORKLOADS[workload] if isinstance(workload, str) else int(workload)
    o = _Opt()
    o.workload = w
    o.seed = seed
    o.nthreads = nthreads
    for key, val in overrides.items():
        setattr(o, key, val)
    p = _Prob()
    rc = _L().lgs_generate(ctypes.byref(o), ctypes.byref(p))
    if rc != 0:
        raise RuntimeError("lgs_generate failed (%d)" % rc)
    try:
        ncol, ns, k, nobs = p.ncol, p.ns, p.k, p.nobs

        def arr(ptr, shape, dt=np.float32):
            n = int(np.prod(shape))
            if n == 0:
                return np.zeros(shape, dt)
            return np.ctypeslib.as_array(ptr, (n,)).astype(dt, copy=True).reshape(shape)

        vs = []
        for i in range(p.nvars):
            v = p.vars[i]
            vs.append(dict(name=v.name.decode(), grid_s_idx=v.grid_s_idx, levels=v.levels,
                           ana_inc_max=float(v.ana_inc_max),
                           ana_bounds=(float(v.ana_bounds[0]), float(v.ana_bounds[1]))))
        prob = Problem(nx=p.nx, ny=p.ny, nz=p.nz, k=k, ns=ns, vars=vs,
                       lev_depth=arr(p.lev_depth, (p.nz,)), lat=arr(p.lat, (ncol,)), lon=arr(p.lon, (ncol,)),
                       mask=arr(p.mask, (ncol,), np.int32), state=arr(p.state, (ncol, ns, k)),
                       mean=arr(p.mean, (ncol, ns)), sprd=arr(p.sprd, (ncol, ns)), truth=arr(p.truth, (ncol, ns)),
                       olat=arr(p.olat, (nobs,)), olon=arr(p.olon, (nobs,)), oz=arr(p.oz, (nobs,)),
                       otime=arr(p.otime, (nobs,)), oval=arr(p.oval, (nobs,)), oerr=arr(p.oerr, (nobs,)),
                       oobsid=arr(p.oobsid, (nobs,), np.int32), oplatid=arr(p.oplatid, (nobs,), np.int32),
                       hx=arr(p.hx, (nobs, k)), hx_mean=arr(p.hx_mean, (nobs,)),
                       name=workload if isinstance(workload, str) else str(workload))
    finally:
        _L().lgs_free(ctypes.byref(p))
    return prob
