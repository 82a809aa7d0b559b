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
    return _lib


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
