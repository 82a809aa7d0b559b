"""ctypes binding of the CPU oracle (letkf_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() and
by bench.py's CPU-baseline leg, never by the GPU library or its Python
binding.  The oracle restates UMD-LETKF's per-gridpoint analysis
(src/letkf_solver.F90:150-389, src/letkf_core.F90:69-146,
src/letkf_loc.F90:251-378 and the localizer plugins) in plain C.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")

MAXINTERP, MAXIDS, MAXLEV, MAXVARS = 16, 32, 128, 8
LOC_NOVRT, LOC_OCEAN, LOC_VTGC = 0, 1, 2

FP = ctypes.POINTER(ctypes.c_float)
IP = ctypes.POINTER(ctypes.c_int)


class Interp(ctypes.Structure):
    _fields_ = [("npoints", ctypes.c_int),
                ("lat", ctypes.c_float * (MAXINTERP + 2)),
                ("dist", ctypes.c_float * (MAXINTERP + 2))]


class Loc(ctypes.Structure):
    _fields_ = [("cls", ctypes.c_int), ("hz", Interp), ("hz_sat", Interp),
                ("tloc_prof", ctypes.c_float), ("tloc_sat", ctypes.c_float),
                ("vtloc_surf", ctypes.c_int), ("bkg_t_delta", ctypes.c_float),
                ("bkg_t_idx", ctypes.c_int), ("bkg_t_len", ctypes.c_int),
                ("n_sat_obs", ctypes.c_int), ("sat_obs", ctypes.c_int * MAXIDS),
                ("n_sat_plats", ctypes.c_int), ("sat_plats", ctypes.c_int * MAXIDS),
                ("vloc", ctypes.c_float), ("nlev", ctypes.c_int),
                ("lev_depth", ctypes.c_float * MAXLEV), ("maxgroups", ctypes.c_int)]


class Var(ctypes.Structure):
    _fields_ = [("grid_s_idx", ctypes.c_int), ("levels", ctypes.c_int),
                ("ana_inc_max", ctypes.c_float), ("ana_bounds", ctypes.c_float * 2)]


class Problem(ctypes.Structure):
    _fields_ = [("ncol", ctypes.c_int), ("k", ctypes.c_int), ("ns", ctypes.c_int),
                ("nvars", ctypes.c_int), ("nobs", ctypes.c_int), ("vars", Var * MAXVARS),
                ("lat", FP), ("lon", FP), ("mask", IP), ("state", FP), ("mean", FP), ("sprd", FP),
                ("olat", FP), ("olon", FP), ("oz", FP), ("otime", FP), ("oval", FP), ("oerr", FP),
                ("oobsid", IP), ("oplatid", IP), ("hx", FP), ("hx_mean", FP),
                ("rtps", ctypes.c_float), ("rtpp", ctypes.c_float), ("mul", ctypes.c_float)]


class Result(ctypes.Structure):
    _fields_ = [("state", FP), ("mean", FP), ("sprd", FP), ("maxhz", FP), ("obscount", FP),
                ("lg_obscount", FP), ("lg_obsloc", FP)]


def build(force=False):
    """Compile liboracle.so (gcc, OpenMP, no FP contraction)."""
    src = os.path.join(HERE, "letkf_oracle.c")
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(src):
        return LIB
    cmd = ["gcc", "-O3", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-fno-fast-math", "-o", LIB, src, "-lm"]
    subprocess.check_call(cmd, cwd=HERE)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        L.or_create.restype = ctypes.c_void_p
        L.or_create.argtypes = [ctypes.POINTER(Problem), ctypes.POINTER(Loc)]
        L.or_destroy.argtypes = [ctypes.c_void_p]
        L.or_run.argtypes = [ctypes.c_void_p, ctypes.c_int, IP, ctypes.c_int, ctypes.POINTER(Result), ctypes.c_int]
        L.or_obslist.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, IP, FP, ctypes.c_int, IP]
        L.or_gc.restype = ctypes.c_float
        L.or_gc.argtypes = [ctypes.c_float, ctypes.c_float]
        L.or_interp_get.restype = ctypes.c_float
        L.or_interp_get.argtypes = [ctypes.POINTER(Interp), ctypes.c_float]
        L.or_interp_build.argtypes = [ctypes.POINTER(Interp), ctypes.c_int, FP, FP]
        L.or_unitvec.argtypes = [ctypes.c_float, ctypes.c_float, FP]
        L.or_dist.restype = ctypes.c_float
        L.or_dist.argtypes = [FP, FP]
        L.or_eigh.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                              ctypes.POINTER(ctypes.c_double)]
        L.or_core_solve.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, FP, FP, FP, FP, ctypes.c_float, FP]
        L.or_set_lapack.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        _lib = L
    return _lib


PREC_LAPACK = 1   # OR_PREC_LAPACK: the reference's sgemm / ssyev call sequence


def set_lapack():
    """Register an optimised BLAS sgemm and LAPACK ssyev with the oracle
    (the ones SciPy is linked with, taken from scipy.linalg.cython_blas /
    cython_lapack), enabling precision PREC_LAPACK.  Each call runs on the
    calling thread when OPENBLAS_NUM_THREADS=1 was set before SciPy loaded;
    the oracle parallelises over columns.  Returns a description of the
    library."""
    from scipy.linalg import cython_blas, cython_lapack
    get_name = ctypes.pythonapi.PyCapsule_GetName
    get_name.restype = ctypes.c_char_p
    get_name.argtypes = [ctypes.py_object]
    get_ptr = ctypes.pythonapi.PyCapsule_GetPointer
    get_ptr.restype = ctypes.c_void_p
    get_ptr.argtypes = [ctypes.py_object, ctypes.c_char_p]

    def ptr(cap):
        return get_ptr(cap, get_name(cap))

    rc = lib().or_set_lapack(ptr(cython_blas.__pyx_capi__["sgemm"]), ptr(cython_lapack.__pyx_capi__["ssyev"]))
    if rc != 0:
        raise RuntimeError("sgemm / ssyev not found in SciPy")
    desc = "SciPy's BLAS / LAPACK"
    try:
        import scipy
        cfg = scipy.show_config(mode="dicts")
        blas = cfg.get("Build Dependencies", {}).get("blas", {})
        desc = "%s %s (SciPy %s)" % (blas.get("name", "BLAS"), blas.get("version", ""), scipy.__version__)
    except Exception:
        pass
    return desc


def _fp(a):
    return a.ctypes.data_as(FP)


def _ip(a):
    return a.ctypes.data_as(IP)


def interp(points):
    """linearinterp_lat table from [(lat, radius), ...] (src/letkf_loc.F90:251-294)."""
    t = Interp()
    lat = np.ascontiguousarray([p[0] for p in points], np.float32)
    rad = np.ascontiguousarray([p[1] for p in points], np.float32)
    lib().or_interp_build(ctypes.byref(t), len(points), _fp(lat), _fp(rad))
    return t


def make_loc(desc, prob):
    """Oracle localizer table from a host-side localizer description
    (dictionary with the reference's YAML keys, see letkf_gb300.localizers)."""
    L = Loc()
    cls = desc["class"].lower()
    if cls == "loc_novrt":
        L.cls = LOC_NOVRT
        L.hz = interp(desc["hzloc"])
        L.maxgroups = 1
    elif cls == "loc_ocean":
        L.cls = LOC_OCEAN
        L.hz = interp(desc["hzloc_prof"])
        L.hz_sat = interp(desc["hzloc_sat"])
        L.tloc_prof = desc.get("tloc_prof", -1.0)
        L.tloc_sat = desc.get("tloc_sat", -1.0)
        so = desc.get("sat_obs", []) or []
        sp = desc.get("sat_plats", []) or []
        L.n_sat_obs = len(so)
        L.n_sat_plats = len(sp)
        for i, v in enumerate(so):
            L.sat_obs[i] = v
        for i, v in enumerate(sp):
            L.sat_plats[i] = v
        vt = desc.get("vtloc_surf")
        if vt and vt.get("type") == "bkg_t":
            L.vtloc_surf = 1
            L.bkg_t_delta = vt["bkg_t_delta"]
            v = prob.vars[vt["bkg_t_var"]]
            L.bkg_t_idx, L.bkg_t_len = v["grid_s_idx"], v["levels"]
            L.maxgroups = 2
        else:
            L.maxgroups = 1
    elif cls == "loc_vtgc":
        L.cls = LOC_VTGC
        L.hz = interp(desc["hzloc"])
        L.vloc = desc["vtloc"]
        lev = np.asarray(prob.lev_depth, np.float32)
        L.nlev = len(lev)
        for i, v in enumerate(lev):
            L.lev_depth[i] = v
        L.maxgroups = len(lev)
    else:
        raise ValueError("localizer class %s not found." % desc["class"])
    return L


class Oracle:
    """CPU oracle over one synthetic problem (letkf_gb300.synth.Problem)."""

    def __init__(self, prob, loc_desc, rtps=0.0, rtpp=0.0, mul=1.0, variables=None):
        self.prob = prob
        self._keep = []
        P = Problem()
        P.ncol, P.k, P.ns, P.nobs = prob.ncol, prob.k, prob.ns, prob.nobs
        vs = variables if variables is not None else prob.vars
        P.nvars = len(vs)
        for i, v in enumerate(vs):
            P.vars[i].grid_s_idx = v["grid_s_idx"]
            P.vars[i].levels = v["levels"]
            P.vars[i].ana_inc_max = v.get("ana_inc_max", 9.99e36)
            b = v.get("ana_bounds", (-9.99e36, 9.99e36))
            P.vars[i].ana_bounds[0], P.vars[i].ana_bounds[1] = b[0], b[1]
        for name in ("lat", "lon", "state", "mean", "sprd", "olat", "olon", "oz", "otime", "oval", "oerr",
                     "hx", "hx_mean"):
            a = np.ascontiguousarray(getattr(prob, name), np.float32)
            self._keep.append(a)
            setattr(P, name, _fp(a))
        for name in ("mask", "oobsid", "oplatid"):
            a = np.ascontiguousarray(getattr(prob, name), np.int32)
            self._keep.append(a)
            setattr(P, name, _ip(a))
        P.rtps, P.rtpp, P.mul = rtps, rtpp, mul
        self.P = P
        self.L = make_loc(loc_desc, prob)
        self.maxgroups = self.L.maxgroups
        self.ctx = lib().or_create(ctypes.byref(self.P), ctypes.byref(self.L))
        if not self.ctx:
            raise MemoryError("or_create failed")

    def close(self):
        if self.ctx:
            lib().or_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def run(self, precision=32, cols=None, nthreads=0):
        """Analysis of the listed columns (default all).  Returns a dict of
        compact arrays: state [ncl, ns, k], mean/sprd [ncl, ns], maxhz,
        obscount [ncl], lg_obscount/lg_obsloc [ncl, maxgroups]."""
        p = self.prob
        if cols is None:
            cols = np.arange(p.ncol, dtype=np.int32)
        cols = np.ascontiguousarray(cols, np.int32)
        n = len(cols)
        out = dict(state=np.zeros((n, p.ns, p.k), np.float32), mean=np.zeros((n, p.ns), np.float32),
                   sprd=np.zeros((n, p.ns), np.float32), maxhz=np.zeros(n, np.float32),
                   obscount=np.zeros(n, np.float32),
                   lg_obscount=np.zeros((n, self.maxgroups), np.float32),
                   lg_obsloc=np.zeros((n, self.maxgroups), np.float32))
        R = Result()
        for key in out:
            setattr(R, key, _fp(out[key]))
        rc = lib().or_run(self.ctx, precision, _ip(cols), n, ctypes.byref(R), nthreads)
        if rc < 0 or (rc & 12):
            raise RuntimeError("oracle run failed: %d" % rc)
        out["eig_rc"] = rc
        return out

    def obslist(self, col, group=0):
        p = self.prob
        cap = p.nobs if p.nobs > 0 else 1
        idx = np.zeros(cap, np.int32)
        r = np.zeros(cap, np.float32)
        nc = ctypes.c_int(0)
        n = lib().or_obslist(self.ctx, int(col), int(group), _ip(idx), _fp(r), cap, ctypes.byref(nc))
        return idx[:n].copy(), r[:n].copy(), nc.value


def gc(z, L):
    return lib().or_gc(float(z), float(L))


def unitvec(lat, lon):
    out = np.zeros(3, np.float32)
    lib().or_unitvec(float(lat), float(lon), _fp(out))
    return out


def dist(a, b):
    a = np.ascontiguousarray(a, np.float32)
    b = np.ascontiguousarray(b, np.float32)
    return lib().or_dist(_fp(a), _fp(b))


def eigh(A):
    A = np.asfortranarray(A, np.float64)
    k = A.shape[0]
    lam = np.zeros(k)
    V = np.zeros((k, k), order="F")
    DP = ctypes.POINTER(ctypes.c_double)
    rc = lib().or_eigh(k, A.ctypes.data_as(DP), lam.ctypes.data_as(DP), V.ctypes.data_as(DP))
    return lam, V, rc


def core_solve(hdxb, rdiag, rloc, dep, precision=32, infl=1.0):
    """letkf_core_solve: hdxb [n, k] (obs-major), returns trans [k, k] with
    trans[i, j] = T(i, j) (Fortran trans(i,j))."""
    hdxb = np.ascontiguousarray(hdxb, np.float32)
    n, k = hdxb.shape
    tr = np.zeros(k * k, np.float32)
    lib().or_core_solve(precision, k, n, _fp(hdxb), _fp(np.ascontiguousarray(rdiag, np.float32)),
                        _fp(np.ascontiguousarray(rloc, np.float32)), _fp(np.ascontiguousarray(dep, np.float32)),
                        infl, _fp(tr))
    return tr.reshape(k, k).T.copy()   # column-major -> [i, j]
