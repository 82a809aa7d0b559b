"""letkf_gb300 -- Python binding of the GB300 (sm_103a) LETKF analysis library.

The library (liblgpu.so, built in-tree from umd-letkf_gb300/csrc) replaces
UMD-LETKF's per-gridpoint analysis path; include/letkf_gpu.h is its C ABI.
This module is a thin ctypes layer over that ABI that mirrors the reference's
host-side interface:

  reference                                  here
  letkf_solver_init(config)                  Solver.solver_init(solver_cfg)
  letkf_loc_init(config) / plugin %init      Solver.loc_init(localization_cfg, vars, lev_depth)
  module globals (state_ij, obs_def, ...)    Solver.set_grid / set_state / set_obs
  letkf_solver_run()                         Solver.run()
  letkf_solver_final()                       Solver.final()

Configuration dictionaries use the reference's YAML keys
(solver: inflation: {mul, rtps, rtpp}; localization: class, hzloc, ...).
There is no CPU fallback: if the CUDA library is missing or no GPU is
usable, LgpuError is raised.
"""
import ctypes
import os

import numpy as np

from ._build import lgpu_lib_path, build_lgpu, build_synth  # noqa: F401

__all__ = ["Solver", "LgpuError", "ConfigError", "normalize_loc", "normalize_solver", "analyse", "lib"]

LGPU_OK = 0
STATUS = {0: "OK", 1: "ERR_ARG", 2: "ERR_CUDA", 3: "ERR_NOMEM", 4: "ERR_UNSUPPORTED_LOCALIZER", 5: "ERR_CONFIG",
          6: "ERR_ORDER", 7: "ERR_CAPACITY", 8: "ERR_NONFINITE", 9: "ERR_EIG", 10: "ERR_UNSUPPORTED"}
MAX_INTERP, MAX_IDS, MAX_LEVELS, MAX_K = 16, 32, 128, 128

FP = ctypes.POINTER(ctypes.c_float)
IP = ctypes.POINTER(ctypes.c_int)


class LgpuError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s: %s" % (STATUS.get(code, code), msg))
        self.code = code
        self.msg = msg


class ConfigError(ValueError):
    pass


class _SolverCfg(ctypes.Structure):
    _fields_ = [("rtps", ctypes.c_float), ("rtpp", ctypes.c_float), ("mul", ctypes.c_float), ("save_diag", ctypes.c_int)]


class _Interp(ctypes.Structure):
    _fields_ = [("lat", ctypes.c_float), ("radius", ctypes.c_float)]


class _LocCfg(ctypes.Structure):
    _fields_ = [("cls", ctypes.c_char_p), ("n_hz", ctypes.c_int), ("hz", ctypes.POINTER(_Interp)),
                ("n_hz_sat", ctypes.c_int), ("hz_sat", ctypes.POINTER(_Interp)),
                ("tloc_prof", ctypes.c_float), ("tloc_sat", ctypes.c_float), ("vtloc_surf", ctypes.c_int),
                ("bkg_t_delta", ctypes.c_float), ("bkg_t_var", ctypes.c_int),
                ("n_sat_obs", ctypes.c_int), ("sat_obs", IP), ("n_sat_plats", ctypes.c_int), ("sat_plats", IP),
                ("vtloc", ctypes.c_float), ("nlev", ctypes.c_int), ("lev_depth", FP)]


class _Var(ctypes.Structure):
    _fields_ = [("grid_s_idx", ctypes.c_int), ("levels", ctypes.c_int), ("ana_inc_max", ctypes.c_float),
                ("ana_bounds", ctypes.c_float * 2)]


class _Obs(ctypes.Structure):
    _fields_ = [(n, FP) for n in ("lat", "lon", "zdim", "time", "val", "err")] + [("obsid", IP), ("platid", IP)]


class Timings(ctypes.Structure):
    _fields_ = [("total_ms", ctypes.c_float), ("index_ms", ctypes.c_float), ("prep_ms", ctypes.c_float),
                ("gram_ms", ctypes.c_float), ("eig_ms", ctypes.c_float), ("update_ms", ctypes.c_float),
                ("launches", ctypes.c_int), ("units", ctypes.c_int), ("kept_pairs", ctypes.c_longlong),
                ("variant", ctypes.c_int), ("tiles_ms", ctypes.c_float), ("mma_chunks", ctypes.c_longlong),
                ("mma_n", ctypes.c_int), ("precision", ctypes.c_int), ("fp64_units", ctypes.c_int),
                ("fp64_ms", ctypes.c_float), ("h2d_obs_ms", ctypes.c_float), ("host_obs_ms", ctypes.c_float),
                ("h2d_state_ms", ctypes.c_float), ("d2h_state_ms", ctypes.c_float), ("span_ms", ctypes.c_float),
                ("host_run_ms", ctypes.c_float), ("h2d_state_bytes", ctypes.c_longlong),
                ("d2h_state_bytes", ctypes.c_longlong)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


VARIANT_AUTO, VARIANT_PLAIN, VARIANT_BATCHED_TC, VARIANT_LEARNED = 0, 1, 2, 3
VARIANTS = {"auto": 0, "plain": 1, "batched": 2, "learned": 3}
PREC_FP32, PREC_FP32_RESOLVE, PREC_FP64 = 0, 1, 2
PRECISIONS = {"fp32": 0, "fp32_resolve": 1, "fp64": 2}


class _LearnCfg(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("stride", ctypes.c_int), ("hidden", ctypes.c_int),
                ("judge_frac", ctypes.c_float), ("gate_frac", ctypes.c_float), ("sample_frac", ctypes.c_float),
                ("train_cap", ctypes.c_int), ("seed", ctypes.c_uint64)]


class LearnStats(ctypes.Structure):
    _fields_ = [("coarse", ctypes.c_int), ("judged", ctypes.c_int), ("fallback", ctypes.c_int),
                ("gated", ctypes.c_int), ("inferred", ctypes.c_int), ("judge_rms", ctypes.c_float),
                ("judge_ref_rms", ctypes.c_float), ("tau", ctypes.c_float), ("train_rows", ctypes.c_longlong),
                ("exact_ms", ctypes.c_float), ("feature_ms", ctypes.c_float), ("network_ms", ctypes.c_float),
                ("apply_ms", ctypes.c_float)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}

EXPORTS = ["lgpu_set_variant", "lgpu_create", "lgpu_destroy", "lgpu_last_error", "lgpu_solver_init", "lgpu_loc_init",
           "lgpu_loc_maxgroups", "lgpu_set_grid", "lgpu_set_state", "lgpu_set_obs", "lgpu_solver_run",
           "lgpu_get_state", "lgpu_get_diag", "lgpu_get_timings", "lgpu_solver_final", "lgpu_get_obslist",
           "lgpu_debug_metric", "lgpu_debug_gc", "lgpu_host_alloc", "lgpu_host_free", "lgpu_flush_l2",
           "lgpu_get_obslist_noalloc", "lgpu_set_obs_raw", "lgpu_set_state_members", "lgpu_get_background",
           "lgpu_get_obs_prepared", "lgpu_debug_transform", "lgpu_bind_state",
           "lgpu_debug_weight", "lgpu_learn_init", "lgpu_learn_collect", "lgpu_learn_train", "lgpu_learn_stats_get",
           "lgpu_learn_param_count", "lgpu_learn_get_params", "lgpu_learn_set_params", "lgpu_mlp_debug",
           "lgpu_learn_set_network", "lgpu_set_precision", "lgpu_write_diag", "lgpu_get_loc_diag",
           "lgpu_write_loc_diag", "lgpu_io_last_error", "lgpu_ens_filename", "lgpu_nc_dim_len", "lgpu_nc_var_info",
           "lgpu_nc_read_float", "lgpu_nc_read_int", "lgpu_read_obs_nc", "lgpu_read_hx_nc", "lgpu_read_state_nc",
           "lgpu_write_state_nc", "lgpu_write_diag_nc", "lgpu_write_loc_diag_nc"]

_lib = None


def lib(path=None):
    """Load liblgpu.so (in-tree).  Raises LgpuError if it is missing."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or lgpu_lib_path()
    if not os.path.exists(p):
        raise LgpuError(2, "CUDA library %s is missing: build it with __graft_entry__.build()" % p)
    L = ctypes.CDLL(p)
    H = ctypes.c_void_p
    L.lgpu_create.argtypes = [ctypes.c_int, ctypes.POINTER(H)]
    L.lgpu_destroy.argtypes = [H]
    L.lgpu_destroy.restype = None
    L.lgpu_last_error.argtypes = [H]
    L.lgpu_last_error.restype = ctypes.c_char_p
    L.lgpu_solver_init.argtypes = [H, ctypes.POINTER(_SolverCfg)]
    L.lgpu_loc_init.argtypes = [H, ctypes.POINTER(_LocCfg)]
    L.lgpu_loc_maxgroups.argtypes = [H]
    L.lgpu_set_variant.argtypes = [H, ctypes.c_int]
    L.lgpu_set_precision.argtypes = [H, ctypes.c_int, ctypes.c_float]
    L.lgpu_set_grid.argtypes = [H, ctypes.c_int, FP, FP, IP]
    L.lgpu_set_state.argtypes = [H, ctypes.c_int, ctypes.c_int, FP, FP, FP, ctypes.c_int, ctypes.POINTER(_Var)]
    L.lgpu_set_obs.argtypes = [H, ctypes.c_int, ctypes.POINTER(_Obs), FP, FP]
    L.lgpu_solver_run.argtypes = [H]
    L.lgpu_get_state.argtypes = [H, FP, FP, FP]
    L.lgpu_get_diag.argtypes = [H, FP, FP, FP, FP]
    L.lgpu_get_timings.argtypes = [H, ctypes.POINTER(Timings)]
    L.lgpu_solver_final.argtypes = [H]
    L.lgpu_get_obslist.argtypes = [H, ctypes.c_int, ctypes.c_int, IP, FP, ctypes.c_int, IP, IP]
    L.lgpu_debug_metric.argtypes = [H, ctypes.c_int, FP, FP, FP, FP, FP]
    L.lgpu_debug_gc.argtypes = [H, ctypes.c_int, FP, FP, FP]
    L.lgpu_debug_weight.argtypes = [H, ctypes.c_int, FP, FP, FP, FP, FP, FP]
    L.lgpu_host_alloc.argtypes = [ctypes.c_size_t, ctypes.POINTER(ctypes.c_void_p)]
    L.lgpu_host_free.argtypes = [ctypes.c_void_p]
    L.lgpu_flush_l2.argtypes = [H, ctypes.c_size_t]
    L.lgpu_get_obslist_noalloc.argtypes = [H, ctypes.c_int, ctypes.c_int, IP, FP, ctypes.c_int, IP, IP]
    L.lgpu_set_obs_raw.argtypes = [H, ctypes.c_int, ctypes.POINTER(_Obs), IP, FP, IP]
    L.lgpu_set_state_members.argtypes = [H, ctypes.c_int, ctypes.c_int, FP, ctypes.c_int, ctypes.POINTER(_Var)]
    L.lgpu_get_background.argtypes = [H, FP, FP, FP]
    L.lgpu_debug_transform.argtypes = [H, ctypes.c_int, ctypes.c_int, FP, FP]
    L.lgpu_get_obs_prepared.argtypes = [H, FP, FP, FP, FP, FP, FP]
    L.lgpu_bind_state.argtypes = [H, ctypes.c_int, ctypes.c_int, FP, FP, FP, ctypes.c_int, ctypes.POINTER(_Var)]
    L.lgpu_learn_init.argtypes = [H, ctypes.POINTER(_LearnCfg)]
    L.lgpu_learn_collect.argtypes = [H, ctypes.POINTER(ctypes.c_longlong)]
    L.lgpu_learn_train.argtypes = [H, ctypes.c_int, ctypes.c_int, ctypes.c_float, FP]
    L.lgpu_learn_stats_get.argtypes = [H, ctypes.POINTER(LearnStats)]
    L.lgpu_learn_set_network.argtypes = [H, ctypes.c_int]
    L.lgpu_learn_param_count.argtypes = [H]
    L.lgpu_learn_param_count.restype = ctypes.c_longlong
    L.lgpu_learn_get_params.argtypes = [H, FP, ctypes.c_longlong]
    L.lgpu_learn_set_params.argtypes = [H, FP, ctypes.c_longlong]
    L.lgpu_mlp_debug.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, FP, FP, FP, FP,
                                 FP, FP, FP]
    C, LLP = ctypes.c_char_p, ctypes.POINTER(ctypes.c_longlong)
    CPP = ctypes.POINTER(ctypes.c_char_p)
    FPP = ctypes.POINTER(FP)
    L.lgpu_write_diag.argtypes = [H, C, ctypes.c_int, ctypes.c_int, FP, FP]
    L.lgpu_get_loc_diag.argtypes = [H, FP]
    L.lgpu_write_loc_diag.argtypes = [H, C, ctypes.c_int, ctypes.c_int, FP, FP, ctypes.c_int, FP]
    L.lgpu_io_last_error.argtypes = []
    L.lgpu_io_last_error.restype = ctypes.c_char_p
    L.lgpu_ens_filename.argtypes = [C, ctypes.c_int, ctypes.c_char_p, ctypes.c_int]
    L.lgpu_nc_dim_len.argtypes = [C, C, LLP]
    L.lgpu_nc_var_info.argtypes = [C, C, IP, LLP, ctypes.c_int]
    L.lgpu_nc_read_float.argtypes = [C, C, FP, ctypes.c_longlong]
    L.lgpu_nc_read_int.argtypes = [C, C, IP, ctypes.c_longlong]
    L.lgpu_read_obs_nc.argtypes = [C, ctypes.c_int, IP, FP, FP, FP, FP, FP, FP, IP, IP, IP]
    L.lgpu_read_hx_nc.argtypes = [C, ctypes.c_int, ctypes.c_int, FP]
    L.lgpu_read_state_nc.argtypes = [C, C, ctypes.c_int, ctypes.c_int, ctypes.c_int, FP]
    L.lgpu_write_state_nc.argtypes = [C, ctypes.c_int, ctypes.c_int, FP, FP, ctypes.c_int, CPP, IP, FPP,
                                      ctypes.c_int, CPP, IP, FPP]
    L.lgpu_write_diag_nc.argtypes = [C, ctypes.c_int, ctypes.c_int, ctypes.c_int, FP, FP, FP, FP, FP, FP]
    L.lgpu_write_loc_diag_nc.argtypes = [C, ctypes.c_int, ctypes.c_int, FP, FP, FP, FP]
    if path is None:
        _lib = L
    return L


def _fp(a):
    return a.ctypes.data_as(FP)


def _ip(a):
    return a.ctypes.data_as(IP)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


# ---------------------------------------------------------------- configs --
def _interp_points(cfg, key):
    """linearinterp_lat table from a YAML-style entry
    {type: linearinterp_lat, value: [{lat, radius}, ...]} or a list of
    (lat, radius) pairs."""
    v = cfg.get(key)
    if v is None:
        raise ConfigError('missing "%s"' % key)
    if isinstance(v, dict):
        t = v.get("type")
        if t != "linearinterp_lat":
            raise ConfigError('Unrecognized %s type: "%s"' % (key, t))
        v = v.get("value", [])
    pts = []
    for p in v:
        if isinstance(p, dict):
            pts.append((float(p["lat"]), float(p["radius"])))
        else:
            pts.append((float(p[0]), float(p[1])))
    return pts


def normalize_loc(cfg, variables=None):
    """localization: section -> flat description with the reference's meaning.
    variables (list of dicts with 'name') resolves vtloc_surf.bkg_t_var."""
    cls = str(cfg.get("class", "")).lower()
    out = {"class": cls}
    if cls in ("loc_novrt", "loc_vtgc"):
        out["hzloc"] = _interp_points(cfg, "hzloc")
        if cls == "loc_vtgc":
            out["vtloc"] = float(cfg["vtloc"])
    elif cls == "loc_ocean":
        out["hzloc_prof"] = _interp_points(cfg, "hzloc_prof")
        out["hzloc_sat"] = _interp_points(cfg, "hzloc_sat")
        out["tloc_prof"] = float(cfg.get("tloc_prof", -1.0))
        out["tloc_sat"] = float(cfg.get("tloc_sat", -1.0))
        out["sat_obs"] = [int(x) for x in (cfg.get("sat_obs") or [])]
        out["sat_plats"] = [int(x) for x in (cfg.get("sat_plats") or [])]
        vt = cfg.get("vtloc_surf")
        if vt:
            t = vt.get("type")
            if t == "bkg_t":
                var = vt["bkg_t_var"]
                if isinstance(var, str):
                    names = [v["name"] for v in (variables or [])]
                    if var not in names:
                        raise ConfigError('state variable "%s" not found' % var)
                    var = names.index(var)
                out["vtloc_surf"] = {"type": "bkg_t", "bkg_t_delta": float(vt["bkg_t_delta"]), "bkg_t_var": int(var)}
            elif t != "none":
                raise ConfigError("illegal vtloc_surf 'type' given: %s" % t)
    return out


def normalize_solver(cfg):
    """solver: section -> (rtps, rtpp, mul, save_diag) with the reference's
    defaults (src/letkf_solver.F90:86-101)."""
    cfg = cfg or {}
    infl = cfg.get("inflation", cfg)
    return dict(rtps=float(infl.get("rtps", 0.0)), rtpp=float(infl.get("rtpp", 0.0)),
                mul=float(infl.get("mul", 1.0)), save_diag=bool(cfg.get("save_diag", True)))


# ----------------------------------------------------------------- solver --
class Solver:
    """One device handle running the analysis path on one GPU."""

    def __init__(self, device=0):
        self.L = lib()
        self.h = ctypes.c_void_p()
        rc = self.L.lgpu_create(int(device), ctypes.byref(self.h))
        if rc != LGPU_OK:
            raise LgpuError(rc, "lgpu_create failed (no usable sm_103a device?)")
        self._keep = []
        self.ncol = self.k = self.ns = self.nobs = 0
        self.maxgroups = 0

    # -- plumbing
    def _ck(self, rc):
        if rc != LGPU_OK:
            msg = self.L.lgpu_last_error(self.h)
            raise LgpuError(rc, msg.decode() if msg else "")
        return rc

    def close(self):
        if self.h:
            self.L.lgpu_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_variant(self, variant):
        """Gram kernel: 'plain' (per column, FP32 CUDA cores), 'batched'
        (128-column tiles on the tensor cores) or 'auto'."""
        v = VARIANTS[variant] if isinstance(variant, str) else int(variant)
        return self._ck(self.L.lgpu_set_variant(self.h, v))

    def set_precision(self, mode, gap_threshold=1e-6):
        """Eigensolve precision: 'fp32' (the reference's), 'fp32_resolve'
        (FP32, FP64 re-solve of units with a failed solve or a relative
        eigenvalue gap <= gap_threshold) or 'fp64' (every unit)."""
        m = PRECISIONS[mode] if isinstance(mode, str) else int(mode)
        return self._ck(self.L.lgpu_set_precision(self.h, m, float(gap_threshold)))

    # -- letkf_solver_init
    def solver_init(self, cfg=None, **kw):
        c = normalize_solver(cfg)
        c.update(kw)
        self.solver_cfg = c
        s = _SolverCfg(c["rtps"], c["rtpp"], c["mul"], int(c["save_diag"]))
        return self._ck(self.L.lgpu_solver_init(self.h, ctypes.byref(s)))

    # -- letkf_loc_init
    def loc_init(self, cfg, variables=None, lev_depth=None):
        d = normalize_loc(cfg, variables)
        c = _LocCfg()
        keep = []
        c.cls = d["class"].encode()
        keep.append(c.cls)

        def table(pts):
            arr = (_Interp * max(1, len(pts)))()
            for i, (la, r) in enumerate(pts):
                arr[i].lat, arr[i].radius = la, r
            keep.append(arr)
            return len(pts), arr

        c.tloc_prof = c.tloc_sat = -1.0
        if d["class"] in ("loc_novrt", "loc_vtgc"):
            c.n_hz, c.hz = table(d["hzloc"])
        if d["class"] == "loc_vtgc":
            c.vtloc = d["vtloc"]
            lev = _f32(lev_depth if lev_depth is not None else cfg["lev_depth"])
            keep.append(lev)
            c.nlev, c.lev_depth = len(lev), _fp(lev)
        if d["class"] == "loc_ocean":
            c.n_hz, c.hz = table(d["hzloc_prof"])
            c.n_hz_sat, c.hz_sat = table(d["hzloc_sat"])
            c.tloc_prof, c.tloc_sat = d.get("tloc_prof", -1.0), d.get("tloc_sat", -1.0)
            so, sp = _i32(d.get("sat_obs", []) or [0]), _i32(d.get("sat_plats", []) or [0])
            keep += [so, sp]
            c.n_sat_obs, c.sat_obs = len(d.get("sat_obs", [])), _ip(so)
            c.n_sat_plats, c.sat_plats = len(d.get("sat_plats", [])), _ip(sp)
            vt = d.get("vtloc_surf")
            if vt and vt.get("type") == "bkg_t":
                c.vtloc_surf, c.bkg_t_delta, c.bkg_t_var = 1, vt["bkg_t_delta"], vt["bkg_t_var"]
        self._ck(self.L.lgpu_loc_init(self.h, ctypes.byref(c)))
        self.maxgroups = self.L.lgpu_loc_maxgroups(self.h)
        self.loc_desc = d
        return LGPU_OK

    # -- module globals
    def set_grid(self, lat, lon, mask=None):
        lat, lon = _f32(lat), _f32(lon)
        m = _i32(mask if mask is not None else np.zeros(len(lat), np.int32))
        self.ncol = len(lat)
        return self._ck(self.L.lgpu_set_grid(self.h, len(lat), _fp(lat), _fp(lon), _ip(m)))

    def set_state(self, state, mean, sprd, variables):
        state, mean, sprd = _f32(state), _f32(mean), _f32(sprd)
        ncol, ns, k = state.shape
        vs = (_Var * len(variables))()
        for i, v in enumerate(variables):
            vs[i].grid_s_idx, vs[i].levels = v["grid_s_idx"], v["levels"]
            vs[i].ana_inc_max = v.get("ana_inc_max", 9.99e36)
            b = v.get("ana_bounds", (-9.99e36, 9.99e36))
            vs[i].ana_bounds[0], vs[i].ana_bounds[1] = b[0], b[1]
        self.k, self.ns = k, ns
        self._bound = None
        return self._ck(self.L.lgpu_set_state(self.h, k, ns, _fp(state), _fp(mean), _fp(sprd), len(variables), vs))

    def bind_state(self, state, mean, sprd, variables):
        """lgpu_bind_state: every following run() reads the background from
        these arrays and overwrites them with the analysis (in place, like the
        reference's state_ij).  They must be writable float32 C-contiguous
        arrays (page-locked ones, PinnedArray.array, give full link speed) and
        stay alive while bound."""
        for a in (state, mean, sprd):
            if not (isinstance(a, np.ndarray) and a.dtype == np.float32 and a.flags.c_contiguous and a.flags.writeable):
                raise ValueError("bind_state needs writable float32 C-contiguous arrays")
        ncol, ns, k = state.shape
        self.k, self.ns = k, ns
        self._bound = (state, mean, sprd)
        return self._ck(self.L.lgpu_bind_state(self.h, k, ns, _fp(state), _fp(mean), _fp(sprd), len(variables),
                                               self._vars(variables)))

    def set_obs(self, lat, lon, zdim, time, val, err, obsid, platid, hx, hx_mean):
        arrs = [_f32(a) for a in (lat, lon, zdim, time, val, err)] + [_i32(obsid), _i32(platid)]
        hx, hx_mean = _f32(hx), _f32(hx_mean)
        o = _Obs(*[_fp(a) for a in arrs[:6]], _ip(arrs[6]), _ip(arrs[7]))
        self.nobs = len(arrs[0])
        return self._ck(self.L.lgpu_set_obs(self.h, self.nobs, ctypes.byref(o), _fp(hx), _fp(hx_mean)))

    @staticmethod
    def _vars(variables):
        vs = (_Var * len(variables))()
        for i, v in enumerate(variables):
            vs[i].grid_s_idx, vs[i].levels = v["grid_s_idx"], v["levels"]
            vs[i].ana_inc_max = v.get("ana_inc_max", 9.99e36)
            b = v.get("ana_bounds", (-9.99e36, 9.99e36))
            vs[i].ana_bounds[0], vs[i].ana_bounds[1] = b[0], b[1]
        return vs

    def set_state_members(self, members, variables):
        """Full ensemble members [ij, slab, member]; the background mean,
        perturbations and spread are formed on the device
        (src/letkf_state.F90:326-334)."""
        members = _f32(members)
        ncol, ns, k = members.shape
        self.k, self.ns = k, ns
        return self._ck(self.L.lgpu_set_state_members(self.h, k, ns, _fp(members), len(variables),
                                                      self._vars(variables)))

    def set_obs_raw(self, lat, lon, zdim, time, val, err, obsid, platid, hx_members, qc=None):
        """Observations with full member H(x) values [obs, member] and QC
        flags; the mean/perturbation split and the QC compaction run on the
        device (src/letkf_obs.F90:459-488).  Returns the kept count."""
        arrs = [_f32(a) for a in (lat, lon, zdim, time, val, err)] + [_i32(obsid), _i32(platid)]
        hx = _f32(hx_members)
        o = _Obs(*[_fp(a) for a in arrs[:6]], _ip(arrs[6]), _ip(arrs[7]))
        q = _i32(qc) if qc is not None else None
        kept = ctypes.c_int(0)
        self._ck(self.L.lgpu_set_obs_raw(self.h, len(arrs[0]), ctypes.byref(o), _ip(q) if q is not None else None,
                                         _fp(hx), ctypes.byref(kept)))
        self.nobs = kept.value
        return kept.value

    def get_background(self):
        x = np.empty((self.ncol, self.ns, self.k), np.float32)
        m = np.empty((self.ncol, self.ns), np.float32)
        sp = np.empty((self.ncol, self.ns), np.float32)
        self._ck(self.L.lgpu_get_background(self.h, _fp(x), _fp(m), _fp(sp)))
        return x, m, sp

    def get_obs_prepared(self):
        n = self.nobs
        out = dict(hx=np.empty((n, self.k), np.float32), hx_mean=np.empty(n, np.float32),
                   lat=np.empty(n, np.float32), lon=np.empty(n, np.float32), val=np.empty(n, np.float32),
                   err=np.empty(n, np.float32))
        self._ck(self.L.lgpu_get_obs_prepared(self.h, *[_fp(out[k]) for k in ("hx", "hx_mean", "lat", "lon", "val",
                                                                              "err")]))
        return out

    def set_problem(self, prob, variables=None):
        """Upload a letkf_gb300.synth.Problem (grid, state, observations)."""
        self.set_grid(prob.lat, prob.lon, prob.mask)
        self.set_state(prob.state, prob.mean, prob.sprd, variables if variables is not None else prob.vars)
        self.set_obs(prob.olat, prob.olon, prob.oz, prob.otime, prob.oval, prob.oerr, prob.oobsid, prob.oplatid,
                     prob.hx, prob.hx_mean)

    # -- letkf_solver_run
    def run(self):
        return self._ck(self.L.lgpu_solver_run(self.h))

    def get_state(self, out=None):
        if out is None:
            out = (np.empty((self.ncol, self.ns, self.k), np.float32), np.empty((self.ncol, self.ns), np.float32),
                   np.empty((self.ncol, self.ns), np.float32))
        x, m, s = out
        self._ck(self.L.lgpu_get_state(self.h, _fp(x), _fp(m), _fp(s)))
        return x, m, s

    def get_diag(self):
        g = self.maxgroups
        d = dict(maxhz=np.empty(self.ncol, np.float32), obscount=np.empty(self.ncol, np.float32),
                 lg_obscount=np.empty((g, self.ncol), np.float32), lg_obsloc=np.empty((g, self.ncol), np.float32))
        self._ck(self.L.lgpu_get_diag(self.h, _fp(d["maxhz"]), _fp(d["obscount"]), _fp(d["lg_obscount"]),
                                      _fp(d["lg_obsloc"])))
        return d

    def write_diag(self, path, nx, ny, lat_nom, lon_nom):
        """letkf_solver_final's diag.solver.nc of the last run (lgpu_write_diag)."""
        la, lo = _f32(lat_nom), _f32(lon_nom)
        return self._ck(self.L.lgpu_write_diag(self.h, str(path).encode(), int(nx), int(ny), _fp(la), _fp(lo)))

    def get_loc_diag(self):
        """loc_ocean: level count of each column's surface localisation group."""
        out = np.empty(self.ncol, np.float32)
        self._ck(self.L.lgpu_get_loc_diag(self.h, _fp(out)))
        return out

    def write_loc_diag(self, path, nx, ny, lat_nom, lon_nom, vert_nom):
        """loc_ocean_final's diag.loc_ocean.nc of the last run (lgpu_write_loc_diag)."""
        la, lo, vz = _f32(lat_nom), _f32(lon_nom), _f32(vert_nom)
        return self._ck(self.L.lgpu_write_loc_diag(self.h, str(path).encode(), int(nx), int(ny), _fp(la), _fp(lo),
                                                   len(vz), _fp(vz)))

    # -- learned form (no counterpart in the reference)
    def learn_init(self, nx, ny, stride=4, hidden=512, judge_frac=0.02, gate_frac=0.05, sample_frac=0.25,
                   train_cap=200000, seed=0):
        c = _LearnCfg(int(nx), int(ny), int(stride), int(hidden), float(judge_frac), float(gate_frac),
                      float(sample_frac), int(train_cap), int(seed))
        return self._ck(self.L.lgpu_learn_init(self.h, ctypes.byref(c)))

    def learn_collect(self):
        n = ctypes.c_longlong(0)
        self._ck(self.L.lgpu_learn_collect(self.h, ctypes.byref(n)))
        return n.value

    def learn_train(self, epochs=4, batch=1024, lr=1e-3):
        loss = np.zeros(1, np.float32)
        self._ck(self.L.lgpu_learn_train(self.h, int(epochs), int(batch), float(lr), _fp(loss)))
        return float(loss[0])

    def learn_stats(self):
        st = LearnStats()
        self._ck(self.L.lgpu_learn_stats_get(self.h, ctypes.byref(st)))
        return st.as_dict()

    def learn_set_network(self, on=True):
        self._ck(self.L.lgpu_learn_set_network(self.h, 1 if on else 0))

    def learn_params(self):
        n = self.L.lgpu_learn_param_count(self.h)
        if n < 0:
            raise LgpuError(6, "learn_params before learn_init")
        p = np.empty(n, np.float32)
        self._ck(self.L.lgpu_learn_get_params(self.h, _fp(p), n))
        return p

    def learn_set_params(self, p):
        p = _f32(p)
        self._ck(self.L.lgpu_learn_set_params(self.h, _fp(p), p.size))

    def timings(self):
        t = Timings()
        self._ck(self.L.lgpu_get_timings(self.h, ctypes.byref(t)))
        return t.as_dict()

    def obslist(self, ij, group=0):
        cap = max(self.nobs, 1)
        idx = np.zeros(cap, np.int32)
        r = np.zeros(cap, np.float32)
        n, nc = ctypes.c_int(0), ctypes.c_int(0)
        self._ck(self.L.lgpu_get_obslist(self.h, int(ij), int(group), _ip(idx), _fp(r), cap, ctypes.byref(n),
                                         ctypes.byref(nc)))
        m = min(n.value, cap)
        return idx[:m].copy(), r[:m].copy(), nc.value

    def obslist_noalloc(self, ij, group=0, out=None):
        """lgpu_get_obslist_noalloc: same list as obslist() without any device
        allocation; `out` = (idx int32, rloc float32) caller buffers."""
        if out is None:
            cap = max(self.nobs, 1)
            out = (np.zeros(cap, np.int32), np.zeros(cap, np.float32))
        idx, r = out
        n, nc = ctypes.c_int(0), ctypes.c_int(0)
        self._ck(self.L.lgpu_get_obslist_noalloc(self.h, int(ij), int(group), _ip(idx), _fp(r), len(idx),
                                                 ctypes.byref(n), ctypes.byref(nc)))
        m = min(n.value, len(idx))
        return idx[:m].copy(), r[:m].copy(), nc.value

    def final(self):
        return self._ck(self.L.lgpu_solver_final(self.h))

    def flush_l2(self, nbytes=256 << 20):
        return self._ck(self.L.lgpu_flush_l2(self.h, nbytes))

    # -- verification helpers
    def debug_metric(self, lat1, lon1, lat2, lon2):
        a = [_f32(x) for x in (lat1, lon1, lat2, lon2)]
        n = len(a[0])
        out = np.zeros(n, np.float32)
        self._ck(self.L.lgpu_debug_metric(self.h, n, *[_fp(x) for x in a], _fp(out)))
        return out

    def debug_transform(self, gram_packed):
        """Eigensolve stage on packed Gram blocks [nunits, k(k+3)/2] -> T [nunits, k, k]."""
        g = _f32(gram_packed)
        nunits, nf = g.shape
        k = int(round((-3 + (9 + 8 * nf) ** 0.5) / 2))
        out = np.zeros((nunits, k, k), np.float32)
        self._ck(self.L.lgpu_debug_transform(self.h, nunits, k, _fp(g), _fp(out)))
        return out

    def debug_weight(self, lat1, lon1, lat2, lon2, L):
        """Batched-path fast weights: (exact dist, fast dist, exact GC, fast GC,
        fast dist with the short asin series)."""
        a = [_f32(x) for x in (lat1, lon1, lat2, lon2, L)]
        n = len(a[0])
        out = np.zeros(5 * n, np.float32)
        self._ck(self.L.lgpu_debug_weight(self.h, n, *[_fp(x) for x in a], _fp(out)))
        return tuple(out[q * n:(q + 1) * n] for q in range(5))

    def debug_gc(self, z, L):
        z, L = _f32(z), _f32(L)
        n = len(z)
        out = np.zeros(2 * n, np.float32)
        self._ck(self.L.lgpu_debug_gc(self.h, n, _fp(z), _fp(L), _fp(out)))
        return out[:n], out[n:]


def mlp_param_shapes(din, hidden, dout):
    """Shapes of the network parameters in their flat order (W1, b1, W2, b2,
    W3, b3; weights row-major [out][in])."""
    return [(hidden, din), (hidden,), (hidden, hidden), (hidden,), (dout, hidden), (dout,)]


def mlp_debug(params, x, t=None, hidden=512, device=0):
    """The network kernels on one batch (verification): returns loss, the
    gradient from the training kernels, the CUDA-core forward output and the
    tensor-core forward output."""
    L = lib()
    x = _f32(x)
    rows, din = x.shape
    params = _f32(params)
    # dout from the parameter count: H*din + H + H*H + H + dout*H + dout
    rest = params.size - (hidden * din + hidden + hidden * hidden + hidden)
    dout = rest // (hidden + 1)
    if rest != dout * (hidden + 1):
        raise ValueError("parameter count does not match din=%d hidden=%d" % (din, hidden))
    t = np.zeros((rows, dout), np.float32) if t is None else _f32(t)
    loss = np.zeros(1, np.float32)
    grad = np.empty(params.size, np.float32)
    ys = np.empty((rows, dout), np.float32)
    yt = np.empty((rows, dout), np.float32)
    rc = L.lgpu_mlp_debug(int(device), din, int(hidden), int(dout), rows, _fp(params), _fp(x), _fp(t), _fp(loss),
                          _fp(grad), _fp(ys), _fp(yt))
    if rc != LGPU_OK:
        raise LgpuError(rc, "lgpu_mlp_debug failed")
    return {"loss": float(loss[0]), "grad": grad, "y_simt": ys, "y_tc": yt}


class PinnedArray:
    """numpy view over page-locked host memory from lgpu_host_alloc."""

    def __init__(self, shape, dtype=np.float32):
        self.L = lib()
        n = int(np.prod(shape)) * np.dtype(dtype).itemsize
        self.ptr = ctypes.c_void_p()
        rc = self.L.lgpu_host_alloc(n, ctypes.byref(self.ptr))
        if rc != LGPU_OK:
            raise LgpuError(rc, "lgpu_host_alloc(%d) failed" % n)
        buf = (ctypes.c_char * n).from_address(self.ptr.value)
        self.array = np.frombuffer(buf, dtype=dtype).reshape(shape)

    def free(self):
        if self.ptr:
            self.array = None
            self.L.lgpu_host_free(self.ptr)
            self.ptr = ctypes.c_void_p()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def analyse(prob, localization, solver=None, variables=None, device=0):
    """Run one analysis of a synthetic Problem; returns (state, mean, sprd,
    diag, timings)."""
    with Solver(device) as s:
        s.solver_init(solver)
        s.loc_init(localization, variables if variables is not None else prob.vars, prob.lev_depth)
        s.set_problem(prob, variables)
        s.run()
        x, m, sp = s.get_state()
        d = s.get_diag()
        t = s.timings()
    return x, m, sp, d, t
