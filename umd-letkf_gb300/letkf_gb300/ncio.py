"""The file formats either side of the analysis path, through the library's
NetCDF classic reader and writer (C ABI, host code; no device needed):

  ens_filename(pattern, ensmem)      parse_ens_filename (src/letkf_state_helper.F90:445-510)
  read_obs(path)                     obsio_nc_read_obs (src/subclass.letkf_obsio/letkf_obsio_nc.F90:150-237)
  read_hx(pattern, k, nobs, inc)     obsio_nc_read_hx for members 1..k (:244-306) -> [nobs][k]
  read_state_members(pattern, var, k, nx, ny, nz)
                                     stateio_nc_read_state for members 1..k
                                     (src/subclass.letkf_stateio/letkf_stateio_nc.F90:196-245) -> [k][nz][ny][nx]
  write_state(path, ...)             stateio_nc_write_state (:252-370), classic format
  write_diag_arrays(path, ...)       letkf_solver_final's diag.solver.nc from host arrays
  write_loc_diag_arrays(path, ...)   loc_ocean_final's diag.loc_ocean.nc from host arrays

Members are numbered from 1 as the reference numbers them.  Errors raise
LgpuError with the library's message (lgpu_io_last_error)."""
import ctypes

import numpy as np

from . import FP, IP, LGPU_OK, LgpuError, _f32, _fp, _i32, _ip, lib


def _ck(rc):
    if rc != LGPU_OK:
        msg = lib().lgpu_io_last_error()
        raise LgpuError(rc, msg.decode() if msg else "")
    return rc


def _b(s):
    return str(s).encode()


def ens_filename(pattern, ensmem):
    buf = ctypes.create_string_buffer(4096)
    _ck(lib().lgpu_ens_filename(_b(pattern), int(ensmem), buf, len(buf)))
    return buf.value.decode()


def dim_len(path, dim):
    n = ctypes.c_longlong(0)
    _ck(lib().lgpu_nc_dim_len(_b(path), _b(dim), ctypes.byref(n)))
    return n.value


def var_shape(path, var):
    nd = ctypes.c_int(0)
    d = (ctypes.c_longlong * 8)()
    _ck(lib().lgpu_nc_var_info(_b(path), _b(var), ctypes.byref(nd), d, 8))
    return tuple(int(d[i]) for i in range(nd.value))


def read_var(path, var, dtype=np.float32):
    shape = var_shape(path, var)
    out = np.empty(shape, np.int32 if np.dtype(dtype).kind == "i" else np.float32)
    n = int(np.prod(shape))
    if out.dtype == np.int32:
        _ck(lib().lgpu_nc_read_int(_b(path), _b(var), _ip(out), n))
    else:
        _ck(lib().lgpu_nc_read_float(_b(path), _b(var), _fp(out), n))
    return out


def read_obs(path):
    """One observation file: dict with obsid, platid, lat, lon, zdim, time,
    val, err, qc (the letkf_observation fields, src/letkf_obs.F90:57-68)."""
    L = lib()
    n = ctypes.c_int(0)
    _ck(L.lgpu_read_obs_nc(_b(path), 0, ctypes.byref(n), None, None, None, None, None, None, None, None, None))
    m = n.value
    f = {k: np.empty(m, np.float32) for k in ("lat", "lon", "zdim", "time", "val", "err")}
    i = {k: np.empty(m, np.int32) for k in ("obsid", "platid", "qc")}
    _ck(L.lgpu_read_obs_nc(_b(path), m, ctypes.byref(n), _fp(f["lat"]), _fp(f["lon"]), _fp(f["zdim"]),
                           _fp(f["time"]), _fp(f["val"]), _fp(f["err"]), _ip(i["obsid"]), _ip(i["platid"]),
                           _ip(i["qc"])))
    return dict(f, **i)


def read_hx(pattern, k, nobs, read_inc=False):
    """H(x) of members 1..k from the files `pattern` names (#ENSn#): [nobs][k]."""
    hx = np.empty((k, nobs), np.float32)
    for m in range(k):
        _ck(lib().lgpu_read_hx_nc(_b(ens_filename(pattern, m + 1)), int(nobs), int(bool(read_inc)), _fp(hx[m])))
    return np.ascontiguousarray(hx.T)


def read_state_members(pattern, var, k, nx, ny, nz):
    """Variable `var` of members 1..k: [k][nz][ny][nx]."""
    out = np.empty((k, nz, ny, nx), np.float32)
    for m in range(k):
        _ck(lib().lgpu_read_state_nc(_b(ens_filename(pattern, m + 1)), _b(var), int(nx), int(ny), int(nz),
                                     _fp(out[m])))
    return out


def write_state(path, lon_nom, lat_nom, vtgrids, variables):
    """vtgrids: list of (name, nominal depths); variables: list of (name,
    vtgrid index, values [nz][ny][nx] or [ny][nx] on a one-level grid)."""
    lon, lat = _f32(lon_nom), _f32(lat_nom)
    nx, ny = len(lon), len(lat)
    vt_names = (ctypes.c_char_p * max(1, len(vtgrids)))(*[_b(n) for n, _ in vtgrids])
    vt_arrays = [_f32(v) for _, v in vtgrids]
    vt_len = _i32([len(v) for v in vt_arrays])
    vt_ptr = (FP * max(1, len(vtgrids)))(*[_fp(v) for v in vt_arrays])
    names = (ctypes.c_char_p * max(1, len(variables)))(*[_b(n) for n, _, _ in variables])
    var_vt = _i32([g for _, g, _ in variables])
    vals = []
    for n, g, v in variables:
        a = _f32(v)
        if a.size != len(vt_arrays[g]) * ny * nx:
            raise ValueError("variable %s: %d values, grid holds %d" % (n, a.size, len(vt_arrays[g]) * ny * nx))
        vals.append(a)
    val_ptr = (FP * max(1, len(vals)))(*[_fp(v) for v in vals])
    _ck(lib().lgpu_write_state_nc(_b(path), nx, ny, _fp(lon), _fp(lat), len(vtgrids), vt_names, _ip(vt_len),
                                  vt_ptr, len(variables), names, _ip(var_vt), val_ptr))


def write_diag_arrays(path, lat_nom, lon_nom, maxhz, obscount, lg_obscount, lg_obsloc):
    lat, lon = _f32(lat_nom), _f32(lon_nom)
    a, b, c, d = (_f32(x) for x in (maxhz, obscount, lg_obscount, lg_obsloc))
    groups = c.size // (len(lat) * len(lon))
    _ck(lib().lgpu_write_diag_nc(_b(path), len(lon), len(lat), groups, _fp(lat), _fp(lon), _fp(a), _fp(b), _fp(c),
                                 _fp(d)))


def write_loc_diag_arrays(path, lat_nom, lon_nom, surf_lvl, surf_depth):
    lat, lon = _f32(lat_nom), _f32(lon_nom)
    a, b = _f32(surf_lvl), _f32(surf_depth)
    _ck(lib().lgpu_write_loc_diag_nc(_b(path), len(lon), len(lat), _fp(lat), _fp(lon), _fp(a), _fp(b)))
