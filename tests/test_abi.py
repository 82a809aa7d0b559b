"""CPU checks of the C ABI and the host-side logic (no GPU needed): the
library builds for sm_103a and exports every entry point include/letkf_gpu.h
declares; configuration handling mirrors the reference's messages."""
import ctypes
import os
import re

import pytest

from conftest import ROOT


def header_functions():
    src = open(os.path.join(ROOT, "include", "letkf_gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(lgpu_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_header_function():
    from letkf_gb300 import EXPORTS, _build
    path = _build.lgpu_lib_path()
    if not os.path.exists(path):
        _build.build_lgpu()
    lib = ctypes.CDLL(path)
    names = header_functions()
    assert len(names) >= 17
    for n in names:
        assert hasattr(lib, n), n
    assert set(EXPORTS) == set(names)


def test_build_targets_sm103a_only():
    from letkf_gb300 import _build
    assert "-gencode=arch=compute_103a,code=sm_103a" in _build.NVCC_FLAGS
    assert not any("sm_90" in f or "sm_100" in f for f in _build.NVCC_FLAGS)


def test_config_normalization_messages():
    from letkf_gb300 import ConfigError, normalize_loc, normalize_solver
    assert normalize_solver({}) == dict(rtps=0.0, rtpp=0.0, mul=1.0, save_diag=True)
    assert normalize_solver({"inflation": {"rtps": 0.6}})["rtps"] == 0.6
    d = normalize_loc({"class": "LOC_NOVRT", "hzloc": {"type": "linearinterp_lat",
                                                      "value": [{"lat": 0, "radius": 5e5}]}})
    assert d == {"class": "loc_novrt", "hzloc": [(0.0, 5e5)]}
    with pytest.raises(ConfigError, match='Unrecognized hzloc type: "gaussian"'):
        normalize_loc({"class": "loc_novrt", "hzloc": {"type": "gaussian", "value": []}})
    with pytest.raises(ConfigError, match="illegal vtloc_surf 'type' given: dpth"):
        normalize_loc({"class": "loc_ocean", "hzloc_prof": [(0, 1e5)], "hzloc_sat": [(0, 1e5)],
                       "vtloc_surf": {"type": "dpth"}})
    d = normalize_loc({"class": "loc_ocean", "hzloc_prof": [(0, 1e5)], "hzloc_sat": [(0, 1e5)],
                       "vtloc_surf": {"type": "bkg_t", "bkg_t_delta": 0.2, "bkg_t_var": "T"}},
                      variables=[{"name": "S"}, {"name": "T"}])
    assert d["vtloc_surf"]["bkg_t_var"] == 1


def test_missing_library_fails_loudly(tmp_path):
    from letkf_gb300 import LgpuError, lib
    with pytest.raises(LgpuError):
        lib(str(tmp_path / "nope.so"))


def test_no_device_fails_loudly_and_null_handles_are_rejected():
    """Without a GPU the library refuses to start (there is no CPU path), and
    every setter rejects a null handle with LGPU_ERR_ARG."""
    from letkf_gb300 import _build
    path = _build.lgpu_lib_path()
    if not os.path.exists(path):
        _build.build_lgpu()
    lib = ctypes.CDLL(path)
    H = ctypes.c_void_p
    lib.lgpu_set_precision.argtypes = [H, ctypes.c_int, ctypes.c_float]
    lib.lgpu_set_variant.argtypes = [H, ctypes.c_int]
    lib.lgpu_solver_run.argtypes = [H]
    lib.lgpu_create.argtypes = [ctypes.c_int, ctypes.POINTER(H)]
    lib.lgpu_destroy.argtypes = [H]
    assert lib.lgpu_set_precision(None, 1, 1e-6) == 1
    assert lib.lgpu_set_variant(None, 2) == 1
    assert lib.lgpu_solver_run(None) == 1
    h = H()
    rc = lib.lgpu_create(0, ctypes.byref(h))
    if rc == 0:   # a GPU is present: nothing to check here
        lib.lgpu_destroy(h)
        pytest.skip("a CUDA device is present")
    assert rc == 2 and not h.value   # LGPU_ERR_CUDA, no handle


# ---- the header pinned in compiled code: tests/abi_c/test_abi.c is built with
# gcc against include/letkf_gpu.h and prints every struct's layout; the
# ctypes mirror of the Python host and the Fortran BIND(C) types of
# umd-letkf_gb300/fortran/letkf_gpu_c.F90 must match it field by field

def build_abi_program(tmpdir):
    import shutil
    import subprocess
    from letkf_gb300 import _build
    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    lib_dir = os.path.dirname(_build.lgpu_lib_path())
    if not os.path.exists(_build.lgpu_lib_path()):
        _build.build_lgpu()
    exe = os.path.join(str(tmpdir), "test_abi")
    subprocess.check_call(["gcc", "-std=c11", "-Wall", "-Wextra", "-Werror", "-O1", "-I",
                           os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "abi_c", "test_abi.c"),
                           "-L", lib_dir, "-llgpu", "-Wl,-rpath," + lib_dir, "-lm", "-o", exe])
    return exe


def c_layout(exe):
    import subprocess
    out = subprocess.check_output([exe, "layout"], text=True)
    lay = {}
    for line in out.split("\n"):
        if not line.strip():
            continue
        st, field, off, size = line.split()
        lay.setdefault(st, {})[field] = (int(off), int(size))
    return lay


FORTRAN_KINDS = {"c_int": (4, 4), "c_float": (4, 4), "c_double": (8, 8), "c_long_long": (8, 8),
                 "c_size_t": (8, 8), "c_ptr": (8, 8)}


def fortran_layout(path):
    """Offsets of the BIND(C) derived types under the C layout rules (each
    component aligned to its size, the struct padded to its largest
    alignment)."""
    src = open(path).read()
    types = {}
    for m in re.finditer(r"TYPE, BIND\(C\) :: (\w+)\n(.*?)END TYPE", src, flags=re.S):
        name, body = m.group(1), m.group(2)
        off, align, fields = 0, 1, {}
        for line in body.split("\n"):
            line = line.split("!")[0].strip()
            if not line:
                continue
            km = re.match(r"(?:REAL|INTEGER|TYPE)\((\w+)\)\s*::\s*(.*)", line)
            assert km, line
            size, al = FORTRAN_KINDS[km.group(1)]
            for comp in [c.strip() for c in re.split(r",(?![^(]*\))", km.group(2))]:
                cm = re.match(r"(\w+)(?:\((\d+)\))?$", comp)
                n = int(cm.group(2) or 1)
                off = (off + al - 1) // al * al
                fields[cm.group(1).lower()] = (off, size * n)
                off += size * n
                align = max(align, al)
        fields["-"] = (0, (off + align - 1) // align * align)
        types[name] = fields
    return types


def test_header_layout_matches_ctypes_and_fortran(tmp_path):
    import letkf_gb300 as L
    lay = c_layout(build_abi_program(tmp_path))
    mirrors = {"lgpu_solver_config": L._SolverCfg, "lgpu_interp_point": L._Interp, "lgpu_loc_config": L._LocCfg,
               "lgpu_statevar": L._Var, "lgpu_obs": L._Obs, "lgpu_timings": L.Timings,
               "lgpu_learn_config": L._LearnCfg, "lgpu_learn_stats": L.LearnStats}
    assert set(mirrors) == set(lay)
    for st, cls in mirrors.items():
        got = {n: (getattr(cls, n).offset, getattr(cls, n).size) for n, _ in cls._fields_}
        got["-"] = (0, ctypes.sizeof(cls))
        assert got == lay[st], st
    fl = fortran_layout(os.path.join(ROOT, "umd-letkf_gb300", "fortran", "letkf_gpu_c.F90"))
    assert set(fl) == set(lay)
    for st in lay:
        assert fl[st] == lay[st], st


def test_fortran_interfaces_cover_the_solver_path():
    """Every solver-path entry point of the header has a BIND(C) interface
    with the C name in the Fortran module."""
    src = open(os.path.join(ROOT, "umd-letkf_gb300", "fortran", "letkf_gpu_c.F90")).read()
    bound = set(re.findall(r'BIND\(C, name="(lgpu_\w+)"\)', src))
    need = {"lgpu_create", "lgpu_destroy", "lgpu_last_error", "lgpu_solver_init", "lgpu_loc_init",
            "lgpu_loc_maxgroups", "lgpu_set_variant", "lgpu_set_precision", "lgpu_set_grid", "lgpu_set_state",
            "lgpu_bind_state", "lgpu_set_state_members", "lgpu_set_obs", "lgpu_set_obs_raw", "lgpu_solver_run",
            "lgpu_get_state", "lgpu_get_diag", "lgpu_get_timings", "lgpu_solver_final", "lgpu_get_obslist",
            "lgpu_write_diag", "lgpu_write_loc_diag", "lgpu_host_alloc", "lgpu_host_free"}
    assert need <= bound, sorted(need - bound)
    assert bound <= set(header_functions())


def test_fortran_solver_module_uses_bound_entry_points():
    """The replacement solver module (letkf_solver_gpu.F90) calls only entry
    points the binding module declares, and keeps the reference's three
    public procedures."""
    d = os.path.join(ROOT, "umd-letkf_gb300", "fortran")
    binding = open(os.path.join(d, "letkf_gpu_c.F90")).read()
    solver = open(os.path.join(d, "letkf_solver_gpu.F90")).read()
    bound = set(re.findall(r"FUNCTION (lgpu_\w+)\(|SUBROUTINE (lgpu_\w+)\(", binding))
    bound = {a or b for a, b in bound}
    called = set(re.findall(r"\b(lgpu_\w+)\s*\(", solver))
    assert called and called <= bound, sorted(called - bound)
    assert re.search(r"^MODULE letkf_solver$", solver, flags=re.M)
    for name in ("letkf_solver_init", "letkf_solver_run", "letkf_solver_final"):
        assert "PUBLIC :: %s" % name in solver
