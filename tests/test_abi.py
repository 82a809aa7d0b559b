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
