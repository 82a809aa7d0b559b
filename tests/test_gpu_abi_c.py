"""GPU: the C ABI driven from plain C (tests/abi_c/test_abi.c, compiled with
gcc against include/letkf_gpu.h and linked to liblgpu.so): status codes, a
small analysis into a bound state, diagnostics, timings and the list query,
as a Fortran or C host would call them."""
import subprocess

import pytest

from test_abi import build_abi_program

pytestmark = pytest.mark.gpu


def test_abi_from_c(tmp_path):
    exe = build_abi_program(tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    print(r.stdout, r.stderr)
    assert r.returncode == 0, r.stderr
    assert r.stdout.startswith("abi ok")
