"""Shared test setup: import paths, the `gpu` marker, cached workloads.

CPU tests (-m "not gpu") check the oracle against known answers, the host
logic and the C ABI's exported symbols.  GPU tests (-m gpu) call the CUDA
library through its C ABI and compare with the oracle."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "umd-letkf_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs an sm_103a GPU and the built CUDA library")


_cache = {}


def workload(name, **kw):
    """Generate (once per session) a synthetic workload."""
    from letkf_gb300 import synth
    key = (name, tuple(sorted(kw.items())))
    if key not in _cache:
        _cache[key] = synth.generate(name, **kw)
    return _cache[key]


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle as O
    O.build()
    return O
