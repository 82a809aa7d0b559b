"""lgpu_get_obslist_noalloc: the local-observation-list query for callers that
cannot allocate device memory (hosts that hand out their own pre-allocated
device pool, or whose memory footprint is fixed once they start).  Its scratch is a fixed
__device__ array inside the library; these tests call it through the C ABI
and check it against lgpu_get_obslist (same lists, same order, same weights,
same candidate counts) on consecutive calls, and that tables larger than the
fixed capacity are refused.

Collected last on purpose (file name), so a run that stops at the first
failure has already run every other test; it also passes on its own in a
fresh process."""
from dataclasses import replace

import numpy as np
import pytest

from conftest import workload
from helpers import gpu_run, workload_cfg

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["simple3d", "c1"])
def test_noalloc_matches_obslist_on_consecutive_calls(name):
    cfg = workload_cfg(name)
    prob = workload(cfg["gen"]["workload"], **{k: v for k, v in cfg["gen"].items() if k != "workload"})
    res = gpu_run(prob, cfg["localization"], cfg["solver"], keep_open=True)
    s = res["solver"]
    try:
        rng = np.random.default_rng(3)
        active = np.nonzero(prob.mask == 0)[0]
        cols = list(rng.choice(active, size=6, replace=False))
        # the column next to the first observation has a non-empty list
        cols.insert(0, int(np.argmin((prob.lat - prob.olat[0]) ** 2 + (prob.lon - prob.olon[0] % 360) ** 2)))
        groups = [0, s.maxgroups - 1]
        nonempty = 0
        for c in cols:
            for g in groups:
                ref = s.obslist(int(c), g)
                first = s.obslist_noalloc(int(c), g)     # two calls in a row share the scratch
                second = s.obslist_noalloc(int(c), g)
                for got in (first, second):
                    assert np.array_equal(got[0], ref[0])
                    assert np.array_equal(got[1].view(np.uint32), ref[1].view(np.uint32))
                    assert got[2] == ref[2]
                nonempty += len(ref[0]) > 0
        assert nonempty > 0
        # a short caller buffer receives the first entries of the canonical list
        c = cols[0]
        ref = s.obslist(int(c), 0)
        if len(ref[0]) > 1:
            idx = np.zeros(1, np.int32)
            r = np.zeros(1, np.float32)
            got = s.obslist_noalloc(int(c), 0, out=(idx, r))
            assert got[0][0] == ref[0][0] and got[1][0] == ref[1][0]
    finally:
        s.close()


def test_noalloc_rejects_tables_over_capacity():
    from letkf_gb300 import LgpuError
    prob = workload("simple3d")
    rng = np.random.default_rng(11)
    n = 262144 + 4096                  # above the fixed list capacity with a margin
    hx = rng.standard_normal((n, prob.k)).astype(np.float32)
    hx -= hx.mean(1, keepdims=True)
    big = replace(prob, olat=np.degrees(np.arcsin(rng.uniform(-1, 1, n))).astype(np.float32),
                  olon=rng.uniform(0, 360, n).astype(np.float32), oz=np.ones(n, np.float32),
                  otime=np.zeros(n, np.float32), oval=rng.standard_normal(n).astype(np.float32),
                  oerr=np.ones(n, np.float32), oobsid=np.ones(n, np.int32), oplatid=np.ones(n, np.int32),
                  hx=hx, hx_mean=np.zeros(n, np.float32))
    cfg = workload_cfg("simple3d")
    res = gpu_run(big, cfg["localization"], {}, keep_open=True, variant="batched")
    s = res["solver"]
    try:
        assert s.nobs > 262144, "the table must exceed the fixed capacity for the refusal to be tested"
        with pytest.raises(LgpuError) as e:
            s.obslist_noalloc(0, 0)
        assert e.value.code == 7 and "exceed" in e.value.msg
    finally:
        s.close()
