"""GPU: the pre-processing upstream of the analysis, on the device, through the
C ABI (lgpu_set_state_members, lgpu_set_obs_raw) against the numpy
restatement of the reference (src/letkf_state.F90:326-334,
src/letkf_obs.F90:459-488): bit-exact statistics, order-preserving QC
compaction, and a bit-identical analysis compared with uploading the
host-prepared arrays."""
import numpy as np
import pytest

from conftest import workload
from helpers import workload_cfg
from prep_ref import background_stats, hx_stats

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["c1", "ocean"])
def test_device_preparation_matches_reference(name):
    from letkf_gb300 import Solver
    cfg = workload_cfg(name)
    p = workload(cfg["gen"]["workload"], **{k: v for k, v in cfg["gen"].items() if k != "workload"})
    members = (p.state + p.mean[:, :, None]).astype(np.float32)
    hxm = (p.hx + p.hx_mean[:, None]).astype(np.float32)
    rng = np.random.default_rng(9)
    qc = (rng.random(p.nobs) < 0.1).astype(np.int32) * rng.integers(1, 4, p.nobs).astype(np.int32)
    pert, mean, sprd = background_stats(members)
    hp, hm, keep = hx_stats(hxm, qc)

    # one Gram form in both runs (AUTO picks the faster form by timing, which
    # may differ between the two solvers)
    with Solver(0) as s:
        s.solver_init(cfg["solver"])
        s.loc_init(cfg["localization"], p.vars, p.lev_depth)
        s.set_variant("batched")
        s.set_grid(p.lat, p.lon, p.mask)
        s.set_state_members(members, p.vars)
        gx, gm, gs = s.get_background()
        assert np.array_equal(gx.view(np.uint32), pert.view(np.uint32))
        assert np.array_equal(gm.view(np.uint32), mean.view(np.uint32))
        assert np.array_equal(gs.view(np.uint32), sprd.view(np.uint32))
        kept = s.set_obs_raw(p.olat, p.olon, p.oz, p.otime, p.oval, p.oerr, p.oobsid, p.oplatid, hxm, qc)
        assert kept == int(keep.sum())
        o = s.get_obs_prepared()
        assert np.array_equal(o["hx"].view(np.uint32), hp[keep].view(np.uint32))
        assert np.array_equal(o["hx_mean"].view(np.uint32), hm[keep].view(np.uint32))
        for key, src in (("lat", p.olat), ("lon", p.olon), ("val", p.oval), ("err", p.oerr)):
            assert np.array_equal(o[key], src[keep])
        s.run()
        xa, ma, sa = s.get_state()

    with Solver(0) as s:
        s.solver_init(cfg["solver"])
        s.loc_init(cfg["localization"], p.vars, p.lev_depth)
        s.set_variant("batched")
        s.set_grid(p.lat, p.lon, p.mask)
        s.set_state(pert, mean, sprd, p.vars)
        s.set_obs(p.olat[keep], p.olon[keep], p.oz[keep], p.otime[keep], p.oval[keep], p.oerr[keep], p.oobsid[keep],
                  p.oplatid[keep], hp[keep], hm[keep])
        s.run()
        xb, mb, sb = s.get_state()
    assert np.array_equal(xa, xb) and np.array_equal(ma, mb) and np.array_equal(sa, sb)
