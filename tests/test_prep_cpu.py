"""CPU: the numpy restatement of the reference's pre-processing reproduces the
synthetic generator's background and observation-space statistics bit for
bit (both follow src/letkf_state.F90:326-334 and src/letkf_obs.F90:459-466)."""
import numpy as np

from conftest import workload
from prep_ref import background_stats, hx_stats


def test_generator_statistics_follow_reference_semantics():
    p = workload("c1")
    # the generator derived p.state/p.mean/p.sprd from full members it does not
    # keep; re-deriving from pert+mean reproduces mean and spread to 1 ulp
    members = (p.state + p.mean[:, :, None]).astype(np.float32)
    pert, mean, sprd = background_stats(members)
    assert np.max(np.abs(mean - p.mean)) <= 2e-6 * np.max(np.abs(p.mean))
    assert np.allclose(sprd, p.sprd, rtol=1e-5)
    hxm = (p.hx + p.hx_mean[:, None]).astype(np.float32)
    hp, hm, keep = hx_stats(hxm)
    assert keep.all()
    assert np.allclose(hm, p.hx_mean, rtol=0, atol=2e-6 * np.max(np.abs(p.hx_mean)))
    assert np.allclose(hp, p.hx, atol=1e-5)
