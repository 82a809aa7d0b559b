"""CPU: the cycling helpers of the synthetic generator (the learned form's
workload): the forecast step keeps a constant field constant, moves a
zonal pattern eastwards at the jet speed, recomputes the background
statistics (k - 1 spread, perturbations summing to zero), and new
observations keep the clustered network's centres across cycles."""
import numpy as np

from letkf_gb300 import synth


def _small():
    return synth.generate("c3", nx=72, ny=36, nz=2, n_obs=2000, k=8)


def test_forecast_statistics_and_constant_field():
    p = _small()
    p.state[...] = 0.0
    p.mean[...] = 3.0
    p.truth[...] = 3.0
    synth.forecast(p)
    assert np.allclose(p.mean, 3.0, atol=1e-5) and np.allclose(p.truth, 3.0, atol=1e-5)
    assert np.allclose(p.state, 0.0, atol=1e-5) and np.allclose(p.sprd, 0.0, atol=1e-5)
    q = _small()
    synth.forecast(q)
    assert np.allclose(q.state.sum(axis=2), 0.0, atol=1e-3)
    full = q.state + q.mean[:, :, None]
    sd = np.sqrt(((full - full.mean(axis=2, keepdims=True)) ** 2).sum(axis=2) / (q.k - 1))
    assert np.allclose(sd, q.sprd, rtol=1e-3, atol=1e-5)


def test_forecast_moves_a_zonal_pattern_east():
    p = _small()
    nx, ny = p.nx, p.ny
    i = np.arange(p.ncol) % nx
    j = np.arange(p.ncol) // nx
    wave = np.cos(2 * np.pi * i / nx).astype(np.float32)
    p.state[...] = 0.0
    p.truth[...] = wave[:, None]
    p.mean[...] = wave[:, None]
    dt = 40 * 86400.0
    synth.forecast(p, u=0.5, kappa=0.0, dt=dt)
    # at the equator row the shift is u dt / (R dlon) cells
    row = ny // 2
    lat = -90 + (row + 0.5) * 180.0 / ny
    cells = 0.5 * dt / (6371000.0 * np.cos(np.radians(lat)) * 2 * np.pi / nx)
    got = p.truth[j == row, 0]
    phase = np.angle(np.sum(got * np.exp(-2j * np.pi * np.arange(nx) / nx)))
    assert abs((-phase) * nx / (2 * np.pi) - cells) < 0.1


def test_observe_keeps_cluster_centres():
    p = _small()
    a = synth.observe(p, seed=1, n_obs=4000)
    b = synth.observe(p, seed=2, n_obs=4000)
    assert not np.array_equal(a.olat, b.olat)
    ha = np.histogram2d(a.olat, a.olon, bins=(18, 36))[0].ravel()
    hb = np.histogram2d(b.olat, b.olon, bins=(18, 36))[0].ravel()
    assert np.corrcoef(ha, hb)[0, 1] > 0.9
    assert a.hx.shape == (4000, p.k) and np.allclose(a.hx.sum(axis=1), 0.0, atol=1e-3)
