"""GPU: the analysis between files, as the reference runs it: ensemble
members in per-member state files (stateio_nc), observations and per-member
hx files (obsio_nc), read through the library's NetCDF classic reader into
the device-side preparation (src/letkf_state.F90:326-334,
src/letkf_obs.F90:459-488), analysed, and the diagnostics files of
letkf_solver_final and loc_ocean_final written and read back with
scipy.io.netcdf_file.

Bars (written here):
  - the analysis from files equals the in-memory analysis of the same
    workload within the parity bar (1e-5 relative L2 over the perturbations
    and the mean; the device forms mean and spread from the members, the
    in-memory path takes the generator's), observation lists bit-identical;
  - diag.solver.nc holds the run's diagnostics exactly, with the reference's
    dimensions and attributes;
  - diag.loc_ocean.nc's vtloc_surf_lvl equals calc_mldlvl_bkgt
    (src/subclass.letkf_localizer/letkf_loc_ocean.F90:408-427) evaluated in
    numpy on the background mean; vtloc_surf_depth is the level's depth.
"""
import numpy as np
import pytest

from conftest import workload
from helpers import gpu_run, rel_l2, workload_cfg

pytestmark = pytest.mark.gpu
netcdf_file = pytest.importorskip("scipy.io").netcdf_file


def _mld_levels(mean, t_idx, t_len, delta):
    """calc_mldlvl_bkgt on every column of the background mean [ncol][ns]."""
    t0 = mean[:, t_idx].astype(np.float32)
    out = np.full(mean.shape[0], t_len, np.int32)
    done = np.zeros(mean.shape[0], bool)
    for i in range(1, t_len):
        hit = ~done & (np.abs(t0 - mean[:, t_idx + i].astype(np.float32)) > np.float32(delta))
        out[hit] = i
        done |= hit
    return out


def test_files_in_analysis_and_diagnostics_out(tmp_path):
    from letkf_gb300 import Solver, ncio
    cfg = workload_cfg("c2ocean")
    prob = workload(cfg["gen"]["workload"], **{k: v for k, v in cfg["gen"].items() if k != "workload"})
    nx, ny, nz, k = prob.nx, prob.ny, prob.nz, prob.k
    lat_nom = prob.lat.reshape(ny, nx)[:, 0].copy()
    lon_nom = prob.lon.reshape(ny, nx)[0, :].copy()
    v = {x["name"]: x for x in prob.vars}
    # ensemble members on files, [nz][ny][nx] per variable
    members = prob.state + prob.mean[:, :, None]                    # [ncol][ns][k]
    for m in range(k):
        def field(name):
            i0, n = v[name]["grid_s_idx"], v[name]["levels"]
            return np.ascontiguousarray(members[:, i0:i0 + n, m].T.reshape(n, ny, nx))
        ncio.write_state(tmp_path / ("bkg.%03d.nc" % (m + 1)), lon_nom, lat_nom,
                         [("depth", prob.lev_depth), ("surface", np.zeros(1, np.float32))],
                         [("T", 0, field("T")), ("S", 0, field("S")), ("SSH", 1, field("SSH"))])
    # observations and hx files, written by scipy (an independent writer)
    n = prob.nobs
    hx_full = prob.hx + prob.hx_mean[:, None]
    with netcdf_file(str(tmp_path / "obs.nc"), "w") as f:
        f.createDimension("obs", n)
        for name, arr, typ in (("obid", prob.oobsid, "i4"), ("plat", prob.oplatid, "i4"), ("lat", prob.olat, "f4"),
                               ("lon", prob.olon, "f4"), ("depth", prob.oz, "f4"), ("hr", prob.otime, "f4"),
                               ("val", prob.oval, "f4"), ("err", prob.oerr, "f4"),
                               ("qc", np.zeros(n, np.int32), "i4")):
            f.createVariable(name, typ, ("obs",))[:] = arr
    for m in range(k):
        with netcdf_file(str(tmp_path / ("hx.%03d.nc" % (m + 1))), "w") as f:
            f.createDimension("obs", n)
            f.createVariable("hx", "f4", ("obs",))[:] = hx_full[:, m]
    # read back through the library
    fields = {name: ncio.read_state_members(str(tmp_path / "bkg.#ENS3#.nc"), name, k, nx, ny, v[name]["levels"])
              for name in ("T", "S", "SSH")}
    mem = np.empty_like(members)
    for name, a in fields.items():
        i0, nl = v[name]["grid_s_idx"], v[name]["levels"]
        mem[:, i0:i0 + nl, :] = a.reshape(k, nl, ny * nx).transpose(2, 1, 0)
    assert np.array_equal(mem, members)
    obs = ncio.read_obs(tmp_path / "obs.nc")
    hx = ncio.read_hx(str(tmp_path / "hx.#ENS3#.nc"), k, obs["lat"].size)
    assert np.array_equal(hx, hx_full.astype(np.float32))
    ref = gpu_run(prob, cfg["localization"], cfg["solver"], keep_open=True)
    sref = ref["solver"]
    with Solver(0) as s:
        s.solver_init(cfg["solver"])
        s.loc_init(cfg["localization"], prob.vars, prob.lev_depth)
        s.set_grid(prob.lat, prob.lon, prob.mask)
        s.set_state_members(mem, prob.vars)
        kept = s.set_obs_raw(obs["lat"], obs["lon"], obs["zdim"], obs["time"], obs["val"], obs["err"], obs["obsid"],
                             obs["platid"], hx, obs["qc"])
        assert kept == n
        s.run()
        x, m_, sp = s.get_state()
        act = np.nonzero(prob.mask == 0)[0]
        pa = x[act].astype(np.float64) - m_[act][:, :, None]
        pr = ref["state"][act].astype(np.float64) - ref["mean"][act][:, :, None]
        assert rel_l2(pa, pr) <= 1e-5 and rel_l2(m_[act], ref["mean"][act]) <= 1e-5
        for c in act[:: max(1, len(act) // 20)]:
            assert np.array_equal(s.obslist(int(c), 0)[0], sref.obslist(int(c), 0)[0])
        # diagnostics files
        d = s.get_diag()
        s.write_diag(tmp_path / "diag.solver.nc", nx, ny, lat_nom, lon_nom)
        with netcdf_file(str(tmp_path / "diag.solver.nc"), "r", mmap=False) as f:
            assert f.dimensions == {"time": 1, "lat": ny, "lon": nx, "loc_group": 2}
            assert np.array_equal(f.variables["col_maxhz"][0].reshape(-1), d["maxhz"])
            assert np.array_equal(f.variables["col_obscount"][0].reshape(-1), d["obscount"])
            assert np.array_equal(f.variables["lg_obscount"][0].reshape(2, -1), d["lg_obscount"])
            assert np.array_equal(f.variables["lg_obsloc"][0].reshape(2, -1), d["lg_obsloc"])
            assert np.array_equal(f.variables["lat"][:], lat_nom)
        lvl = s.get_loc_diag()
        s.write_loc_diag(tmp_path / "diag.loc_ocean.nc", nx, ny, lat_nom, lon_nom, prob.lev_depth)
        with netcdf_file(str(tmp_path / "diag.loc_ocean.nc"), "r", mmap=False) as f:
            fl = f.variables["vtloc_surf_lvl"][0].reshape(-1)
            fd = f.variables["vtloc_surf_depth"][0].reshape(-1)
        # the background mean the device formed from the members
        _, mean_b, _ = s.get_background()
    sref.close()
    tv = v["T"]
    expect = _mld_levels(mean_b, tv["grid_s_idx"], tv["levels"], cfg["localization"]["vtloc_surf"]["bkg_t_delta"])
    assert np.array_equal(lvl[act], expect[act].astype(np.float32))
    assert np.all(lvl[prob.mask != 0] == 0)
    assert np.array_equal(fl, lvl)
    assert np.array_equal(fd[act], prob.lev_depth[expect[act] - 1])
    assert len(np.unique(expect[act])) > 1   # the mixed layer varies over the grid
