"""CPU: the NetCDF classic reader and writer of the library (host code,
through the C ABI) against scipy.io.netcdf_file, an independent
implementation of the same published format, in both directions:

  - diag.solver.nc / diag.loc_ocean.nc as letkf_solver_final and
    loc_ocean_final write them (src/letkf_solver.F90:397-527,
    src/subclass.letkf_localizer/letkf_loc_ocean.F90:249-322): dimensions,
    variable shapes, attributes and values;
  - observation files and per-member hx files as obsio_nc reads them
    (src/subclass.letkf_obsio/letkf_obsio_nc.F90:150-306), CDF-1 and CDF-2,
    with and without read_inc, member file names from #ENSn#;
  - state files as stateio_nc reads and writes them
    (src/subclass.letkf_stateio/letkf_stateio_nc.F90:196-370), integer and
    double variables converted, a record dimension, a 2-D variable;
  - the file-name patterns of parse_ens_filename
    (src/letkf_state_helper.F90:445-510);
  - refusals: a NetCDF-4/HDF5 file, a missing variable, a size mismatch.
"""
import numpy as np
import pytest

from letkf_gb300 import LgpuError, ncio

netcdf_file = pytest.importorskip("scipy.io").netcdf_file


def test_ens_filename_patterns():
    assert ncio.ens_filename("bkg/#ENS3#/ocn.nc", 7) == "bkg/007/ocn.nc"
    assert ncio.ens_filename("mem#ENS2#_#ENS2#.nc", 12) == "mem12_12.nc"
    assert ncio.ens_filename("x.#ENS4#.#TYPE#.nc", 5) == "x.0005.ana.nc"
    assert ncio.ens_filename("x.#ENS4#.#TYPE#.nc", -1) == "x.mean.bkg.nc"
    assert ncio.ens_filename("x.#ENS4#.#TYPE#.nc", -2) == "x.mean.ana.nc"
    assert ncio.ens_filename("x.#ENS4#.#TYPE#.nc", -3) == "x.sprd.bkg.nc"
    assert ncio.ens_filename("x.#ENS4#.#TYPE#.nc", -4) == "x.sprd.ana.nc"
    assert ncio.ens_filename("plain.nc", 3) == "plain.nc"
    with pytest.raises(LgpuError, match="Illegal 'ensmem'"):
        ncio.ens_filename("a#ENS1#", -9)
    with pytest.raises(LgpuError, match="illegal ensmem"):
        ncio.ens_filename("plain.nc", -9)


def test_diag_files_read_back_with_scipy(tmp_path):
    rng = np.random.default_rng(0)
    nx, ny, G = 12, 7, 3
    lat = np.linspace(-80, 80, ny).astype(np.float32)
    lon = np.linspace(0, 330, nx).astype(np.float32)
    maxhz = rng.uniform(1e5, 8e5, nx * ny).astype(np.float32)
    obsc = rng.integers(0, 500, nx * ny).astype(np.float32)
    lgc = rng.integers(0, 400, (G, nx * ny)).astype(np.float32)
    lgl = rng.uniform(0, 50, (G, nx * ny)).astype(np.float32)
    p = tmp_path / "diag.solver.nc"
    ncio.write_diag_arrays(p, lat, lon, maxhz, obsc, lgc, lgl)
    with netcdf_file(str(p), "r", mmap=False) as f:
        assert f.version_byte == 1
        assert f.dimensions == {"time": 1, "lat": ny, "lon": nx, "loc_group": G}
        assert f.variables["col_maxhz"].dimensions == ("time", "lat", "lon")
        assert f.variables["lg_obsloc"].dimensions == ("time", "loc_group", "lat", "lon")
        assert f.variables["lat"].axis == b"Y" and f.variables["lat"].units == b"degrees_north"
        assert f.variables["lon"].axis == b"X" and f.variables["lon"].units == b"degrees_east"
        assert f.variables["col_maxhz"].units == b"m"
        assert f.variables["col_maxhz"].long_name == b"max observation search radius for the column"
        assert f.variables["lg_obscount"].long_name == b"observations per localization group"
        assert np.array_equal(f.variables["lat"][:], lat)
        assert np.array_equal(f.variables["lon"][:], lon)
        assert np.array_equal(f.variables["col_maxhz"][:].reshape(-1), maxhz)
        assert np.array_equal(f.variables["col_obscount"][:].reshape(-1), obsc)
        assert np.array_equal(f.variables["lg_obscount"][:].reshape(G, -1), lgc)
        assert np.array_equal(f.variables["lg_obsloc"][:].reshape(G, -1), lgl)
    # our reader on our file
    assert ncio.var_shape(p, "lg_obsloc") == (1, G, ny, nx)
    assert np.array_equal(ncio.read_var(p, "lg_obsloc").reshape(G, -1), lgl)
    q = tmp_path / "diag.loc_ocean.nc"
    lvl = rng.integers(0, 10, nx * ny).astype(np.float32)
    dep = (lvl * 10.0).astype(np.float32)
    ncio.write_loc_diag_arrays(q, lat, lon, lvl, dep)
    with netcdf_file(str(q), "r", mmap=False) as f:
        assert f.dimensions == {"time": 1, "lat": ny, "lon": nx}
        assert f.variables["vtloc_surf_depth"].units == b"meters"
        assert np.array_equal(f.variables["vtloc_surf_lvl"][:].reshape(-1), lvl)
        assert np.array_equal(f.variables["vtloc_surf_depth"][:].reshape(-1), dep)


def _obs_file(path, obs, version):
    with netcdf_file(str(path), "w", version=version) as f:
        n = len(obs["lat"])
        f.createDimension("obs", n)
        for name, key, typ in (("obid", "obsid", "i4"), ("plat", "platid", "i4"), ("lat", "lat", "f4"),
                               ("lon", "lon", "f4"), ("depth", "zdim", "f4"), ("hr", "time", "f4"),
                               ("val", "val", "f4"), ("err", "err", "f4"), ("qc", "qc", "i4")):
            v = f.createVariable(name, typ, ("obs",))
            v[:] = obs[key]


@pytest.mark.parametrize("version", [1, 2])
def test_obs_and_hx_files(tmp_path, version):
    rng = np.random.default_rng(version)
    n, k = 1000, 6
    obs = dict(obsid=rng.integers(1, 5, n).astype(np.int32), platid=rng.integers(1, 3, n).astype(np.int32),
               lat=rng.uniform(-90, 90, n).astype(np.float32), lon=rng.uniform(0, 360, n).astype(np.float32),
               zdim=rng.uniform(0, 2000, n).astype(np.float32), time=rng.uniform(-3, 3, n).astype(np.float32),
               val=rng.standard_normal(n).astype(np.float32), err=rng.uniform(0.1, 1, n).astype(np.float32),
               qc=(rng.random(n) < 0.1).astype(np.int32))
    p = tmp_path / "obs.nc"
    _obs_file(p, obs, version)
    got = ncio.read_obs(p)
    for key, v in obs.items():
        assert np.array_equal(got[key], v), key
    hx = rng.standard_normal((n, k)).astype(np.float32)
    inc = rng.standard_normal((n, k)).astype(np.float32)
    for m in range(k):
        with netcdf_file(str(tmp_path / ("hx.%03d.nc" % (m + 1))), "w", version=version) as f:
            f.createDimension("obs", n)
            f.createVariable("hx", "f4", ("obs",))[:] = hx[:, m]
            f.createVariable("val", "f4", ("obs",))[:] = obs["val"]
            f.createVariable("inc", "f4", ("obs",))[:] = inc[:, m]
    pat = str(tmp_path / "hx.#ENS3#.nc")
    assert np.array_equal(ncio.read_hx(pat, k, n), hx)
    got = ncio.read_hx(pat, k, n, read_inc=True)
    assert np.array_equal(got, inc + obs["val"][:, None])
    with pytest.raises(LgpuError, match="obs in file does not match expected"):
        ncio.read_hx(pat, k, n + 1)


def test_state_files_both_directions(tmp_path):
    rng = np.random.default_rng(5)
    nx, ny, nz, k = 16, 9, 5, 3
    lon = np.arange(nx, dtype=np.float32) * (360.0 / nx)
    lat = np.linspace(-80, 80, ny).astype(np.float32)
    depth = np.array([5, 15, 30, 60, 100], np.float32)
    T = rng.standard_normal((k, nz, ny, nx)).astype(np.float32)
    S = rng.standard_normal((k, nz, ny, nx))                     # stored as double
    ssh = rng.integers(-300, 300, (k, 1, ny, nx)).astype(np.int16)   # stored as short
    for m in range(k):
        with netcdf_file(str(tmp_path / ("ens%02d.nc" % (m + 1))), "w", version=2) as f:
            f.createDimension("time", None)
            f.createDimension("z", nz)
            f.createDimension("y", ny)
            f.createDimension("x", nx)
            f.createDimension("z1", 1)
            t = f.createVariable("temp", "f4", ("time", "z", "y", "x"))
            t[0] = T[m]
            f.createVariable("salt", "f8", ("time", "z", "y", "x"))[0] = S[m]
            f.createVariable("ssh", "i2", ("time", "z1", "y", "x"))[0] = ssh[m]
    pat = str(tmp_path / "ens#ENS2#.nc")
    assert np.array_equal(ncio.read_state_members(pat, "temp", k, nx, ny, nz), T)
    assert np.array_equal(ncio.read_state_members(pat, "salt", k, nx, ny, nz), S.astype(np.float32))
    assert np.array_equal(ncio.read_state_members(pat, "ssh", k, nx, ny, 1), ssh.astype(np.float32))
    with pytest.raises(LgpuError, match="grid holds"):
        ncio.read_state_members(pat, "temp", k, nx, ny, nz + 1)
    with pytest.raises(LgpuError, match="not in"):
        ncio.read_state_members(pat, "nope", k, nx, ny, nz)
    # the writer: one analysis member, two variables on two vertical grids
    out = tmp_path / "ana.nc"
    ncio.write_state(out, lon, lat, [("depth", depth), ("surface", np.zeros(1, np.float32))],
                     [("Temp", 0, T[0]), ("SSH", 1, ssh[0].astype(np.float32))])
    with netcdf_file(str(out), "r", mmap=False) as f:
        assert f.dimensions["time"] is None and f.dimensions["lon"] == nx and f.dimensions["depth"] == nz
        assert f.variables["Temp"].dimensions == ("time", "depth", "lat", "lon")
        assert f.variables["lon"].units == b"degrees_east" and f.variables["lat"].axis == b"Y"
        assert f.variables["depth"].axis == b"Z" and f.variables["time"].axis == b"T"
        assert np.array_equal(f.variables["Temp"][0], T[0])
        assert np.array_equal(f.variables["SSH"][0, 0], ssh[0, 0].astype(np.float32))
        assert np.array_equal(f.variables["depth"][:], depth)
    assert np.array_equal(ncio.read_var(out, "Temp")[0], T[0])
    assert ncio.dim_len(out, "time") == 1


def test_cdf5_header(tmp_path):
    """CDF-5 (64-bit data) packed by hand from the format description: 8-byte
    counts and sizes, 8-byte offsets, an int64 and a double variable."""
    import struct

    def name(s):
        b = s.encode()
        return struct.pack(">Q", len(b)) + b + bytes((-len(b)) % 4)

    n = 5
    vals64 = np.array([-3, 0, 7, 2 ** 40, 11], ">i8")
    valsd = np.array([0.5, -1.25, 3.0, 1e10, -7.0], ">f8")
    hdr = b"CDF\x05" + struct.pack(">Q", 0)
    hdr += struct.pack(">IQ", 0x0A, 1) + name("obs") + struct.pack(">Q", n)
    hdr += struct.pack(">IQ", 0, 0)                      # no global attributes
    hdr += struct.pack(">IQ", 0x0B, 2)

    def var(nm, typ, size, begin):
        return name(nm) + struct.pack(">QQ", 1, 0) + struct.pack(">IQ", 0, 0) + struct.pack(">IQQ", typ, size, begin)

    probe = hdr + var("qc", 10, 8 * n, 0) + var("val", 6, 8 * n, 0)
    b0 = len(probe)
    hdr += var("qc", 10, 8 * n, b0) + var("val", 6, 8 * n, b0 + 8 * n)
    p = tmp_path / "five.nc"
    p.write_bytes(hdr + vals64.tobytes() + valsd.tobytes())
    assert ncio.dim_len(p, "obs") == n
    assert np.array_equal(ncio.read_var(p, "qc", np.int32), vals64.astype(np.int64).clip(-2**31, 2**31 - 1))
    assert np.array_equal(ncio.read_var(p, "val"), valsd.astype(np.float32))


def test_refusals(tmp_path):
    h5 = tmp_path / "four.nc"
    h5.write_bytes(b"\x89HDF\r\n\x1a\n" + bytes(64))
    with pytest.raises(LgpuError, match="HDF5") as e:
        ncio.read_obs(h5)
    assert e.value.code == 10
    bad = tmp_path / "bad.nc"
    bad.write_bytes(b"not a netcdf file")
    with pytest.raises(LgpuError, match="not a netCDF"):
        ncio.read_obs(bad)
    with pytest.raises(LgpuError, match="cannot open"):
        ncio.read_obs(tmp_path / "missing.nc")
    p = tmp_path / "obs.nc"
    with netcdf_file(str(p), "w") as f:
        f.createDimension("obs", 3)
        f.createVariable("lat", "f4", ("obs",))[:] = [1, 2, 3]
    with pytest.raises(LgpuError, match='"obid"'):
        ncio.read_obs(p)
