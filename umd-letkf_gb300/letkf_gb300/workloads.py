"""Named analysis workloads: generator options + the localization and solver
sections a reference YAML configuration would carry for them.

  c1        90x45x10 grid, one 3-D temperature, k=20, 5,000 point obs,
            horizontal GC 500 km x vertical GC 200 m (loc_vtgc), RTPS 0.6
  c2        720x360x40 ocean (T, S, SSH; 81 slabs), k=40, 3,000 T/S profiles
            + 200,000 SSH/SST swath obs, loc_novrt 800 km (equator) to
            200 km (poles), default inflation
  c3        720x360x40 ocean, k=32 (or 64), 500,000 clustered obs, loc_novrt
            with a constant 60 km length scale (support ~219 km)
  c4        1440x720x50 (T, S; 100 slabs), k=100, 1,000,000 clustered obs,
            loc_novrt 60 km as c3
  c5        learned form: 720x360x40, k=32, c3's clustered network (persistent
            clusters), loc_novrt 400 km, stride-4 coarse lattice, 5 exact
            training cycles
  c2learn   the learned form on the headline lattice: 720x360x40, k=40,
            C2's localisation, 440,000 observations in wide clusters
            (close to uniform), stride 4, 5 exact training cycles
  c5mid     c5 with 10 levels and 2 training cycles (profiling-sized: the same
            network rows per analysis)
  c2mid     c2 observations on a 360x180x10 grid (profiling-sized: the same
            local observation counts per column, a fifth of the columns)
  simple3d  test/simple3d-style (k=50, three 3-D variables, two synthetic
            obs, loc_novrt 500 km -> 50 km)
  ocean     test/ocean/vtloc-style (k=10, T/S/u/v, five synthetic obs,
            loc_ocean with the mixed-layer split)
  c2ocean   c2small's grid and observations under loc_ocean with temporal
            localisation (tloc_prof 2 h, tloc_sat 1.5 h; observation times
            of both signs) and both surface-id lists set (sat_obs = [3],
            sat_plats = [2]: the SSH swath obs are surface obs, the SST swath
            obs of the same platform are not), mixed-layer split on T
  c4mid     c4's 50 levels and k = 100 on a 240x120 grid (profiling-sized:
            the same slabs and members per column)
  c2small / c1small / c3small / c4small  reduced grids with the same
            generators for fast tests
"""

C2_LOC = {"class": "loc_novrt",
          "hzloc": {"type": "linearinterp_lat", "value": [{"lat": 0.0, "radius": 800.0e3},
                                                          {"lat": 90.0, "radius": 200.0e3}]}}

WORKLOADS = {
    "c1": dict(gen=dict(workload="c1"),
               localization={"class": "loc_vtgc",
                             "hzloc": {"type": "linearinterp_lat", "value": [{"lat": 0.0, "radius": 500.0e3}]},
                             "vtloc": 200.0},
               solver={"inflation": {"rtps": 0.6}}),
    "c2": dict(gen=dict(workload="c2"), localization=C2_LOC, solver={}),
    "c2small": dict(gen=dict(workload="c2", nx=144, ny=72, nz=10, n_profiles=300, n_swaths=10, swath_len=800),
                    localization=C2_LOC, solver={}),
    "c2mid": dict(gen=dict(workload="c2", nx=360, ny=180, nz=10), localization=C2_LOC, solver={}),
    "c2ocean": dict(gen=dict(workload="c2", nx=144, ny=72, nz=10, n_profiles=300, n_swaths=10, swath_len=800),
                    localization={"class": "loc_ocean",
                                  "hzloc_prof": C2_LOC["hzloc"],
                                  "hzloc_sat": {"type": "linearinterp_lat",
                                                "value": [{"lat": 0.0, "radius": 500.0e3},
                                                          {"lat": 90.0, "radius": 100.0e3}]},
                                  "tloc_prof": 2.0, "tloc_sat": 1.5,
                                  "sat_obs": [3], "sat_plats": [2],
                                  "vtloc_surf": {"type": "bkg_t", "bkg_t_delta": 0.2, "bkg_t_var": "T"}},
                    solver={}),
    "c3": dict(gen=dict(workload="c3"),
               localization={"class": "loc_novrt",
                             "hzloc": {"type": "linearinterp_lat", "value": [{"lat": 0.0, "radius": 60.0e3}]}},
               solver={}),
    "c3k64": dict(gen=dict(workload="c3", k=64),
                  localization={"class": "loc_novrt",
                                "hzloc": {"type": "linearinterp_lat", "value": [{"lat": 0.0, "radius": 60.0e3}]}},
                  solver={}),
    "c4": dict(gen=dict(workload="c4"),
               localization={"class": "loc_novrt",
                             "hzloc": {"type": "linearinterp_lat", "value": [{"lat": 0.0, "radius": 60.0e3}]}},
               solver={}),
    # learned form: the clustered network of c3 with k = 32 and a 400 km
    # localisation scale (the transform then varies on scales the stride-4
    # coarse lattice, 2 degrees, resolves); 5 exact training cycles, truth and
    # members advanced by a zonal jet of 0.5 m/s with diffusion 1e3 m^2/s
    # over 6 h between cycles
    "c5": dict(gen=dict(workload="c3", k=32),
               localization={"class": "loc_novrt",
                             "hzloc": {"type": "linearinterp_lat", "value": [{"lat": 0.0, "radius": 400.0e3}]}},
               solver={},
               learn=dict(stride=4, hidden=512, judge_frac=0.02, gate_frac=0.1, sample_frac=0.6, train_cap=600000,
                          seed=5),
               cycles=dict(train=5, u=0.5, kappa=1.0e3, dt=21600.0, epochs=15, batch=1024, lr=1e-3)),
    # the learned form on the headline lattice and ensemble: 720x360x40, k = 40,
    # C2's localisation (800 km at the equator to 200 km at the poles),
    # 440,000 observations from the cycling observer in 12 clusters of
    # 3,000 km (close to uniform, C2's density), stride-4 coarse lattice
    "c2learn": dict(gen=dict(workload="c3", k=40, n_obs=440000, cluster_sigma_m=3.0e6),
                    localization=C2_LOC, solver={},
                    learn=dict(stride=4, hidden=512, judge_frac=0.02, gate_frac=0.1, sample_frac=0.6,
                               train_cap=600000, seed=5),
                    cycles=dict(train=5, u=0.5, kappa=1.0e3, dt=21600.0, epochs=15, batch=1024, lr=1e-3,
                                cluster_sigma_m=3.0e6)),
    "c5mid": dict(gen=dict(workload="c3", k=32, nz=10),
                  localization={"class": "loc_novrt",
                                "hzloc": {"type": "linearinterp_lat", "value": [{"lat": 0.0, "radius": 400.0e3}]}},
                  solver={},
                  learn=dict(stride=4, hidden=512, judge_frac=0.02, gate_frac=0.05, sample_frac=0.3,
                             train_cap=300000, seed=5),
                  cycles=dict(train=2, u=0.5, kappa=1.0e3, dt=21600.0, epochs=2, batch=1024, lr=1e-3)),
    "c4mid": dict(gen=dict(workload="c4", nx=240, ny=120, n_obs=40000),
                  localization={"class": "loc_novrt",
                                "hzloc": {"type": "linearinterp_lat", "value": [{"lat": 0.0, "radius": 150.0e3}]}},
                  solver={}),
    "c4small": dict(gen=dict(workload="c4", nx=180, ny=90, nz=5, n_obs=40000),
                    localization={"class": "loc_novrt",
                                  "hzloc": {"type": "linearinterp_lat", "value": [{"lat": 0.0, "radius": 150.0e3}]}},
                    solver={}),
    "c3small": dict(gen=dict(workload="c3", nx=180, ny=90, nz=10, n_obs=40000),
                    localization={"class": "loc_novrt",
                                  "hzloc": {"type": "linearinterp_lat", "value": [{"lat": 0.0, "radius": 150.0e3}]}},
                    solver={}),
    "simple3d": dict(gen=dict(workload="simple3d"),
                     localization={"class": "loc_novrt",
                                   "hzloc": {"type": "linearinterp_lat",
                                             "value": [{"lat": 0.0, "radius": 500.0e3},
                                                       {"lat": 90.0, "radius": 50.0e3}]}},
                     solver={}),
    "ocean": dict(gen=dict(workload="ocean"),
                  localization={"class": "loc_ocean", "save_diag": True,
                                "hzloc_prof": {"type": "linearinterp_lat",
                                               "value": [{"lat": 0.0, "radius": 720.0e3},
                                                         {"lat": 90.0, "radius": 200.0e3}]},
                                "hzloc_sat": {"type": "linearinterp_lat",
                                              "value": [{"lat": 0.0, "radius": 500.0e3},
                                                        {"lat": 90.0, "radius": 50.0e3}]},
                                "sat_obs": [], "sat_plats": [1],
                                "vtloc_surf": {"type": "bkg_t", "bkg_t_delta": 0.2, "bkg_t_var": "ocn_t"}},
                  solver={"inflation": {"rtps": 0.0, "rtpp": 0.0, "mul": 1.0}}),
}

# test/simple3d solver/state variants (default.yaml, bounds_check.yaml,
# inflation_{rtps,rtpp,mul}.yaml)
SIMPLE3D_VARIANTS = {
    "default": dict(solver={}, bounds=None),
    "bounds_check": dict(solver={}, bounds={0: dict(ana_bounds=(-2.0, 2.0)), 1: dict(ana_inc_max=2.0),
                                            2: dict(ana_inc_max=0.2, ana_bounds=(-2.0, 2.0))}),
    "inflation_rtps": dict(solver={"inflation": {"rtps": 0.8}}, bounds=None),
    "inflation_rtpp": dict(solver={"inflation": {"rtpp": 0.8}}, bounds=None),
    "inflation_mul": dict(solver={"inflation": {"mul": 1.05}}, bounds=None),
}


def apply_bounds(variables, bounds):
    """Copy of a variable list with per-variable ana_inc_max / ana_bounds."""
    out = [dict(v) for v in variables]
    for i, b in (bounds or {}).items():
        out[i].update(b)
    return out
