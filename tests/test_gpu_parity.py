"""GPU parity: the CUDA library through its C ABI against the CPU oracle.

Bars (written here, checked per variable and level):
  - distances, local observation lists (indices and canonical order),
    search-candidate counts and maxhz: bit-exact;
  - localisation weights: |r_gpu - r_oracle| <= 4e-7 (one GC factor) /
    1e-6 (products), keep/drop decisions exact;
  - analysis perturbations and analysis mean: relative L2 <= 1e-5 per slab
    against the FP32 oracle (reference arithmetic) and the FP64 oracle,
    for slabs whose perturbation norm is not negligible, both Gram forms
    (the batched tensor-core form accumulates in segments of at most 64
    chunks of 16 observations, summed in FP64);
  - mean increment: reported; relative L2 <= 2e-3 per slab (FP32 Gram
    accumulation error of ill-conditioned columns, shared by the
    reference's own FP32 path).
"""
import numpy as np
import pytest

from conftest import workload
from helpers import compare, gpu_run, oracle_for, workload_cfg

pytestmark = pytest.mark.gpu

PERT_TOL = 1e-5          # plain FP32 path
PERT_TOL_TC = PERT_TOL   # batched tensor-core path: TF32 x3 split, segmented FP32 tensor-core accumulation
MEAN_TOL = 1e-5
INC_TOL = 2e-3


@pytest.fixture(scope="module")
def solver():
    from letkf_gb300 import Solver
    s = Solver(0)
    yield s
    s.close()


def test_metric_bitexact(solver):
    from oracle import oracle as O
    rng = np.random.default_rng(7)
    n = 20000
    la1 = rng.uniform(-90, 90, n).astype(np.float32)
    lo1 = rng.uniform(-180, 360, n).astype(np.float32)
    la2 = np.clip(la1 + rng.normal(0, 20, n), -90, 90).astype(np.float32)
    lo2 = (lo1 + rng.normal(0, 30, n)).astype(np.float32)
    got = solver.debug_metric(la1, lo1, la2, lo2)
    ref = np.array([O.dist(O.unitvec(a, b), O.unitvec(c, d)) for a, b, c, d in zip(la1, lo1, la2, lo2)], np.float32)
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))


def test_gc_fast_and_exact(solver):
    from oracle import oracle as O
    rng = np.random.default_rng(8)
    n = 200000
    L = rng.choice(np.array([50e3, 200e3, 500e3, 800e3, 200.0], np.float32), n)
    z = (rng.random(n) * 2.05 * L / np.sqrt(0.3)).astype(np.float32)
    fast, exact = solver.debug_gc(z, L)
    assert np.max(np.abs(fast.astype(np.float64) - exact)) <= 4e-7
    ref = np.array([O.gc(a, b) for a, b in zip(z[:20000], L[:20000])], np.float32)
    assert np.array_equal(exact[:20000].view(np.uint32), ref.view(np.uint32))


def test_fast_weight_path_bounds(solver):
    """The batched Gram's fast distance and weight against the exact ones,
    near the search radius and the 1e-4 keep threshold (the bands that send a
    pair to the exact path hold a 5x margin over these bounds)."""
    rng = np.random.default_rng(21)
    n = 400000
    L = rng.choice(np.array([60e3, 200e3, 500e3, 800e3], np.float32), n)
    lat1 = rng.uniform(-89.0, 89.0, n)
    lon1 = rng.uniform(0.0, 360.0, n)
    # separations spread over the whole support, denser near the keep threshold (z/c ~ 1.78-1.83)
    zc = np.where(rng.random(n) < 0.5, rng.uniform(0.0, 2.0, n), rng.uniform(1.70, 1.90, n))
    dist = zc * L / np.sqrt(0.3)
    brg = rng.uniform(0.0, 2 * np.pi, n)
    dlat = np.degrees(dist / 6371e3) * np.cos(brg)
    lat2 = np.clip(lat1 + dlat, -89.9, 89.9)
    lon2 = (lon1 + np.degrees(dist / 6371e3) * np.sin(brg) / np.cos(np.radians(lat1))) % 360.0
    de, df, re, rf, ds = solver.debug_weight(lat1, lon1, lat2, lon2, L)
    ok = de > 1.0
    assert np.max(np.abs(df[ok].astype(np.float64) / de[ok] - 1.0)) <= 1e-6
    # short asin series: half-chords up to 0.25 (separations up to ~3,220 km)
    sh = ok & (de < 2 * 6371e3 * np.arcsin(0.25))
    assert sh.sum() > 100000
    assert np.max(np.abs(ds[sh].astype(np.float64) / de[sh] - 1.0)) <= 1e-6
    near = (re > 2e-5) & (re < 5e-4)
    assert near.sum() > 10000
    assert np.max(np.abs(rf[near].astype(np.float64) - re[near])) <= 2e-8
    assert np.max(np.abs(rf.astype(np.float64) - re)) <= 1e-6


LIST_CASES = [("simple3d", None), ("ocean", None), ("c1", None), ("c2small", 150), ("c3small", 150),
              ("c2ocean", 150)]


@pytest.mark.parametrize("variant", ["plain", "batched"])
@pytest.mark.parametrize("name,nsample", LIST_CASES)
def test_obslists_bitexact(name, nsample, variant):
    cfg = workload_cfg(name)
    prob = workload(cfg["gen"]["workload"], **{k: v for k, v in cfg["gen"].items() if k != "workload"})
    res = gpu_run(prob, cfg["localization"], cfg["solver"], keep_open=True, variant=variant)
    s = res["solver"]
    o = oracle_for(prob, cfg["localization"], cfg["solver"])
    rng = np.random.default_rng(1)
    active = np.nonzero(prob.mask == 0)[0]
    if nsample is None:
        # every column near an observation plus a random sample
        cols = rng.choice(active, size=min(200, len(active)), replace=False)
        near = []
        for la, lo in zip(prob.olat[:50], prob.olon[:50]):
            d = (prob.lat - la) ** 2 + ((prob.lon - lo + 180) % 360 - 180) ** 2
            near.append(int(np.argmin(d)))
        cols = np.unique(np.concatenate([cols, near]))
    else:
        cols = rng.choice(active, size=nsample, replace=False)
    G = s.maxgroups
    groups = range(G) if G <= 2 else [0, G // 2, G - 1]
    nonempty = 0
    for c in cols:
        for g in groups:
            gi, gr, gn = s.obslist(int(c), g)
            oi, orr, on = o.obslist(int(c), g)
            assert gn == on, (c, g)
            assert np.array_equal(gi, oi), (c, g, len(gi), len(oi))
            tol = 1e-6 if (name == "c1") else 4e-7
            assert np.all(np.abs(gr.astype(np.float64) - orr) <= tol), (c, g)
            nonempty += len(gi) > 0
    assert nonempty > 0
    # diagnostics: maxhz and candidate counts bit-exact, kept counts exact
    ref = o.run(32, cols=cols)
    d = res["diag"]
    assert np.array_equal(d["maxhz"][cols], ref["maxhz"])
    assert np.array_equal(d["obscount"][cols], ref["obscount"])
    assert np.array_equal(d["lg_obscount"][:, cols].T, ref["lg_obscount"])
    assert np.allclose(d["lg_obsloc"][:, cols].T, ref["lg_obsloc"], rtol=2e-5, atol=1e-5)
    s.close()
    o.close()


def _check_analysis(prob, cfg_loc, cfg_solver, cols, variables=None, label="", variant="auto"):
    gpu = gpu_run(prob, cfg_loc, cfg_solver, variables=variables, variant=variant)
    assert gpu["timings"]["variant"] == (1 if variant == "plain" else 2)
    o = oracle_for(prob, cfg_loc, cfg_solver, variables=variables)
    for prec in (32, 64):
        ref = o.run(prec, cols=cols)
        cmp = compare(prob, gpu, ref, cols)
        # slabs with negligible perturbations (e.g. fully clipped) are skipped
        pr = ref["state"] - ref["mean"][:, :, None]
        pn = np.sqrt(np.sum(pr.astype(np.float64) ** 2, axis=(0, 2)))
        ok = pn > 1e-6 * max(pn.max(), 1e-30)
        tol = PERT_TOL if variant == "plain" else PERT_TOL_TC
        assert np.all(cmp["pert"][ok] <= tol), (label, prec, cmp["pert"].max(), np.argmax(cmp["pert"]))
        assert np.all(cmp["mean"] <= MEAN_TOL), (label, prec, cmp["mean"].max())
        big = cmp["inc_norm"] > 1e-3 * max(cmp["inc_norm"].max(), 1e-30)
        assert np.all(cmp["inc"][big] <= INC_TOL), (label, prec, cmp["inc"][big].max())
    # masked columns keep the background exactly (src/letkf_solver.F90:207)
    mc = np.nonzero(prob.mask)[0]
    if len(mc):
        assert np.array_equal(gpu["state"][mc], prob.state[mc])
        assert np.array_equal(gpu["mean"][mc], prob.mean[mc])
        assert np.array_equal(gpu["sprd"][mc], prob.sprd[mc])
    assert np.all(np.isfinite(gpu["state"]))
    o.close()
    return gpu


@pytest.mark.parametrize("gram", ["plain", "batched"])
@pytest.mark.parametrize("variant", ["default", "bounds_check", "inflation_rtps", "inflation_rtpp", "inflation_mul"])
def test_simple3d_variants(variant, gram):
    from letkf_gb300.workloads import SIMPLE3D_VARIANTS, apply_bounds
    cfg = workload_cfg("simple3d")
    prob = workload("simple3d")
    v = SIMPLE3D_VARIANTS[variant]
    variables = apply_bounds(prob.vars, v["bounds"])
    cols = np.arange(prob.ncol)[::3]
    _check_analysis(prob, cfg["localization"], v["solver"], cols, variables=variables, label=variant, variant=gram)


@pytest.mark.parametrize("gram", ["plain", "batched"])
@pytest.mark.parametrize("name", ["ocean", "c1", "c2small", "c3small", "c2ocean"])
def test_analysis_parity(name, gram):
    cfg = workload_cfg(name)
    prob = workload(cfg["gen"]["workload"], **{k: v for k, v in cfg["gen"].items() if k != "workload"})
    active = np.nonzero(prob.mask == 0)[0]
    rng = np.random.default_rng(2)
    cols = np.sort(rng.choice(active, size=min(600, len(active)), replace=False))
    _check_analysis(prob, cfg["localization"], cfg["solver"], cols, label=name, variant=gram)


@pytest.mark.parametrize("gram", ["plain", "batched"])
def test_ocean_time_and_surface_ids(gram):
    """loc_ocean with temporal localisation and both surface-id lists
    (src/subclass.letkf_localizer/letkf_loc_ocean.F90:467-499), through the
    GPU: SSH swath obs (id 3, platform 2) are surface obs and never enter the
    sub-mixed-layer group; SST swath obs (id 4, platform 2) fail the id list
    and are used in both groups with the profile radius; the weights carry
    the temporal factor (lower than without tloc, same keep decisions as the
    oracle, which the list tests check bit-exactly)."""
    from dataclasses import replace
    cfg = workload_cfg("c2ocean")
    prob = workload(cfg["gen"]["workload"], **{k: v for k, v in cfg["gen"].items() if k != "workload"})
    assert np.any(prob.otime > 0.5) and np.any(prob.otime < -0.5)
    loc_nt = dict(cfg["localization"], tloc_prof=-1.0, tloc_sat=-1.0)
    res = gpu_run(prob, cfg["localization"], cfg["solver"], keep_open=True, variant=gram)
    res_nt = gpu_run(prob, loc_nt, cfg["solver"], keep_open=True, variant=gram)
    s, s_nt = res["solver"], res_nt["solver"]
    try:
        assert s.maxgroups == 2
        # columns next to swath observations of both kinds
        cols = []
        for kind in (3, 4):
            for i in np.nonzero(prob.oobsid == kind)[0][::97][:12]:
                d = (prob.lat - prob.olat[i]) ** 2 + ((prob.lon - prob.olon[i] + 180) % 360 - 180) ** 2
                c = int(np.argmin(d + 1e9 * prob.mask))
                cols.append(c)
        sst_below, lower = 0, 0
        for c in cols:
            for g in (0, 1):
                gi, gr, _ = s.obslist(c, g)
                ni, nr, _ = s_nt.obslist(c, g)
                kinds = prob.oobsid[gi]
                if g == 1:
                    assert not np.any(kinds == 3), c      # surface obs never below the mixed layer
                    sst_below += int(np.sum(kinds == 4))
                # the temporal factor only lowers weights (and can drop
                # entries); 1e-6 covers the fast/exact evaluations near the
                # keep threshold
                assert set(gi.tolist()) <= set(ni.tolist())
                wt = dict(zip(ni.tolist(), nr.tolist()))
                for i, r in zip(gi.tolist(), gr.tolist()):
                    assert r <= wt[i] + 1e-6
                    lower += r < 0.999 * wt[i]
        assert sst_below > 0 and lower > 0
    finally:
        s.close()
        s_nt.close()


@pytest.mark.parametrize("k", [12, 20])
def test_ocean_groups_with_k_multiple_of_4(k):
    """loc_ocean (two localisation groups) with k a multiple of 4: the update
    stages both groups' transforms with bulk async copies."""
    cfg = workload_cfg("ocean")
    prob = workload("ocean", k=k)
    active = np.nonzero(prob.mask == 0)[0]
    cols = active[:: max(1, len(active) // 400)]
    for gram in ("plain", "batched"):
        _check_analysis(prob, cfg["localization"], cfg["solver"], cols, label="ocean k=%d" % k, variant=gram)


@pytest.mark.parametrize("name", ["c2small", "c3small"])
def test_auto_variant_choice(name):
    """AUTO times both Gram forms on the first analysis and keeps the faster;
    its analysis, on the first run and on the next (which reuses the choice),
    is bit-identical to an explicit run of the chosen form."""
    cfg = workload_cfg(name)
    prob = workload(cfg["gen"]["workload"], **{k: v for k, v in cfg["gen"].items() if k != "workload"})
    res = gpu_run(prob, cfg["localization"], cfg["solver"], variant="auto", keep_open=True)
    s = res["solver"]
    try:
        chosen = res["timings"]["variant"]
        assert chosen in (1, 2)
        s.run()
        assert s.timings()["variant"] == chosen
        second = s.get_state()
    finally:
        s.close()
    ref = gpu_run(prob, cfg["localization"], cfg["solver"], variant="plain" if chosen == 1 else "batched")
    for got in ((res["state"], res["mean"], res["sprd"]), second):
        for a, b in zip(got, (ref["state"], ref["mean"], ref["sprd"])):
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


@pytest.mark.parametrize("k", [65, 99, 100, 128])
def test_large_ensembles(k):
    """Ensembles past 64 members: four rows per lane in the eigensolver, up
    to five register tile sets in the plain Gram, the k > 64 update forms
    (thread per slab for k a multiple of 4 with one group, the shuffle form
    for the per-level groups of loc_vtgc and for odd k)."""
    c1 = workload_cfg("c1")
    p = workload("c1", k=k)
    cols = np.arange(0, p.ncol, 53)
    for gram in ("plain", "batched"):
        _check_analysis(p, c1["localization"], c1["solver"], cols, label="c1 k=%d %s" % (k, gram), variant=gram)


@pytest.mark.parametrize("name", ["c4small", "ocean"])
def test_k100_workloads(name):
    """k = 100 (the 0.25-degree configuration's ensemble): clustered obs with
    one group (thread-per-slab update, 40 KB of transforms) and loc_ocean's
    two groups (80 KB of transforms in shared memory)."""
    cfg = workload_cfg(name)
    gen = {kk: v for kk, v in cfg["gen"].items() if kk != "workload"}
    if name == "ocean":
        gen["k"] = 100
    prob = workload(cfg["gen"]["workload"], **gen)
    active = np.nonzero(prob.mask == 0)[0]
    rng = np.random.default_rng(5)
    cols = rng.choice(active, size=min(300, len(active)), replace=False)
    if name == "ocean":   # five observations: add the columns within 600 km of one
        la, lo = np.radians(prob.lat[active])[:, None], np.radians(prob.lon[active])[:, None]
        ola, olo = np.radians(prob.olat)[None, :], np.radians(prob.olon)[None, :]
        c = np.sin(la) * np.sin(ola) + np.cos(la) * np.cos(ola) * np.cos(lo - olo)
        near = active[np.any(np.arccos(np.clip(c, -1, 1)) * 6.371e6 < 6e5, axis=1)]
        cols = np.concatenate([cols, near[:: max(1, len(near) // 300)]])
    cols = np.unique(cols)
    for gram in ("plain", "batched"):
        _check_analysis(prob, cfg["localization"], cfg["solver"], cols, label="%s k=100" % name, variant=gram)


def test_single_observation_closed_form():
    """One obs, one column in range: the GPU mean increment at the observed
    slab equals the scalar Kalman update."""
    prob = workload("simple3d")
    cfg = workload_cfg("simple3d")
    gpu = gpu_run(prob, cfg["localization"], {})
    o = oracle_for(prob, cfg["localization"], {})
    col = int(np.argmin((prob.lat - 41.0) ** 2 + (prob.lon - 221.0) ** 2))
    idx, rr, _ = o.obslist(col, 0)
    assert list(idx) == [0]
    y = prob.hx[0].astype(np.float64)
    s2 = y @ y / (prob.k - 1)
    d = float(prob.oval[0]) - float(prob.hx_mean[0])
    expect = d * s2 / (s2 + float(prob.oerr[0]) / float(rr[0]))
    inc = float(gpu["mean"][col, 0]) - float(prob.mean[col, 0])
    assert abs(inc - expect) < 2e-5 * max(1.0, abs(expect))
    o.close()


def test_edge_cases():
    """No observations; every column masked; ensemble sizes 2 and odd."""
    from dataclasses import replace
    cfg = workload_cfg("simple3d")
    prob = workload("simple3d")
    empty = replace(prob, olat=prob.olat[:0], olon=prob.olon[:0], oz=prob.oz[:0], otime=prob.otime[:0],
                    oval=prob.oval[:0], oerr=prob.oerr[:0], oobsid=prob.oobsid[:0], oplatid=prob.oplatid[:0],
                    hx=prob.hx[:0], hx_mean=prob.hx_mean[:0])
    g = gpu_run(empty, cfg["localization"], {})
    full_b = prob.state + prob.mean[:, :, None]
    assert np.allclose(g["state"], full_b, atol=3e-6)
    assert np.all(g["diag"]["obscount"] == 0)
    masked = replace(prob, mask=np.ones_like(prob.mask))
    g = gpu_run(masked, cfg["localization"], {})
    assert np.array_equal(g["state"], prob.state)
    for k in (2, 7, 33, 64):
        p = workload("c1", k=k)
        c1 = workload_cfg("c1")
        cols = np.arange(0, p.ncol, 37)
        for gram in ("plain", "batched"):
            _check_analysis(p, c1["localization"], c1["solver"], cols, label="k=%d %s" % (k, gram), variant=gram)


def test_errors_and_validation():
    from letkf_gb300 import LgpuError, Solver
    with Solver(0) as s:
        for bad in ({"inflation": {"rtps": 1.5}}, {"inflation": {"rtpp": -0.1}},
                    {"inflation": {"rtps": 0.5, "rtpp": 0.5}}, {"inflation": {"mul": 0.9}}):
            with pytest.raises(LgpuError) as e:
                s.solver_init(bad)
            assert e.value.code == 5
        with pytest.raises(LgpuError) as e:
            s.loc_init({"class": "loc_nosuch", "hzloc": [(0.0, 1e5)]})
        assert e.value.code == 4 and "LOC_NOSUCH not found" in e.value.msg
        with pytest.raises(LgpuError) as e:
            s.run()
        assert e.value.code == 6
        prob = workload("simple3d")
        s.solver_init({})
        s.loc_init(workload_cfg("simple3d")["localization"], prob.vars)
        with pytest.raises(LgpuError) as e:
            s.set_state(prob.state, prob.mean, prob.sprd, prob.vars)
        assert e.value.code == 6          # state before grid
        s.set_grid(prob.lat, prob.lon, prob.mask)
        big = np.zeros((prob.ncol, 1, 129), np.float32)
        with pytest.raises(LgpuError) as e:
            s.set_state(big, np.zeros((prob.ncol, 1), np.float32), np.zeros((prob.ncol, 1), np.float32),
                        [dict(grid_s_idx=0, levels=1)])
        assert e.value.code == 10
        s.set_state(prob.state, prob.mean, prob.sprd, prob.vars)
        bad_err = prob.oerr.copy()
        bad_err[0] = 0.0
        with pytest.raises(LgpuError) as e:
            s.set_obs(prob.olat, prob.olon, prob.oz, prob.otime, prob.oval, bad_err, prob.oobsid, prob.oplatid,
                      prob.hx, prob.hx_mean)
        assert e.value.code == 1
