"""Known-answer tests that pin the CPU oracle to the reference's arithmetic.

The reference's regression data (downloaded NetCDF backgrounds and norms)
is not available, so the oracle is pinned by answers derived independently
from the reference source and documentation:
  - letkf_loc_gc (src/letkf_loc.F90:348-378) evaluated in exact rational
    arithmetic with the same truncated coefficients;
  - linearinterp_lat (src/letkf_loc.F90:251-320) padding and interpolation;
  - the eigensolver against LAPACK dsyev/ssyev (the routine family
    src/letkf_core.F90:107 calls), through scipy;
  - letkf_core_solve against its closed form for one observation;
  - solver-loop identities (no obs, RTPS/RTPP with alpha=1, multiplicative
    inflation, bounds) and the scalar Kalman update at an observed point.
"""
import math
from fractions import Fraction

import numpy as np
import pytest

from conftest import workload

f32 = np.float32


def gc_rational(z, L):
    """letkf_loc_gc in exact arithmetic on the float inputs (the reference
    evaluates in REAL(8); the exact value rounded to float agrees except at
    rare double-rounding ties)."""
    c = Fraction(float(f32(L))) / Fraction(math.sqrt(0.3))
    az = abs(Fraction(float(f32(z))))
    zc = az / c
    if az >= 2 * c:
        return 0.0
    if az > c:
        v = (Fraction(0.08333) * zc ** 5 - Fraction(0.5) * zc ** 4 + Fraction(0.625) * zc ** 3 +
             Fraction(1.66667) * zc ** 2 - 5 * zc + 4 - Fraction(0.66667) * c / az)
    else:
        v = -Fraction(0.25) * zc ** 5 + Fraction(0.5) * zc ** 4 + Fraction(0.625) * zc ** 3 - Fraction(1.66667) * zc ** 2 + 1
    return float(v)


def test_gc_known_answers(oracle_mod):
    O = oracle_mod
    L = 500e3
    c = L / math.sqrt(0.3)
    assert O.gc(0.0, L) == 1.0
    assert O.gc(2 * c * 1.000001, L) == 0.0
    assert O.gc(-2 * c * 1.000001, L) == 0.0
    # both branches meet at z = c: 0.20833 with the truncated coefficients
    assert abs(O.gc(c * 0.9999999, L) - 0.20833) < 1e-5
    assert abs(O.gc(c * 1.0000001, L) - 0.20833) < 1e-5
    rng = np.random.default_rng(5)
    for L in (50e3, 200e3, 500e3, 800e3, 200.0, 3.0):
        for z in rng.random(400) * 2.1 * L / math.sqrt(0.3):
            got = O.gc(float(z), L)
            ref = gc_rational(z, L)
            assert abs(got - ref) <= 1.2e-7 * max(1.0, abs(ref)), (z, L, got, ref)


def test_interp_padding_and_values(oracle_mod):
    O = oracle_mod
    t = O.interp([(0.0, 500e3), (90.0, 50e3)])
    assert t.npoints == 2
    assert O.lib().or_interp_get(t, 0.0) == f32(500e3)
    assert O.lib().or_interp_get(t, 90.0) == f32(50e3)
    assert O.lib().or_interp_get(t, -45.0) == f32(275e3)
    # a first point above 0 degrees gets a 0-degree point with the same radius,
    # a last point below 90 a 90-degree point with the last radius
    t = O.interp([(10.0, 100e3), (40.0, 300e3)])
    assert t.npoints == 4
    assert list(t.lat[:4]) == [0.0, 10.0, 40.0, 90.0]
    assert list(t.dist[:4]) == [100e3, 100e3, 300e3, 300e3]
    assert O.lib().or_interp_get(t, 5.0) == f32(100e3)
    assert abs(O.lib().or_interp_get(t, 25.0) - 200e3) < 0.05
    assert O.lib().or_interp_get(t, 60.0) == f32(300e3)
    # a single point spans the globe
    t = O.interp([(0.0, 500e3)])
    assert t.npoints == 2 and O.lib().or_interp_get(t, 77.0) == f32(500e3)


def test_metric_properties(oracle_mod):
    O = oracle_mod
    R = 6371000.0
    a, b = O.unitvec(0.0, 0.0), O.unitvec(0.0, 90.0)
    assert abs(O.dist(a, b) - R * math.pi / 2) < 2.0
    assert O.dist(a, a) == 0.0
    assert abs(O.dist(O.unitvec(90.0, 0.0), O.unitvec(-90.0, 0.0)) - R * math.pi) < 4.0
    rng = np.random.default_rng(3)
    for _ in range(300):
        la1, lo1 = rng.uniform(-90, 90), rng.uniform(-180, 360)
        la2, lo2 = la1 + rng.normal(0, 10), lo1 + rng.normal(0, 10)
        la2 = max(-90.0, min(90.0, la2))
        u1, u2 = O.unitvec(la1, lo1), O.unitvec(la2, lo2)
        d = O.dist(u1, u2)
        assert d == O.dist(u2, u1)
        # haversine in double on the float inputs
        p1, p2 = math.radians(f32(la1)), math.radians(f32(la2))
        dl = math.radians(float(f32(lo2)) - float(f32(lo1)))
        h = math.sin((p2 - p1) / 2) ** 2 + math.cos(p1) * math.cos(p2) * math.sin(dl / 2) ** 2
        ref = 2 * R * math.asin(min(1.0, math.sqrt(h)))
        assert abs(d - ref) <= 1e-6 * ref + 1.0, (la1, lo1, la2, lo2, d, ref)


def test_unitvec_matches_libm(oracle_mod):
    O = oracle_mod
    rng = np.random.default_rng(4)
    for la, lo in zip(rng.uniform(-90, 90, 500), rng.uniform(-720, 720, 500)):
        u = O.unitvec(la, lo)
        p, l = math.radians(float(f32(la))), math.radians(float(f32(lo)))
        ref = np.array([math.cos(p) * math.cos(l), math.cos(p) * math.sin(l), math.sin(p)], np.float32)
        assert np.max(np.abs(u - ref)) <= 6e-8


def test_eigh_against_lapack(oracle_mod):
    scipy_lapack = pytest.importorskip("scipy.linalg.lapack")
    O = oracle_mod
    rng = np.random.default_rng(11)
    for k in (2, 5, 20, 40, 64):
        Y = rng.standard_normal((k, 3 * k))
        A = Y @ Y.T + (k - 1) * np.eye(k)
        lam, V, rc = O.eigh(A)
        assert rc == 0
        w, v, info = scipy_lapack.dsyev(A)
        assert info == 0
        assert np.allclose(lam, w, rtol=1e-12, atol=1e-10)
        # eigenvectors up to sign
        assert np.allclose(np.abs(np.sum(V * v, 0)), 1.0, atol=1e-9)
        ws, vs, info = scipy_lapack.ssyev(A.astype(np.float32))
        assert info == 0
        assert np.allclose(lam, ws, rtol=2e-5)


def test_core_solve_single_observation(oracle_mod):
    """One observation: A = (k-1)I + w y y^T has eigenvalue (k-1) + w|y|^2 on y
    and k-1 elsewhere, so W = I + (sqrt((k-1)/lam1) - 1) yy^T/|y|^2 and
    wbar = w d y / lam1."""
    O = oracle_mod
    rng = np.random.default_rng(2)
    for k in (5, 20, 40):
        y = rng.standard_normal(k).astype(np.float32)
        y -= y.mean(dtype=np.float32)
        err, r, d = f32(0.5), f32(0.7), f32(1.3)
        w = float(r) / float(err)
        yy = y.astype(np.float64)
        lam1 = (k - 1) + w * yy @ yy
        u = yy / np.linalg.norm(yy)
        W = np.eye(k) + (math.sqrt((k - 1) / lam1) - 1.0) * np.outer(u, u)
        wbar = w * float(d) * yy / lam1
        T = W + wbar[:, None]
        for prec, tol in ((64, 2e-7), (32, 2e-6)):   # results are returned as REAL
            got = O.core_solve(y[None, :], [err], [r], [d], precision=prec)
            assert np.allclose(got, T, atol=tol, rtol=0), (prec, np.abs(got - T).max())
        # W 1 = 1 for perturbations that sum to zero (sum of members preserved)
        got = O.core_solve(y[None, :], [err], [r], [0.0], precision=64)
        assert np.allclose(got @ np.ones(k), np.ones(k), atol=1e-6)


def _oracle(prob, loc, **infl):
    from letkf_gb300 import normalize_loc
    from oracle import oracle as O
    return O.Oracle(prob, normalize_loc(loc, prob.vars), **infl)


LOC_SIMPLE = {"class": "loc_novrt", "hzloc": [(0.0, 500e3), (90.0, 50e3)]}


def test_solver_identities():
    prob = workload("simple3d")
    # no observations anywhere: analysis = background
    from dataclasses import replace
    empty = replace(prob, olat=prob.olat[:0], olon=prob.olon[:0], oz=prob.oz[:0], otime=prob.otime[:0],
                    oval=prob.oval[:0], oerr=prob.oerr[:0], oobsid=prob.oobsid[:0], oplatid=prob.oplatid[:0],
                    hx=prob.hx[:0], hx_mean=prob.hx_mean[:0])
    o = _oracle(empty, LOC_SIMPLE)
    r = o.run(32, cols=np.arange(0, prob.ncol, 97))
    cols = np.arange(0, prob.ncol, 97)
    full_b = prob.state[cols] + prob.mean[cols][:, :, None]
    assert np.allclose(r["state"], full_b, atol=3e-6)
    assert np.allclose(r["mean"], prob.mean[cols], atol=3e-7)
    assert np.allclose(r["sprd"], prob.sprd[cols], rtol=3e-6)
    assert np.all(r["obscount"] == 0)
    o.close()
    # RTPS alpha=1 restores the background spread; RTPP alpha=1 the perturbations
    cols = np.arange(prob.ncol)[np.abs(prob.lat) < 60][::50]
    o = _oracle(prob, LOC_SIMPLE, rtps=1.0)
    r = o.run(64, cols=cols)
    assert np.allclose(r["sprd"], prob.sprd[cols], rtol=1e-5)
    o.close()
    o = _oracle(prob, LOC_SIMPLE, rtpp=1.0)
    r = o.run(64, cols=cols)
    pert = r["state"] - r["mean"][:, :, None]
    assert np.allclose(pert, prob.state[cols], atol=2e-5)
    o.close()
    # multiplicative inflation scales the spread
    o1 = _oracle(prob, LOC_SIMPLE)
    o2 = _oracle(prob, LOC_SIMPLE, mul=1.05)
    a, b = o1.run(64, cols=cols), o2.run(64, cols=cols)
    assert np.allclose(b["sprd"], 1.05 * a["sprd"], rtol=1e-5)
    assert np.allclose(b["mean"], a["mean"], atol=1e-6)
    # perturbations sum to zero, members = perturbation + mean
    assert np.allclose((a["state"] - a["mean"][:, :, None]).sum(-1), 0.0, atol=1e-4)


def test_scalar_kalman_update_at_observation():
    """simple3d obs1 sits 0.5 deg from grid point (41N, 221E).  With the only
    obs in range, the LETKF mean increment at a slab observed exactly is the
    scalar Kalman update d * s2 / (s2 + err/r), s2 = sum(y^2)/(k-1)
    (R^-1 = r/err with err used as given, src/letkf_core.F90:92-94)."""
    from oracle import oracle as O
    prob = workload("simple3d")
    o = _oracle(prob, LOC_SIMPLE)
    # column nearest obs 0
    col = int(np.argmin((prob.lat - 41.0) ** 2 + (prob.lon - 221.0) ** 2))
    idx, rr, nc = o.obslist(col, 0)
    assert list(idx) == [0]
    r = o.run(64, cols=[col])
    y = prob.hx[0].astype(np.float64)
    s2 = y @ y / (prob.k - 1)
    d = float(prob.oval[0]) - float(prob.hx_mean[0])
    expect = d * s2 / (s2 + float(prob.oerr[0]) / float(rr[0]))
    slab = 0    # obs 0 observes state1 at level 0 (depth 1 m)
    inc = float(r["mean"][0, slab]) - float(prob.mean[col, slab])
    assert abs(inc - expect) < 1e-5 * max(1.0, abs(expect))
    # the localisation weight is the GC weight of the documented metric
    dist = O.dist(O.unitvec(prob.lat[col], prob.lon[col]), O.unitvec(prob.olat[0], prob.olon[0]))
    L = O.lib().or_interp_get(O.interp([(0.0, 500e3), (90.0, 50e3)]), float(prob.lat[col]))
    assert rr[0] == f32(O.gc(dist, L))
    o.close()


def test_ocean_temporal_gc_and_surface_ids():
    """loc_ocean (src/subclass.letkf_localizer/letkf_loc_ocean.F90:451-499):
    an observation is a surface observation only when its id is in sat_obs AND
    its platform in sat_plats; a surface observation takes the satellite radius
    and tloc_sat and is dropped below the mixed layer, any other the profile
    radius and tloc_prof.  The temporal factor is letkf_loc_gc(time, tloc),
    which takes |time|: the sign of the time does not matter.  The weight is
    the REAL product of the two REAL factors."""
    from dataclasses import replace
    from oracle import oracle as O
    prob = workload("simple3d")
    col = int(np.argmin((prob.lat - 41.0) ** 2 + (prob.lon - 221.0) ** 2))
    loc = {"class": "loc_ocean", "hzloc_prof": [(0.0, 500e3), (90.0, 50e3)], "hzloc_sat": [(0.0, 300e3)],
           "tloc_prof": 2.0, "tloc_sat": 1.5, "sat_obs": [3], "sat_plats": [2],
           "vtloc_surf": {"type": "bkg_t", "bkg_t_delta": 0.2, "bkg_t_var": prob.vars[0]["name"]}}
    dist = O.dist(O.unitvec(prob.lat[col], prob.lon[col]), O.unitvec(prob.olat[0], prob.olon[0]))
    Lp = O.lib().or_interp_get(O.interp([(0.0, 500e3), (90.0, 50e3)]), float(prob.lat[col]))
    Ls = O.lib().or_interp_get(O.interp([(0.0, 300e3)]), float(prob.lat[col]))
    seen = {}
    for obsid, platid, surf in [(1, 1, False), (3, 2, True), (4, 2, False), (3, 1, False)]:
        for t in (1.25, -1.25, 0.0):
            ids = prob.oobsid.copy()
            plats = prob.oplatid.copy()
            times = prob.otime.copy()
            ids[0], plats[0], times[0] = obsid, platid, t
            o = _oracle(replace(prob, oobsid=ids, oplatid=plats, otime=times), loc)
            assert o.maxgroups == 2
            idx, rr, _ = o.obslist(col, 0)
            rh = np.float32(O.gc(dist, Ls if surf else Lp))
            rt = np.float32(O.gc(t, 1.5 if surf else 2.0))
            assert 0 in list(idx), (obsid, platid, t)
            got = rr[list(idx).index(0)]
            assert got == np.float32(rh * rt), (obsid, platid, t, got, rh * rt)
            seen[(obsid, platid, abs(t))] = seen.get((obsid, platid, abs(t)), got)
            assert seen[(obsid, platid, abs(t))] == got      # t and -t give the same weight
            # below the mixed layer: surface observations are dropped
            idx1 = list(o.obslist(col, 1)[0])
            assert (0 in idx1) == (not surf), (obsid, platid, t)
            o.close()
    # the temporal factor is active: a nonzero time lowers the weight
    assert seen[(1, 1, 1.25)] < seen[(1, 1, 0.0)]
    assert seen[(3, 2, 1.25)] < seen[(3, 2, 0.0)]


def test_bounds_semantics():
    """bounds_check: clipped means stay inside ana_bounds and inside
    bkg_mean +- ana_inc_max; members stay inside the bounds."""
    from letkf_gb300.workloads import SIMPLE3D_VARIANTS, apply_bounds
    prob = workload("simple3d")
    vs = apply_bounds(prob.vars, SIMPLE3D_VARIANTS["bounds_check"]["bounds"])
    from letkf_gb300 import normalize_loc
    from oracle import oracle as O
    o = O.Oracle(prob, normalize_loc(LOC_SIMPLE), variables=vs)
    cols = np.arange(prob.ncol)[::7]
    for prec in (32, 64):
        r = o.run(prec, cols=cols)
        for v in vs:
            s0, s1 = v["grid_s_idx"], v["grid_s_idx"] + v["levels"]
            lo, hi = v.get("ana_bounds", (-9.99e36, 9.99e36))
            m = r["mean"][:, s0:s1]
            x = r["state"][:, s0:s1]
            assert np.all(m >= lo - 1e-5) and np.all(m <= hi + 1e-5)
            assert np.all(x >= lo - 1e-4) and np.all(x <= hi + 1e-4)
            inc = v.get("ana_inc_max", 9.99e36)
            if inc < 1e30:
                assert np.all(np.abs(m - prob.mean[cols, s0:s1]) <= inc + 1e-5)
    o.close()


def test_fp32_mirror_close_to_fp64():
    from letkf_gb300.workloads import WORKLOADS
    prob = workload("c1")
    wl = WORKLOADS["c1"]
    o = _oracle(prob, wl["localization"], rtps=0.6)
    cols = np.arange(0, prob.ncol, 5)
    a, b = o.run(32, cols=cols), o.run(64, cols=cols)
    pa, pb = a["state"] - a["mean"][:, :, None], b["state"] - b["mean"][:, :, None]
    assert np.linalg.norm(pa - pb) / np.linalg.norm(pb) < 1e-5
    assert np.linalg.norm(a["mean"] - b["mean"]) / np.linalg.norm(b["mean"]) < 1e-6
    o.close()


def test_lapack_call_sequence():
    """The oracle's library-call form (the reference's sgemm / ssyev('V','U')
    sequence through SciPy's BLAS / LAPACK, the timed CPU baseline) agrees
    with the FP64 oracle as closely as the FP32 restatement does."""
    pytest.importorskip("scipy")
    from letkf_gb300.workloads import WORKLOADS
    from oracle import oracle as O
    O.set_lapack()
    rng = np.random.default_rng(3)
    for k in (3, 10, 40):
        # the FP64 form is pinned to the closed form above
        y = rng.standard_normal(k).astype(f32)
        err, r, d = f32(0.7), f32(0.9), f32(-0.4)
        got64 = O.core_solve(y[None, :], [err], [r], [d], precision=64)
        got = O.core_solve(y[None, :], [err], [r], [d], precision=O.PREC_LAPACK)
        assert np.allclose(got, got64, atol=2e-6, rtol=0), (k, np.abs(got - got64).max())
    prob = workload("c1")
    wl = WORKLOADS["c1"]
    o = _oracle(prob, wl["localization"], rtps=0.6)
    cols = np.arange(0, prob.ncol, 5)
    a, b = o.run(O.PREC_LAPACK, cols=cols, nthreads=1), o.run(64, cols=cols)
    pa, pb = a["state"] - a["mean"][:, :, None], b["state"] - b["mean"][:, :, None]
    assert np.linalg.norm(pa - pb) / np.linalg.norm(pb) < 1e-5
    assert np.linalg.norm(a["mean"] - b["mean"]) / np.linalg.norm(b["mean"]) < 1e-6
    assert np.array_equal(a["lg_obscount"], b["lg_obscount"])
    o.close()
