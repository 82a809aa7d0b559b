#!/usr/bin/env python
"""Headline benchmark: LETKF analysis throughput (grid columns per second) of
the GB300 library on the 720x360x40 ocean workload (k=40, T/S/SSH = 81 slabs,
3,000 T/S profiles + 200,000 SSH/SST swath observations, loc_novrt 800 km ->
200 km), synthetic seeded inputs.

One step = one complete analysis (observation index build, search,
localisation, Gram, eigensolve, transform and update epilogue) over every
ocean column, inputs resident in HBM; the L2 is flushed (256 MB write)
between timed steps.  `e2e` repeats the step through the public C ABI with
host buffers: the state and observations are copied in from page-locked host
memory and the analysis is copied back every step.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

--impl reference times the reference algorithm on the host cores, on a
bounded column sample of the same workload: the oracle's column loop with
the reference's own sequence of library calls (sgemm, ssyev('V','U'),
sgemm x3, one sgemm per slab, all FP32) through the optimised BLAS / LAPACK
SciPy is linked with, single-threaded per call, OpenMP over columns.  With N > 1 (torchrun) every rank runs
an independent replica on its own GPU (weak scaling, no collectives on the
data path); rank 0 prints the line.
"""
import argparse
import json
import os

# the CPU legs call BLAS / LAPACK from every OpenMP thread: one thread per call
os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "umd-letkf_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "gridpoints/s on 1 GB300: batched+learned vs plain LETKF at fixed analysis error"
UNIT = "gridpoints/s"


# nominal FP32 CUDA-core peak: 152 SMs x 128 lanes x 2 flop x 2.07 GHz
SIMT_FP32_TFLOPS = 152 * 128 * 2 * 2.07e9 / 1e12


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return d["hbm_gbs"], d["bf16_tflops"], "measured"
    except Exception:
        return 6800.0, 1900.0, "fallback"


class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch
            import torch.distributed as td
            backend = "nccl" if torch.cuda.is_available() else "gloo"
            if backend == "nccl":
                torch.cuda.set_device(self.local)
            td.init_process_group(backend)
            self.td, self.torch = td, torch
            self.dev = torch.device("cuda", self.local) if backend == "nccl" else torch.device("cpu")

    def barrier(self):
        if self.world > 1:
            self.td.barrier()

    def max(self, x):
        if self.world == 1:
            return x
        t = self.torch.tensor([float(x)], dtype=self.torch.float64, device=self.dev)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.world > 1:
            self.td.destroy_process_group()


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, gpu):
        self.proc = None
        # the raw samples (the JSON line carries their summary)
        self.path = os.environ.get("LGPU_CLOCKS_CSV", "/tmp/lgpu_clocks.csv")
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(gpu), "--query-gpu=" + q, "--format=csv,noheader",
                                          "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1].split()[0]))
                smax = float(parts[2].split()[0])
            except Exception:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def make_problem(name, nthreads=0):
    from letkf_gb300 import synth
    from letkf_gb300.workloads import WORKLOADS
    cfg = WORKLOADS[name]
    gen = dict(cfg["gen"])
    w = gen.pop("workload")
    prob = synth.generate(w, nthreads=nthreads, **gen)
    return prob, cfg


def cpu_oracle(prob, cfg):
    """The oracle over `prob` in the reference's library-call form: returns
    (oracle, precision code, description of the arithmetic).  Without SciPy's
    BLAS / LAPACK the FP32 restatement (plain loops, Jacobi) stands in."""
    from letkf_gb300 import normalize_loc, normalize_solver
    from oracle import oracle as O
    inf = normalize_solver(cfg["solver"])
    o = O.Oracle(prob, normalize_loc(cfg["localization"], prob.vars), rtps=inf["rtps"], rtpp=inf["rtpp"],
                 mul=inf["mul"])
    try:
        lib = O.set_lapack()
        return o, O.PREC_LAPACK, ("the reference's call sequence (sgemm, ssyev('V','U'), sgemm x3, sgemm per slab; "
                                  "FP32) through %s, one thread per call, OpenMP over columns "
                                  "(oracle/letkf_oracle.c)" % lib)
    except Exception as e:   # no SciPy on this host
        return o, 32, ("FP32 C restatement of the reference algorithm with plain loops and a Jacobi eigensolve "
                       "(oracle/letkf_oracle.c; no BLAS / LAPACK: %s), OpenMP over columns" % type(e).__name__)


def size_sample(o, prec, active, nth, target_s):
    """An evenly spread column sample worth about target_s of host work."""
    probe = active[:: max(1, len(active) // (4 * nth))][: 4 * nth]
    t0 = time.perf_counter()
    o.run(prec, cols=probe, nthreads=nth)
    rate = len(probe) / max(time.perf_counter() - t0, 1e-9)
    n = int(min(len(active), max(4 * nth, rate * target_s)))
    return active[:: max(1, len(active) // n)][:n]


def cpu_rate(prob, cfg, target_s=15.0, nthreads=0):
    """The reference's arithmetic on the host cores over a bounded, evenly
    spread sample of ocean columns; returns (columns/s, sample size, threads,
    seconds, description)."""
    o, prec, desc = cpu_oracle(prob, cfg)
    active = np.nonzero(prob.mask == 0)[0]
    nth = nthreads or os.cpu_count() or 1
    sample = size_sample(o, prec, active, nth, target_s)
    t0 = time.perf_counter()
    o.run(prec, cols=sample, nthreads=nth)
    dt = time.perf_counter() - t0
    o.close()
    return len(sample) / dt, len(sample), nth, dt, desc


def reference_arm(args, dist):
    if dist.rank != 0:
        return 0
    prob, cfg = make_problem(args.workload)
    o, prec, how = cpu_oracle(prob, cfg)
    active = np.nonzero(prob.mask == 0)[0]
    nth = os.cpu_count() or 1
    # one step is about 6 s of host work
    sample = size_sample(o, prec, active, nth, 6.0)
    for _ in range(args.warmup):
        o.run(prec, cols=sample[: max(nth, len(sample) // 8)], nthreads=nth)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        o.run(prec, cols=sample, nthreads=nth)
        times.append(time.perf_counter() - t0)
    o.close()
    ms = 1000.0 * statistics.mean(times)
    value = len(sample) / (ms / 1000.0)
    desc = "%d of %d ocean columns (evenly spaced) per step; %s" % (len(sample), len(active), how)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": workload_config(args, prob, cfg),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": nth, "kind": "port", "sample": desc},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def describe_loc(loc):
    """One-line description of a localization section."""
    pts = loc.get("hzloc", loc.get("hzloc_prof", {})).get("value", [])
    rad = " -> ".join("%g km (%g deg)" % (p["radius"] / 1e3, p["lat"]) for p in pts)
    out = "%s %s" % (loc["class"], rad)
    if "vtloc" in loc:
        out += ", vertical GC %g m" % loc["vtloc"]
    return out


def workload_config(args, prob, cfg):
    nact = int(np.sum(prob.mask == 0))
    names = "/".join(v["name"] for v in prob.vars) if prob.vars and "name" in prob.vars[0] else "%d variables" % len(
        prob.vars)
    state_gb = 2.0 * prob.ncol * prob.ns * prob.k * 4 / 1e9
    return {"workload": "%s: %dx%dx%d grid, %s (%d slabs), k=%d, %d obs, %s" % (
                args.workload, prob.nx, prob.ny, prob.nz, names, prob.ns, prob.k, prob.nobs,
                describe_loc(cfg["localization"])),
            "columns_total": int(prob.ncol), "columns_active": nact, "ensemble": int(prob.k), "slabs": int(prob.ns),
            "observations": int(prob.nobs), "l2": "flushed (256 MB device write) before every timed step; "
                                                  "state in+out %.1f GB per step" % state_gb,
            "parallelism": "replicas" if args.gpus > 1 else "single",
            "eig_precision": args.precision}


def gpu_arm(args, dist):
    from letkf_gb300 import PinnedArray, Solver
    prob, cfg = make_problem(args.workload)
    hbm, bf16, peak_kind = peaks()
    dev = dist.local if dist.world > 1 else 0
    s = Solver(dev)
    s.set_variant(args.variant)
    s.set_precision(args.precision)
    s.solver_init(cfg["solver"])
    s.loc_init(cfg["localization"], prob.vars, prob.lev_depth)
    s.set_problem(prob)
    nact = int(np.sum(prob.mask == 0))
    # ---- device-resident steps
    for _ in range(max(args.warmup, 3)):
        s.run()
    dist.barrier()
    clocks = Clocks(dev)
    tims = []
    for _ in range(args.steps):
        s.flush_l2(256 << 20)
        s.run()
        tims.append(s.timings())
    dist.barrier()
    ck = clocks.stop()
    ms = statistics.mean(t["total_ms"] for t in tims)
    ms_max = dist.max(ms)
    value = dist.world * nact / (ms_max / 1000.0)
    stage = {k: statistics.mean(t[k] for t in tims)
             for k in ("index_ms", "prep_ms", "gram_ms", "tiles_ms", "eig_ms", "update_ms")}
    launches = tims[-1]["launches"]
    diag = s.get_diag()
    kept = float(np.sum(diag["lg_obscount"], dtype=np.float64))
    cand = float(np.sum(diag["obscount"], dtype=np.float64))
    k, ns, ncol = prob.k, prob.ns, prob.ncol
    units = tims[-1]["units"]
    # algorithmic work per launch: the Gram kernel does one
    # multiply-add per packed feature (k(k+3)/2 of them: upper triangle of G
    # and the right-hand side) per kept (column, observation) pair; the
    # eigensolve ~9k^3 + transform 4k^3 per unit; the update reads the
    # background members and writes the analysis members, mean and spread.
    gram_flop = float(k * (k + 3)) * kept
    eig_flop = 13.0 * k ** 3 * units
    upd_bytes = 2.0 * ncol * ns * k * 4 + 4.0 * ncol * ns * 4
    gram_kernel_ms = stage["gram_ms"] - stage["tiles_ms"]
    # executed tensor work of the batched Gram: 3 TF32 products x 2 flop x
    # M=128 x N=features per pass x K=16 per chunk that ran MMAs
    mma_flop = float(tims[-1]["mma_chunks"]) * 3 * 2 * 128 * tims[-1]["mma_n"] * 16
    stages = {
        "tile_streams": {"ms": stage["tiles_ms"]},
        "gram": {"ms": gram_kernel_ms, "tflops": gram_flop / (gram_kernel_ms * 1e-3) / 1e12},
        "eig": {"ms": stage["eig_ms"], "tflops": eig_flop / (stage["eig_ms"] * 1e-3) / 1e12,
                "fp64_units": tims[-1]["fp64_units"], "fp64_ms": tims[-1]["fp64_ms"]},
        "update": {"ms": stage["update_ms"], "gbs": upd_bytes / (stage["update_ms"] * 1e-3) / 1e9},
        "index": {"ms": stage["index_ms"]}, "prep": {"ms": stage["prep_ms"]},
        "kept_pairs": kept, "candidate_pairs": cand}
    times = {"gram": gram_kernel_ms, "eig": stage["eig_ms"], "update": stage["update_ms"]}
    dom = max(times, key=times.get)
    kname = {"gram": "k_gram_tc" if tims[-1]["variant"] == 2 else "k_gram", "eig": "k_eig", "update": "k_update"}[dom]
    traffic = read_traffic(kname) if args.workload == "c2" else None   # the committed captures are of C2
    if dom == "update":
        ach = upd_bytes / (stage["update_ms"] * 1e-3) / 1e9
        roof = {"kernel": kname, "bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s",
                "frac": ach / hbm, "traffic": traffic, "peak_source": peak_kind + " hbm_gbs (burst)"}
    else:
        fl = gram_flop if dom == "gram" else eig_flop
        ach = fl / (times[dom] * 1e-3) / 1e12
        simt = SIMT_FP32_TFLOPS
        roof = {"kernel": kname, "bound": "tensor", "achieved": ach, "peak": bf16, "unit": "TFLOP/s",
                "frac": ach / bf16, "traffic": traffic,
                "peak_source": peak_kind + " bf16_tflops (burst)",
                "note": ("TF32 three-term split on tcgen05; dense TF32 is half the bf16 rate and the split triples "
                         "the MMAs, so bf16/6 bounds this kernel's algorithmic rate" if dom == "gram" else
                         "FP32 on the CUDA cores (no tensor work); nominal FP32 SIMT peak %.1f TFLOP/s, "
                         "frac of it %.4f" % (simt, ach / simt))}
    if dom == "gram" and mma_flop > 0:
        ex = mma_flop / (gram_kernel_ms * 1e-3) / 1e12
        roof["tensor_executed"] = {"tflops": ex, "peak_tf32_tflops": bf16 / 2, "frac": ex / (bf16 / 2),
                                   "note": "MMA work issued (3 TF32 products per FP32 product, zero weights "
                                           "and padding included) over the Gram kernels' time; TF32 dense "
                                           "peak taken as half the measured bf16 peak"}
    variant = {1: "plain", 2: "batched_tc"}.get(tims[-1]["variant"], "?")
    plain = None
    if variant != "plain" and not args.no_plain:
        # the plain per-column FP32 path on the same inputs (the headline ratio's denominator)
        s.set_variant("plain")
        for _ in range(2):
            s.run()
        pt = []
        for _ in range(max(1, min(args.steps, 3))):
            s.flush_l2(256 << 20)
            s.run()
            pt.append(s.timings()["total_ms"])
        pms = dist.max(statistics.mean(pt))
        plain = {"value": dist.world * nact / (pms / 1000.0), "ms_per_step": pms,
                 "speedup_of_headline": (dist.world * nact / (ms_max / 1000.0)) / (dist.world * nact / (pms / 1000.0))}
        s.set_variant(args.variant)
        s.run()
    # ---- end to end through the C ABI with page-locked host buffers: the
    # state is bound in place (lgpu_bind_state, the reference's in-place
    # letkf_solver_run); every step uploads the observations and the
    # background and downloads the analysis into the bound arrays
    pin = {n: PinnedArray(getattr(prob, n).shape, getattr(prob, n).dtype) for n in
           ("olat", "olon", "oz", "otime", "oval", "oerr", "oobsid", "oplatid", "hx", "hx_mean")}
    for n, p in pin.items():
        p.array[...] = getattr(prob, n)
    outp = [PinnedArray(prob.state.shape), PinnedArray(prob.mean.shape), PinnedArray(prob.sprd.shape)]
    h2d = sum(p.array.nbytes for p in pin.values()) + sum(p.array.nbytes for p in outp)
    d2h = sum(p.array.nbytes for p in outp)

    def refill():   # the same background every step (outside the timed region)
        for p, src in zip(outp, (prob.state, prob.mean, prob.sprd)):
            np.copyto(p.array, src)

    s.bind_state(outp[0].array, outp[1].array, outp[2].array, prob.vars)

    def e2e_step():
        s.set_obs(pin["olat"].array, pin["olon"].array, pin["oz"].array, pin["otime"].array, pin["oval"].array,
                  pin["oerr"].array, pin["oobsid"].array, pin["oplatid"].array, pin["hx"].array,
                  pin["hx_mean"].array)
        s.run()

    for _ in range(max(6, args.warmup)):
        refill()
        e2e_step()
    dist.barrier()
    et, ev, etim = [], [], []
    for _ in range(args.steps):
        refill()
        s.flush_l2(256 << 20)
        t0 = time.perf_counter()
        e2e_step()
        et.append(time.perf_counter() - t0)
        tm = s.timings()
        ev.append(tm["variant"])
        etim.append(tm)
    dist.barrier()
    e2e_ms = dist.max(1000.0 * statistics.mean(et))
    e2e_val = dist.world * nact / (e2e_ms / 1000.0)
    link = link_summary(etim)
    ok = bool(np.all(np.isfinite(outp[1].array)))
    for p in list(pin.values()) + outp:
        p.free()
    s.close()
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": dist.world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded generator, no public dataset)",
            "config": workload_config(args, prob, cfg), "clocks": ck, "gpu_launches": launches * args.steps,
            "e2e": {"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                    "ms_per_step": e2e_ms, "step_ms": [round(1000.0 * t, 3) for t in et],
                    "variant": [{1: "plain", 2: "batched_tc"}.get(v, "?") for v in ev], "link": link},
            "roofline": roof, "stages": stages, "analysis_finite": ok, "variant": variant, "plain_variant": plain}
    if dist.rank == 0 and dist.world == 1 and not args.no_cpu_baseline:
        rate, n, nth, dt, how = cpu_rate(prob, cfg)
        line["cpu_baseline"] = {"value": rate, "unit": UNIT, "cores": nth, "kind": "port",
                                "sample": "%d of %d ocean columns (evenly spaced), %.1f s; %s" % (n, nact, dt, how)}
    if dist.rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def link_summary(tims):
    """Where the end-to-end step goes, from the library's CUDA events and host
    clocks (means over the timed steps): observation upload, background
    upload and analysis download with their rates, the device span of the run
    (start to the last download) and the host time of the two calls."""
    m = lambda key: statistics.mean(t[key] for t in tims)
    up, down = m("h2d_state_ms"), m("d2h_state_ms")
    ub, db = m("h2d_state_bytes"), m("d2h_state_bytes")
    return {"h2d_obs_ms": m("h2d_obs_ms"), "h2d_state_ms": up, "d2h_state_ms": down,
            "h2d_state_gbs": ub / (up * 1e-3) / 1e9 if up > 0 else None,
            "d2h_state_gbs": db / (down * 1e-3) / 1e9 if down > 0 else None,
            "device_span_ms": m("span_ms"), "device_compute_ms": m("total_ms"),
            "host_set_obs_ms": m("host_obs_ms"), "host_run_ms": m("host_run_ms"),
            "stage_ms": {k: m(k + "_ms") for k in ("tiles", "gram", "eig", "update", "index", "prep")},
            "span_ms_per_step": [round(t["span_ms"], 2) for t in tims],
            "host_run_ms_per_step": [round(t["host_run_ms"], 2) for t in tims]}


def learned_arm(args, dist):
    """C5: the learned form in a cycling experiment.  Cycles 0-4 run the exact
    analysis (AUTO form) and collect training rows; the network is trained on
    the GPU; on the next cycle the exact (AUTO), plain and learned analyses
    are timed on the same inputs and the learned analysis is compared with
    the exact one (RMS of the analysis-mean difference over the background
    spread; the interpolation without the network alongside)."""
    from letkf_gb300 import PinnedArray, Solver, synth
    from letkf_gb300.workloads import WORKLOADS
    cfg = WORKLOADS[args.workload]
    gen = dict(cfg["gen"])
    w = gen.pop("workload")
    cy = cfg["cycles"]
    t_setup = time.perf_counter()
    prob = synth.generate(w, **gen)
    nobs = prob.nobs
    prob = synth.observe(prob, seed=2000, n_obs=nobs, **{k: cy[k] for k in ("n_clusters", "cluster_sigma_m") if k in cy})
    dev = dist.local if dist.world > 1 else 0
    s = Solver(dev)
    s.solver_init(cfg["solver"])
    s.loc_init(cfg["localization"], prob.vars, prob.lev_depth)
    s.set_problem(prob)
    s.learn_init(prob.nx, prob.ny, **cfg["learn"])

    obs_kw = {k: cy[k] for k in ("n_clusters", "cluster_sigma_m") if k in cy}

    def next_cycle(p, ana, c):
        x, m, sp = ana
        p.state[...] = x - m[:, :, None]
        p.mean[...] = m
        p.sprd[...] = sp
        synth.forecast(p, u=cy["u"], kappa=cy["kappa"], dt=cy["dt"])
        return synth.observe(p, seed=2000 + c, n_obs=nobs, **obs_kw)

    for c in range(cy["train"]):
        if c:
            prob = next_cycle(prob, ana, c)
            s.set_problem(prob)
        s.set_variant("auto")
        rows = s.learn_collect()
        ana = s.get_state()
    t_tr = time.perf_counter()
    loss = s.learn_train(epochs=cy["epochs"], batch=cy["batch"], lr=cy["lr"])
    t_tr = time.perf_counter() - t_tr
    prob = next_cycle(prob, ana, cy["train"])
    s.set_problem(prob)
    t_setup = time.perf_counter() - t_setup
    nact = int(np.sum(prob.mask == 0))

    def timed(variant, steps, warm):
        s.set_variant(variant)
        for _ in range(max(warm, 3)):
            s.run()
        dist.barrier()
        ts = []
        for _ in range(steps):
            s.flush_l2(256 << 20)
            s.run()
            ts.append(s.timings())
        dist.barrier()
        return ts

    ex_t = timed("auto", args.steps, args.warmup)
    ex = s.get_state()
    exact_variant = {1: "plain", 2: "batched_tc"}.get(ex_t[-1]["variant"], "?")
    pl_t = timed("plain", max(1, min(args.steps, 3)), 1)
    clocks = Clocks(dev)
    le_t = timed("learned", args.steps, args.warmup)
    ck = clocks.stop()
    le = s.get_state()
    st = s.learn_stats()
    s.learn_set_network(False)
    s.run()
    ip = s.get_state()
    s.learn_set_network(True)
    act = prob.mask == 0
    spread = float(np.sqrt(np.mean(prob.sprd[act].astype(np.float64) ** 2)))
    err = lambda a: float(np.sqrt(np.mean((a[1][act].astype(np.float64) - ex[1][act]) ** 2))) / spread
    # end to end through the C ABI: state and observations from page-locked
    # host buffers, analysis back into page-locked buffers, every step
    names = ("olat", "olon", "oz", "otime", "oval", "oerr", "oobsid", "oplatid", "hx", "hx_mean")
    pin = {n: PinnedArray(getattr(prob, n).shape, getattr(prob, n).dtype) for n in names + ("state", "mean", "sprd")}
    for n, p_ in pin.items():
        p_.array[...] = getattr(prob, n)
    outp = [PinnedArray(prob.state.shape), PinnedArray(prob.mean.shape), PinnedArray(prob.sprd.shape)]
    h2d = sum(p_.array.nbytes for p_ in pin.values())
    d2h = sum(p_.array.nbytes for p_ in outp)

    def e2e_step():
        s.set_state(pin["state"].array, pin["mean"].array, pin["sprd"].array, prob.vars)
        s.set_obs(*(pin[n].array for n in names))
        s.run()
        s.get_state(tuple(p_.array for p_ in outp))

    s.set_variant("learned")
    for _ in range(max(3, args.warmup)):
        e2e_step()
    et = []
    for _ in range(args.steps):
        s.flush_l2(256 << 20)
        t0 = time.perf_counter()
        e2e_step()
        et.append(time.perf_counter() - t0)
    for p_ in list(pin.values()) + outp:
        p_.free()
    s.close()
    ms = dist.max(statistics.mean(t["total_ms"] for t in le_t))
    ms_ex = statistics.mean(t["total_ms"] for t in ex_t)
    ms_pl = statistics.mean(t["total_ms"] for t in pl_t)
    e2e_ms = dist.max(1000.0 * statistics.mean(et))
    line = {"metric": METRIC, "value": dist.world * nact / (ms / 1000.0), "unit": UNIT, "n_gpus": dist.world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 (exact solves), bf16 x bf16 -> f32 (network)",
            "data": "synthetic (seeded generator; cycling with a zonal jet, persistent clustered network)",
            "config": dict(workload_config(args, prob, cfg), learn=cfg["learn"], cycles=cy),
            "clocks": ck, "gpu_launches": le_t[-1]["launches"] * args.steps, "variant": "learned",
            "e2e": {"value": dist.world * nact / (e2e_ms / 1000.0), "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h), "ms_per_step": e2e_ms,
                    "step_ms": [round(1000.0 * t, 3) for t in et]},
            "exact": {"variant": exact_variant, "ms_per_step": ms_ex, "value": nact / (ms_ex / 1000.0)},
            "plain_variant": {"ms_per_step": ms_pl, "value": nact / (ms_pl / 1000.0),
                              "speedup_of_headline": ms_pl / ms},
            "analysis_error": {"learned_mean_rms_over_spread": err(le), "interpolation_only": err(ip),
                               "bar": 0.01},
            "learn": dict(st, train_loss=loss, train_s=t_tr, train_rows=rows, setup_s=t_setup),
            "stages": {"learned_exact_ms": st["exact_ms"], "features_ms": st["feature_ms"],
                       "network_ms": st["network_ms"], "apply_ms": st["apply_ms"],
                       "update_ms": statistics.mean(t["update_ms"] for t in le_t)}}
    if dist.rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def single_run(args):
    """One lgpu_solver_run of the workload, for kernel profiles; prints the
    library's stage timings."""
    from letkf_gb300 import Solver
    prob, cfg = make_problem(args.workload)
    s = Solver(0)
    try:
        s.set_variant(args.variant)
        s.set_precision(args.precision)
        s.solver_init(cfg["solver"])
        s.loc_init(cfg["localization"], prob.vars, prob.lev_depth)
        s.set_problem(prob)
        s.run()
        print(json.dumps({"workload": args.workload, "timings": s.timings()}), flush=True)
    finally:
        s.close()
    return 0


def read_traffic(kernel):
    """DRAM bytes per launch of the dominant kernel from the committed ncu
    summary (profiles/<kernel>_c2.md, line 'traffic_bytes_per_launch: N')."""
    p = os.path.join(ROOT, "profiles", "%s_c2.md" % kernel)
    try:
        for line in open(p):
            if line.startswith("traffic_bytes_per_launch:"):
                return float(line.split(":", 1)[1].split()[0])
    except Exception:
        pass
    return None


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="c2")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--variant", default="auto", choices=["auto", "plain", "batched"])
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp32_resolve", "fp64"],
                    help="eigensolve precision (FP32 as the reference; FP64 re-solve of flagged units; FP64)")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain-variant comparison run")
    ap.add_argument("--single-run", action="store_true",
                    help="one analysis of --workload (no timing loop): the case profiled under ncu")
    args = ap.parse_args()
    if args.single_run:
        return single_run(args)
    dist = Dist()
    try:
        if args.impl == "reference":
            return reference_arm(args, dist)
        from letkf_gb300.workloads import WORKLOADS
        if "learn" in WORKLOADS.get(args.workload, {}):
            return learned_arm(args, dist)
        return gpu_arm(args, dist)
    finally:
        dist.close()


if __name__ == "__main__":
    sys.exit(main())
