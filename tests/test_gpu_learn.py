"""GPU: the learned analysis form (no counterpart in the reference, which
solves every column exactly).

(1) The network kernels against the numpy oracle (oracle/mlp_oracle.py):
    loss, CUDA-core forward, tensor-core forward, gradient of every parameter
    tensor.  Bars (relative L2): outputs 3e-3 (BF16 hidden activations can
    round differently where FP32 and FP64 pre-activations straddle a BF16
    rounding boundary), gradients 1e-2, loss 1e-3.
(2) A cycling experiment on a reduced grid of the learned workload (1-degree
    lattice, k = 32, clustered observations, 400 km localisation, coarse
    stride 2): the network is trained on exact analyses of cycles 0-4; on
    cycle 5 the learned analysis is compared with the exact one and with the
    interpolation alone (the method without the network), by the RMS of the
    analysis-mean difference over the background spread.
"""
import numpy as np
import pytest

from oracle import mlp_oracle as M

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


@pytest.mark.parametrize("din,hidden,dout,rows", [(40, 64, 36, 300), (1072, 512, 1056, 256)])
def test_network_against_oracle(din, hidden, dout, rows):
    from letkf_gb300 import mlp_debug, mlp_param_shapes
    rng = np.random.default_rng(din + rows)
    parts = []
    for s in mlp_param_shapes(din, hidden, dout):
        if len(s) == 2:
            a = np.sqrt(6.0 / (s[0] + s[1]))
            parts.append(rng.uniform(-a, a, size=s).ravel())
        else:
            parts.append(0.1 * rng.standard_normal(s))
    p = np.concatenate(parts).astype(np.float32)
    x = rng.standard_normal((rows, din)).astype(np.float32)
    t = rng.standard_normal((rows, dout)).astype(np.float32)
    g = mlp_debug(p, x, t, hidden=hidden)
    loss, grad, y = M.loss_grad(p, x, t, hidden, dout)
    assert rel(g["y_simt"], y) <= 3e-3
    assert rel(g["y_tc"], y) <= 3e-3
    assert abs(g["loss"] - loss) <= 1e-3 * loss
    o = 0
    for s in mlp_param_shapes(din, hidden, dout):
        n = int(np.prod(s))
        assert rel(g["grad"][o:o + n], grad[o:o + n]) <= 1e-2, (s, rel(g["grad"][o:o + n], grad[o:o + n]))
        o += n


def _cycle_problem(cycle, base=None, ana=None):
    """Background of `cycle`: the reduced learned workload's first background
    for cycle 0, else the forecast of the previous analysis; observations of
    the persistent clustered network drawn anew every cycle."""
    from letkf_gb300 import synth
    if base is None:
        p = synth.generate("c3", nx=360, ny=180, nz=5, n_obs=40000, k=32)
    else:
        p = base
        x, m, s = ana
        p.state[...] = x - m[:, :, None]
        p.mean[...] = m
        p.sprd[...] = s
        synth.forecast(p)
    return synth.observe(p, seed=1000 + cycle, n_obs=40000)


LOC = {"class": "loc_novrt", "hzloc": {"type": "linearinterp_lat", "value": [{"lat": 0.0, "radius": 400.0e3}]}}


def test_learned_form_cycling():
    from letkf_gb300 import Solver
    s = Solver(0)
    try:
        s.solver_init({})
        p = _cycle_problem(0)
        s.loc_init(LOC, p.vars)
        s.set_variant("plain")
        s.set_problem(p)
        s.learn_init(p.nx, p.ny, stride=2, hidden=512, judge_frac=0.05, gate_frac=0.05, sample_frac=1.0,
                     train_cap=300000, seed=5)
        # cycles 0-4: exact analyses, collected
        for c in range(5):
            if c > 0:
                p = _cycle_problem(c, p, ana)
                s.set_problem(p)
            s.set_variant("plain")
            s.learn_collect()
            ana = s.get_state()
        first = s.learn_train(epochs=1, batch=512, lr=1e-3)
        loss = s.learn_train(epochs=29, batch=512, lr=1e-3)
        assert np.isfinite(loss) and loss < 0.6 * first
        # cycle 5 (not trained on): exact, learned, interpolation only
        p = _cycle_problem(5, p, ana)
        s.set_problem(p)
        s.set_variant("plain")
        s.run()
        ex = s.get_state()
        s.set_variant("learned")
        s.learn_set_network(True)
        s.run()
        le = s.get_state()
        st = s.learn_stats()
        s.learn_set_network(False)
        s.run()
        ip = s.get_state()
        s.learn_set_network(True)
        # the exact solves of the learned form in FP64: every one counted
        s.set_precision("fp64")
        s.run()
        le64 = s.get_state()
        st64, t64 = s.learn_stats(), s.timings()
        s.set_precision("fp32")
    finally:
        s.close()
    act = p.mask == 0
    spread = float(np.sqrt(np.mean(p.sprd[act] ** 2)))
    err_l = float(np.sqrt(np.mean((le[1][act] - ex[1][act]) ** 2))) / spread
    err_i = float(np.sqrt(np.mean((ip[1][act] - ex[1][act]) ** 2))) / spread
    print("learned", err_l, "interpolation", err_i, st)
    assert st["inferred"] > 0.5 * (st["inferred"] + st["gated"] + st["coarse"] + st["judged"] + st["fallback"])
    assert st["judged"] > 0 and st["judge_rms"] > 0.0
    # the network improves on the interpolation alone (measured 1.15% against
    # 1.36% of the background spread at 60 epochs, 1.23% at 25)
    assert err_l < 0.97 * err_i
    assert err_l <= 0.02
    assert t64["precision"] == 2
    assert t64["fp64_units"] == st64["coarse"] + st64["judged"] + st64["fallback"] + st64["gated"]
    assert np.all(np.isfinite(le64[0])) and np.all(np.isfinite(le64[1]))
    err_64 = float(np.sqrt(np.mean((le64[1][act] - ex[1][act]) ** 2))) / spread
    assert err_64 <= 0.02
