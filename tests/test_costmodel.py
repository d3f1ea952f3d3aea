"""The learned pass-time model: its forward and backward kernels against a
numpy reference (gradient check), its training on timings the engine records
itself, and what the learned planner gains over the fixed-width greedy one."""
import numpy as np
import pytest

import dmsim_workloads as W

I, H = 17, 32
NP = H * I + H + H * H + H + H + 1  # network parameters


def unpack(p):
    o = 0
    W1 = p[o:o + H * I].reshape(H, I); o += H * I
    b1 = p[o:o + H]; o += H
    W2 = p[o:o + H * H].reshape(H, H); o += H * H
    b2 = p[o:o + H]; o += H
    W3 = p[o:o + H]; o += H
    b3 = p[o]
    return W1, b1, W2, b2, W3, b3


def np_forward(p, X):
    W1, b1, W2, b2, W3, b3 = unpack(p.astype(np.float64))
    a1 = np.maximum(X @ W1.T + b1, 0)
    a2 = np.maximum(a1 @ W2.T + b2, 0)
    return a2 @ W3 + b3, a1, a2


def np_grad(p, X, T):
    """d(mean (y - T)^2)/d(params), in float64: the CPU reference of the backward kernel."""
    W1, b1, W2, b2, W3, b3 = unpack(p.astype(np.float64))
    y, a1, a2 = np_forward(p, X)
    B = len(X)
    r = y - T
    dy = 2 * r / B
    gW3 = a2.T @ dy
    gb3 = dy.sum()
    d2 = np.outer(dy, W3) * (a2 > 0)
    gW2 = d2.T @ a1
    gb2 = d2.sum(0)
    d1 = (d2 @ W2) * (a1 > 0)
    gW1 = d1.T @ X
    gb1 = d1.sum(0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3, [gb3]])
    return g, float((r ** 2).mean())


def test_numpy_reference_gradient_is_a_gradient():
    """Finite differences pin the numpy reference itself (CPU)."""
    rng = np.random.default_rng(0)
    p = rng.normal(size=NP) * 0.2
    X = rng.random((7, I))
    T = rng.normal(size=7)
    g, _ = np_grad(p, X, T)
    for idx in rng.choice(NP, 25, replace=False):
        e = np.zeros(NP)
        e[idx] = 1e-6
        num = (np_grad(p + e, X, T)[1] - np_grad(p - e, X, T)[1]) / 2e-6
        assert abs(num - g[idx]) <= 1e-5 * max(1.0, abs(g[idx]))


@pytest.mark.gpu
def test_gpu_forward_and_gradient_match_cpu(engine):
    rng = np.random.default_rng(1)
    p = (rng.normal(size=NP) * 0.3).astype(np.float32)
    X = rng.random((1000, I)).astype(np.float32)
    T = rng.normal(size=1000).astype(np.float32)
    y = engine.mlp_forward(p, X)
    yr, _, _ = np_forward(p, X.astype(np.float64))
    assert np.abs(y - yr).max() <= 1e-4 * max(1.0, np.abs(yr).max())
    g, loss = engine.mlp_grad(p, X, T)
    gr, lr = np_grad(p, X.astype(np.float64), T.astype(np.float64))
    assert abs(loss - lr) <= 1e-4 * max(1.0, lr)
    assert np.abs(g - gr).max() <= 1e-4 * max(1.0, np.abs(gr).max())


@pytest.mark.gpu
def test_collect_train_predict(engine, tmp_path):
    feats, ms = engine.cost_collect(10, n_circuits=2, gates=40, seed=3)
    assert len(ms) > 100 and np.all(ms > 0)
    loss = engine.cost_train(feats, ms, steps=1500, lr=3e-3, seed=1)
    assert loss[1] < loss[0] and loss[1] < 0.5
    pred = engine.cost_predict(feats)
    rel = np.abs(np.log(pred) - np.log(ms))
    assert np.median(rel) < 0.5
    path = str(tmp_path / "m.bin")
    engine.cost_save(path)
    engine.cost_load(path)
    assert np.allclose(engine.cost_predict(feats[:10]), pred[:10], rtol=1e-5)


@pytest.mark.gpu
def test_learned_planner_vs_fixed_width_greedy(engine, oracle):
    """Train on the engine's own FP64 timings (pipe kernels and FP64-width
    tensor passes), then plan a 12-qubit mixed-table circuit with the learned
    planner and with the greedy k<=4 planner: both match the oracle and the
    learned plan is no slower than the fixed rule (measured).  On GB300 the
    fixed rule -- widest fusion, tensor cores for every dense 3/4-qubit block
    -- is within a few percent of every plan the learned planner scores."""
    n = 12
    feats, ms = [], []
    for seed, nn in ((11, 10), (12, 12)):
        f, m = engine.cost_collect(nn, n_circuits=2, gates=60, seed=seed, arith=engine.AR_FP64)
        feats.append(f)
        ms.append(m)
    engine.cost_train(np.concatenate(feats), np.concatenate(ms), steps=3000, lr=3e-3, seed=2)
    try:
        circ = W.table_mix(n, 300, seed=77)
        times = {}
        states = {}
        for planner in ("greedy", "learned"):
            with engine.Simulation(n, mode="fused", planner=planner) as s:
                s.extend(circ)
                s.upload()
                s.run()
                t = []
                for _ in range(3):
                    s.reset_dm()
                    s.run()
                    t.append(s.last_timings()["ms"])
                times[planner] = min(t)
                states[planner] = s.get_dm()
        ref = oracle.dm_sim(n, circ)
        for st in states.values():
            assert max(np.abs(st[0] - ref[0]).max(), np.abs(st[1] - ref[1]).max()) <= 1e-12
        assert times["learned"] <= times["greedy"] * 1.05, times
    finally:
        engine.cost_load_default()


@pytest.mark.gpu
@pytest.mark.slow
def test_shipped_model_gain_double_float_14q(engine):
    """The shipped model on the 14-qubit mixed-table workload in double-float
    arithmetic, where the fixed density rule sends some sparse 4-qubit blocks
    to the wrong unit: the learned plan is measured faster than the greedy one
    (3.5% when the model was trained: 3.47 s against 3.59 s)."""
    n = 14
    circ = W.table_mix(n, 2000, seed=2)
    times = {}
    for planner in ("greedy", "learned"):
        with engine.Simulation(n, mode="fused", planner=planner, fused_arith="df64") as s:
            s.extend(circ)
            s.upload()
            s.run()
            t = []
            for _ in range(2):
                s.run()
                t.append(s.last_timings()["ms"])
            times[planner] = min(t)
    assert times["learned"] <= times["greedy"] * 0.99, times
