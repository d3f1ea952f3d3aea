"""FP64-width tensor-core passes (tensor64.cu: FP64 state, 7 BF16 digits per
operand, exact order sums, integer combination, one rounding to FP64):
parity with the CPU oracle, with the FP64-pipe fused passes and with the
plain path, at sizes from one tile to many tiles per block."""
import numpy as np
import pytest

import dmsim_workloads as W

pytestmark = pytest.mark.gpu


def run(engine, n, circ, mode="fused", tensor="all", planner="greedy", max_k=4, arith="fp64"):
    with engine.Simulation(n, mode=mode, max_k=max_k, planner=planner, tensor=tensor, fused_arith=arith,
                           plain_arith=arith) as s:
        s.extend(circ)
        s.upload()
        s.set_option(engine.OPT_RECORD, 1)
        s.run()
        rec = s.pass_records()
        re, im = s.get_dm()
    return re, im, rec


def maxerr(a, b):
    return max(np.abs(a[0] - b[0]).max(), np.abs(a[1] - b[1]).max())


@pytest.mark.parametrize("n,seed,max_k", [(5, 1, 3), (6, 2, 4), (7, 3, 4), (8, 4, 3), (8, 5, 4)])
def test_fp64_tensor_passes_match_oracle(engine, oracle, n, seed, max_k):
    """Every eligible 3/4-qubit pass on the FP64-width tensor kernel; the
    reference CPU engine's result to 1e-12 (the plain path's tolerance)."""
    circ = W.table_mix(n, 150, seed=seed)
    re, im, rec = run(engine, n, circ, max_k=max_k)
    assert rec[:, 8].sum() > 0, "no pass ran on the tensor cores"
    assert (rec[:, 1] != 16).all(), "an FP64 run converts nothing"
    ref = oracle.dm_sim(n, circ)
    scale = max(1.0, np.abs(ref[0]).max())
    assert maxerr((re, im), ref) <= 1e-12 * scale


@pytest.mark.parametrize("n", [10, 12])
def test_fp64_tensor_passes_match_fp64_pipe_passes(engine, n):
    """The same fused plan with its dense passes on the tensor cores and on
    GB300's FP64 pipe: both FP64-width, within 1e-13."""
    circ = W.layered_u3_cx(n, 160, seed=21)
    a = run(engine, n, circ, tensor="all")
    b = run(engine, n, circ, tensor=0)
    assert a[2][:, 8].sum() > 0 and b[2][:, 8].sum() == 0
    assert maxerr(a[:2], b[:2]) <= 1e-13


def test_fp64_tensor_fused_vs_plain_14q_sample(engine, oracle):
    """A 13-qubit mixed-gate circuit (2^26 entries, hundreds of tiles per
    block): the FP64-width fused run against the plain FP64 path, on the
    device; and the statevector oracle's fidelity."""
    n = 13
    circ = W.table_mix(n, 300, seed=17)
    sr, si = oracle.sv_sim(n, circ)
    with engine.Simulation(n, mode="fused", tensor=True, fused_arith="fp64") as f, \
            engine.Simulation(n, mode="plain", plain_arith="fp64") as p:
        for s in (f, p):
            s.extend(circ)
            s.upload()
            s.run()
        d = f.compare(p)
        m = f.pure_metrics(sr + 1j * si)
    assert d["max_abs_err"] <= 1e-13, d
    assert abs(1 - m["fidelity"]) <= 1e-12 and m["max_abs_err"] <= 1e-13, m
