"""Tensor-core passes (3- and 4-qubit dense operators, BF16 slices with exact
FP32 sums, double-float recombination): parity with the FP32-pipe
double-float kernels, with the plain FP64 path and with the CPU oracle."""
import numpy as np
import pytest

import dmsim_workloads as W

pytestmark = pytest.mark.gpu


def run_fused(engine, n, circ, tensor, max_k=4, planner="greedy"):
    with engine.Simulation(n, mode="fused", max_k=max_k, planner=planner, tensor=tensor) as s:
        s.extend(circ)
        s.upload()
        s.set_option(engine.OPT_RECORD, 1)
        s.run()
        rec = s.pass_records()
        re, im = s.get_dm()
    return re, im, rec


def maxerr(a, b):
    return max(np.abs(a[0] - b[0]).max(), np.abs(a[1] - b[1]).max())


@pytest.mark.parametrize("n,seed", [(6, 1), (7, 2), (8, 3)])
def test_all_eligible_passes_on_tensor_cores_match_oracle(engine, oracle, n, seed):
    circ = W.table_mix(n, 120, seed=seed)
    re, im, rec = run_fused(engine, n, circ, tensor="all")
    assert rec[:, 8].sum() > 0, "no pass ran on the tensor cores"
    ref = oracle.dm_sim(n, circ)
    scale = max(1.0, np.abs(ref[0]).max())
    assert maxerr((re, im), ref) <= 1e-10 * scale


@pytest.mark.parametrize("max_k", [3, 4])
def test_tensor_matches_fp32_pipe_kernels(engine, max_k):
    n = 9
    circ = W.layered_u3_cx(n, 200, seed=11)
    a = run_fused(engine, n, circ, tensor="all", max_k=max_k)
    b = run_fused(engine, n, circ, tensor=0, max_k=max_k)
    assert a[2][:, 8].sum() > 0 and b[2][:, 8].sum() == 0
    assert maxerr(a[:2], b[:2]) <= 1e-10


def test_dense_two_qubit_blocks_vs_plain(engine):
    """Random dense C2 unitaries fuse into dense 4-qubit blocks."""
    n = 10
    rng = np.random.default_rng(7)
    with engine.Simulation(n, mode="plain") as p, engine.Simulation(n, mode="fused", tensor="all") as f:
        for _ in range(80):
            q = rng.choice(n, 2, replace=False)
            A = rng.normal(size=(4, 4)) + 1j * rng.normal(size=(4, 4))
            U, _ = np.linalg.qr(A)
            p.append_c2(int(q[0]), int(q[1]), U)
            f.append_c2(int(q[0]), int(q[1]), U)
        p.upload()
        f.upload()
        f.set_option(engine.OPT_RECORD, 1)
        p.run()
        f.run()
        assert f.pass_records()[:, 8].sum() > 0
        err = f.compare(p)
    assert err["max_abs_err"] <= 1e-10, err


def test_tensor_twelve_qubits_vs_plain(engine):
    n = 12
    circ = W.table_mix(n, 300, seed=21)
    with engine.Simulation(n, mode="plain") as p, engine.Simulation(n, mode="fused", tensor="all") as f:
        p.extend(circ)
        f.extend(circ)
        p.upload()
        f.upload()
        p.run()
        f.run()
        err = f.compare(p)
    assert err["max_abs_err"] <= 1e-10, err


def test_chained_runs_and_small_states(engine, oracle):
    """n = 5 (4-qubit passes fall back, 3-qubit ones are eligible) and a
    second run on the resident state."""
    n = 5
    circ = W.table_mix(n, 60, seed=4)
    with engine.Simulation(n, mode="fused", tensor="all") as s:
        s.extend(circ)
        s.upload()
        s.run()
        s.run()
        re, im = s.get_dm()
    r1 = oracle.dm_sim(n, circ)
    ref = oracle.dm_sim(n, circ + circ)
    assert maxerr((re, im), ref) <= 1e-10 * max(1.0, np.abs(r1[0]).max())


def test_complex64_tensor_passes(engine):
    """complex64 (FP32 state, 3 BF16 slices per operand): the tensor-core
    passes are as accurate as the FP32-pipe ones against an FP64 run."""
    n = 10
    circ = W.u3_cx_ccx(n, 300, seed=3)
    errs = {}
    with engine.Simulation(n, mode="plain") as ref:
        ref.extend(circ)
        ref.upload()
        ref.run()
        for tensor in (0, "all"):
            with engine.Simulation(n, mode="fused", precision="c64", tensor=tensor) as s:
                s.extend(circ)
                s.upload()
                s.set_option(engine.OPT_RECORD, 1)
                s.run()
                ran_tc = s.pass_records()[:, 8].sum() > 0
                errs[tensor] = (s.compare(ref)["max_abs_err"], ran_tc)
    assert errs["all"][1] and not errs[0][1]
    assert errs["all"][0] <= 1e-5 and errs[0][0] <= 1e-5, errs
    assert errs["all"][0] <= 4 * errs[0][0] + 1e-7, errs


@pytest.mark.parametrize("max_k", [3, 4])
def test_complex64_tensor_kernel_12q(engine, max_k):
    """The complex64 tensor-core kernel (tensor32.cu: 3 true-scale BF16 slices,
    exact FP32 order sums) at 12 qubits, every 3- or 4-qubit pass on it:
    against an FP64 run of the same circuit, at the FP32-pipe passes' error
    level (complex64: tolerance 1e-5 max element)."""
    n = 12
    circ = W.u3_cx_ccx(n, 400, seed=21)
    errs = {}
    with engine.Simulation(n, mode="fused", max_k=max_k) as ref:
        ref.extend(circ)
        ref.upload()
        ref.run()
        for tensor in (0, "all"):
            with engine.Simulation(n, mode="fused", max_k=max_k, precision="c64", tensor=tensor) as s:
                s.extend(circ)
                s.upload()
                s.set_option(engine.OPT_RECORD, 1)
                s.run()
                rec = s.pass_records()
                ntc = int(rec[:, 8].sum())
                widths = set(int(k) for k in rec[rec[:, 8] > 0, 0])
                errs[tensor] = (s.compare(ref)["max_abs_err"], ntc, widths)
    assert errs[0][1] == 0 and errs["all"][1] > 0, errs
    assert max_k in errs["all"][2], errs
    assert errs["all"][0] <= 1e-5 and errs[0][0] <= 1e-5, errs
    assert errs["all"][0] <= 4 * errs[0][0] + 1e-7, errs


@pytest.mark.parametrize("n,seed", [(6, 5), (8, 6)])
def test_complex64_tensor_kernel_vs_oracle(engine, oracle, n, seed):
    """complex64 state, every eligible pass on the complex64 tensor kernel,
    against the CPU oracle (FP64) on the mixed-gate table: within complex64
    accuracy."""
    circ = W.table_mix(n, 150, seed=seed)
    with engine.Simulation(n, mode="fused", precision="c64", tensor="all") as s:
        s.extend(circ)
        s.upload()
        s.set_option(engine.OPT_RECORD, 1)
        s.run()
        assert s.pass_records()[:, 8].sum() > 0
        re, im = s.get_dm()
    ref = oracle.dm_sim(n, circ)
    assert maxerr((re, im), ref) <= 2e-5 * max(1.0, np.abs(ref[0]).max())
