"""GPU parity: the sm_103a engine against the CPU oracle (the reference's CPU
algorithm restated and pinned), through the C ABI.

Tolerances: plain gate-by-gate <= 1e-12 max-element error; fused <= 1e-10;
complex64 <= 1e-5 trace distance (bounded by sqrt(1-F) for pure references).
"""
import math

import numpy as np
import pytest

import dmsim_workloads as W

pytestmark = pytest.mark.gpu

NO_SRN = [o for o in range(38) if o != W.OP["SRN"]]


def run_engine(engine, n, circ, mode="plain", max_k=4, precision="fp64", init=None):
    with engine.Simulation(n, mode=mode, max_k=max_k, precision=precision) as s:
        if init is not None:
            s.set_dm(*init)
        for g in circ:
            if g[0] == 64:
                s.append_c1(g[1][0], g[5])
            elif g[0] == 65:
                s.append_c2(g[1][0], g[1][1], g[5])
            else:
                s.append(g[0], g[1], g[2], g[3], g[4])
        s.upload()
        s.run()
        return s.get_dm()


def maxerr(a, b):
    """Max element error, scaled by the entries' magnitude when it exceeds 1
    (DM-Sim's R gate is diag(1, i*theta), not unitary, so rho can grow)."""
    scale = max(1.0, np.abs(b[0]).max(), np.abs(b[1]).max())
    return max(np.abs(a[0] - b[0]).max(), np.abs(a[1] - b[1]).max()) / scale


@pytest.mark.parametrize("name", [x for x in W.OP_NAMES if x != "SRN"])
@pytest.mark.parametrize("n", [5, 7])
def test_each_gate_plain(engine, oracle, name, n):
    """One gate on a generic state, on low and high qubits, plain path."""
    op = W.OP[name]
    ar = W.ARITY[op]
    pre = W.random_circuit(n, 12, ops=[W.OP["U3"], W.OP["CX"]], seed=5)
    init = oracle.dm_sim(n, pre)
    rng = np.random.default_rng(op)
    for qs in (tuple(range(ar)), tuple(range(n - 1, n - 1 - ar, -1)), tuple(rng.choice(n, ar, replace=False))):
        circ = [W.make_gate(op, qs, rng)]
        ref = oracle.dm_sim(n, circ, *init)
        got = run_engine(engine, n, circ, init=init)
        assert maxerr(got, ref) <= 1e-12, (name, qs)


@pytest.mark.parametrize("mode,max_k", [("plain", 4), ("fused", 2), ("fused", 3), ("fused", 4)])
@pytest.mark.parametrize("n,seed", [(3, 0), (5, 1), (6, 2), (8, 3)])
def test_random_circuits(engine, oracle, mode, max_k, n, seed):
    circ = W.random_circuit(n, 80, ops=NO_SRN, seed=300 + seed)
    ref = oracle.dm_sim(n, circ)
    got = run_engine(engine, n, circ, mode, max_k)
    assert maxerr(got, ref) <= (1e-12 if mode == "plain" else 1e-10)


@pytest.mark.parametrize("mode", ["plain", "fused"])
def test_srn_circuits_reference_order(engine, oracle, mode):
    """All 38 gates, SRN included: a circuit with SRN runs in the reference's
    own forward / conjugate-transpose / forward order and matches it."""
    n = 6
    for seed in range(2):
        circ = W.random_circuit(n, 60, seed=600 + seed)
        circ.insert(3, (W.OP["SRN"], (seed,), 0.0, 0.0, 0.0))
        ref = oracle.dm_sim(n, circ)
        got = run_engine(engine, n, circ, mode)
        assert maxerr(got, ref) <= 1e-12


@pytest.mark.parametrize("n,seed", [(4, 0), (7, 1), (9, 2)])
def test_plain_double_float_option(engine, oracle, n, seed):
    """The plain method computed in double-float (DMSIM_OPT_PLAIN_ARITH) keeps
    the plain path's 1e-12 bar."""
    circ = W.random_circuit(n, 80, ops=NO_SRN, seed=800 + seed)
    ref = oracle.dm_sim(n, circ)
    with engine.Simulation(n, mode="plain", plain_arith="df64") as s:
        s.extend(circ)
        s.upload()
        s.run()
        got = s.get_dm()
    assert maxerr(got, ref) <= 1e-12


def test_c1_c2(engine, oracle):
    rng = np.random.default_rng(8)

    def ru(d):
        q, _ = np.linalg.qr(rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d)))
        return q

    n = 6
    circ = []
    for i in range(30):
        if i % 2:
            q = tuple(int(x) for x in rng.choice(n, 2, replace=False))
            circ.append((65, q, 0, 0, 0, ru(4)))
        else:
            circ.append((64, (int(rng.integers(n)),), 0, 0, 0, ru(2)))
    ref = oracle.dm_sim(n, circ)
    for mode in ("plain", "fused"):
        got = run_engine(engine, n, circ, mode)
        assert maxerr(got, ref) <= (1e-12 if mode == "plain" else 1e-10), mode


def test_chained_runs(engine, oracle):
    """run -> clear_circuit -> append -> run keeps rho on the device
    (example/adder_n10_omp.py:59-80)."""
    n = 6
    c1 = W.random_circuit(n, 40, ops=NO_SRN, seed=21)
    c2 = W.random_circuit(n, 40, ops=NO_SRN, seed=22)
    ref = oracle.dm_sim(n, c2, *oracle.dm_sim(n, c1))
    for mode in ("plain", "fused"):
        with engine.Simulation(n, mode=mode) as s:
            s.extend(c1)
            s.upload()
            s.run()
            s.clear_circuit()
            s.extend(c2)
            s.upload()
            s.run()
            got = s.get_dm()
        assert maxerr(got, ref) <= (1e-12 if mode == "plain" else 1e-10)


def test_measure_bit_exact_with_injected_uniforms(engine, oracle):
    n = 7
    circ = W.random_circuit(n, 60, ops=NO_SRN, seed=31)
    ref_re, _ = oracle.dm_sim(n, circ)
    u = oracle.libc_uniforms(4242, 500)
    with engine.Simulation(n) as s:
        s.extend(circ)
        s.upload()
        s.run()
        got = s.measure(500, u)
        re, _ = s.get_dm()
    # same sampling algorithm given the same diagonal: identical outcomes
    mine, _ = oracle.measure(n, re, u)
    assert got == [int(x) for x in mine]
    # and against the oracle's own diagonal (agrees to 1e-12, so outcomes match
    # unless a draw lands within 1e-12 of a bucket edge)
    theirs, _ = oracle.measure(n, ref_re, u)
    assert got == [int(x) for x in theirs]


def test_adder_known_answer(engine):
    """README.md:228-247: every shot of the 10-qubit adder reads 1000000010."""
    import libdmsim_py_nvgpu_omp as dm
    sim = dm.Simulation(10, 1)
    for q in (1, 5, 6, 7, 8):
        sim.append(sim.X(q))
    sim.upload()
    sim.run()
    sim.clear_circuit()

    def maj(a, b, c):
        sim.append(sim.CX(c, b)); sim.append(sim.CX(c, a)); sim.append(sim.CCX(a, b, c))

    def unmaj(a, b, c):
        sim.append(sim.CCX(a, b, c)); sim.append(sim.CX(c, a)); sim.append(sim.CX(a, b))

    maj(0, 5, 1); maj(1, 6, 2); maj(2, 7, 3); maj(3, 8, 4)
    sim.append(sim.CX(4, 9))
    unmaj(3, 8, 4); unmaj(2, 7, 3); unmaj(1, 6, 2); unmaj(0, 5, 1)
    sim.upload()
    sim.run()
    res = sim.measure(10)
    assert res == [0b1000000010] * 10


def test_layered_10q_vs_oracle(engine, oracle):
    """The 10-qubit layered U3+CX workload, 200 gates: rho and diagonal <= 1e-12."""
    n = 10
    circ = W.layered_u3_cx(n, 200)
    ref = oracle.dm_sim(n, circ)
    got = run_engine(engine, n, circ)
    assert maxerr(got, ref) <= 1e-12
    d = 1 << n
    assert np.abs(got[0].reshape(d, d).diagonal() - ref[0].reshape(d, d).diagonal()).max() <= 1e-12
    fused = run_engine(engine, n, circ, "fused")
    assert maxerr(fused, ref) <= 1e-10


def test_pure_state_metrics_full_size(engine, oracle):
    """12 qubits, mixed table: plain and fused against the statevector oracle on
    the device (fidelity, trace, max element error)."""
    n = 12
    circ = W.table_mix(n, 300, seed=41)
    sr, si = oracle.sv_sim(n, circ)
    psi = sr + 1j * si
    for mode, tol in (("plain", 1e-12), ("fused", 1e-10)):
        with engine.Simulation(n, mode=mode) as s:
            s.extend(circ)
            s.upload()
            s.run()
            m = s.pure_metrics(psi)
        assert m["max_abs_err"] <= tol, (mode, m)
        assert abs(m["trace"] - 1) <= 1e-10
        assert abs(m["fidelity"] - 1) <= 1e-10


def test_complex64_mode(engine, oracle):
    n = 9
    circ = W.u3_cx_ccx(n, 200, seed=51)
    sr, si = oracle.sv_sim(n, circ)
    psi = sr + 1j * si
    for mode in ("plain", "fused"):
        with engine.Simulation(n, mode=mode, precision="c64") as s:
            s.extend(circ)
            s.upload()
            s.run()
            m = s.pure_metrics(psi)
        td_bound = math.sqrt(max(0.0, 1 - m["fidelity"]))
        assert td_bound <= 1e-5 or m["frob_err"] <= 1e-5, (mode, m)


def test_errors_are_status_codes(engine):
    with engine.Simulation(3) as s:
        with pytest.raises(engine.DMSimError) as e:
            s.append(W.OP["CX"], (0, 3))
        assert e.value.status == engine.ERR_ARG
        with pytest.raises(engine.DMSimError) as e:
            s.run()
        assert e.value.status == engine.ERR_STATE
        s.append(W.OP["H"], (0,))
        s.upload()
        with pytest.raises(engine.DMSimError) as e:
            s.upload()
        assert e.value.status == engine.ERR_STATE
        s.run()
        s.reset()
        re, im = s.get_dm()
        assert re[0] == 1 and np.count_nonzero(re) == 1 and np.count_nonzero(im) == 0
