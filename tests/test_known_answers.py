"""Known answers from the reference's own tests, checked exactly on the
density matrix (no shot noise): the deuteron ansatz's 20-point <X0 X1> curve
(xacc/tests/DmSimCpuAcceleratorTester.cpp:20-49), the RX / controlled-RZ /
U3(theta, -pi/2, pi/2) <Z> curves (xacc/nvidia_omp/tests/
DmSimAcceleratorTester.cpp:69-151), <Z> of H, X, XX (:29-67), the Bell state
(:8-27) and the deterministic shot tests (xacc/tests/
DmSimCpuAcceleratorTester.cpp:51-108).  The oracle is checked on the CPU,
the engine on the GPU in plain and fused modes."""
import math

import numpy as np
import pytest

import dmsim_workloads as W

OP = W.OP
ANGLES = np.linspace(-math.pi, math.pi, 20)
# reference: expected results of the deuteron ansatz (6 printed digits)
DEUTERON = [0.0, -0.324699, -0.614213, -0.837166, -0.9694, -0.996584, -0.915773, -0.735724, -0.475947, -0.164595,
            0.164595, 0.475947, 0.735724, 0.915773, 0.996584, 0.9694, 0.837166, 0.614213, 0.324699, 0.0]


def g(name, qubits, theta=0.0, phi=0.0, lam=0.0):
    return (OP[name], tuple(qubits), theta, phi, lam)


def deuteron(t):
    # X(q0); Ry(q1, t); CX(q1, q0); H(q0); H(q1): parity of the two qubits
    return 2, [g("X", [0]), g("RY", [1], theta=t), g("CX", [1, 0]), g("H", [0]), g("H", [1])]


def expect_z(diag, n, qubits):
    idx = np.arange(1 << n)
    sign = np.ones(1 << n)
    for q in qubits:
        sign *= 1 - 2 * ((idx >> q) & 1)
    return float(np.dot(diag, sign))


CASES = (
    [("deuteron", t, deuteron(t), [0, 1], DEUTERON[i], 1e-6) for i, t in enumerate(ANGLES)]
    + [("rx", t, (1, [g("RX", [0], theta=t)]), [0], math.cos(t), 1e-12) for t in ANGLES]
    + [("crz", t, (2, [g("X", [0]), g("H", [1]), g("CRZ", [0, 1], lam=t), g("H", [1])]), [1], math.cos(t), 1e-12)
       for t in ANGLES]
    + [("u3", t, (1, [g("U3", [0], theta=t, phi=-math.pi / 2, lam=math.pi / 2)]), [0], math.cos(t), 1e-12)
       for t in ANGLES]
    + [("h", 0, (1, [g("H", [0])]), [0], 0.0, 1e-12), ("x", 0, (1, [g("X", [0])]), [0], -1.0, 1e-12),
       ("xx", 0, (1, [g("X", [0]), g("X", [0])]), [0], 1.0, 1e-12)]
)


def diag_of(re, n):
    d = 1 << n
    return re.reshape(d, d).diagonal().copy()


def test_oracle_known_answers(oracle):
    for name, t, (n, circ), qubits, want, tol in CASES:
        re, _ = oracle.dm_sim(n, circ)
        got = expect_z(diag_of(re, n), n, qubits)
        assert abs(got - want) <= tol, (name, t, got, want)


def test_oracle_bell_and_deterministic_states(oracle):
    # nothing: |00>; X0 CX01: |11>; H0 CX01: (|00> + |11>)/sqrt2
    for circ, want in (([], [1, 0, 0, 0]), ([g("X", [0]), g("CX", [0, 1])], [0, 0, 0, 1]),
                       ([g("H", [0]), g("CX", [0, 1])], [0.5, 0, 0, 0.5])):
        re, _ = oracle.dm_sim(2, circ)
        assert np.abs(diag_of(re, 2) - want).max() <= 1e-15


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["plain", "fused"])
def test_engine_known_answers(engine, mode):
    for name, t, (n, circ), qubits, want, tol in CASES:
        with engine.Simulation(n, mode=mode) as s:
            s.extend(circ)
            s.upload()
            s.run()
            got = expect_z(s.get_diag(), n, qubits)
        assert abs(got - want) <= max(tol, 1e-12), (mode, name, t, got, want)


@pytest.mark.gpu
def test_engine_deterministic_shots(engine):
    """Every shot of |11> is 3 and of |00> is 0; the Bell state gives only 0 and 3."""
    for circ, allowed in (([], {0}), ([g("X", [0]), g("CX", [0, 1])], {3}), ([g("H", [0]), g("CX", [0, 1])], {0, 3})):
        with engine.Simulation(2, mode="plain") as s:
            s.extend(circ)
            s.upload()
            s.run()
            shots = s.measure(100)
        assert set(int(x) for x in shots) <= allowed, (circ, shots)
