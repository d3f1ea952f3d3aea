"""Noise channels (no counterpart in the reference): rho -> sum K rho K^+ as a
superoperator pass, against a numpy Kraus reference for the channel steps and
the oracle for the gate segments in between."""
import numpy as np
import pytest

import dmsim_workloads as W

NO_SRN = [o for o in range(38) if o not in (W.OP["SRN"], W.OP["R"])]
I2 = np.eye(2)
X = np.array([[0, 1], [1, 0]], complex)
Y = np.array([[0, -1j], [1j, 0]])
Z = np.diag([1.0, -1.0]).astype(complex)


def kraus_of(kind, p):
    if kind == "depolarizing":
        return [np.sqrt(1 - 3 * p / 4) * I2, np.sqrt(p / 4) * X, np.sqrt(p / 4) * Y, np.sqrt(p / 4) * Z]
    if kind == "amplitude_damping":
        return [np.array([[1, 0], [0, np.sqrt(1 - p)]]), np.array([[0, np.sqrt(p)], [0, 0]])]
    if kind == "phase_damping":
        return [np.array([[1, 0], [0, np.sqrt(1 - p)]]), np.array([[0, 0], [0, np.sqrt(p)]])]
    if kind == "bit_flip":
        return [np.sqrt(1 - p) * I2, np.sqrt(p) * X]
    if kind == "phase_flip":
        return [np.sqrt(1 - p) * I2, np.sqrt(p) * Z]
    if kind == "depolarizing2":
        P = [I2, X, Y, Z]
        return [np.sqrt((1 - 15 * p / 16) if (i == 0 and j == 0) else p / 16) * np.kron(P[i], P[j])
                for i in range(4) for j in range(4)]
    raise ValueError(kind)


def embed(m, qubits, n):
    """Full 2^n operator of m on qubits (2-qubit m in the index 2*bit(q0)+bit(q1) order)."""
    d = 1 << n
    k = len(qubits)
    full = np.zeros((d, d), complex)
    for col in range(d):
        ci = 0
        for t, q in enumerate(qubits):
            ci |= ((col >> q) & 1) << (k - 1 - t)
        for ri in range(1 << k):
            row = col
            for t, q in enumerate(qubits):
                bit = (ri >> (k - 1 - t)) & 1
                row = (row & ~(1 << q)) | (bit << q)
            full[row, col] += m[ri, ci]
    return full


def reference(oracle, n, program):
    """program: list of ('gates', circuit) and ('chan', qubits, kraus) steps."""
    d = 1 << n
    re, im = oracle.zero_state(n)
    for step in program:
        if step[0] == "gates":
            re, im = oracle.dm_sim(n, step[1], re, im)
        else:
            rho = oracle.rho_from_result(n, re, im)
            out = sum(embed(K, step[1], n) @ rho @ embed(K, step[1], n).conj().T for K in step[2])
            A = out.T  # back to the dm_real_res layout
            re, im = np.ascontiguousarray(A.real).ravel(), np.ascontiguousarray(A.imag).ravel()
    return oracle.rho_from_result(n, re, im)


def build_program(n, seed):
    rng = np.random.default_rng(seed)
    kinds = ["depolarizing", "amplitude_damping", "phase_damping", "bit_flip", "phase_flip", "depolarizing2"]
    prog = []
    for i in range(6):
        prog.append(("gates", W.random_circuit(n, 8, ops=NO_SRN, seed=seed * 100 + i)))
        kind = kinds[i % len(kinds)]
        qs = [int(x) for x in rng.choice(n, 2 if kind == "depolarizing2" else 1, replace=False)]
        prog.append(("chan", qs, kraus_of(kind, float(rng.uniform(0.05, 0.4))), kind))
    return prog


def test_channel_planning_is_a_barrier(engine):
    """Host side: a channel is its own SUPER pass between fused groups."""
    # plan_inspect takes gates only; the channel path is covered on the GPU below
    p = engine.plan_inspect(4, [(W.OP["H"], (0,), 0, 0, 0)], mode="fused")
    assert p[0]["cls"] in ("DENSE",)
    assert "SUPER" in engine.CLASS_NAMES


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["plain", "fused"])
@pytest.mark.parametrize("seed", [1, 2])
def test_channels_match_kraus_reference(engine, oracle, mode, seed):
    n = 5
    prog = build_program(n, seed)
    ref = reference(oracle, n, prog)
    with engine.Simulation(n, mode=mode) as s:
        for step in prog:
            if step[0] == "gates":
                s.extend(step[1])
            elif step[3] in ("depolarizing", "depolarizing2") and seed == 1:
                s.append_noise(step[3], step[1], _p_of(step))
            else:
                s.append_channel(step[1], step[2])
        s.upload()
        s.run()
        rho = s.rho()
    tol = 1e-12 if mode == "plain" else 1e-10
    assert np.abs(rho - ref).max() <= tol
    assert abs(np.trace(rho).real - 1) <= 1e-12


def _p_of(step):
    # recover p from the identity Kraus weight of the depolarizing channels
    k0 = step[2][0]
    w = abs(k0[0, 0]) ** 2
    return (1 - w) * 4 / 3 if step[3] == "depolarizing" else (1 - w) * 16 / 15


@pytest.mark.gpu
def test_depolarizing_drives_to_maximally_mixed(engine):
    n = 3
    with engine.Simulation(n) as s:
        s.append(W.OP["H"], (0,))
        for q in range(n):
            s.append_noise("depolarizing", (q,), 1.0)
        s.upload()
        s.run()
        rho = s.rho()
    assert np.abs(rho - np.eye(8) / 8).max() <= 1e-14
