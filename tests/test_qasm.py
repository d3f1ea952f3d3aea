"""OpenQASM 2 frontend: programs parse into the engine's gate stream with
DM-Sim's semantics (checked against the oracle), errors are reported, and a
parsed program runs on the GPU."""
import math

import numpy as np
import pytest

import dmsim_qasm as Q
import dmsim_workloads as W

ADDER = """
OPENQASM 2.0;
include "qelib1.inc";
// ripple-carry adder (Cuccaro et al.): carry-in q0, A = q[1..4], B = q[5..8], carry-out q9
gate majority a,b,c { cx c,b; cx c,a; ccx a,b,c; }
gate unmaj a,b,c { ccx a,b,c; cx c,a; cx a,b; }
qreg q[10];
creg m[10];
x q[1]; x q[5]; x q[6]; x q[7]; x q[8];
majority q[0],q[5],q[1];
majority q[1],q[6],q[2];
majority q[2],q[7],q[3];
majority q[3],q[8],q[4];
cx q[4],q[9];
unmaj q[3],q[8],q[4];
unmaj q[2],q[7],q[3];
unmaj q[1],q[6],q[2];
unmaj q[0],q[5],q[1];
measure q -> m;
"""


def test_adder_program_known_answer(oracle):
    n, circ, measured = Q.parse_qasm(ADDER)
    assert n == 10 and measured == list(range(10))
    assert sum(1 for g in circ if g[0] == W.OP["CCX"]) == 8
    re, _ = oracle.dm_sim(n, circ)
    out, _ = oracle.measure(n, re, oracle.libc_uniforms(3, 16))
    assert set(int(x) for x in out) == {0b1000000010}


def test_parameters_slots_and_broadcast(oracle):
    prog = """OPENQASM 2.0; include "qelib1.inc";
    qreg a[2]; qreg b[1];
    h a;
    rz(-pi/4) b[0];
    crz(pi/2) a[0], b[0];
    u3(0.1, 2*pi/3, -pi^2/10) a[1];
    cu1(sqrt(2)) a[1], a[0];
    rxx(cos(pi/3)) a[0], b[0];
    barrier a, b;
    cx a, b;
    """
    n, circ, _ = Q.parse_qasm(prog)
    assert n == 3
    assert circ[0] == (W.OP["H"], (0,), 0.0, 0.0, 0.0) and circ[1] == (W.OP["H"], (1,), 0.0, 0.0, 0.0)
    assert circ[2] == (W.OP["RZ"], (2,), 0.0, -math.pi / 4, 0.0)          # RZ uses phi
    assert circ[3] == (W.OP["CRZ"], (0, 2), 0.0, 0.0, math.pi / 2)        # CRZ uses lambda
    assert circ[4][0] == W.OP["U3"] and circ[4][2:] == (0.1, 2 * math.pi / 3, -math.pi ** 2 / 10)
    assert circ[5] == (W.OP["CU1"], (1, 0), 0.0, 0.0, math.sqrt(2))
    assert circ[6] == (W.OP["RXX"], (0, 2), math.cos(math.pi / 3), 0.0, 0.0)
    assert circ[7] == (W.OP["CX"], (0, 2), 0.0, 0.0, 0.0) and circ[8] == (W.OP["CX"], (1, 2), 0.0, 0.0, 0.0)
    # the parsed stream runs in the oracle like the same gates appended by hand
    re, im = oracle.dm_sim(n, circ)
    assert abs(re.reshape(8, 8).trace() - 1) < 1e-12


def test_nested_gate_definitions(oracle):
    prog = """OPENQASM 2.0; include "qelib1.inc";
    gate bell a,b { h a; cx a,b; }
    gate rot(t) a { rx(t/2) a; ry(-t) a; }
    gate both(t) a,b { bell a,b; rot(t) b; }
    qreg q[2];
    both(0.7) q[0], q[1];
    """
    n, circ, _ = Q.parse_qasm(prog)
    names = [W.OP_NAMES[g[0]] for g in circ]
    assert names == ["H", "CX", "RX", "RY"]
    assert circ[2][2] == pytest.approx(0.35) and circ[3][2] == pytest.approx(-0.7)


@pytest.mark.parametrize("prog,msg", [
    ("qreg q[2]; foo q[0];", "unknown gate"),
    ("qreg q[2]; h q[2];", "out of range"),
    ("qreg q[2]; reset q[0];", "unsupported"),
    ("qreg q[2]; cx q[0], q[0];", "repeats"),
    ("qreg q[2]; rx(pi/) q[0];", "bad parameter"),
])
def test_errors(prog, msg):
    with pytest.raises(Q.QasmError, match=msg):
        Q.parse_qasm(prog)


@pytest.mark.gpu
def test_qasm_program_runs_on_the_engine(engine):
    for mode in ("plain", "fused"):
        sim, measured = Q.load_qasm(ADDER, mode=mode)
        sim.run()
        assert sim.measure(8) == [0b1000000010] * 8
        sim.close()
