"""The OpenQASM 2 frontend on the reference's own circuits (benchmark/*.qasm,
tool/vqe_uccsd_n8.qasm and the QASMBench suite it ships under qasmbench/,
small, medium and large, 55 programs), where the reference checkout is
present (CPU; skipped elsewhere -- the circuits are not copied into this
repository): every circuit parses -- those with classically controlled
statements or resets under the reference translator's rule of dropping them
(tool/dmsim_qasm.py:104, :321-322) -- and for circuits of up to 10 qubits the
density-matrix oracle on the parsed circuit equals psi psi^+ of the
statevector oracle."""
import glob
import os
import subprocess

import numpy as np
import pytest

import dmsim_qasm as Q

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def reference_dir():
    d = os.environ.get("DMSIM_REFERENCE_DIR")
    if not d:
        r = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref-dir"], capture_output=True,
                           text=True)
        d = r.stdout.strip()
    return d if d and os.path.isdir(os.path.join(d, "benchmark")) else None


REF = reference_dir()
FILES = sorted(glob.glob(os.path.join(REF, "benchmark", "*.qasm"))) + [os.path.join(REF, "tool", "vqe_uccsd_n8.qasm")] \
    + sorted(glob.glob(os.path.join(REF, "qasmbench", "*", "*", "*.qasm"))) if REF else []


@pytest.mark.skipif(not REF, reason="the reference checkout is not present")
@pytest.mark.parametrize("path", FILES, ids=[os.path.relpath(f, REF) for f in FILES])
def test_reference_circuit_parses_and_oracles_agree(oracle, path):
    with open(path) as f:
        text = f.read()
    n, circ, _ = Q.parse_qasm(text, conditionals="skip")
    assert n >= 2 and len(circ) > 0
    if n <= 10:
        re_, im_ = oracle.dm_sim(n, circ)
        sr, si = oracle.sv_sim(n, circ)
        psi = sr + 1j * si
        rho = np.outer(psi, psi.conj())  # rho[r][c]; the result layout is rho^T
        d = 1 << n
        A = (re_ + 1j * im_).reshape(d, d).T
        assert np.abs(A - rho).max() <= 1e-12


def test_conditionals_raise_unless_skipped():
    prog = "OPENQASM 2.0;\ninclude \"qelib1.inc\";\nqreg q[2];\ncreg c[2];\nh q[0];\nif(c==1) x q[1];\n"
    with pytest.raises(Q.QasmError):
        Q.parse_qasm(prog)
    n, circ, _ = Q.parse_qasm(prog, conditionals="skip")
    assert n == 2 and len(circ) == 1
