"""The CPU oracle is pinned to the reference: bit-identical density matrices
and measure() outcomes against fixtures made by the reference CPU engine
(tests/golden/make_golden.py), and, where the reference sources were present
at build time, against the live reference engine."""
import glob
import os

import numpy as np
import pytest

import dmsim_workloads as W

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def decode(z):
    circ = []
    for op, q, p in zip(z["ops"], z["qubits"], z["params"]):
        ar = W.ARITY[int(op)]
        circ.append((int(op), tuple(int(x) for x in q[:ar]), float(p[0]), float(p[1]), float(p[2])))
    return circ


def golden_cases():
    return sorted(f for f in glob.glob(os.path.join(GOLDEN, "*.npz")) if "adder" not in f)


@pytest.mark.parametrize("path", golden_cases(), ids=lambda p: os.path.basename(p)[:-4])
def test_oracle_matches_reference_fixture(oracle, path):
    z = np.load(path)
    n = int(z["n"])
    re, im = oracle.dm_sim(n, decode(z))
    # bit-identical on the machine that made the fixtures; libm's sin/cos may
    # differ by an ulp on another CPU, hence the 1e-15 allowance there
    assert np.abs(re - z["re"]).max() <= 1e-15
    assert np.abs(im - z["im"]).max() <= 1e-15


@pytest.mark.parametrize("path", golden_cases(), ids=lambda p: os.path.basename(p)[:-4])
def test_oracle_measure_matches_reference_fixture(oracle, path):
    z = np.load(path)
    n = int(z["n"])
    u = oracle.libc_uniforms(int(z["seed"]), len(z["outcomes"]))
    out, _ = oracle.measure(n, z["re"], u)
    assert (out == z["outcomes"]).all()


def test_adder_known_answer(oracle):
    """README.md:228-247: the 10-qubit adder measures 1000000010 on every shot."""
    z = np.load(os.path.join(GOLDEN, "adder_n10.npz"))
    re, im = oracle.dm_sim(10, decode(z))
    diag = re.reshape(1024, 1024).diagonal()
    assert np.abs(diag - z["diag"]).max() <= 1e-15
    u = oracle.libc_uniforms(int(z["seed"]), len(z["outcomes"]))
    out, tot = oracle.measure(10, re, u)
    assert (out == z["outcomes"]).all()
    assert set(int(x) for x in out) == {0b1000000010}
    assert abs(tot - 1.0) < 1e-12


def _ref(oracle):
    if not oracle.Reference.available():
        pytest.skip("reference CPU engine not built here (its sources are not mounted)")
    return oracle.Reference


@pytest.mark.parametrize("n,seed,ncpu", [(3, 0, 1), (5, 1, 2), (5, 2, 4), (6, 3, 1), (4, 4, 4)])
def test_oracle_bit_exact_vs_live_reference(oracle, n, seed, ncpu):
    Ref = _ref(oracle)
    circ = W.random_circuit(n, 50, seed=1000 + seed)
    r = Ref(n, ncpu)
    r.run(circ)
    rr, ri = r.dm()
    r.close()
    orr, ori = oracle.dm_sim(n, circ)
    assert np.array_equal(rr, orr) and np.array_equal(ri, ori)


def test_reference_chained_runs_are_wrong_and_oracle_is_right(oracle):
    """The reference CPU block_transpose serialises the tile's threads and reads
    smem[tlx][tly] before it is written (src/dmsim_cpu_omp.hpp:791-825), so a
    second sim() from a non-initial state is wrong; the oracle's transpose is
    correct and agrees with the statevector."""
    Ref = _ref(oracle)
    n = 5
    ops = [o for o in range(38) if o not in (W.OP["SRN"], W.OP["R"])]
    c1 = W.random_circuit(n, 30, ops=ops, seed=7)
    c2 = W.random_circuit(n, 30, ops=ops, seed=8)
    r = Ref(n, 1)
    r.run(c1)
    r.clear_circuit()
    r.run(c2)
    rr, ri = r.dm()
    r.close()
    re, im = oracle.dm_sim(n, c1)
    re, im = oracle.dm_sim(n, c2, re, im)
    sr, si = oracle.sv_sim(n, c1 + c2)
    psi = sr + 1j * si
    rho_o = oracle.rho_from_result(n, re, im)
    rho_r = oracle.rho_from_result(n, rr, ri)
    exact = np.outer(psi, psi.conj())
    assert np.abs(rho_o - exact).max() < 1e-13
    assert np.abs(rho_r - exact).max() > 1e-3


def test_statevector_oracle_matches_dm_oracle(oracle):
    n = 5
    ops = [o for o in range(38) if o != W.OP["SRN"]]  # SRN is not complex-linear
    for seed in range(3):
        circ = W.random_circuit(n, 60, ops=ops, seed=seed)
        re, im = oracle.dm_sim(n, circ)
        sr, si = oracle.sv_sim(n, circ)
        psi = sr + 1j * si
        assert np.abs(oracle.rho_from_result(n, re, im) - np.outer(psi, psi.conj())).max() < 1e-13
