"""The no-allocation metrics entry point (dmsim_pure_metrics_noalloc).

Some callers cannot call cudaMalloc: a process whose device memory is already
reserved by another allocator, or a monitoring loop that must not stall the
GPU on cudaMalloc/cudaFree's implicit synchronisation.  For them the library
stages the pure state in a 1 MiB array fixed in its device image instead of a
fresh buffer.  These tests call that entry point through the C ABI and check
it against the allocating dmsim_pure_metrics and against the same numbers
computed on the host from the copied-back state (FP64 and complex64), two
calls in a row (the second call finds the array holding the first call's
data), plus the size limit.

This file is collected last on purpose, and passes alone in a fresh process too.
"""
import ctypes

import numpy as np
import pytest

import dmsim_workloads as W

pytestmark = pytest.mark.gpu


def noalloc(engine, sim, psi):
    pr = np.ascontiguousarray(psi.real)
    pi = np.ascontiguousarray(psi.imag)
    out = np.zeros(4)
    P = ctypes.POINTER(ctypes.c_double)
    st = engine.lib().dmsim_pure_metrics_noalloc(sim._h, pr.ctypes.data_as(P), pi.ctypes.data_as(P),
                                                 out.ctypes.data_as(P))
    return st, {"fidelity": out[0], "trace": out[1], "max_abs_err": out[2], "frob_err": out[3]}


def close(a, b, tol):
    return all(abs(a[k] - b[k]) <= tol * max(1.0, abs(b[k])) for k in a)


def test_noalloc_metrics_match_allocating_entry_point(engine, oracle):
    # two different states and pure references, one call after the other
    cases = [(8, W.table_mix(8, 60, seed=91), "plain"), (10, W.layered_u3_cx(10, 80, seed=92), "fused")]
    for n, circ, mode in cases:
        sr, si = oracle.sv_sim(n, circ)
        psi = sr + 1j * si
        # a slightly wrong reference state as well, so the error outputs are not all ~0
        psi_off = psi.copy()
        psi_off[1] += 1e-3
        with engine.Simulation(n, mode=mode) as s:
            s.extend(circ)
            s.upload()
            s.run()
            for ref_psi in (psi, psi_off):
                want = s.pure_metrics(ref_psi)
                for _ in range(2):
                    st, got = noalloc(engine, s, ref_psi)
                    assert st == engine.OK, engine.lib().dmsim_last_error(s._h)
                    assert close(got, want, 1e-12), (got, want)
            assert abs(want["trace"] - 1) < 1e-10


def numpy_metrics(rho, psi):
    """fidelity, trace, max |rho - psi psi^+|, ||rho - psi psi^+||_F on the host."""
    d = rho - np.outer(psi, psi.conj())
    return {"fidelity": float(np.real(psi.conj() @ rho @ psi)), "trace": float(np.real(np.trace(rho))),
            "max_abs_err": float(np.abs(d).max()), "frob_err": float(np.linalg.norm(d))}


@pytest.mark.parametrize("precision", ["fp64", "c64"])
def test_noalloc_metrics_match_host_arithmetic(engine, oracle, precision):
    """Independent of the device kernel the two entry points share: the same
    four numbers computed on the host from the copied-back rho, for an FP64
    and a complex64 state, two calls in a row."""
    n = 7
    circ = W.table_mix(n, 80, seed=93)
    sr, si = oracle.sv_sim(n, circ)
    psi = sr + 1j * si
    psi_off = psi.copy()
    psi_off[3] += 1e-3
    with engine.Simulation(n, mode="fused", precision=precision) as s:
        s.extend(circ)
        s.upload()
        s.run()
        re, im = s.get_dm()
        d = 1 << n
        rho = (re + 1j * im).reshape(d, d).T  # the result layout is rho^T
        tol = 1e-12 if precision == "fp64" else 1e-6
        for ref_psi in (psi, psi_off):
            want = numpy_metrics(rho, ref_psi)
            for _ in range(2):
                st, got = noalloc(engine, s, ref_psi)
                assert st == engine.OK, engine.lib().dmsim_last_error(s._h)
                assert close(got, want, tol), (got, want)


def test_noalloc_rejects_states_beyond_its_scratch(engine):
    # 17 qubits: the handle allocates rho lazily, so nothing large is allocated here
    with engine.Simulation(17) as s:
        psi = np.zeros(1 << 17, dtype=np.complex128)
        st, _ = noalloc(engine, s, psi)
        assert st == engine.ERR_ARG
        assert b"16 qubits" in engine.lib().dmsim_last_error(s._h)
