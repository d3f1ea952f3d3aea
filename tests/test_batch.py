"""The batched sweep: many circuits of uneven qubit counts in one persistent
work-queue launch, each checked against the oracle; diagonal and <Z_i Z_{i+1}>
outputs; the sweep workload's shape at a reduced size."""
import numpy as np
import pytest

import dmsim_workloads as W

pytestmark = pytest.mark.gpu


def zz_from_diag(diag, n):
    idx = np.arange(1 << n)
    return np.array([np.sum(diag * (1 - 2 * (((idx >> i) ^ (idx >> (i + 1))) & 1))) for i in range(n - 1)])


@pytest.mark.parametrize("mode", ["plain", "fused"])
def test_batch_matches_oracle(engine, oracle, mode):
    rng = np.random.default_rng(5)
    sweep = []
    for i in range(12):
        n = int(rng.integers(3, 9))
        if i % 2:
            sweep.append((n, W.hea(n, int(rng.integers(2, 5)), rng)))
        else:
            sweep.append((n, W.random_circuit(n, 30, ops=[o for o in range(38) if o != W.OP["SRN"]], seed=700 + i)))
    with engine.Batch([n for n, _ in sweep], mode=mode) as b:
        for c, (n, circ) in enumerate(sweep):
            b.extend(c, circ)
        b.upload()
        for _ in range(2):  # the graph resets every state: two runs give the same result
            b.run()
            for c, (n, circ) in enumerate(sweep):
                ref = oracle.dm_sim(n, circ)
                re, im = b.dm(c)
                scale = max(1.0, np.abs(ref[0]).max())
                tol = (1e-12 if mode == "plain" else 1e-10) * scale
                assert np.abs(re - ref[0]).max() <= tol and np.abs(im - ref[1]).max() <= tol, (c, n)
                d = 1 << n
                rd = ref[0].reshape(d, d).diagonal()
                assert np.abs(b.diag(c) - rd).max() <= tol
                if n > 1:
                    assert np.abs(b.zz(c) - zz_from_diag(rd, n)).max() <= 10 * tol


@pytest.mark.parametrize("arith", ["fp64", "df64"])
def test_wide_circuits_on_engine_kernels(engine, oracle, arith):
    """Circuits at or above the wide threshold run on the engine's own pass
    kernels (tensor-core passes included) as concurrent graph branches, the
    rest in the work-queue kernel; both kinds against the oracle, twice."""
    rng = np.random.default_rng(8)
    sweep = [(n, W.hea(n, 3, rng)) for n in (4, 7, 5, 8, 6, 9, 7)]
    with engine.Batch([n for n, _ in sweep], mode="fused", fused_arith=arith, wide_qubits=7) as b:
        for c, (n, circ) in enumerate(sweep):
            b.extend(c, circ)
        b.upload()
        for _ in range(2):
            b.run()
            for c, (n, circ) in enumerate(sweep):
                ref = oracle.dm_sim(n, circ)
                re, im = b.dm(c)
                assert max(np.abs(re - ref[0]).max(), np.abs(im - ref[1]).max()) <= 1e-10, (c, n)
                d = 1 << n
                rd = ref[0].reshape(d, d).diagonal()
                assert np.abs(b.diag(c) - rd).max() <= 1e-10
                assert np.abs(b.zz(c) - zz_from_diag(rd, n)).max() <= 1e-9


def test_hea_sweep_shape(engine, oracle):
    """The parameter-sweep workload's shape (HEA, qubits uniform in {6..12}),
    64 circuits: every output against the oracle's diagonal."""
    sweep = W.hea_sweep(64, seed=9, nmin=6, nmax=10)
    with engine.Batch([n for n, _ in sweep], mode="fused") as b:
        for c, (n, circ) in enumerate(sweep):
            b.extend(c, circ)
        b.upload()
        b.run()
        st = b.stats()
        assert st["ms"] > 0 and st["items"] > 0
        for c in (0, 7, 31, 63):
            n, circ = sweep[c]
            sr, si = oracle.sv_sim(n, circ)
            p = sr ** 2 + si ** 2
            assert np.abs(b.diag(c) - p).max() <= 1e-10
            assert np.abs(b.zz(c) - zz_from_diag(p, n)).max() <= 1e-9


@pytest.mark.slow
def test_hea_sweep_full_config(engine, oracle):
    """The sweep at its full size: 512 hardware-efficient-ansatz circuits,
    qubits uniform in {6..12}, 4-10 layers, in one persistent launch.  Every
    circuit's diagonal and <Z_i Z_{i+1}> against the statevector oracle."""
    sweep = W.hea_sweep(512, seed=4)
    with engine.Batch([n for n, _ in sweep], mode="fused") as b:
        for c, (n, circ) in enumerate(sweep):
            b.extend(c, circ)
        b.upload()
        b.run()
        worst_d = worst_z = 0.0
        for c, (n, circ) in enumerate(sweep):
            sr, si = oracle.sv_sim(n, circ)
            p = sr ** 2 + si ** 2
            worst_d = max(worst_d, float(np.abs(b.diag(c) - p).max()))
            worst_z = max(worst_z, float(np.abs(b.zz(c) - zz_from_diag(p, n)).max()))
    assert worst_d <= 1e-10 and worst_z <= 1e-9, (worst_d, worst_z)


@pytest.mark.gpu
def test_dependency_wait_runs_out_and_gpu_stays_usable(engine):
    """Failure detection without a GPU fault: a wait whose count never
    arrives gives up after the wait limit, the run reports a timeout, and the
    next batch on the same device runs correctly."""
    rng = np.random.default_rng(1)
    sweep = [(4, W.hea(4, 3, rng)), (5, W.hea(5, 3, rng))]
    with engine.Batch([n for n, _ in sweep], mode="plain", wait_limit=1 << 12, test_stall=True) as b:
        for c, (n, circ) in enumerate(sweep):
            b.extend(c, circ)
        b.upload()
        with pytest.raises(engine.DMSimError) as e:
            b.run()
        assert e.value.status == engine.ERR_TIMEOUT
        # no plausible-looking output survives an expired wait
        assert np.isnan(b.diag(0)).all() and np.isnan(b.zz(1)).all()
    with engine.Batch([n for n, _ in sweep], mode="plain") as b:
        for c, (n, circ) in enumerate(sweep):
            b.extend(c, circ)
        b.upload()
        b.run()
        with engine.Simulation(4, mode="plain") as s:
            s.extend(sweep[0][1])
            s.upload()
            s.run()
            assert np.abs(s.get_diag() - b.diag(0)).max() <= 1e-12
