"""Real operators (H, RY, CX, SWAP and their fused products) run the
real-coefficient kernel instances (two multiply-adds per complex term):
parity with the oracle in plain FP64, plain double-float and fused modes."""
import numpy as np
import pytest

import dmsim_workloads as W

pytestmark = pytest.mark.gpu


def real_circuit(n, gates, seed):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(gates):
        k = rng.integers(0, 4)
        if k == 0:
            out.append((W.OP["H"], (int(rng.integers(n)),), 0.0, 0.0, 0.0))
        elif k == 1:
            out.append((W.OP["RY"], (int(rng.integers(n)),), float(rng.uniform(0, 2 * np.pi)), 0.0, 0.0))
        elif k == 2:
            q = rng.choice(n, 2, replace=False)
            out.append((W.OP["CX"], (int(q[0]), int(q[1])), 0.0, 0.0, 0.0))
        else:
            q = rng.choice(n, 2, replace=False)
            out.append((W.OP["SWAP"], (int(q[0]), int(q[1])), 0.0, 0.0, 0.0))
    return out


@pytest.mark.parametrize("mode,plain_arith,tol", [("plain", "fp64", 1e-12), ("plain", "df64", 1e-12),
                                                   ("fused", "fp64", 1e-10)])
def test_real_operators_match_oracle(engine, oracle, mode, plain_arith, tol):
    n = 7
    circ = real_circuit(n, 150, seed=5)
    with engine.Simulation(n, mode=mode, max_k=2, plain_arith=plain_arith) as s:
        s.extend(circ)
        s.upload()
        s.run()
        re, im = s.get_dm()
    ref = oracle.dm_sim(n, circ)
    assert max(np.abs(re - ref[0]).max(), np.abs(im - ref[1]).max()) <= tol
