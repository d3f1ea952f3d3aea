"""Generate the golden fixtures in tests/golden/ from the REFERENCE CPU engine.

Runs DM-Sim's own CPU engine (src/dmsim_cpu_omp.hpp, compiled from the
reference sources by ``make -C oracle ref`` into oracle/_ref/) on small seeded
circuits and stores, per case, the circuit itself, the reference's
dm_real_res/dm_imag_res and (for some cases) measure() outcomes for a fixed
seed.  Needs the reference sources, so it runs only where they are mounted;
the fixtures it writes are committed and used everywhere.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [os.path.join(ROOT, "oracle"), os.path.join(ROOT, "dm-sim_gb300", "python")]

import oracle as O  # noqa: E402
import dmsim_workloads as W  # noqa: E402


def encode(circ):
    m = len(circ)
    ops = np.array([g[0] for g in circ], dtype=np.int32)
    qs = np.zeros((m, 5), dtype=np.uint32)
    ps = np.zeros((m, 3))
    for i, g in enumerate(circ):
        qs[i, :len(g[1])] = g[1]
        ps[i] = g[2], g[3], g[4]
    return ops, qs, ps


def adder_n10():
    """The 10-qubit Cuccaro ripple-carry adder of example/adder_n10_cpu_omp.cpp:22-61."""
    c = []
    X, CX, CCX = W.OP["X"], W.OP["CX"], W.OP["CCX"]
    for q in (1, 5, 6, 7, 8):
        c.append((X, (q,), 0.0, 0.0, 0.0))

    def maj(a, b, cc):
        c.extend([(CX, (cc, b), 0.0, 0.0, 0.0), (CX, (cc, a), 0.0, 0.0, 0.0), (CCX, (a, b, cc), 0.0, 0.0, 0.0)])

    def unmaj(a, b, cc):
        c.extend([(CCX, (a, b, cc), 0.0, 0.0, 0.0), (CX, (cc, a), 0.0, 0.0, 0.0), (CX, (a, b), 0.0, 0.0, 0.0)])

    maj(0, 5, 1); maj(1, 6, 2); maj(2, 7, 3); maj(3, 8, 4)
    c.append((CX, (4, 9), 0.0, 0.0, 0.0))
    unmaj(3, 8, 4); unmaj(2, 7, 3); unmaj(1, 6, 2); unmaj(0, 5, 1)
    return c


CASES = {
    # every gate of the table, small n
    "all_gates_n4_s0": (4, lambda: W.random_circuit(4, 60, seed=100)),
    "all_gates_n5_s1": (5, lambda: W.random_circuit(5, 60, seed=101)),
    "all_gates_n5_s2": (5, lambda: W.random_circuit(5, 40, seed=102)),
    # the workload shapes at small n
    "layered_u3_cx_n6": (6, lambda: W.layered_u3_cx(6, 60, seed=103)),
    "table_mix_n6": (6, lambda: W.table_mix(6, 40, seed=104)),
    "qft_layers_n5": (5, lambda: W.qft_then_layers(5, 30, seed=105)),
    "u3_cx_ccx_n5": (5, lambda: W.u3_cx_ccx(5, 40, seed=106)),
}


def main():
    if not O.Reference.available():
        sys.exit("the reference CPU engine is not built (make -C oracle ref)")
    for name, (n, gen) in CASES.items():
        circ = gen()
        ref = O.Reference(n, 1)
        ref.run(circ)
        re, im = ref.dm()
        seed = 12345
        outcomes = ref.measure(seed, 64)
        ref.close()
        ops, qs, ps = encode(circ)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), n=n, ops=ops, qubits=qs, params=ps, re=re, im=im,
                            seed=seed, outcomes=outcomes)
        print(name, n, len(circ))
    # the adder: full rho is 2 x 8 MB, keep the diagonal and the shots
    circ = adder_n10()
    ref = O.Reference(10, 1)
    ref.run(circ)
    re, _ = ref.dm()
    outcomes = ref.measure(777, 32)
    ref.close()
    ops, qs, ps = encode(circ)
    diag = re.reshape(1024, 1024).diagonal().copy()
    np.savez_compressed(os.path.join(HERE, "adder_n10.npz"), n=10, ops=ops, qubits=qs, params=ps, diag=diag,
                        seed=777, outcomes=outcomes)
    print("adder_n10", sorted(set(int(x) for x in outcomes)))


if __name__ == "__main__":
    main()
