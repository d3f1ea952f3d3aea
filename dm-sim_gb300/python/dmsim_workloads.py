"""Seeded synthetic circuits for the density-matrix engine's workloads.

A circuit is a list of ``(op, qubits, theta, phi, lam)`` tuples, with ``op`` the
gate id of DM-Sim's ``enum OP`` (src/dmsim_nvgpu_omp.cuh:42-48) and the angles
in the parameter slots that DM-Sim's static factories use
(src/dmsim_nvgpu_omp.cuh:580-767): RZ uses ``phi``; CRX/CRY/CRZ/CU1 use ``lam``;
RX/RY/RXX/RZZ/RYY/R use ``theta``.  Controls come first, the target last.

Workloads (sizes as named):
  * ``layered_u3_cx(n=10, ngates=200)`` -- alternating layers of U3 on every
    qubit and CX on a random disjoint pairing;
  * ``table_mix(n=14, ngates=2000)`` -- gates uniform over the 29-entry mixed
    table on uniformly random distinct qubits;
  * ``qft_then_layers(n=16, nlayer_gates=1000)`` -- X on each qubit with p=0.5,
    QFT (H + CU1(pi/2^k) ladder + final SWAPs), then U3+CX layer gates;
  * ``hea_sweep(ncirc=512)`` -- hardware-efficient ansatz circuits with qubit
    counts uniform in {6..12}, 4-10 layers of RY/RZ ~ U[-pi,pi) + CX ladder;
  * ``u3_cx_ccx(n=17, ngates=1000)`` -- random U3, CX and CCX gates.
"""
import math

import numpy as np

OP_NAMES = ["U3", "U2", "U1", "CX", "ID", "X", "Y", "Z", "H", "S",
            "SDG", "T", "TDG", "RX", "RY", "RZ", "CZ", "CY", "SWAP", "CH",
            "CCX", "CSWAP", "CRX", "CRY", "CRZ", "CU1", "CU3", "RXX", "RZZ", "RCCX",
            "RC3X", "C3X", "C3SQRTX", "C4X", "R", "SRN", "W", "RYY"]
OP = {name: i for i, name in enumerate(OP_NAMES)}

ARITY = {}
for _n in ["U3", "U2", "U1", "ID", "X", "Y", "Z", "H", "S", "SDG", "T", "TDG", "RX", "RY", "RZ", "R", "SRN", "W"]:
    ARITY[OP[_n]] = 1
for _n in ["CX", "CZ", "CY", "SWAP", "CH", "CRX", "CRY", "CRZ", "CU1", "CU3", "RXX", "RZZ", "RYY"]:
    ARITY[OP[_n]] = 2
for _n in ["CCX", "CSWAP", "RCCX"]:
    ARITY[OP[_n]] = 3
for _n in ["RC3X", "C3X", "C3SQRTX"]:
    ARITY[OP[_n]] = 4
ARITY[OP["C4X"]] = 5

# which angle slots a gate reads
PARAMS = {OP["U3"]: "tpl", OP["U2"]: "pl", OP["U1"]: "l", OP["RX"]: "t", OP["RY"]: "t", OP["RZ"]: "p",
          OP["CRX"]: "l", OP["CRY"]: "l", OP["CRZ"]: "l", OP["CU1"]: "l", OP["CU3"]: "tpl",
          OP["RXX"]: "t", OP["RZZ"]: "t", OP["RYY"]: "t", OP["R"]: "t"}

# the 29-entry mixed table of the 14-qubit workload
TABLE29 = [OP[x] for x in ["U1", "U2", "U3", "RX", "RY", "RZ", "H", "S", "T", "X", "Y", "Z",
                           "CX", "CY", "CZ", "CH", "SWAP", "CRX", "CRY", "CRZ", "CU1", "CU3",
                           "RXX", "RYY", "RZZ", "CCX", "CSWAP", "C3X", "C4X"]]

ALL_OPS = list(range(38))


def make_gate(op, qubits, rng, lo=0.0, hi=2 * math.pi):
    slots = PARAMS.get(op, "")
    th = rng.uniform(lo, hi) if "t" in slots else 0.0
    ph = rng.uniform(lo, hi) if "p" in slots else 0.0
    la = rng.uniform(lo, hi) if "l" in slots else 0.0
    return (op, tuple(int(q) for q in qubits), th, ph, la)


def random_circuit(n, ngates, ops=ALL_OPS, seed=0, lo=0.0, hi=2 * math.pi):
    """Gates drawn uniformly from ``ops`` on uniformly random distinct qubits."""
    rng = np.random.default_rng(seed)
    ops = [o for o in ops if ARITY[o] <= n]
    out = []
    for _ in range(ngates):
        op = ops[rng.integers(len(ops))]
        qs = rng.choice(n, size=ARITY[op], replace=False)
        out.append(make_gate(op, qs, rng, lo, hi))
    return out


def layered_u3_cx(n=10, ngates=200, seed=1):
    """Alternating layers: U3(theta,phi,lambda ~ U[0,2pi)) on every qubit, then CX
    on a random disjoint pairing of the qubits; truncated to ``ngates``."""
    rng = np.random.default_rng(seed)
    out = []
    while len(out) < ngates:
        for q in range(n):
            out.append(make_gate(OP["U3"], (q,), rng))
        perm = rng.permutation(n)
        for i in range(0, n - 1, 2):
            out.append((OP["CX"], (int(perm[i]), int(perm[i + 1])), 0.0, 0.0, 0.0))
    return out[:ngates]


def table_mix(n=14, ngates=2000, seed=2):
    return random_circuit(n, ngates, TABLE29, seed=seed)


def qft(n, qubits=None):
    """Textbook QFT: H, then CU1(pi/2^k) from each later qubit, then SWAPs."""
    qs = list(range(n)) if qubits is None else list(qubits)
    out = []
    for i in range(len(qs)):
        out.append((OP["H"], (qs[i],), 0.0, 0.0, 0.0))
        for j in range(i + 1, len(qs)):
            out.append((OP["CU1"], (qs[j], qs[i]), 0.0, 0.0, math.pi / (2 ** (j - i))))
    for i in range(len(qs) // 2):
        out.append((OP["SWAP"], (qs[i], qs[len(qs) - 1 - i]), 0.0, 0.0, 0.0))
    return out


def qft_then_layers(n=16, nlayer_gates=1000, seed=3):
    rng = np.random.default_rng(seed)
    out = []
    for q in range(n):
        if rng.random() < 0.5:
            out.append((OP["X"], (q,), 0.0, 0.0, 0.0))
    out += qft(n)
    out += layered_u3_cx(n, nlayer_gates, seed=seed + 1000)
    return out


def hea(n, layers, rng):
    out = []
    for _ in range(layers):
        for q in range(n):
            out.append(make_gate(OP["RY"], (q,), rng, -math.pi, math.pi))
        for q in range(n):
            out.append(make_gate(OP["RZ"], (q,), rng, -math.pi, math.pi))
        for q in range(n - 1):
            out.append((OP["CX"], (q, q + 1), 0.0, 0.0, 0.0))
    return out


def hea_sweep(ncirc=512, seed=4, nmin=6, nmax=12, lmin=4, lmax=10):
    """List of (n, circuit) for the batched parameter sweep."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(ncirc):
        n = int(rng.integers(nmin, nmax + 1))
        layers = int(rng.integers(lmin, lmax + 1))
        out.append((n, hea(n, layers, rng)))
    return out


def u3_cx_ccx(n=17, ngates=1000, seed=5):
    return random_circuit(n, ngates, [OP["U3"], OP["CX"], OP["CCX"]], seed=seed)


def sparse_triples(n=14, ngates=600, seed=6):
    """Controlled rotations, phases and CX inside fixed disjoint qubit triples
    (0-2, 3-5, ...), in random order across the triples: every fused block is
    a sparse 3-qubit operator (at most 2 nonzeros per row), the case where the
    tensor-core passes lose to the pipe kernels."""
    rng = np.random.default_rng(seed)
    ops = [OP["CRY"], OP["CRZ"], OP["CU1"], OP["CRX"], OP["CX"], OP["CZ"]]
    ntri = n // 3
    out = []
    for _ in range(ngates):
        t = int(rng.integers(0, ntri))
        a, b = (int(x) for x in rng.choice(3, size=2, replace=False))
        out.append(make_gate(int(rng.choice(ops)), (3 * t + a, 3 * t + b), rng))
    return out
