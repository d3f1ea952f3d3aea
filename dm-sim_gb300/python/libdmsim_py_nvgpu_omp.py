"""Drop-in replacement for DM-Sim's pybind11 module ``libdmsim_py_nvgpu_omp``.

Same names, argument order and meaning as the reference module
(src/py_nvgpu_omp_wrapper.cu:29-90): ``Gate(op, qb0..qb4, theta, phi, lambda)``,
``Simulation(n_qubits, n_gpus)`` with ``append / upload / clear_circuit / run /
reset / measure(rep) -> list`` and the 38 static gate factories.  Additions:
``C1`` / ``C2`` arbitrary gates, ``reset_dm``, ``reset_sim`` (alias of
``reset``), ``dump``, and ``measure(rep, uniforms)`` with injected uniforms.

Errors raise ``RuntimeError`` subclasses instead of exiting the process.
"""
import numpy as np

import dmsim_gb300 as _eng

OP = _eng.OP
OP_NAMES = _eng.OP_NAMES


class Gate:
    """Gate(op, qb0, qb1, qb2, qb3, qb4, theta, phi, lambda) -- src/dmsim_nvgpu_omp.cuh:99-191."""

    __slots__ = ("op_name", "qb0", "qb1", "qb2", "qb3", "qb4", "theta", "phi", "lam", "matrix")

    def __init__(self, op, qb0=0, qb1=0, qb2=0, qb3=0, qb4=0, theta=0.0, phi=0.0, lam=0.0, matrix=None):
        self.op_name = int(op)
        self.qb0, self.qb1, self.qb2, self.qb3, self.qb4 = int(qb0), int(qb1), int(qb2), int(qb3), int(qb4)
        self.theta, self.phi, self.lam = float(theta), float(phi), float(lam)
        self.matrix = matrix

    def dump(self):
        name = OP_NAMES[self.op_name] if self.op_name < len(OP_NAMES) else ("C1" if self.op_name == 64 else "C2")
        return f"{name}({self.qb0},{self.qb1},{self.qb2},{self.qb3},{self.qb4},{self.theta:g},{self.phi:g},{self.lam:g});"


def _g(name, qs=(), theta=0.0, phi=0.0, lam=0.0):
    q = list(qs) + [0] * (5 - len(qs))
    return Gate(OP[name], *q, theta, phi, lam)


class Simulation:
    """Simulation(n_qubits, n_gpus) -- src/dmsim_nvgpu_omp.cuh:196-271 (n_gpus must be 1)."""

    def __init__(self, n_qubits, n_gpus=1, **options):
        self._sim = _eng.Simulation(n_qubits, n_gpus, **options)
        self.n_qubits = int(n_qubits)
        self.dim = 1 << self.n_qubits

    # circuit management (append :331-344, upload :345-377, clear_circuit :496-520)
    def append(self, g):
        if g.op_name == 64:
            self._sim.append_c1(g.qb0, g.matrix)
        elif g.op_name == 65:
            self._sim.append_c2(g.qb0, g.qb1, g.matrix)
        else:
            self._sim.append(g.op_name, (g.qb0, g.qb1, g.qb2, g.qb3, g.qb4), g.theta, g.phi, g.lam)

    def upload(self):
        self._sim.upload()
        return self

    def clear_circuit(self):
        self._sim.clear_circuit()

    def run(self):
        """sim() -- :390-494."""
        self._sim.run()

    def reset(self):
        """reset() -- :303-307: clear the circuit and return rho to |0..0><0..0|."""
        self._sim.reset()

    reset_sim = reset

    def reset_dm(self):
        self._sim.reset_dm()

    def measure(self, repetition=10, uniforms=None):
        """measure(rep) -- :521-549.  With ``uniforms`` (rep values in [0,1)) the
        draws replace rand()/RAND_MAX and the outcomes are reproducible."""
        return self._sim.measure(repetition, uniforms)

    def dump(self):
        return self._sim.dump()

    @property
    def n_gates(self):
        return self._sim.n_gates()

    @property
    def dm_real_res(self):
        return self._sim.get_dm()[0]

    @property
    def dm_imag_res(self):
        return self._sim.get_dm()[1]

    def get_dm(self):
        return self._sim.get_dm()

    # ------------------------------------------------ standard gates (:580-658)
    @staticmethod
    def U3(theta, phi, lam, m): return _g("U3", (m,), theta, phi, lam)
    @staticmethod
    def U2(phi, lam, m): return _g("U2", (m,), 0.0, phi, lam)
    @staticmethod
    def U1(lam, m): return _g("U1", (m,), 0.0, 0.0, lam)
    @staticmethod
    def CX(m, n): return _g("CX", (m, n))
    @staticmethod
    def ID(m): return _g("ID", (m,))
    @staticmethod
    def X(m): return _g("X", (m,))
    @staticmethod
    def Y(m): return _g("Y", (m,))
    @staticmethod
    def Z(m): return _g("Z", (m,))
    @staticmethod
    def H(m): return _g("H", (m,))
    @staticmethod
    def S(m): return _g("S", (m,))
    @staticmethod
    def SDG(m): return _g("SDG", (m,))
    @staticmethod
    def T(m): return _g("T", (m,))
    @staticmethod
    def TDG(m): return _g("TDG", (m,))
    @staticmethod
    def RX(theta, m): return _g("RX", (m,), theta)
    @staticmethod
    def RY(theta, m): return _g("RY", (m,), theta)
    @staticmethod
    def RZ(phi, m): return _g("RZ", (m,), 0.0, phi)
    # ------------------------------------------------ composition gates (:660-747)
    @staticmethod
    def CZ(m, n): return _g("CZ", (m, n))
    @staticmethod
    def CY(m, n): return _g("CY", (m, n))
    @staticmethod
    def SWAP(m, n): return _g("SWAP", (m, n))
    @staticmethod
    def CH(m, n): return _g("CH", (m, n))
    @staticmethod
    def CCX(l, m, n): return _g("CCX", (l, m, n))
    @staticmethod
    def CSWAP(l, m, n): return _g("CSWAP", (l, m, n))
    @staticmethod
    def CRX(lam, m, n): return _g("CRX", (m, n), 0.0, 0.0, lam)
    @staticmethod
    def CRY(lam, m, n): return _g("CRY", (m, n), 0.0, 0.0, lam)
    @staticmethod
    def CRZ(lam, m, n): return _g("CRZ", (m, n), 0.0, 0.0, lam)
    @staticmethod
    def CU1(lam, m, n): return _g("CU1", (m, n), 0.0, 0.0, lam)
    @staticmethod
    def CU3(theta, phi, lam, m, n): return _g("CU3", (m, n), theta, phi, lam)
    @staticmethod
    def RXX(theta, m, n): return _g("RXX", (m, n), theta)
    @staticmethod
    def RZZ(theta, m, n): return _g("RZZ", (m, n), theta)
    @staticmethod
    def RCCX(l, m, n): return _g("RCCX", (l, m, n))
    @staticmethod
    def RC3X(l, m, n, o): return _g("RC3X", (l, m, n, o))
    @staticmethod
    def C3X(l, m, n, o): return _g("C3X", (l, m, n, o))
    @staticmethod
    def C3SQRTX(l, m, n, o): return _g("C3SQRTX", (l, m, n, o))
    @staticmethod
    def C4X(l, m, n, o, p): return _g("C4X", (l, m, n, o, p))
    # ------------------------------------------------ DM-Sim native gates (:749-767)
    @staticmethod
    def R(theta, m): return _g("R", (m,), theta)
    @staticmethod
    def SRN(m): return _g("SRN", (m,))
    @staticmethod
    def W(m): return _g("W", (m,))
    @staticmethod
    def RYY(theta, m, n): return _g("RYY", (m, n), theta)
    # ------------------------------------------------ additions: arbitrary gates
    @staticmethod
    def C1(m, q):
        """Arbitrary 1-qubit gate: m is a 2x2 complex matrix."""
        return Gate(64, q, matrix=np.asarray(m, dtype=np.complex128).reshape(2, 2))

    @staticmethod
    def C2(m, q1, q2):
        """Arbitrary 2-qubit gate: m is 4x4 complex, basis index 2*bit(q1) + bit(q2)."""
        return Gate(65, q1, q2, matrix=np.asarray(m, dtype=np.complex128).reshape(4, 4))
