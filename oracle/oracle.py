"""ctypes bindings for the CPU ORACLE (test infrastructure only).

Loads ``oracle/liboracle.so`` (the plain-C restatement of DM-Sim's CPU engine,
src/dmsim_cpu_omp.hpp) and, when it has been built, ``oracle/_ref/libdmsim_ref.so``
(the reference CPU engine compiled from its own sources).  Only tests, the
smoke check and the benchmark's CPU-baseline leg import this module; the GPU
engine never does.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libdmsim_ref.so")

# enum OP of src/dmsim_cpu_omp.hpp:41-47 (the order is the ABI)
OP_NAMES = ["U3", "U2", "U1", "CX", "ID", "X", "Y", "Z", "H", "S",
            "SDG", "T", "TDG", "RX", "RY", "RZ", "CZ", "CY", "SWAP", "CH",
            "CCX", "CSWAP", "CRX", "CRY", "CRZ", "CU1", "CU3", "RXX", "RZZ", "RCCX",
            "RC3X", "C3X", "C3SQRTX", "C4X", "R", "SRN", "W", "RYY"]
OP = {name: i for i, name in enumerate(OP_NAMES)}
OP_C1, OP_C2 = 64, 65


class DmoGate(ctypes.Structure):
    _fields_ = [("op", ctypes.c_int32), ("qb", ctypes.c_uint32 * 5),
                ("theta", ctypes.c_double), ("phi", ctypes.c_double), ("lam", ctypes.c_double),
                ("m", ctypes.c_double * 32)]


def build(force=False):
    """Compile liboracle.so (gcc) if it is missing."""
    if force or not os.path.exists(LIB_PATH):
        subprocess.check_call(["make", "-s", "-C", HERE, "liboracle.so"])
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.POINTER
        L.dmo_basic_count.argtypes = [P(DmoGate)]
        L.dmo_basic_count.restype = ctypes.c_int
        for name in ("dmo_apply_columns", "dmo_dm_sim"):
            f = getattr(L, name)
            f.argtypes = [ctypes.c_int, P(DmoGate), ctypes.c_int, P(ctypes.c_double), P(ctypes.c_double), ctypes.c_int]
            f.restype = None
        L.dmo_sv_sim.argtypes = [ctypes.c_int, P(DmoGate), ctypes.c_int, P(ctypes.c_double), P(ctypes.c_double)]
        L.dmo_measure.argtypes = [ctypes.c_int, P(ctypes.c_double), ctypes.c_int, P(ctypes.c_double), P(ctypes.c_uint64)]
        L.dmo_measure.restype = ctypes.c_double
        L.dmo_libc_uniforms.argtypes = [ctypes.c_uint, ctypes.c_int, P(ctypes.c_double)]
        _lib = L
    return _lib


def _dptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def to_gates(circuit):
    """circuit: list of (op, qubits, theta, phi, lam[, matrix]) -> ctypes array."""
    arr = (DmoGate * max(1, len(circuit)))()
    for i, g in enumerate(circuit):
        op, qs, th, ph, la = g[0], g[1], g[2], g[3], g[4]
        arr[i].op = op
        for k, q in enumerate(list(qs)[:5]):
            arr[i].qb[k] = q
        arr[i].theta, arr[i].phi, arr[i].lam = th, ph, la
        if len(g) > 5 and g[5] is not None:
            m = np.asarray(g[5], dtype=np.complex128).reshape(-1)
            flat = np.empty(2 * m.size)
            flat[0::2], flat[1::2] = m.real, m.imag
            for k in range(flat.size):
                arr[i].m[k] = flat[k]
    return arr


def zero_state(n):
    N = 1 << (2 * n)
    re = np.zeros(N)
    im = np.zeros(N)
    re[0] = 1.0
    return re, im


def dm_sim(n, circuit, re=None, im=None, nthreads=0):
    """The reference sim() restated; returns (re, im) in dm_real_res layout."""
    if re is None:
        re, im = zero_state(n)
    else:
        re, im = np.ascontiguousarray(re, dtype=np.float64).copy(), np.ascontiguousarray(im, dtype=np.float64).copy()
    g = to_gates(circuit)
    lib().dmo_dm_sim(n, g, len(circuit), _dptr(re), _dptr(im), nthreads)
    return re, im


def sv_sim(n, circuit, re=None, im=None):
    d = 1 << n
    if re is None:
        re = np.zeros(d)
        im = np.zeros(d)
        re[0] = 1.0
    else:
        re, im = re.copy(), im.copy()
    g = to_gates(circuit)
    lib().dmo_sv_sim(n, g, len(circuit), _dptr(re), _dptr(im))
    return re, im


def basic_count(gate):
    g = to_gates([gate])
    return lib().dmo_basic_count(g)


def measure(n, dm_re, uniforms):
    u = np.ascontiguousarray(uniforms, dtype=np.float64)
    out = np.zeros(len(u), dtype=np.uint64)
    tot = lib().dmo_measure(n, _dptr(np.ascontiguousarray(dm_re)), len(u), _dptr(u),
                            out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)))
    return out, tot


def libc_uniforms(seed, rep):
    out = np.zeros(rep)
    lib().dmo_libc_uniforms(seed, rep, _dptr(out))
    return out


def rho_from_result(n, re, im):
    """dm_real_res layout -> rho as a complex matrix (rho[j][i] = res[i*dim+j])."""
    d = 1 << n
    return (re.reshape(d, d) + 1j * im.reshape(d, d)).T


# ---------------------------------------------------------------- reference
class Reference:
    """The reference CPU engine (oracle/_ref/libdmsim_ref.so), driven through its
    own Simulation object.  Only available where the reference sources were
    present at build time (``make -C oracle ref``)."""

    _L = None

    @classmethod
    def available(cls):
        return os.path.exists(REF_PATH)

    @classmethod
    def _lib(cls):
        if cls._L is None:
            L = ctypes.CDLL(REF_PATH)
            P = ctypes.POINTER
            L.ref_create.argtypes = [ctypes.c_uint, ctypes.c_uint]
            L.ref_create.restype = ctypes.c_void_p
            L.ref_destroy.argtypes = [ctypes.c_void_p]
            L.ref_append.argtypes = [ctypes.c_void_p, ctypes.c_int, P(ctypes.c_uint32), ctypes.c_double, ctypes.c_double, ctypes.c_double]
            for nm in ("ref_upload", "ref_sim", "ref_clear_circuit", "ref_reset"):
                getattr(L, nm).argtypes = [ctypes.c_void_p]
            L.ref_get_dm.argtypes = [ctypes.c_void_p, P(ctypes.c_double), P(ctypes.c_double)]
            L.ref_measure.argtypes = [ctypes.c_void_p, ctypes.c_uint, ctypes.c_uint, P(ctypes.c_uint64)]
            cls._L = L
        return cls._L

    def __init__(self, n, ncpus=1):
        self.n = n
        self.h = self._lib().ref_create(n, ncpus)

    def append(self, op, qs, th=0.0, ph=0.0, la=0.0):
        q = (ctypes.c_uint32 * 5)(*(list(qs) + [0] * (5 - len(qs))))
        self._lib().ref_append(self.h, op, q, th, ph, la)

    def run(self, circuit):
        for g in circuit:
            self.append(g[0], g[1], g[2], g[3], g[4])
        self._lib().ref_upload(self.h)
        self._lib().ref_sim(self.h)

    def clear_circuit(self):
        self._lib().ref_clear_circuit(self.h)

    def dm(self):
        N = 1 << (2 * self.n)
        re, im = np.zeros(N), np.zeros(N)
        self._lib().ref_get_dm(self.h, _dptr(re), _dptr(im))
        return re, im

    def measure(self, seed, rep):
        out = np.zeros(rep, dtype=np.uint64)
        self._lib().ref_measure(self.h, seed, rep, out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)))
        return out

    def close(self):
        if self.h:
            self._lib().ref_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
