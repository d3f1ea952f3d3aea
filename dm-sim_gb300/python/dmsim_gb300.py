"""Python binding of the GB300 density-matrix engine's C ABI (include/dmsim_gb300.h).

Every call goes to ``libdmsim_gb300.so`` (hand-written sm_103a kernels behind a
C ABI).  There is no fallback: if the library is missing, importing this
module raises ``ImportError`` with the build command.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.normpath(os.path.join(_HERE, "..", "lib", "libdmsim_gb300.so"))

OK, ERR_ARG, ERR_STATE, ERR_OOM, ERR_CUDA, ERR_TIMEOUT, ERR_UNSUPPORTED = range(7)
(OPT_MODE, OPT_PRECISION, OPT_MAX_K, OPT_PLANNER, OPT_RECORD, OPT_SEED, OPT_GRAPH, OPT_VERBOSE, OPT_FUSED_ARITH,
 OPT_RENORM, OPT_PLAIN_ARITH, OPT_TENSOR, OPT_DIRECT1) = range(1, 14)
AR_FP64, AR_FP32, AR_DF64 = 0, 1, 2
BATCH_OPT_WAIT_LIMIT, BATCH_OPT_TEST_STALL, BATCH_OPT_WIDE_QUBITS = 100, 101, 102
PASS_RECORD = 10  # doubles per pass record: K, class, nnz, max_lo_bit, min_hi_bit, n, ms, bytes, tensor, blocks

OP_NAMES = ["U3", "U2", "U1", "CX", "ID", "X", "Y", "Z", "H", "S",
            "SDG", "T", "TDG", "RX", "RY", "RZ", "CZ", "CY", "SWAP", "CH",
            "CCX", "CSWAP", "CRX", "CRY", "CRZ", "CU1", "CU3", "RXX", "RZZ", "RCCX",
            "RC3X", "C3X", "C3SQRTX", "C4X", "R", "SRN", "W", "RYY"]
OP = {n: i for i, n in enumerate(OP_NAMES)}

CLASS_NAMES = ["MOVE", "SIGNED", "PHASE", "DENSE", "SPARSE", "RLIN", "SUPER"]
NOISE = {"depolarizing": 0, "amplitude_damping": 1, "phase_damping": 2, "bit_flip": 3, "phase_flip": 4,
         "depolarizing2": 5}


class DMSimError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"dmsim error {status}: {msg}")
        self.status = status


_lib = None


def lib():
    """The loaded engine library (ctypes), with argument types declared."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: build it with "
                          f"`python -c 'import __graft_entry__ as g; g.build()'` at the repository root")
    L = ctypes.CDLL(LIB_PATH)
    P = ctypes.POINTER
    H = ctypes.c_void_p
    d, u32, u64, i64 = ctypes.c_double, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int64
    sig = {
        "dmsim_create": [u32, u32, P(H)],
        "dmsim_destroy": [H],
        "dmsim_set_option": [H, ctypes.c_int, i64],
        "dmsim_get_option": [H, ctypes.c_int, P(i64)],
        "dmsim_append": [H, ctypes.c_int, P(u32), d, d, d],
        "dmsim_append_c1": [H, u32, P(d)],
        "dmsim_append_c2": [H, u32, u32, P(d)],
        "dmsim_upload": [H],
        "dmsim_run": [H],
        "dmsim_clear_circuit": [H],
        "dmsim_reset": [H],
        "dmsim_reset_dm": [H],
        "dmsim_measure": [H, u32, P(d), P(u64)],
        "dmsim_get_dm": [H, P(d), P(d)],
        "dmsim_set_dm": [H, P(d), P(d)],
        "dmsim_get_diag": [H, P(d)],
        "dmsim_dump": [H, ctypes.c_char_p, ctypes.c_size_t, P(ctypes.c_size_t)],
        "dmsim_n_qubits": [H, P(u32)],
        "dmsim_n_gates": [H, P(u32)],
        "dmsim_plan_stats": [H, P(u32), P(u32)],
        "dmsim_last_timings": [H, P(d)],
        "dmsim_upload_bytes": [H, P(u64)],
        "dmsim_pass_records": [H, P(d), u32, P(u32)],
        "dmsim_pure_metrics": [H, P(d), P(d), P(d)],
        "dmsim_pure_metrics_noalloc": [H, P(d), P(d), P(d)],
        "dmsim_device_state": [H, P(ctypes.c_void_p), P(ctypes.c_void_p)],
        "dmsim_compare_states": [H, H, P(d)],
        "dmsim_alloc_host": [ctypes.c_size_t, P(ctypes.c_void_p)],
        "dmsim_free_host": [ctypes.c_void_p],
        "dmsim_cost_collect": [u32, u32, u32, u64, ctypes.c_int, P(d), P(d), u32, P(u32)],
        "dmsim_cost_train": [P(d), P(d), u32, u32, d, u64, P(d)],
        "dmsim_cost_predict": [P(d), u32, P(d)],
        "dmsim_cost_save": [ctypes.c_char_p],
        "dmsim_cost_load": [ctypes.c_char_p],
        "dmsim_mlp_forward": [P(ctypes.c_float), P(ctypes.c_float), u32, P(ctypes.c_float)],
        "dmsim_mlp_grad": [P(ctypes.c_float), P(ctypes.c_float), P(ctypes.c_float), u32, P(ctypes.c_float),
                           P(ctypes.c_float)],
        "dmsim_plan_predicted_ms": [H, P(d)],
        "dmsim_batch_create": [u32, P(u32), P(H)],
        "dmsim_batch_destroy": [H],
        "dmsim_batch_set_option": [H, ctypes.c_int, i64],
        "dmsim_batch_append": [H, u32, ctypes.c_int, P(u32), d, d, d],
        "dmsim_batch_upload": [H],
        "dmsim_batch_run": [H],
        "dmsim_batch_get_diag": [H, u32, P(d)],
        "dmsim_batch_get_zz": [H, u32, P(d)],
        "dmsim_batch_get_dm": [H, u32, P(d), P(d)],
        "dmsim_batch_stats": [H, P(d)],
        "dmsim_batch_autotune": [H, P(d)],
        "dmsim_append_channel": [H, u32, P(u32), u32, P(d)],
        "dmsim_append_noise": [H, ctypes.c_int, P(u32), d],
        "dmsim_probe_rate": [ctypes.c_int, P(d)],
        "dmsim_plan_inspect": [u32, P(ctypes.c_int32), P(u32), P(d), P(d), u32, ctypes.c_int, ctypes.c_int,
                               ctypes.c_int, P(d), u32, P(u32)],
    }
    for name, args in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = ctypes.c_int
    L.dmsim_last_error.argtypes = [H]
    L.dmsim_last_error.restype = ctypes.c_char_p
    L.dmsim_batch_last_error.argtypes = [H]
    L.dmsim_batch_last_error.restype = ctypes.c_char_p
    L.dmsim_status_string.argtypes = [ctypes.c_int]
    L.dmsim_status_string.restype = ctypes.c_char_p
    _lib = L
    return L


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class Simulation:
    """One density matrix on the current CUDA device.

    ``precision`` is "fp64" or "c64"; ``mode`` is "plain" (one pass per basic
    gate, the reference's method) or "fused"; ``planner`` is "greedy" or
    "learned" (fused mode only); ``tensor`` runs 3- and 4-qubit dense passes
    on the tensor cores (True: where the planner's rule or cost model picks
    them, "all" or 2: every eligible pass, False: none); ``fused_arith`` and
    ``plain_arith`` are "fp64" (FP64 width, the default) or "df64"
    (double-float, 48-bit significands, faster).
    """

    def __init__(self, n_qubits, n_gpus=1, precision="fp64", mode="plain", max_k=4, planner="greedy",
                 graph=True, fused_arith="fp64", renorm=64, plain_arith="fp64", tensor=True, direct1=True):
        self._h = ctypes.c_void_p()
        self.n = int(n_qubits)
        st = lib().dmsim_create(self.n, int(n_gpus), ctypes.byref(self._h))
        if st != OK:
            raise DMSimError(st, lib().dmsim_status_string(st).decode())
        try:
            self.set_option(OPT_PRECISION, 1 if precision == "c64" else 0)
            self.set_option(OPT_MODE, 1 if mode == "fused" else 0)
            self.set_option(OPT_MAX_K, int(max_k))
            self.set_option(OPT_PLANNER, 1 if planner == "learned" else 0)
            self.set_option(OPT_GRAPH, 1 if graph else 0)
            self.set_option(OPT_FUSED_ARITH, 1 if fused_arith == "df64" else 0)
            self.set_option(OPT_RENORM, int(renorm))
            self.set_option(OPT_PLAIN_ARITH, 1 if plain_arith == "df64" else 0)
            self.set_option(OPT_TENSOR, 2 if tensor == "all" else int(tensor))
            self.set_option(OPT_DIRECT1, 1 if direct1 else 0)
        except Exception:
            self.close()
            raise

    # -- plumbing
    def _check(self, st):
        if st != OK:
            raise DMSimError(st, lib().dmsim_last_error(self._h).decode())

    def close(self):
        if self._h:
            lib().dmsim_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_option(self, key, value):
        self._check(lib().dmsim_set_option(self._h, key, int(value)))

    def get_option(self, key):
        v = ctypes.c_int64()
        self._check(lib().dmsim_get_option(self._h, key, ctypes.byref(v)))
        return v.value

    # -- circuit
    def append(self, op, qubits, theta=0.0, phi=0.0, lam=0.0):
        q = list(qubits) + [0] * (5 - len(qubits))
        self._check(lib().dmsim_append(self._h, int(op), (ctypes.c_uint32 * 5)(*q), theta, phi, lam))

    def append_c1(self, q, m):
        m = np.asarray(m, dtype=np.complex128).reshape(4)
        flat = np.empty(8)
        flat[0::2], flat[1::2] = m.real, m.imag
        self._check(lib().dmsim_append_c1(self._h, int(q), _dp(flat)))

    def append_c2(self, q1, q2, m):
        m = np.asarray(m, dtype=np.complex128).reshape(16)
        flat = np.empty(32)
        flat[0::2], flat[1::2] = m.real, m.imag
        self._check(lib().dmsim_append_c2(self._h, int(q1), int(q2), _dp(flat)))

    def append_channel(self, qubits, kraus):
        """rho -> sum_i K_i rho K_i^+ on 1 or 2 qubits (2-qubit matrices in the
        C2 basis order, index 2*bit(qubits[0]) + bit(qubits[1]))."""
        qs = list(qubits)
        k = np.asarray(kraus, dtype=np.complex128).reshape(len(kraus), -1)
        flat = np.empty(2 * k.size)
        flat[0::2], flat[1::2] = k.real.ravel(), k.imag.ravel()
        q = (ctypes.c_uint32 * 2)(*(qs + [0] * (2 - len(qs))))
        self._check(lib().dmsim_append_channel(self._h, len(qs), q, len(k), _dp(flat)))

    def append_noise(self, kind, qubits, p):
        """A named channel: depolarizing, amplitude_damping, phase_damping,
        bit_flip, phase_flip (one qubit) or depolarizing2 (two qubits)."""
        qs = list(qubits)
        q = (ctypes.c_uint32 * 2)(*(qs + [0] * (2 - len(qs))))
        self._check(lib().dmsim_append_noise(self._h, NOISE[kind], q, float(p)))

    def extend(self, circuit):
        for g in circuit:
            self.append(g[0], g[1], g[2], g[3], g[4])

    def upload(self):
        self._check(lib().dmsim_upload(self._h))

    def run(self):
        self._check(lib().dmsim_run(self._h))

    def clear_circuit(self):
        self._check(lib().dmsim_clear_circuit(self._h))

    def reset(self):
        self._check(lib().dmsim_reset(self._h))

    def reset_dm(self):
        self._check(lib().dmsim_reset_dm(self._h))

    # -- results
    def measure(self, rep=10, uniforms=None):
        out = np.zeros(rep, dtype=np.uint64)
        up = None
        if uniforms is not None:
            u = np.ascontiguousarray(uniforms, dtype=np.float64)
            assert len(u) == rep
            up = _dp(u)
        self._check(lib().dmsim_measure(self._h, rep, up, out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))))
        return [int(x) for x in out]

    def get_dm(self):
        N = 1 << (2 * self.n)
        re, im = np.empty(N), np.empty(N)
        self._check(lib().dmsim_get_dm(self._h, _dp(re), _dp(im)))
        return re, im

    def set_dm(self, re, im):
        re = np.ascontiguousarray(re, dtype=np.float64)
        im = np.ascontiguousarray(im, dtype=np.float64)
        assert re.size == 1 << (2 * self.n) and im.size == re.size
        self._check(lib().dmsim_set_dm(self._h, _dp(re), _dp(im)))

    def get_diag(self):
        d = np.empty(1 << self.n)
        self._check(lib().dmsim_get_diag(self._h, _dp(d)))
        return d

    def rho(self):
        """rho as a complex (2^n x 2^n) matrix: rho[r][c] = A[c*2^n + r]."""
        re, im = self.get_dm()
        d = 1 << self.n
        return (re.reshape(d, d) + 1j * im.reshape(d, d)).T

    def dump(self):
        need = ctypes.c_size_t()
        self._check(lib().dmsim_dump(self._h, None, 0, ctypes.byref(need)))
        buf = ctypes.create_string_buffer(need.value)
        self._check(lib().dmsim_dump(self._h, buf, need.value, None))
        return buf.value.decode()

    def n_gates(self):
        v = ctypes.c_uint32()
        self._check(lib().dmsim_n_gates(self._h, ctypes.byref(v)))
        return v.value

    def plan_stats(self):
        a, b = ctypes.c_uint32(), ctypes.c_uint32()
        self._check(lib().dmsim_plan_stats(self._h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def upload_bytes(self):
        v = ctypes.c_uint64()
        self._check(lib().dmsim_upload_bytes(self._h, ctypes.byref(v)))
        return v.value

    def last_timings(self):
        o = np.zeros(3)
        self._check(lib().dmsim_last_timings(self._h, _dp(o)))
        return {"ms": o[0], "passes": int(o[1]), "bytes": o[2]}

    def pass_records(self):
        cnt = ctypes.c_uint32()
        self._check(lib().dmsim_pass_records(self._h, None, 0, ctypes.byref(cnt)))
        out = np.zeros((cnt.value, PASS_RECORD))
        if cnt.value:
            self._check(lib().dmsim_pass_records(self._h, _dp(out), cnt.value, ctypes.byref(cnt)))
        return out

    def pure_metrics(self, psi):
        psi = np.asarray(psi, dtype=np.complex128)
        pr, pi = np.ascontiguousarray(psi.real), np.ascontiguousarray(psi.imag)
        o = np.zeros(4)
        self._check(lib().dmsim_pure_metrics(self._h, _dp(pr), _dp(pi), _dp(o)))
        return {"fidelity": o[0], "trace": o[1], "max_abs_err": o[2], "frob_err": o[3]}

    def compare(self, other):
        """max |A - B| and ||A - B||_F between this state and another, on the device."""
        o = np.zeros(2)
        self._check(lib().dmsim_compare_states(self._h, other._h, _dp(o)))
        return {"max_abs_err": o[0], "frob_err": o[1]}

    def get_dm_into(self, re, im):
        """Copy rho into caller-provided float64 buffers (e.g. PinnedBuffer arrays)."""
        self._check(lib().dmsim_get_dm(self._h, _dp(re), _dp(im)))

    def predicted_ms(self):
        v = ctypes.c_double()
        self._check(lib().dmsim_plan_predicted_ms(self._h, ctypes.byref(v)))
        return v.value

    def device_state(self):
        re, im = ctypes.c_void_p(), ctypes.c_void_p()
        self._check(lib().dmsim_device_state(self._h, ctypes.byref(re), ctypes.byref(im)))
        return re.value, im.value


PASS_REC = 1040


def plan_inspect(n, circuit, mode="fused", max_k=4, planner="greedy"):
    """Plan a circuit on the host only (no GPU): list of passes with their
    width, class, qubits and operator, as dmsim_upload would build them.

    ``circuit`` holds (op, qubits, theta, phi, lam[, matrix]) tuples."""
    m = len(circuit)
    ops = np.zeros(max(m, 1), dtype=np.int32)
    qs = np.zeros(5 * max(m, 1), dtype=np.uint32)
    ps = np.zeros(3 * max(m, 1))
    mats = np.zeros(32 * max(m, 1))
    for i, g in enumerate(circuit):
        ops[i] = g[0]
        for k, q in enumerate(g[1]):
            qs[5 * i + k] = q
        ps[3 * i:3 * i + 3] = g[2], g[3], g[4]
        if len(g) > 5 and g[5] is not None:
            mm = np.asarray(g[5], dtype=np.complex128).reshape(-1)
            mats[32 * i:32 * i + 2 * mm.size:2] = mm.real
            mats[32 * i + 1:32 * i + 2 * mm.size:2] = mm.imag
    L = lib()
    P = ctypes.POINTER
    cnt = ctypes.c_uint32()
    args = (n, ops.ctypes.data_as(P(ctypes.c_int32)), qs.ctypes.data_as(P(ctypes.c_uint32)), _dp(ps), _dp(mats), m,
            1 if mode == "fused" else 0, int(max_k), 1 if planner == "learned" else 0)
    st = L.dmsim_plan_inspect(*args, None, 0, ctypes.byref(cnt))
    if st != OK:
        raise DMSimError(st, L.dmsim_status_string(st).decode())
    out = np.zeros((max(cnt.value, 1), PASS_REC))
    st = L.dmsim_plan_inspect(*args, _dp(out), cnt.value, ctypes.byref(cnt))
    if st != OK:
        raise DMSimError(st, L.dmsim_status_string(st).decode())
    passes = []
    for r in out[:cnt.value]:
        K = int(r[0])
        D = 1 << K
        rec = {"K": K, "cls": CLASS_NAMES[int(r[1])], "nbasic": int(r[2]), "nnz": int(r[3]),
               "qubits": [int(x) for x in r[4:4 + K]], "ket_only": bool(r[8]), "transpose": bool(r[9]),
               "tensor": bool(r[10])}
        if rec["transpose"]:
            rec["cls"] = "TRANSPOSE"
        elif rec["cls"] == "RLIN":
            rec["rl"] = r[16:32].reshape(4, 4).copy()
            rec["rlb"] = r[528:544].reshape(4, 4).copy()
        else:
            u = r[16:16 + 2 * D * D]
            v = r[528:528 + 2 * D * D]
            rec["U"] = (u[0::2] + 1j * u[1::2]).reshape(D, D)
            rec["V"] = (v[0::2] + 1j * v[1::2]).reshape(D, D)
        passes.append(rec)
    return passes


class PinnedBuffer:
    """A page-locked host float64 array (cudaHostAlloc) for fast copies."""

    def __init__(self, count):
        self._p = ctypes.c_void_p()
        st = lib().dmsim_alloc_host(int(count) * 8, ctypes.byref(self._p))
        if st != OK:
            raise DMSimError(st, "pinned host allocation failed")
        self.array = np.ctypeslib.as_array(ctypes.cast(self._p, ctypes.POINTER(ctypes.c_double)), shape=(int(count),))

    def close(self):
        if self._p:
            self.array = None
            lib().dmsim_free_host(self._p)
            self._p = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------- cost model
COST_FEATURES = 17
MLP_PARAMS = 1665


def _fp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def _ok(st, what):
    if st != OK:
        raise DMSimError(st, f"{what}: {lib().dmsim_status_string(st).decode()}")


def cost_collect(n, n_circuits=2, gates=60, seed=0, arith=AR_DF64, cap=200000):
    """Per-pass (features, ms) samples the engine records on its own random
    circuits under several fusion plans, timed with CUDA events on the GPU,
    in the given arithmetic (AR_FP64 or AR_DF64)."""
    feats = np.zeros((cap, COST_FEATURES))
    ms = np.zeros(cap)
    cnt = ctypes.c_uint32()
    _ok(lib().dmsim_cost_collect(n, n_circuits, gates, seed, arith, _dp(feats), _dp(ms), cap, ctypes.byref(cnt)),
        "cost_collect")
    k = min(cnt.value, cap)
    return feats[:k].copy(), ms[:k].copy()


def cost_train(feats, ms, steps=3000, lr=3e-3, seed=1):
    feats = np.ascontiguousarray(feats, dtype=np.float64)
    ms = np.ascontiguousarray(ms, dtype=np.float64)
    loss = np.zeros(2)
    _ok(lib().dmsim_cost_train(_dp(feats), _dp(ms), len(ms), steps, lr, seed, _dp(loss)), "cost_train")
    return loss


def cost_predict(feats):
    feats = np.ascontiguousarray(feats, dtype=np.float64)
    out = np.zeros(len(feats))
    _ok(lib().dmsim_cost_predict(_dp(feats), len(feats), _dp(out)), "cost_predict")
    return out


def cost_save(path):
    _ok(lib().dmsim_cost_save(path.encode()), "cost_save")


def cost_load(path):
    _ok(lib().dmsim_cost_load(path.encode()), "cost_load")


def cost_load_default():
    """Reload the model the library ships with ($DMSIM_COST_MODEL, else
    dm-sim_gb300/model/cost_mlp.bin), e.g. after training another one."""
    path = os.environ.get("DMSIM_COST_MODEL") or os.path.normpath(os.path.join(_HERE, "..", "model", "cost_mlp.bin"))
    cost_load(path)


def mlp_forward(params, X):
    params = np.ascontiguousarray(params, dtype=np.float32)
    X = np.ascontiguousarray(X, dtype=np.float32)
    y = np.zeros(len(X), dtype=np.float32)
    _ok(lib().dmsim_mlp_forward(_fp(params), _fp(X), len(X), _fp(y)), "mlp_forward")
    return y


def mlp_grad(params, X, T):
    params = np.ascontiguousarray(params, dtype=np.float32)
    X = np.ascontiguousarray(X, dtype=np.float32)
    T = np.ascontiguousarray(T, dtype=np.float32)
    g = np.zeros(MLP_PARAMS, dtype=np.float32)
    loss = np.zeros(1, dtype=np.float32)
    _ok(lib().dmsim_mlp_grad(_fp(params), _fp(X), _fp(T), len(X), _fp(g), _fp(loss)), "mlp_grad")
    return g, float(loss[0])


PROBES = ["fp64_fma", "fp32_fma", "dmma_flops", "int_lop3", "int_add", "int_shf", "int_prmt", "int_mad",
          "cvt_s64_to_f64", "cvt_f32_f64", "cvt_f32_s32", "mix_fadd_lop3"]


def probe_rates():
    """Execution-unit throughputs of the current GPU (dmsim_probe_rate):
    {probe name: operations per second}."""
    out = {}
    for i, name in enumerate(PROBES):
        v = ctypes.c_double()
        _ok(lib().dmsim_probe_rate(i, ctypes.byref(v)), "dmsim_probe_rate")
        out[name] = v.value
    return out


class Batch:
    """Many independent circuits (1..16 qubits each, uneven counts allowed),
    each from |0..0><0..0|, run together from one captured CUDA graph: the
    circuits below ``wide_qubits`` (default 10) by one persistent work-queue
    kernel, each wider one by the engine's own pass kernels on a concurrent
    branch.  Outputs per circuit: the diagonal and <Z_i Z_{i+1}>."""

    def __init__(self, n_qubits_list, mode="fused", max_k=4, planner="greedy", wait_limit=None, test_stall=False,
                 fused_arith="fp64", wide_qubits=None):
        self.nq = [int(x) for x in n_qubits_list]
        self._h = ctypes.c_void_p()
        arr = (ctypes.c_uint32 * len(self.nq))(*self.nq)
        st = lib().dmsim_batch_create(len(self.nq), arr, ctypes.byref(self._h))
        if st != OK:
            raise DMSimError(st, lib().dmsim_status_string(st).decode())
        self._check(lib().dmsim_batch_set_option(self._h, OPT_MODE, 1 if mode == "fused" else 0))
        self._check(lib().dmsim_batch_set_option(self._h, OPT_MAX_K, int(max_k)))
        self._check(lib().dmsim_batch_set_option(self._h, OPT_PLANNER, 1 if planner == "learned" else 0))
        if wait_limit is not None:
            self._check(lib().dmsim_batch_set_option(self._h, BATCH_OPT_WAIT_LIMIT, int(wait_limit)))
        if test_stall:
            self._check(lib().dmsim_batch_set_option(self._h, BATCH_OPT_TEST_STALL, 1))
        self._check(lib().dmsim_batch_set_option(self._h, OPT_FUSED_ARITH, 1 if fused_arith == "df64" else 0))
        if wide_qubits is not None:
            self._check(lib().dmsim_batch_set_option(self._h, BATCH_OPT_WIDE_QUBITS, int(wide_qubits)))

    def _check(self, st):
        if st != OK:
            raise DMSimError(st, lib().dmsim_batch_last_error(self._h).decode())

    def close(self):
        if self._h:
            lib().dmsim_batch_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def append(self, c, op, qubits, theta=0.0, phi=0.0, lam=0.0):
        q = list(qubits) + [0] * (5 - len(qubits))
        self._check(lib().dmsim_batch_append(self._h, c, int(op), (ctypes.c_uint32 * 5)(*q), theta, phi, lam))

    def extend(self, c, circuit):
        for g in circuit:
            self.append(c, g[0], g[1], g[2], g[3], g[4])

    def upload(self):
        self._check(lib().dmsim_batch_upload(self._h))

    def run(self):
        self._check(lib().dmsim_batch_run(self._h))

    def diag(self, c):
        out = np.zeros(1 << self.nq[c])
        self._check(lib().dmsim_batch_get_diag(self._h, c, _dp(out)))
        return out

    def zz(self, c):
        out = np.zeros(max(self.nq[c] - 1, 1))
        self._check(lib().dmsim_batch_get_zz(self._h, c, _dp(out)))
        return out[:max(self.nq[c] - 1, 0)]

    def dm(self, c):
        N = 1 << (2 * self.nq[c])
        re, im = np.zeros(N), np.zeros(N)
        self._check(lib().dmsim_batch_get_dm(self._h, c, _dp(re), _dp(im)))
        return re, im

    def stats(self):
        o = np.zeros(8)
        self._check(lib().dmsim_batch_stats(self._h, _dp(o)))
        return {"ms": o[0], "passes": int(o[1]), "basic": int(o[2]), "items": int(o[3]), "bytes": o[4],
                "grid": int(o[5]), "small_n": int(o[6]), "g_shift": int(o[7])}

    def autotune(self):
        """Pick the tile shape (groups per tile of the small circuits) by timing."""
        v = ctypes.c_double()
        self._check(lib().dmsim_batch_autotune(self._h, ctypes.byref(v)))
        return v.value
