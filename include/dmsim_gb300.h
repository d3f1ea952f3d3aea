/*
 * dmsim_gb300.h -- C ABI of the GB300 density-matrix gate engine.
 *
 * Plain pointers and sizes only; every call returns a status code (0 = ok)
 * and never exits the process.  One handle owns one density matrix on the
 * current CUDA device and one CUDA stream; calls on one handle must be
 * serialised by the caller (the reference object is not thread-safe either).
 *
 * Each entry point replaces a member of DM-Sim's Simulation class
 * (src/dmsim_nvgpu_omp.cuh in pnnl/DM-Sim); the citation is given per entry.
 */
#ifndef DMSIM_GB300_H
#define DMSIM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct dmsim_sim* dmsim_handle;

enum dmsim_status {
  DMSIM_OK = 0,
  DMSIM_ERR_ARG = 1,          /* bad qubit index, unknown gate id, null pointer, bad size */
  DMSIM_ERR_STATE = 2,        /* call out of order (upload twice, run before upload) */
  DMSIM_ERR_OOM = 3,          /* device or pinned host allocation failed */
  DMSIM_ERR_CUDA = 4,         /* CUDA runtime error (message in dmsim_last_error) */
  DMSIM_ERR_TIMEOUT = 5,      /* a bounded device wait ran out; the run's results are undefined (a
                                 single-circuit handle's rho must be reset or set before further use) */
  DMSIM_ERR_UNSUPPORTED = 6   /* e.g. n_gpus != 1: this engine is single-GPU */
};

/* Runtime options (dmsim_set_option).  Defaults in brackets. */
enum dmsim_option {
  DMSIM_OPT_MODE = 1,       /* 0 = plain gate-by-gate [0], 1 = fused */
  DMSIM_OPT_PRECISION = 2,  /* 0 = FP64 [0], 1 = complex64 (FP32 passes, FP64 reductions); set before the first append */
  DMSIM_OPT_MAX_K = 3,      /* widest fused operator, 1..4 [4] */
  DMSIM_OPT_PLANNER = 4,    /* 0 = greedy fixed width [0], 1 = learned cost model */
  DMSIM_OPT_RECORD = 5,     /* 1 = time every pass of the next runs (no graph) [0] */
  DMSIM_OPT_SEED = 6,       /* seed of measure() without uniforms; -1 = time(0) like the reference [-1] */
  DMSIM_OPT_GRAPH = 7,      /* 1 = replay uploaded circuits from a captured CUDA graph [1] */
  DMSIM_OPT_VERBOSE = 8,    /* 1 = print the reference's per-run timing banner [0] */
  DMSIM_OPT_FUSED_ARITH = 9, /* fused FP64 runs: 0 = FP64 width [0] (3/4-qubit passes on the tensor cores with
                                 7 BF16 digits per operand and exact integer sums, the rest in FP64), 1 = double-float
                                 passes on the FP32 pipe and tensor cores (48-bit significands) */
  DMSIM_OPT_RENORM = 10,     /* complex64: FP64 trace + Hermitian renormalisation every R passes and at the end [64]; 0 = off */
  DMSIM_OPT_PLAIN_ARITH = 11, /* plain FP64 runs (FP64 state at rest): 0 = FP64 passes [0] (dense passes bound by
                                 GB300's FP64 pipe), 1 = double-float passes on the FP32 pipe (HBM-bound) */
  DMSIM_OPT_TENSOR = 12,      /* 3- and 4-qubit dense/sparse passes on the tensor cores (BF16 digits): 1 =
                                 where the learned planner picks them, else every eligible pass of an
                                 FP64-width run, the 4-qubit passes of a complex64 run (BF16 x 3 split, FP32
                                 accumulation) and, in double-float runs, passes above a density rule [1];
                                 0 = never; 2 = every eligible pass */
  DMSIM_OPT_DIRECT1 = 13      /* 1 = 1-qubit move/sign/phase/dense passes on the register kernel (no shared-memory
                                 tiles) [1], 0 = the tiled kernel */
};

/* Gate ids: the order of enum OP, src/dmsim_nvgpu_omp.cuh:42-48 (ABI). */
enum dmsim_op {
  DMSIM_U3 = 0, DMSIM_U2, DMSIM_U1, DMSIM_CX, DMSIM_ID, DMSIM_X, DMSIM_Y, DMSIM_Z, DMSIM_H, DMSIM_S,
  DMSIM_SDG, DMSIM_T, DMSIM_TDG, DMSIM_RX, DMSIM_RY, DMSIM_RZ, DMSIM_CZ, DMSIM_CY, DMSIM_SWAP, DMSIM_CH,
  DMSIM_CCX, DMSIM_CSWAP, DMSIM_CRX, DMSIM_CRY, DMSIM_CRZ, DMSIM_CU1, DMSIM_CU3, DMSIM_RXX, DMSIM_RZZ, DMSIM_RCCX,
  DMSIM_RC3X, DMSIM_C3X, DMSIM_C3SQRTX, DMSIM_C4X, DMSIM_R, DMSIM_SRN, DMSIM_W, DMSIM_RYY,
  DMSIM_N_OPS
};

/* Simulation(n_qubits, n_gpus) -- src/dmsim_nvgpu_omp.cuh:196-271.  Allocates
 * rho = |0..0><0..0| on the current device.  n_gpus must be 1. */
int dmsim_create(uint32_t n_qubits, uint32_t n_gpus, dmsim_handle* out);
/* ~Simulation() -- :273-301 */
int dmsim_destroy(dmsim_handle h);
int dmsim_set_option(dmsim_handle h, int key, int64_t value);
int dmsim_get_option(dmsim_handle h, int key, int64_t* value);

/* append(Gate*) -- :331-344, with the Gate fields of :99-191 (op, qb0..qb4,
 * theta, phi, lambda).  Qubits must be < n_qubits and distinct where the gate
 * uses them. */
int dmsim_append(dmsim_handle h, int op, const uint32_t qb[5], double theta, double phi, double lambda);
/* Arbitrary 1-qubit gate (README "C1"; element formulas of C1_GATE :1004-1025).
 * m = 2x2 complex, row-major, re/im interleaved (8 doubles). */
int dmsim_append_c1(dmsim_handle h, uint32_t q, const double m[8]);
/* Arbitrary 2-qubit gate (README "C2"; C2_GATE :1028-1122): m = 4x4 complex,
 * row-major, re/im interleaved (32 doubles), basis index 2*bit(q1) + bit(q2). */
int dmsim_append_c2(dmsim_handle h, uint32_t q1, uint32_t q2, const double m[32]);
/* Noise channel (no counterpart in the reference, which has no noise):
 * rho -> sum_i K_i rho K_i^+ on nq = 1 or 2 qubits q[0..nq-1]; kraus holds
 * n_kraus (<= 16) matrices of 2^nq x 2^nq complex, row-major, re/im
 * interleaved, 2-qubit ones in the C2 basis order (index 2*bit(q[0]) +
 * bit(q[1])).  Applied as one superoperator pass; a fusion barrier. */
int dmsim_append_channel(dmsim_handle h, uint32_t nq, const uint32_t q[2], uint32_t n_kraus, const double* kraus);
enum dmsim_noise {
  DMSIM_NOISE_DEPOLARIZING = 0,       /* rho -> (1-p) rho + p I/2 */
  DMSIM_NOISE_AMPLITUDE_DAMPING = 1,  /* gamma = p */
  DMSIM_NOISE_PHASE_DAMPING = 2,      /* lambda = p */
  DMSIM_NOISE_BIT_FLIP = 3,           /* X with probability p */
  DMSIM_NOISE_PHASE_FLIP = 4,         /* Z with probability p */
  DMSIM_NOISE_DEPOLARIZING2 = 5       /* two qubits: rho -> (1-p) rho + p I/4 */
};
/* A named channel of strength p in [0, 1] on q[0] (and q[1] for the 2-qubit kind). */
int dmsim_append_noise(dmsim_handle h, int kind, const uint32_t q[2], double p);
/* upload() -- :345-377.  Plans the passes and copies them to the device once. */
int dmsim_upload(dmsim_handle h);
/* sim() -- :390-494, without the copy of rho to the host (dmsim_get_dm). */
int dmsim_run(dmsim_handle h);
/* clear_circuit() -- :496-520.  rho is kept (chained circuits). */
int dmsim_clear_circuit(dmsim_handle h);
/* reset() -- :303-307: clear_circuit + reset_dm */
int dmsim_reset(dmsim_handle h);
/* reset_dm() -- :308-329: rho = |0..0><0..0| */
int dmsim_reset_dm(dmsim_handle h);
/* measure(rep) -- :521-549.  uniforms[rep] replace rand()/RAND_MAX when not
 * NULL; otherwise srand(seed option) + rand() as the reference.  out[rep].
 * The probability prefix is the reference's sequential FP64 sum. */
int dmsim_measure(dmsim_handle h, uint32_t rep, const double* uniforms, uint64_t* out);
/* dm_real_res / dm_imag_res -- :456-459, :790-791: re[i*dim+j] + i*im[i*dim+j]
 * = rho[j][i].  Buffers hold 4^n doubles each. */
int dmsim_get_dm(dmsim_handle h, double* re, double* im);
/* Load rho from host buffers in the same layout. */
int dmsim_set_dm(dmsim_handle h, const double* re, const double* im);
/* diag[i] = Re rho[i][i], 2^n doubles */
int dmsim_get_diag(dmsim_handle h, double* diag);
/* dump() -- :379-387: one line per gate; returns the length needed (incl. NUL). */
int dmsim_dump(dmsim_handle h, char* buf, size_t len, size_t* needed);
int dmsim_n_qubits(dmsim_handle h, uint32_t* n);
int dmsim_n_gates(dmsim_handle h, uint32_t* n);
/* Passes of the uploaded plan and basic gates they replace. */
int dmsim_plan_stats(dmsim_handle h, uint32_t* n_passes, uint32_t* n_basic);
/* Bytes the last upload() copied to the device (the pass descriptors) */
int dmsim_upload_bytes(dmsim_handle h, uint64_t* bytes);
/* Timing of the last run: out[0] = ms, out[1] = passes, out[2] = bytes moved (algorithmic) */
int dmsim_last_timings(dmsim_handle h, double out[3]);
/* Per-pass records of the last recorded run (DMSIM_OPT_RECORD): for each pass
 * DMSIM_PASS_RECORD doubles {K, class, nnz, max_lo_bit, min_hi_bit, n, ms,
 * bytes, tensor (1: ran on the tensor cores), blocks launched}.  Passes
 * that apply no gates have K = 0 and class 16 (FP64 <-> double-float
 * conversion), 17 (conjugate transpose) or 18 (complex64 renormalisation). */
#define DMSIM_PASS_RECORD 10
int dmsim_pass_records(dmsim_handle h, double* out, uint32_t cap, uint32_t* count);
/* Compare rho with a pure state psi (2^n complex, FP64) on the device:
 * out[0] = fidelity <psi|rho|psi>, out[1] = trace, out[2] = max |rho - psi psi^+|,
 * out[3] = ||rho - psi psi^+||_F. */
int dmsim_pure_metrics(dmsim_handle h, const double* psi_re, const double* psi_im, double out[4]);
/* dmsim_pure_metrics without any allocation.  No counterpart in the reference.
 * For callers that cannot call cudaMalloc: processes whose device memory is
 * already reserved by another allocator (a framework's caching pool), and
 * monitoring loops that must not stall running work on cudaMalloc/cudaFree's
 * implicit synchronisation.  psi is staged in a 1 MiB array fixed in the
 * library's device image (every GPU that loads the library holds it until the
 * process exits), so states are limited to 16 qubits (2^16 amplitudes); larger
 * states get DMSIM_ERR_ARG with a message.  The first call on a device looks
 * up the array's address on that device: make it before any stream capture.
 * Every call reuses the same array (the accumulators are cleared each call,
 * psi is overwritten), so calls that overlap on the GPU -- from two threads or
 * two handles on the same device -- race; serialise them.  Same outputs as
 * dmsim_pure_metrics; rho must already be allocated (DMSIM_ERR_STATE if not).
 * The array's address is looked up once per device and kept for the life of
 * the process: do not call this entry point after cudaDeviceReset (or any
 * other teardown of the device's primary context) in the same process. */
int dmsim_pure_metrics_noalloc(dmsim_handle h, const double* psi_re, const double* psi_im, double out[4]);
/* Compare two states of the same size on the device (either precision, e.g.
 * a complex64 state against an FP64 one): out[0] = max |A - B| over entries,
 * out[1] = ||A - B||_F. */
int dmsim_compare_states(dmsim_handle a, dmsim_handle b, double out[2]);
/* Page-locked host buffers for fast dmsim_get_dm / dmsim_set_dm copies. */
int dmsim_alloc_host(size_t bytes, void** out);
int dmsim_free_host(void* p);
/* Host-only planning (no GPU needed): decompose and plan a circuit exactly as
 * dmsim_upload would and return, per pass, DMSIM_PASS_REC doubles:
 * [0..7] {K, class, n_basic, nnz, q0, q1, q2, q3}, [8] ket-only flag,
 * [9] transpose flag (the reference-order adjoint stage, no operator),
 * [10] tensor-core flag (a fused double-float run with DMSIM_OPT_TENSOR = 1
 * would run the pass on the tensor cores), [16..527] the ket operator U and [528..1039] the bra operator V (16x16
 * complex, re/im interleaved, row stride 2^K; for the real-linear class the
 * 4x4 real ket and bra maps).  ops[i], qubits[5*i..], params[3*i..] = theta,
 * phi, lambda; mats[32*i..] holds C1/C2 matrices (may be NULL when there are
 * none).  Returns the pass count in *npasses. */
#define DMSIM_PASS_REC 1040
int dmsim_plan_inspect(uint32_t n_qubits, const int32_t* ops, const uint32_t* qubits, const double* params,
                       const double* mats, uint32_t ngates, int mode, int max_k, int planner,
                       double* out, uint32_t cap, uint32_t* npasses);
/* ---- learned pass-time model (process-wide) --------------------------------
 * Features: DMSIM_COST_FEATURES doubles per pass (width, class, density,
 * touched fractions, target-bit positions, size, precision, tensor cores).
 * dmsim_cost_collect: run the engine's own random circuits (29-entry mixed
 * table, n qubits, mt19937_64 from seed) under several fusion plans on the
 * current GPU in the given arithmetic (0 FP64, 1 FP32 on a complex64 state,
 * 2 double-float), timing every
 * pass with CUDA events; writes up to cap samples and the total count.  dmsim_cost_train: fit the network on the GPU (Adam,
 * full batch, steps, lr, weights seeded by seed); loss[0..1] = first / last
 * mean squared error of standardised log time.  dmsim_cost_predict: GPU
 * inference, ms per sample.  save / load: the weights file. */
#define DMSIM_COST_FEATURES 17
int dmsim_cost_collect(uint32_t n, uint32_t n_circuits, uint32_t gates, uint64_t seed, int arith, double* feats,
                       double* ms, uint32_t cap, uint32_t* count);
int dmsim_cost_train(const double* feats, const double* ms, uint32_t count, uint32_t steps, double lr, uint64_t seed,
                     double loss[2]);
int dmsim_cost_predict(const double* feats, uint32_t count, double* out_ms);
int dmsim_cost_save(const char* path);
int dmsim_cost_load(const char* path);
/* The network's forward pass and its loss gradient on the GPU for given
 * parameters (DMSIM_MLP_PARAMS floats) -- the hooks the gradient check uses. */
#define DMSIM_MLP_PARAMS 1665
int dmsim_mlp_forward(const float* params, const float* X, uint32_t B, float* y);
int dmsim_mlp_grad(const float* params, const float* X, const float* T, uint32_t B, float* grad, float* loss);
/* Predicted run time of the uploaded plan (learned planner), ms */
int dmsim_plan_predicted_ms(dmsim_handle h, double* ms);
/* ---- batched sweep: many independent circuits in one captured graph -------
 * Circuits of 1..16 qubits (uneven counts allowed), each from |0..0><0..0|,
 * planned like single circuits (DMSIM_OPT_MODE / MAX_K / PLANNER /
 * FUSED_ARITH via dmsim_batch_set_option), run from one captured CUDA graph:
 * the narrow circuits (fewer than DMSIM_BATCH_OPT_WIDE_QUBITS qubits) by one
 * persistent work-queue kernel, each wide circuit by the engine's own pass
 * kernels on a concurrent branch.  Outputs per circuit: the diagonal (2^n)
 * and <Z_i Z_{i+1}> for i < n-1.  stats: {ms of the last run, passes, basic
 * gates, work items of the queue, algorithmic bytes, queue grid, tile-shape
 * small_n, g_shift}.  No reference counterpart: the reference runs circuits
 * one Simulation at a time. */
typedef struct dmsim_batch* dmsim_batch_handle;
/* Batch-only options: the polls (128 ns naps) after which a work-queue
 * dependency wait gives up [2^25, ~4 s] -- the kernel then sets an error flag,
 * skips the item and finishes, and dmsim_batch_run returns
 * DMSIM_ERR_TIMEOUT with every output of that run (diagonals, <ZZ>, states)
 * set to NaN -- and a test hook that makes the last pass of circuit 0
 * wait for one tile more than its predecessor has, so that its waits run
 * out (failure detection without a GPU fault). */
enum { DMSIM_BATCH_OPT_WAIT_LIMIT = 100, DMSIM_BATCH_OPT_TEST_STALL = 101,
       /* circuits of at least this many qubits run on the engine's own pass kernels (tensor-core passes
          included), as concurrent branches of the batch's graph; the rest share the work-queue kernel [10] */
       DMSIM_BATCH_OPT_WIDE_QUBITS = 102 };
int dmsim_batch_create(uint32_t n_circuits, const uint32_t* n_qubits, dmsim_batch_handle* out);
int dmsim_batch_destroy(dmsim_batch_handle b);
int dmsim_batch_set_option(dmsim_batch_handle b, int key, int64_t value);
int dmsim_batch_append(dmsim_batch_handle b, uint32_t circuit, int op, const uint32_t qb[5], double theta, double phi,
                       double lambda);
int dmsim_batch_upload(dmsim_batch_handle b);
int dmsim_batch_run(dmsim_batch_handle b);
int dmsim_batch_get_diag(dmsim_batch_handle b, uint32_t circuit, double* out);
int dmsim_batch_get_zz(dmsim_batch_handle b, uint32_t circuit, double* out);
int dmsim_batch_get_dm(dmsim_batch_handle b, uint32_t circuit, double* re, double* im);
/* The autotuner: times the uploaded batch under a few choices of the wide
 * circuits' threshold and of the queue's tile shape (fewer groups per tile
 * for its smallest circuits) and keeps the fastest. */
int dmsim_batch_autotune(dmsim_batch_handle b, double* best_ms);
int dmsim_batch_stats(dmsim_batch_handle b, double out[8]);
const char* dmsim_batch_last_error(dmsim_batch_handle b);
/* ---- execution-unit throughput probes (no counterpart in the reference) ----
 * The measurements behind the kernels' choice of arithmetic on this GPU: each
 * probe runs fixed-length independent chains of one instruction kind on 8
 * blocks of 256 threads per SM of the current device and returns operations
 * per second (instructions, or FLOPs for the FP64 MMA). */
enum dmsim_probe {
  DMSIM_PROBE_FP64_FMA = 0,      /* fma.rn.f64 */
  DMSIM_PROBE_FP32_FMA = 1,      /* fma.rn.f32 */
  DMSIM_PROBE_DMMA = 2,          /* mma.sync m8n8k4 f64 (FP64 tensor core), FLOPs */
  DMSIM_PROBE_INT_LOP3 = 3,      /* lop3.b32 */
  DMSIM_PROBE_INT_ADD = 4,       /* add.u32 */
  DMSIM_PROBE_INT_SHF = 5,       /* shf.r.clamp.b32 */
  DMSIM_PROBE_INT_PRMT = 6,      /* prmt.b32 */
  DMSIM_PROBE_INT_MAD = 7,       /* mad.lo.u32 */
  DMSIM_PROBE_CVT_S64_F64 = 8,   /* cvt.rn.f64.s64 */
  DMSIM_PROBE_CVT_F32_F64 = 9,   /* cvt.f64.f32 and cvt.rn.f32.f64, counted separately */
  DMSIM_PROBE_CVT_F32_S32 = 10,  /* cvt.rni.s32.f32 and cvt.rn.f32.s32, counted separately */
  DMSIM_PROBE_MIX_FADD_LOP3 = 11,/* add.rn.f32 and lop3.b32 interleaved, counted separately */
  DMSIM_PROBE_COUNT = 12
};
int dmsim_probe_rate(int which, double* ops_per_s);
/* Device pointers of rho (for in-HBM benchmarks and interop) */
int dmsim_device_state(dmsim_handle h, void** re, void** im);
const char* dmsim_last_error(dmsim_handle h);
const char* dmsim_status_string(int status);

#ifdef __cplusplus
}
#endif
#endif
