/*
 * dmsim_oracle.h -- CPU ORACLE FOR TESTS AND THE CPU BASELINE ONLY.
 *
 * This is test infrastructure: a plain-C restatement of DM-Sim's CPU
 * density-matrix algorithm (src/dmsim_cpu_omp.hpp in pnnl/DM-Sim).  Only the
 * tests, the smoke check and the benchmark's CPU-baseline leg may load it.
 * The GPU engine never calls into it.
 *
 * Parity is pinned: tests/test_oracle_pin.py runs the reference CPU engine
 * (compiled from its own sources by oracle/Makefile into oracle/_ref/) and
 * requires bit-identical density matrices for single runs from |0..0><0..0|,
 * plus bit-identical measure() outcomes for the same seed.
 */
#ifndef DMSIM_ORACLE_H
#define DMSIM_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Gate ids: the order of enum OP in src/dmsim_cpu_omp.hpp:41-47 (ABI). */
enum dmo_op {
  DMO_U3 = 0, DMO_U2, DMO_U1, DMO_CX, DMO_ID, DMO_X, DMO_Y, DMO_Z, DMO_H, DMO_S,
  DMO_SDG, DMO_T, DMO_TDG, DMO_RX, DMO_RY, DMO_RZ, DMO_CZ, DMO_CY, DMO_SWAP, DMO_CH,
  DMO_CCX, DMO_CSWAP, DMO_CRX, DMO_CRY, DMO_CRZ, DMO_CU1, DMO_CU3, DMO_RXX, DMO_RZZ, DMO_RCCX,
  DMO_RC3X, DMO_C3X, DMO_C3SQRTX, DMO_C4X, DMO_R, DMO_SRN, DMO_W, DMO_RYY,
  DMO_N_OPS,
  /* additions with no enum value in the reference: arbitrary 1- and 2-qubit
   * gates applied with the element formulas of C1_GATE / C2_GATE
   * (src/dmsim_cpu_omp.hpp:1004-1122) */
  DMO_C1 = 64, DMO_C2 = 65
};

/* One gate as the reference's Gate object holds it (src/dmsim_cpu_omp.hpp:
 * 99-191): op, five qubit slots, theta/phi/lambda.  For DMO_C1 m[0..7] holds
 * the 2x2 matrix (re,im interleaved, row-major); for DMO_C2 m[0..31] holds the
 * 4x4 matrix, with qb0 = qubit1 (the high bit of the 4-dim basis), qb1 = qubit2. */
typedef struct dmo_gate {
  int32_t op;
  uint32_t qb[5];
  double theta, phi, lambda;
  double m[32];
} dmo_gate;

/* Number of basic (C1-kind or CX) gates the reference executes for one gate. */
int dmo_basic_count(const dmo_gate* g);

/* Apply a circuit to every column of the (2^n x 2^n) array re/im, treating
 * index v = col*2^n + row with the gates acting on the row bits, exactly as
 * the reference's forward pass (circuit(), src/dmsim_cpu_omp.hpp:782-788). */
void dmo_apply_columns(int n, const dmo_gate* gates, int ngates, double* re, double* im, int nthreads);

/* Full reference sim(): forward pass, conjugate transpose, second pass
 * (src/dmsim_cpu_omp.hpp:367-447, simulation_kernel :888-935), but with a
 * correct transpose, so chained runs from any state are right.  On return
 * re/im hold the reference's dm_real_res/dm_imag_res layout:
 * re[i*2^n+j] + i*im[i*2^n+j] = rho[j][i]. */
void dmo_dm_sim(int n, const dmo_gate* gates, int ngates, double* re, double* im, int nthreads);

/* Statevector run of the same basic-gate sequence (same formulas). */
void dmo_sv_sim(int n, const dmo_gate* gates, int ngates, double* re, double* im);

/* measure(rep) restated (src/dmsim_cpu_omp.hpp, same as
 * src/dmsim_nvgpu_omp.cuh:521-549): |Re diag| -> sequential FP64 prefix ->
 * linear search per uniform.  uniforms[i] plays rand()/RAND_MAX.
 * Returns the trace sum (scan[dim]). */
double dmo_measure(int n, const double* dm_re, int rep, const double* uniforms, uint64_t* out);

/* The reference's own uniform stream: srand(seed); rand()/RAND_MAX. */
void dmo_libc_uniforms(unsigned seed, int rep, double* out);

#ifdef __cplusplus
}
#endif
#endif
