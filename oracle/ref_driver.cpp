// ref_driver.cpp -- builds the UNMODIFIED reference CPU engine
// (src/dmsim_cpu_omp.hpp of pnnl/DM-Sim, included from the reference tree by
// oracle/Makefile, never copied) into oracle/_ref/libdmsim_ref.so, with a
// small extern "C" surface so the tests can drive the reference's own
// Simulation object: create / append / upload / sim / clear_circuit / measure.
//
// Test infrastructure only (pins the oracle restatement).  Two build-time
// settings, neither of which touches the reference's arithmetic:
//   * RAND_SEED is made a variable so measure() can be reproduced
//     (src/config.hpp:47 defines it as time(0));
//   * PRINT_MEA_PER_CIRCUIT is switched off to keep stdout quiet
//     (src/config.hpp:22).
#include "config.hpp"
#undef RAND_SEED
#undef PRINT_MEA_PER_CIRCUIT
static unsigned dmsim_ref_seed = 1;
#define RAND_SEED (dmsim_ref_seed)
#include "util_cpu.h"
#include "dmsim_cpu_omp.hpp"

#include <cstdint>
#include <cstring>

using namespace DMSim;

extern "C" {

void* ref_create(unsigned n_qubits, unsigned n_cpus) { return new Simulation(n_qubits, n_cpus); }

void ref_destroy(void* h) { delete static_cast<Simulation*>(h); }

void ref_append(void* h, int op, const uint32_t* q, double theta, double phi, double lambda) {
  Gate g(static_cast<enum OP>(op), q[0], q[1], q[2], q[3], q[4], theta, phi, lambda);
  static_cast<Simulation*>(h)->append(&g);
}

void ref_upload(void* h) { static_cast<Simulation*>(h)->upload(); }

void ref_sim(void* h) { static_cast<Simulation*>(h)->sim(); }

void ref_clear_circuit(void* h) { static_cast<Simulation*>(h)->clear_circuit(); }

void ref_reset(void* h) { static_cast<Simulation*>(h)->reset(); }

void ref_get_dm(void* h, double* re, double* im) {
  Simulation* s = static_cast<Simulation*>(h);
  size_t n = (size_t)s->dim * (size_t)s->dim;
  std::memcpy(re, s->dm_real_res, n * sizeof(double));
  std::memcpy(im, s->dm_imag_res, n * sizeof(double));
}

void ref_measure(void* h, unsigned seed, unsigned rep, uint64_t* out) {
  dmsim_ref_seed = seed;
  IdxType* r = static_cast<Simulation*>(h)->measure(rep);
  for (unsigned i = 0; i < rep; i++) out[i] = r[i];
  delete[] r;
}

}  // extern "C"
