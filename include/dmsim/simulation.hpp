// dmsim/simulation.hpp -- header-only C++ drop-in for DM-Sim's Simulation API
// (namespace DMSim, src/dmsim_nvgpu_omp.cuh:29-814 of pnnl/DM-Sim), implemented
// over the C ABI of include/dmsim_gb300.h.
//
// Source compatible with the reference's C++ examples (example/adder_n10_*.cu):
//   Simulation sim(n_qubits, 1);
//   sim.append(Simulation::H(0)); sim.upload(); sim.sim();
//   IdxType* res = sim.measure(5); ... delete[] res;
// Differences: IdxType is 64-bit; errors throw DMSim::Error instead of exit();
// n_gpus must be 1; C1/C2 arbitrary gates, reset_sim(), measure_with() and
// options (fused mode, complex64) are additions.  After sim() the result is
// copied to the host arrays dm_real_res / dm_imag_res as the reference does
// (:456-459); set_copy_back(false) skips that copy for device-only use.
#ifndef DMSIM_SIMULATION_HPP
#define DMSIM_SIMULATION_HPP

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "../dmsim_gb300.h"

namespace DMSim {

using IdxType = unsigned long long;
using ValType = double;

enum OP {
  U3, U2, U1, CX, ID, X, Y, Z, H, S,
  SDG, T, TDG, RX, RY, RZ, CZ, CY, SWAP, CH,
  CCX, CSWAP, CRX, CRY, CRZ, CU1, CU3, RXX, RZZ, RCCX,
  RC3X, C3X, C3SQRTX, C4X, R, SRN, W, RYY,
  C1 = 64, C2 = 65
};

static const char* const OP_NAMES[] = {
    "U3", "U2", "U1", "CX", "ID", "X", "Y", "Z", "H", "S",
    "SDG", "T", "TDG", "RX", "RY", "RZ", "CZ", "CY", "SWAP", "CH",
    "CCX", "CSWAP", "CRX", "CRY", "CRZ", "CU1", "CU3", "RXX", "RZZ", "RCCX",
    "RC3X", "C3X", "C3SQRTX", "C4X", "R", "SRN", "W", "RYY"};

struct Error : std::runtime_error {
  int status;
  Error(int st, const std::string& m) : std::runtime_error(m), status(st) {}
};

// Gate (src/dmsim_nvgpu_omp.cuh:99-191): op, five qubit slots, three angles.
class Gate {
 public:
  Gate(enum OP _op_name, IdxType _qb0, IdxType _qb1, IdxType _qb2, IdxType _qb3, IdxType _qb4, ValType _theta,
       ValType _phi, ValType _lambda)
      : op_name(_op_name), qb0(_qb0), qb1(_qb1), qb2(_qb2), qb3(_qb3), qb4(_qb4), theta(_theta), phi(_phi),
        lambda(_lambda) {
    std::memset(m, 0, sizeof m);
  }
  void dump(std::string& out) const {
    char buf[256];
    const char* name = op_name == C1 ? "C1" : op_name == C2 ? "C2" : OP_NAMES[op_name];
    std::snprintf(buf, sizeof buf, "%s(%llu,%llu,%llu,%llu,%llu,%g,%g,%g);\n", name, qb0, qb1, qb2, qb3, qb4, theta,
                  phi, lambda);
    out += buf;
  }
  enum OP op_name;
  IdxType qb0, qb1, qb2, qb3, qb4;
  ValType theta, phi, lambda;
  double m[32];  // C1: 2x2, C2: 4x4 complex (re, im interleaved, row-major)
};

class Simulation {
 public:
  Simulation(IdxType _n_qubits, IdxType _n_gpus)
      : n_qubits(_n_qubits), n_gpus(_n_gpus), dim(1ull << _n_qubits), half_dim(1ull << (_n_qubits - 1)),
        dm_num(dim * dim), n_gates(0), dm_real_res(nullptr), dm_imag_res(nullptr) {
    check(dmsim_create((uint32_t)_n_qubits, (uint32_t)_n_gpus, &h_), "Simulation");
  }
  ~Simulation() {
    if (dm_real_res) dmsim_free_host(dm_real_res);
    if (dm_imag_res) dmsim_free_host(dm_imag_res);
    dmsim_destroy(h_);
  }
  Simulation(const Simulation&) = delete;
  Simulation& operator=(const Simulation&) = delete;

  void set_option(int key, int64_t value) { check(dmsim_set_option(h_, key, value), "set_option"); }
  void set_copy_back(bool on) { copy_back_ = on; }

  // append(Gate*) (:331-344): the gate is copied, the caller keeps ownership
  void append(Gate* g) {
    if (!g) throw Error(DMSIM_ERR_ARG, "append: null gate");
    if (g->op_name == C1) {
      check(dmsim_append_c1(h_, (uint32_t)g->qb0, g->m), "append");
    } else if (g->op_name == C2) {
      check(dmsim_append_c2(h_, (uint32_t)g->qb0, (uint32_t)g->qb1, g->m), "append");
    } else {
      const uint32_t q[5] = {(uint32_t)g->qb0, (uint32_t)g->qb1, (uint32_t)g->qb2, (uint32_t)g->qb3, (uint32_t)g->qb4};
      check(dmsim_append(h_, (int)g->op_name, q, g->theta, g->phi, g->lambda), "append");
    }
    circuit_.push_back(*g);
    n_gates++;
  }
  Simulation* upload() {
    check(dmsim_upload(h_), "upload");
    return this;
  }
  // sim() (:390-494): run, then copy rho back to dm_real_res / dm_imag_res
  void sim() {
    check(dmsim_run(h_), "sim");
    if (copy_back_) {
      ensure_host();
      check(dmsim_get_dm(h_, dm_real_res, dm_imag_res), "sim");
    }
  }
  void clear_circuit() {
    check(dmsim_clear_circuit(h_), "clear_circuit");
    circuit_.clear();
    n_gates = 0;
  }
  void reset() {
    check(dmsim_reset(h_), "reset");
    circuit_.clear();
    n_gates = 0;
  }
  void reset_sim() { reset(); }
  void reset_dm() { check(dmsim_reset_dm(h_), "reset_dm"); }
  // measure(rep) (:521-549): returns new IdxType[rep], owned by the caller (delete[])
  IdxType* measure(unsigned repetition = 10) { return measure_with(repetition, nullptr); }
  IdxType* measure_with(unsigned repetition, const double* uniforms) {
    std::vector<uint64_t> out(repetition);
    check(dmsim_measure(h_, repetition, uniforms, out.data()), "measure");
    IdxType* res = new IdxType[repetition];
    for (unsigned i = 0; i < repetition; i++) res[i] = out[i];
    return res;
  }
  std::string dump() {
    std::string s;
    for (const Gate& g : circuit_) g.dump(s);
    return s;
  }
  void print_res_sv() {
    ensure_host();
    check(dmsim_get_dm(h_, dm_real_res, dm_imag_res), "print_res_sv");
    printf("----- Real SV ------\n");
    for (IdxType i = 0; i < dim; i++) printf("%lf ", dm_real_res[i * dim + i]);
    printf("\n----- Imag SV ------\n");
    for (IdxType i = 0; i < dim; i++) printf("%lf ", dm_imag_res[i * dim + i]);
    printf("\n");
  }
  void print_res_dm() {
    ensure_host();
    check(dmsim_get_dm(h_, dm_real_res, dm_imag_res), "print_res_dm");
    printf("----- Real DM------\n");
    for (IdxType i = 0; i < dim; i++) {
      for (IdxType j = 0; j < dim; j++) printf("%lf ", dm_real_res[i * dim + j]);
      printf("\n");
    }
    printf("----- Imag DM------\n");
    for (IdxType i = 0; i < dim; i++) {
      for (IdxType j = 0; j < dim; j++) printf("%lf ", dm_imag_res[i * dim + j]);
      printf("\n");
    }
  }

  // ---------------------------------------------------------- factories (:580-767)
  static Gate* U3(ValType theta, ValType phi, ValType lambda, IdxType m) { return new Gate(OP::U3, m, 0, 0, 0, 0, theta, phi, lambda); }
  static Gate* U2(ValType phi, ValType lambda, IdxType m) { return new Gate(OP::U2, m, 0, 0, 0, 0, 0., phi, lambda); }
  static Gate* U1(ValType lambda, IdxType m) { return new Gate(OP::U1, m, 0, 0, 0, 0, 0., 0., lambda); }
  static Gate* CX(IdxType m, IdxType n) { return new Gate(OP::CX, m, n, 0, 0, 0, 0., 0., 0.); }
  static Gate* ID(IdxType m) { return new Gate(OP::ID, m, 0, 0, 0, 0, 0., 0., 0.); }
  static Gate* X(IdxType m) { return new Gate(OP::X, m, 0, 0, 0, 0, 0., 0., 0.); }
  static Gate* Y(IdxType m) { return new Gate(OP::Y, m, 0, 0, 0, 0, 0., 0., 0.); }
  static Gate* Z(IdxType m) { return new Gate(OP::Z, m, 0, 0, 0, 0, 0., 0., 0.); }
  static Gate* H(IdxType m) { return new Gate(OP::H, m, 0, 0, 0, 0, 0., 0., 0.); }
  static Gate* S(IdxType m) { return new Gate(OP::S, m, 0, 0, 0, 0, 0., 0., 0.); }
  static Gate* SDG(IdxType m) { return new Gate(OP::SDG, m, 0, 0, 0, 0, 0., 0., 0.); }
  static Gate* T(IdxType m) { return new Gate(OP::T, m, 0, 0, 0, 0, 0., 0., 0.); }
  static Gate* TDG(IdxType m) { return new Gate(OP::TDG, m, 0, 0, 0, 0, 0., 0., 0.); }
  static Gate* RX(ValType theta, IdxType m) { return new Gate(OP::RX, m, 0, 0, 0, 0, theta, 0., 0.); }
  static Gate* RY(ValType theta, IdxType m) { return new Gate(OP::RY, m, 0, 0, 0, 0, theta, 0., 0.); }
  static Gate* RZ(ValType phi, IdxType m) { return new Gate(OP::RZ, m, 0, 0, 0, 0, 0., phi, 0.); }
  static Gate* CZ(IdxType m, IdxType n) { return new Gate(OP::CZ, m, n, 0, 0, 0, 0., 0., 0.); }
  static Gate* CY(IdxType m, IdxType n) { return new Gate(OP::CY, m, n, 0, 0, 0, 0., 0., 0.); }
  static Gate* SWAP(IdxType m, IdxType n) { return new Gate(OP::SWAP, m, n, 0, 0, 0, 0., 0., 0.); }
  static Gate* CH(IdxType m, IdxType n) { return new Gate(OP::CH, m, n, 0, 0, 0, 0., 0., 0.); }
  static Gate* CCX(IdxType l, IdxType m, IdxType n) { return new Gate(OP::CCX, l, m, n, 0, 0, 0., 0., 0.); }
  static Gate* CSWAP(IdxType l, IdxType m, IdxType n) { return new Gate(OP::CSWAP, l, m, n, 0, 0, 0., 0., 0.); }
  static Gate* CRX(ValType lambda, IdxType m, IdxType n) { return new Gate(OP::CRX, m, n, 0, 0, 0, 0., 0., lambda); }
  static Gate* CRY(ValType lambda, IdxType m, IdxType n) { return new Gate(OP::CRY, m, n, 0, 0, 0, 0., 0., lambda); }
  static Gate* CRZ(ValType lambda, IdxType m, IdxType n) { return new Gate(OP::CRZ, m, n, 0, 0, 0, 0., 0., lambda); }
  static Gate* CU1(ValType lambda, IdxType m, IdxType n) { return new Gate(OP::CU1, m, n, 0, 0, 0, 0., 0., lambda); }
  static Gate* CU3(ValType theta, ValType phi, ValType lambda, IdxType m, IdxType n) { return new Gate(OP::CU3, m, n, 0, 0, 0, theta, phi, lambda); }
  static Gate* RXX(ValType theta, IdxType m, IdxType n) { return new Gate(OP::RXX, m, n, 0, 0, 0, theta, 0., 0.); }
  static Gate* RZZ(ValType theta, IdxType m, IdxType n) { return new Gate(OP::RZZ, m, n, 0, 0, 0, theta, 0., 0.); }
  static Gate* RCCX(IdxType l, IdxType m, IdxType n) { return new Gate(OP::RCCX, l, m, n, 0, 0, 0., 0., 0.); }
  static Gate* RC3X(IdxType l, IdxType m, IdxType n, IdxType o) { return new Gate(OP::RC3X, l, m, n, o, 0, 0., 0., 0.); }
  static Gate* C3X(IdxType l, IdxType m, IdxType n, IdxType o) { return new Gate(OP::C3X, l, m, n, o, 0, 0., 0., 0.); }
  static Gate* C3SQRTX(IdxType l, IdxType m, IdxType n, IdxType o) { return new Gate(OP::C3SQRTX, l, m, n, o, 0, 0., 0., 0.); }
  static Gate* C4X(IdxType l, IdxType m, IdxType n, IdxType o, IdxType p) { return new Gate(OP::C4X, l, m, n, o, p, 0., 0., 0.); }
  static Gate* R(ValType theta, IdxType m) { return new Gate(OP::R, m, 0, 0, 0, 0, theta, 0., 0.); }
  static Gate* SRN(IdxType m) { return new Gate(OP::SRN, m, 0, 0, 0, 0, 0., 0., 0.); }
  static Gate* W(IdxType m) { return new Gate(OP::W, m, 0, 0, 0, 0, 0., 0., 0.); }
  static Gate* RYY(ValType theta, IdxType m, IdxType n) { return new Gate(OP::RYY, m, n, 0, 0, 0, theta, 0., 0.); }
  // additions: arbitrary 1- and 2-qubit gates (matrices re/im interleaved, row-major)
  static Gate* C1Gate(const double m8[8], IdxType q) {
    Gate* g = new Gate(OP::C1, q, 0, 0, 0, 0, 0., 0., 0.);
    std::memcpy(g->m, m8, 8 * sizeof(double));
    return g;
  }
  static Gate* C2Gate(const double m32[32], IdxType q1, IdxType q2) {
    Gate* g = new Gate(OP::C2, q1, q2, 0, 0, 0, 0., 0., 0.);
    std::memcpy(g->m, m32, 32 * sizeof(double));
    return g;
  }

  const IdxType n_qubits;
  const IdxType n_gpus;
  const IdxType dim;
  const IdxType half_dim;
  const IdxType dm_num;
  IdxType n_gates;
  ValType* dm_real_res;  // rho^T layout: dm_real_res[i*dim+j] = Re rho[j][i]
  ValType* dm_imag_res;

 private:
  void check(int st, const char* what) {
    if (st != DMSIM_OK) {
      const char* msg = h_ ? dmsim_last_error(h_) : dmsim_status_string(st);
      throw Error(st, std::string(what) + ": " + (msg && *msg ? msg : dmsim_status_string(st)));
    }
  }
  void ensure_host() {
    if (!dm_real_res) {
      void* p = nullptr;
      check(dmsim_alloc_host(dm_num * sizeof(ValType), &p), "host buffer");
      dm_real_res = static_cast<ValType*>(p);
      check(dmsim_alloc_host(dm_num * sizeof(ValType), &p), "host buffer");
      dm_imag_res = static_cast<ValType*>(p);
    }
  }
  dmsim_handle h_ = nullptr;
  bool copy_back_ = true;
  std::vector<Gate> circuit_;
};

// print_measurement (src/util_nvgpu.cuh): one binary string per shot
inline void print_measurement(const IdxType* res_state, IdxType n_qubits, int repetition) {
  printf("\n===============  Measurement (tests=%d) ================\n", repetition);
  for (int i = 0; i < repetition; i++) {
    printf("Test-%d: ", i);
    for (int b = (int)n_qubits - 1; b >= 0; b--) putchar('0' + (int)((res_state[i] >> b) & 1));
    printf("\n");
  }
}

}  // namespace DMSim

#endif
