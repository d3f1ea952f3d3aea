// dmsim/xacc_backend.hpp -- header-only XACC backend for the GB300 engine,
// over the C++ drop-in (dmsim/simulation.hpp) and so over the C ABI.
//
// Two layers, mirroring pnnl/DM-Sim's XACC plugin:
//   * DmSim::DmSimBackend (init / addGate / measure / finalize, the gate ids
//     of DmSim::OP) -- the interface of xacc/DmSimApi.hpp:47-63, implemented
//     by GB300Backend; getGpuDmSim() returns one, as the reference's
//     xacc/nvidia_omp/NvidiaOmpRunner.cu:173-176 does.  Unlike that runner,
//     every one of the 38 ops is accepted (the reference reaches
//     __builtin_unreachable for ID, CCX, CSWAP, CU3, RXX, RZZ, RCCX, RC3X, C3X,
//     C3SQRTX, C4X, R, SRN, W and RYY, :131-148) and CH applies CH (the
//     reference appends SWAP for it, :106-110).
//   * DmSim::execute -- what xacc/DmSimAccelerator.cpp's execute() does with
//     an XACC IR: visit each enabled instruction, map it to an op
//     (DmSimCircuitVisitor), record the measured qubits (all of them when none
//     is measured), sample `shots` outcomes and turn each into a bit string
//     over the measured qubits in ascending order.  The IR is taken as a
//     plain list of named instructions so that the mapping can be used and
//     tested without XACC; an XACC Accelerator plugin forwards its
//     InstructionIterator to it (INTEGRATION.md shows the glue).
// Parameter conventions (the params vector of addGate, in order): U3 theta,
// phi, lambda; U2 phi, lambda; U1 / CU1 lambda; RX / RY / RZ, CRX / CRY / CRZ,
// RXX / RYY / RZZ and R theta; CU3 theta, phi, lambda.  Qubits: controls
// first, target last, as the Simulation factories.
#ifndef DMSIM_XACC_BACKEND_HPP
#define DMSIM_XACC_BACKEND_HPP

#include <algorithm>
#include <cstdint>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "simulation.hpp"

namespace DmSim {

// The gate ids of the XACC backend interface (the order of enum OP).
enum class OP {
  U3, U2, U1, CX, ID, X, Y, Z, H, S,
  SDG, T, TDG, RX, RY, RZ, CZ, CY, SWAP, CH,
  CCX, CSWAP, CRX, CRY, CRZ, CU1, CU3, RXX, RZZ, RCCX,
  RC3X, C3X, C3SQRTX, C4X, R, SRN, W, RYY
};

class DmSimBackend {
 public:
  virtual ~DmSimBackend() = default;
  virtual void init(int n_qubits, int n_gpus = 1) = 0;
  virtual void addGate(OP op, const std::vector<int>& qubits, const std::vector<double>& params = {}) = 0;
  virtual std::vector<int64_t> measure(int shots) = 0;
  virtual void finalize() = 0;
};

class GB300Backend : public DmSimBackend {
 public:
  // seed: the sampling seed of measure() (-1: time(0), as the reference)
  explicit GB300Backend(int64_t seed = -1) : seed_(seed) {}

  void init(int n_qubits, int n_gpus = 1) override {
    sim_.reset(new DMSim::Simulation((DMSim::IdxType)n_qubits, (DMSim::IdxType)n_gpus));
    sim_->set_copy_back(false);
    sim_->set_option(DMSIM_OPT_SEED, seed_);
  }

  void addGate(OP op, const std::vector<int>& q, const std::vector<double>& p = {}) override {
    if (!sim_) throw DMSim::Error(DMSIM_ERR_STATE, "addGate before init");
    using S = DMSim::Simulation;
    const int nq = arity(op), np = n_params(op);
    if ((int)q.size() != nq || (int)p.size() != np)
      throw DMSim::Error(DMSIM_ERR_ARG, std::string("addGate ") + DMSim::OP_NAMES[(int)op] + ": expects " +
                                            std::to_string(nq) + " qubits and " + std::to_string(np) + " parameters");
    auto Q = [&](int i) { return (DMSim::IdxType)q[i]; };
    DMSim::Gate* g = nullptr;
    switch (op) {
      case OP::U3: g = S::U3(p[0], p[1], p[2], Q(0)); break;
      case OP::U2: g = S::U2(p[0], p[1], Q(0)); break;
      case OP::U1: g = S::U1(p[0], Q(0)); break;
      case OP::CX: g = S::CX(Q(0), Q(1)); break;
      case OP::ID: g = S::ID(Q(0)); break;
      case OP::X: g = S::X(Q(0)); break;
      case OP::Y: g = S::Y(Q(0)); break;
      case OP::Z: g = S::Z(Q(0)); break;
      case OP::H: g = S::H(Q(0)); break;
      case OP::S: g = S::S(Q(0)); break;
      case OP::SDG: g = S::SDG(Q(0)); break;
      case OP::T: g = S::T(Q(0)); break;
      case OP::TDG: g = S::TDG(Q(0)); break;
      case OP::RX: g = S::RX(p[0], Q(0)); break;
      case OP::RY: g = S::RY(p[0], Q(0)); break;
      case OP::RZ: g = S::RZ(p[0], Q(0)); break;
      case OP::CZ: g = S::CZ(Q(0), Q(1)); break;
      case OP::CY: g = S::CY(Q(0), Q(1)); break;
      case OP::SWAP: g = S::SWAP(Q(0), Q(1)); break;
      case OP::CH: g = S::CH(Q(0), Q(1)); break;
      case OP::CCX: g = S::CCX(Q(0), Q(1), Q(2)); break;
      case OP::CSWAP: g = S::CSWAP(Q(0), Q(1), Q(2)); break;
      case OP::CRX: g = S::CRX(p[0], Q(0), Q(1)); break;
      case OP::CRY: g = S::CRY(p[0], Q(0), Q(1)); break;
      case OP::CRZ: g = S::CRZ(p[0], Q(0), Q(1)); break;
      case OP::CU1: g = S::CU1(p[0], Q(0), Q(1)); break;
      case OP::CU3: g = S::CU3(p[0], p[1], p[2], Q(0), Q(1)); break;
      case OP::RXX: g = S::RXX(p[0], Q(0), Q(1)); break;
      case OP::RZZ: g = S::RZZ(p[0], Q(0), Q(1)); break;
      case OP::RCCX: g = S::RCCX(Q(0), Q(1), Q(2)); break;
      case OP::RC3X: g = S::RC3X(Q(0), Q(1), Q(2), Q(3)); break;
      case OP::C3X: g = S::C3X(Q(0), Q(1), Q(2), Q(3)); break;
      case OP::C3SQRTX: g = S::C3SQRTX(Q(0), Q(1), Q(2), Q(3)); break;
      case OP::C4X: g = S::C4X(Q(0), Q(1), Q(2), Q(3), Q(4)); break;
      case OP::R: g = S::R(p[0], Q(0)); break;
      case OP::SRN: g = S::SRN(Q(0)); break;
      case OP::W: g = S::W(Q(0)); break;
      case OP::RYY: g = S::RYY(p[0], Q(0), Q(1)); break;
    }
    std::unique_ptr<DMSim::Gate> own(g);
    sim_->append(g);
  }

  // upload, run from |0..0><0..0|, sample (:150-166 of the reference runner)
  std::vector<int64_t> measure(int shots) override {
    if (!sim_) throw DMSim::Error(DMSIM_ERR_STATE, "measure before init");
    sim_->upload();
    sim_->sim();
    std::unique_ptr<DMSim::IdxType[]> res(sim_->measure((unsigned)shots));
    return std::vector<int64_t>(res.get(), res.get() + shots);
  }

  void finalize() override { sim_.reset(); }

  DMSim::Simulation* simulation() { return sim_.get(); }

  static int arity(OP op) {
    switch (op) {
      case OP::CX: case OP::CZ: case OP::CY: case OP::SWAP: case OP::CH: case OP::CRX: case OP::CRY:
      case OP::CRZ: case OP::CU1: case OP::CU3: case OP::RXX: case OP::RZZ: case OP::RYY:
        return 2;
      case OP::CCX: case OP::CSWAP: case OP::RCCX: return 3;
      case OP::RC3X: case OP::C3X: case OP::C3SQRTX: return 4;
      case OP::C4X: return 5;
      default: return 1;
    }
  }
  static int n_params(OP op) {
    switch (op) {
      case OP::U3: case OP::CU3: return 3;
      case OP::U2: return 2;
      case OP::U1: case OP::CU1: case OP::RX: case OP::RY: case OP::RZ: case OP::CRX: case OP::CRY: case OP::CRZ:
      case OP::RXX: case OP::RZZ: case OP::RYY: case OP::R:
        return 1;
      default: return 0;
    }
  }

 private:
  std::unique_ptr<DMSim::Simulation> sim_;
  int64_t seed_;
};

inline std::shared_ptr<DmSimBackend> getGpuDmSim() { return std::make_shared<GB300Backend>(); }

// ---- the accelerator's execute(), over a plain instruction list
struct Instruction {
  std::string name;            // XACC instruction names: H, X, Y, Z, Rx, Ry, Rz, S, Sdg, T, Tdg, CNOT, CY,
                               // CZ, Swap, CH, CPhase, CRZ, I, U, Measure
  std::vector<int> bits;
  std::vector<double> params;
  bool enabled = true;
};

// The op of an XACC instruction (DmSimCircuitVisitor), or false if it is not a
// gate (Identity, Measure).  Unknown names throw.
inline bool xacc_op(const std::string& name, OP* op) {
  static const std::map<std::string, OP> ops = {
      {"H", OP::H},     {"X", OP::X},        {"Y", OP::Y},     {"Z", OP::Z},       {"Rx", OP::RX},
      {"Ry", OP::RY},   {"Rz", OP::RZ},      {"S", OP::S},     {"Sdg", OP::SDG},   {"T", OP::T},
      {"Tdg", OP::TDG}, {"CNOT", OP::CX},    {"CY", OP::CY},   {"CZ", OP::CZ},     {"Swap", OP::SWAP},
      {"CH", OP::CH},   {"CPhase", OP::CU1}, {"CRZ", OP::CRZ}, {"U", OP::U3}};
  if (name == "I" || name == "Measure") return false;
  auto it = ops.find(name);
  if (it == ops.end()) throw DMSim::Error(DMSIM_ERR_ARG, "unsupported instruction " + name);
  *op = it->second;
  return true;
}

// Run the instructions on n_qubits from |0..0><0..0| and return the counts of
// the measured bit strings (DmSimAccelerator::execute).
inline std::map<std::string, int> execute(DmSimBackend& backend, int n_qubits, const std::vector<Instruction>& ir,
                                          int shots, int n_gpus = 1) {
  backend.init(n_qubits, n_gpus);
  std::vector<int> measured;
  for (const Instruction& ins : ir) {
    if (!ins.enabled) continue;
    if (ins.name == "Measure") {
      measured.push_back(ins.bits.at(0));
      continue;
    }
    OP op;
    if (xacc_op(ins.name, &op)) backend.addGate(op, ins.bits, ins.params);
  }
  if (measured.empty())
    for (int i = 0; i < n_qubits; i++) measured.push_back(i);
  std::sort(measured.begin(), measured.end());
  std::map<std::string, int> counts;
  for (int64_t v : backend.measure(shots)) {
    std::string s;
    for (int b : measured) s.push_back(((uint64_t)v >> b) & 1 ? '1' : '0');
    counts[s]++;
  }
  backend.finalize();
  return counts;
}

// <Z...Z> over the measured bits from counts (AcceleratorBuffer::getExpectationValueZ):
// each outcome weighs +1 for an even number of ones, -1 for an odd number.
inline double expectation_z(const std::map<std::string, int>& counts) {
  double sum = 0, total = 0;
  for (const auto& kv : counts) {
    const int ones = (int)std::count(kv.first.begin(), kv.first.end(), '1');
    sum += (ones % 2 ? -1.0 : 1.0) * kv.second;
    total += kv.second;
  }
  return total > 0 ? sum / total : 0.0;
}

}  // namespace DmSim

#endif
