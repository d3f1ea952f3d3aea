// The reference's 10-qubit adder example (example/adder_n10_nvgpu_omp.cu),
// written against the drop-in header: same calls, same expected output.
#include <cstdio>

#include "dmsim/simulation.hpp"

using namespace DMSim;

void majority(Simulation& sim, const IdxType a, const IdxType b, const IdxType c) {
  sim.append(Simulation::CX(c, b));
  sim.append(Simulation::CX(c, a));
  sim.append(Simulation::CCX(a, b, c));
}
void unmaj(Simulation& sim, const IdxType a, const IdxType b, const IdxType c) {
  sim.append(Simulation::CCX(a, b, c));
  sim.append(Simulation::CX(c, a));
  sim.append(Simulation::CX(a, b));
}

int main() {
  int n_qubits = 10;
  Simulation sim(n_qubits, 1);
  sim.append(Simulation::X(1));
  sim.append(Simulation::X(5));
  sim.append(Simulation::X(6));
  sim.append(Simulation::X(7));
  sim.append(Simulation::X(8));
  majority(sim, 0, 5, 1);
  majority(sim, 1, 6, 2);
  majority(sim, 2, 7, 3);
  majority(sim, 3, 8, 4);
  sim.append(Simulation::CX(4, 9));
  unmaj(sim, 3, 8, 4);
  unmaj(sim, 2, 7, 3);
  unmaj(sim, 1, 6, 2);
  unmaj(sim, 0, 5, 1);
  sim.upload();
  sim.sim();
  auto* res = sim.measure(5);
  print_measurement(res, n_qubits, 5);
  delete[] res;
  return 0;
}
