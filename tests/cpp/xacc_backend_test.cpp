// The XACC backend (include/dmsim/xacc_backend.hpp) on the cases of the
// reference's XACC plugin tests (xacc/tests/DmSimCpuAcceleratorTester.cpp):
// the deuteron ansatz's <X0 X1> curve from 100000 shots, the deterministic
// shot tests (nothing -> 00, X; CX -> 11, Bell -> 00/11 only), plus CH (which
// the reference's GPU runner turned into SWAP) and every op the reference's
// runner could not take.  Prints "name value" lines for tests/test_xacc_backend.py.
#include <cmath>
#include <cstdio>
#include <vector>

#include "dmsim/xacc_backend.hpp"

using DmSim::Instruction;

static void counts_line(const char* name, const std::map<std::string, int>& c) {
  printf("%s", name);
  for (const auto& kv : c) printf(" %s:%d", kv.first.c_str(), kv.second);
  printf("\n");
}

int main() {
  DmSim::GB300Backend backend(/*seed=*/7);
  // deuteron ansatz: X(q0); Ry(q1, t); CX(q1, q0); H(q0); H(q1); measure both
  const double pi = std::acos(-1.0);
  for (int i = 0; i < 20; i++) {
    const double t = -pi + 2 * pi * i / 19.0;
    std::vector<Instruction> ir = {{"X", {0}, {}},      {"Ry", {1}, {t}}, {"CNOT", {1, 0}, {}}, {"H", {0}, {}},
                                   {"H", {1}, {}},      {"Measure", {0}, {}}, {"Measure", {1}, {}}};
    printf("deuteron %d %.6f\n", i, DmSim::expectation_z(DmSim::execute(backend, 2, ir, 100000)));
  }
  counts_line("nothing", DmSim::execute(backend, 2, {{"Measure", {0}, {}}, {"Measure", {1}, {}}}, 100));
  counts_line("x_cx", DmSim::execute(backend, 2, {{"X", {0}, {}}, {"CNOT", {0, 1}, {}}, {"Measure", {0}, {}},
                                                  {"Measure", {1}, {}}}, 100));
  counts_line("bell", DmSim::execute(backend, 2, {{"H", {0}, {}}, {"CNOT", {0, 1}, {}}, {"Measure", {0}, {}},
                                                  {"Measure", {1}, {}}}, 100));
  counts_line("ch", DmSim::execute(backend, 2, {{"X", {0}, {}}, {"CH", {0, 1}, {}}}, 20000));
  // the ops the reference's runner could not take, through the backend interface
  {
    backend.init(3);
    backend.addGate(DmSim::OP::X, {0});
    backend.addGate(DmSim::OP::X, {1});
    backend.addGate(DmSim::OP::CCX, {0, 1, 2});
    std::map<std::string, int> c;
    for (int64_t v : backend.measure(50)) c[std::to_string(v)]++;
    counts_line("ccx", c);
    backend.finalize();
  }
  int ok = 0;
  for (int op = 0; op <= (int)DmSim::OP::RYY; op++) {
    const DmSim::OP o = (DmSim::OP)op;
    backend.init(5);
    std::vector<int> q;
    for (int i = 0; i < DmSim::GB300Backend::arity(o); i++) q.push_back(i);
    std::vector<double> p(DmSim::GB300Backend::n_params(o), 0.3);
    backend.addGate(o, q, p);
    backend.measure(4);
    backend.finalize();
    ok++;
  }
  printf("all_ops %d\n", ok);
  return 0;
}
