// gates.h -- gates of the engine: the user-level gate record and the basic
// gates (one reference pass each) that composites decompose into.
#pragma once
#include <complex>
#include <stdint.h>
#include <vector>

namespace dmg {

using cplx = std::complex<double>;

// A gate as appended by the user: the fields of DM-Sim's Gate
// (src/dmsim_nvgpu_omp.cuh:99-191) plus a matrix for the C1/C2 additions.
struct GateRec {
  int op;              // enum OP value, or OP_C1 / OP_C2
  uint32_t qb[5];
  double theta, phi, lambda;
  double m[32];        // C1: 2x2, C2: 4x4 complex, row-major re/im
  int32_t chan;        // OP_CHANNEL: index of the channel's superoperator
  int32_t nq;          // OP_CHANNEL: 1 or 2 qubits
};

// A channel's superoperator S = sum_i K_i (x) conj(K_i) on K <= 2 qubits:
// S[(a*D+b)*D*D + (c*D+e)] = sum_i K_i[a][c] conj(K_i[b][e]).
struct Channel {
  int K;
  cplx S[256];
};

constexpr int OP_C1 = 64;
constexpr int OP_C2 = 65;
constexpr int OP_CHANNEL = 66;  // a noise channel (no reference counterpart): chan indexes the channel table
constexpr int N_REF_OPS = 38;

extern const char* const kOpNames[N_REF_OPS];

// Basic gate kinds.
enum BasicKind { BK_1Q = 0, BK_2Q = 1, BK_RLIN = 2, BK_SUPER = 3 };

// One basic gate.  BK_1Q: u[0..3] is the 2x2 complex matrix on qubit q[0].
// BK_2Q: u[0..15] is a 4x4 complex matrix on the sub-index a = bit(q[0]) +
// 2*bit(q[1]) (CX(c,t) has q[0] = t, q[1] = c).  BK_RLIN: a real-linear map
// of (re0, im0, re1, im1) on qubit q[0] (rl), with rlb the map it induces on
// the bra side.
struct Basic {
  int kind;
  int op;              // originating basic op (for tracing and cost features)
  int q[2];
  cplx u[16];
  double rl[16], rlb[16];
  const Channel* chan; // BK_SUPER: the channel (sub-index bit i <-> qubit q[i])
};

// Number of qubits a gate id uses (0 for unknown ids).
int gate_arity(int op);

// Decompose one user gate into basic gates, following the composite
// sequences of src/dmsim_nvgpu_omp.cuh:1493-1813.  ID yields nothing (the
// reference's ID_GATE is empty, :1272-1275).
// Channels are looked up in chans.
void decompose(const GateRec& g, std::vector<Basic>& out, const std::vector<Channel>* chans = nullptr);

}  // namespace dmg
