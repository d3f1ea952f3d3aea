// plan.h -- from basic gates to device passes.
#pragma once
#include <stdint.h>

#include <vector>

#include "gates.h"
#include "pass.h"

namespace dmg {

// A pass before it is written to the device: a K-qubit operator on qubits
// q[0..K-1] (sub-index bit i <-> qubit q[i]) and its arithmetic class.
struct PassSpec {
  int K = 0;
  int q[kMaxK] = {0, 0, 0, 0};
  cplx U[kMaxD * kMaxD];       // ket operator, row-major D x D
  cplx V[kMaxD * kMaxD];       // bra operator: conj(U) for a superoperator pass, I for a ket-only pass
  bool ket_only = false;
  bool transpose = false;      // not an operator: the in-place conjugate transpose of rho
  bool rlin = false;
  bool super = false;          // U holds a channel's (4^K x 4^K) superoperator, K <= 2
  double rl[16], rlb[16];
  int cls = CLS_DENSE;
  int nbasic = 0;              // basic gates this pass replaces
  int nnz = 0;                 // nonzeros of U after snapping
  int tc = -1;                 // tensor cores: -1 the engine's rule decides, 0 no, 1 yes (learned planner)
};

// Cost-model features of one pass (also recorded with its measured time).
struct PassFeatures {
  int K, cls, nnz;
  int arith;        // 0 FP64, 1 FP32, 2 double-float
  int max_lo_bit;   // highest target bit below L (-1 if none)
  int min_hi_bit;   // lowest target bit at or above L (2n if none)
  int n;
  double ld_frac, st_frac;  // fraction of the state read / written
  int tc;           // 1: the pass runs on the tensor cores
  int real;         // 1: U and V are real (half the multiply-adds on the FP32 pipe)
};

// Fusion planners.  Both keep program order on every qubit and only reorder
// gates that act on disjoint qubits.
//   greedy: grow each pass with the earliest ready gate that keeps the width <= maxk
//   (prefer gates inside the current qubit set), the fixed-width planner.
std::vector<PassSpec> plan_plain(const std::vector<Basic>& basics);
//   row_cap: a candidate gate is not absorbed if the fused operator would get
//   more than row_cap nonzeros in a row (kMaxD = no cap).
std::vector<PassSpec> plan_greedy(const std::vector<Basic>& basics, int maxk, int row_cap = kMaxD);
// The reference's own order for circuits holding a real-linear gate (SRN):
// every gate on the ket bits only, the conjugate transpose, every gate again
// (src/dmsim_nvgpu_omp.cuh:918-969).  For complex-linear circuits and a
// Hermitian rho this equals plan_plain; with SRN only this order matches.
std::vector<PassSpec> plan_reference_order(const std::vector<Basic>& basics);

// Snap near-exact entries, set V = conj(U) (unless ket_only), detect the
// arithmetic class.
void classify(PassSpec& p, bool fused);

// Size in bytes of the device descriptor of a width-K pass.
size_t desc_size(int K);
// Write the descriptor of pass p for an n-qubit state into out (desc_size bytes).
// Returns the algorithmic bytes per entry-size unit moved by the pass
// (entries read + entries written); features are filled when f != nullptr.
// g_cap caps log2 of the groups per tile (the tile shape; 8 = the largest).
uint64_t build_desc(const PassSpec& p, int n, void* out, PassFeatures* f, uint64_t* ntiles, int* tile_entries,
                    int g_cap = 8);
// Tensor-core passes (dense K = 3, 4 operators on a double-float state):
// whether a pass can run on the tensor cores, the size of its descriptor
// (TcDesc<K>) and the descriptor itself.
bool tc_eligible(const PassSpec& p, int n);
// Whether an eligible pass runs there: option 0 never, 2 always, 1 the
// learned planner's per-pass choice (PassSpec::tc) or, without one, at least
// kTcMinRowNnz nonzeros per row of U (the tensor cores' cost does not depend
// on the density, the FP32-pipe kernel's grows with it).
constexpr int kTcMinRowNnz = 3;
// arith: the run's arithmetic (kernels.h Arith: 0 FP64, 1 FP32, 2 double-float).
// FP64 runs use the FP64-width passes (TcDesc64), the others TcDesc.
bool tc_choose(const PassSpec& p, int n, int tensor_opt, int arith);
size_t tc_desc_bytes(int K, int arith = 2);
// slices = false: geometry and features only (the planner's scoring).
uint64_t build_tc_desc(const PassSpec& p, int n, void* out, PassFeatures* f, uint64_t* ntiles, int* tile_entries,
                       bool slices = true, int arith = 2);
// x rounded to the nearest BF16 value, as a float.
float bf16_round(float x);
// The 7 balanced base-256 digits of an integer |t| <= 2^55 (digit 0 the most
// significant, weight 256^(6-j)): t = sum_j d[j] 256^(6-j), |d[j]| <= 128.
void tc64_digits(int64_t t, int d[7]);

}  // namespace dmg
