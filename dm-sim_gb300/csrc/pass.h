// pass.h -- one superoperator pass over the vectorised density matrix.
//
// The state is the 4^n-entry array A with A[c*2^n + r] = rho[r][c]: the layout
// of DM-Sim's dm_real_res/dm_imag_res after sim() (src/dmsim_nvgpu_omp.cuh:
// 456-459), held as separate real and imaginary arrays.  Ket qubit q is bit q
// of the index and bra qubit q is bit q+n.  A pass applies a K-qubit operator
// U (K <= 4) as U (x) conj(U) on bits {q_i} and {q_i + n} in place.
//
// Tiling.  A tile is the closed set of G * 4^K entries (G = 256/2^K groups)
// that the operator mixes, chosen so that it is made of 2^mhi contiguous runs
// of 2^L entries: the low L index bits (which hold the low target bits plus
// log2(G) free bits) are contiguous in memory and the mhi target bits at or
// above L select the run.  Loads and stores of a run are coalesced 16-byte
// vector accesses whatever qubits the pass targets.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define DMG_HD __host__ __device__
#else
#define DMG_HD
#endif

namespace dmg {

constexpr int kThreads = 256;  // threads per block of every pass kernel
constexpr int kMaxK = 4;       // widest fused operator
constexpr int kMaxD = 16;      // 2^kMaxK

// Arithmetic class of a pass; selects the kernel instance.
enum PassClass : int32_t {
  CLS_MOVE = 0,    // monomial superoperator, every factor exactly 1 (X, CX, SWAP, Toffoli blocks)
  CLS_SIGNED = 1,  // monomial, factors in {1,-1,+i,-i}: sign and re/im swaps only (Y, Z, S, CZ)
  CLS_PHASE = 2,   // monomial with general complex factors (T, U1, controlled phases)
  CLS_DENSE = 3,   // general U, applied ket side then bra side (dense rows)
  CLS_SPARSE = 4,  // general U with sparse rows (per-row column lists)
  CLS_RLIN = 5,    // real-linear 1-qubit map (DM-Sim's SRN gate), K = 1
  CLS_SUPER = 6,   // general superoperator (a noise channel), K <= 2: 4^K x 4^K on the (ket, bra) sub-index
  CLS_COUNT = 7
};

// Kernel instances for DENSE / SPARSE passes whose U and V are real (the
// imaginary parts vanish, e.g. H, RY and their products with permutations):
// two real multiply-adds per complex term instead of four.  The host classes
// stay CLS_DENSE / CLS_SPARSE; PassHeader::flags marks such passes.
constexpr int kClsRealOffset = 16;
constexpr int CLS_DENSE_REAL = kClsRealOffset + CLS_DENSE;
constexpr int CLS_SPARSE_REAL = kClsRealOffset + CLS_SPARSE;
DMG_HD constexpr int base_class(int c) { return c >= kClsRealOffset ? c - kClsRealOffset : c; }
DMG_HD constexpr bool real_class(int c) { return c >= kClsRealOffset; }
constexpr int32_t kPassRealOperator = 1;  // PassHeader::flags bit

// Factor kinds of a monomial superoperator entry f[a][b].
enum FactorKind : int8_t { FK_ONE = 0, FK_NEG = 1, FK_PI = 2, FK_NI = 3, FK_GEN = 4 };

struct PassHeader {
  int32_t K, cls;
  int32_t L;         // low run bits
  int32_t mhi;       // number of target bits >= L
  int32_t g;         // log2 of groups per tile
  int32_t flags;     // kPassRealOperator: U and V are real
  uint64_t ntiles;   // tiles in the state
  int32_t hipos[8];  // global positions of the high target bits, ascending
  int32_t lket[4];   // local bit position of ket target i (qubit q_i)
  int32_t lbra[4];   // local bit position of bra target i (bit q_i + n)
  int32_t freepos[8];// local positions of the g free low bits, ascending
  uint32_t ldmask[8];   // bit h set: run h is read (it holds a source of a stored entry)
  uint32_t stmask[8];   // bit h set: run h is written (it holds an entry the pass changes)
};

// Operator payload for width K (D = 2^K).  A pass applies U to the ket
// sub-index and V to the bra sub-index; a superoperator pass has V = conj(U),
// a ket-only pass (the reference's forward/backward stages) has V = I.
template <int K>
struct PassOp {
  static constexpr int D = 1 << K;
  double ure[D * D], uim[D * D];   // U row-major (DENSE/SPARSE)
  double vre[D * D], vim[D * D];   // V row-major (DENSE/SPARSE)
  double fre[D * D], fim[D * D];   // f[a*D+b] = U[a][src a] * V[b][srcb b] (PHASE)
  double rlin[16];                 // RLIN: ket 4x4 real map on (r0,i0,r1,i1)
  double rlinb[16];                // RLIN: bra 4x4 real map
  int8_t nnz[D], nnzb[D];          // SPARSE: nonzeros per row of U and of V
  int8_t nnzmax, nnzbmax;          // SPARSE: largest row count of U and of V
  // SUPER: S[(a*D+b)*D*D + (c*D+e)] maps entry (c, e) to entry (a, b)
  double sre[K <= 2 ? D * D * D * D : 1], sim[K <= 2 ? D * D * D * D : 1];
  int8_t col[D * D], colb[D * D];  // SPARSE: column lists per row
  int8_t src[D], srcb[D];          // monomial: source index of row a of U / row b of V
  int8_t fk[D * D];                // monomial: factor kind of f[a][b]
};

template <int K>
struct PassDesc {
  PassHeader h;
  PassOp<K> op;
};

// ---- tensor-core passes (K = 3, 4; double-float or complex64 state)
// The ket step multiplies each tile column x (2^K complex entries, as 2R
// reals [re; im]) by the real embedding W = [[Ur, -Ui], [Ui, Ur]] (R x R,
// R = 2^(K+1)); the bra step does the same with V.  Both factors are split
// into BF16 "slices" of 8 bits each on a per-row (W) or per-column (x)
// power-of-two grid, so every slice product is an exact multiple of one unit
// per order i + j and the FP32 tensor-core sums of each order are exact; the
// orders are added in double-float.  The W/V slices are computed on the host.
constexpr int kTcSlices = 6;

// Byte offset of element (row, k) of a K-major, unswizzled BF16 tensor-core
// operand: 8-row x 16-byte core matrices (128 contiguous bytes), 128 bytes
// apart along k, `sbo` bytes apart between 8-row groups.
DMG_HD constexpr uint32_t tc_kmajor_offset(uint32_t row, uint32_t k, uint32_t sbo) {
  return (row >> 3) * sbo + (k >> 3) * 128u + (row & 7) * 16u + (k & 7) * 2u;
}

// ---- FP64-width tensor-core passes (K = 3, 4; FP64 state)
// Every operand value is an integer on a power-of-two grid, split into 7
// balanced base-256 digits (|digit| <= 128, exact in BF16): 55 significant
// bits for the largest value of each column of the state, 56 for each row
// of the operator.  Slice pairs of orders i + j = 0..7 accumulate exactly in
// FP32 (every partial sum is an integer below 2^22), the orders are combined
// in 64-bit integer arithmetic and rounded once to FP64.
constexpr int kTc64Slices = 7;
constexpr int kTc64Orders = 8;

template <int K>
struct TcDesc64 {
  static constexpr int D = 1 << K, R = 2 * D;
  PassHeader h;  // tile geometry, g = 7 - K (128 columns per step)
  // Row exponents: row n of W (0) or V (1) equals 2^ew[side][n mod D] times
  // sum_j digit_j 256^(6-j); rows n and n + D (the real and imaginary parts
  // of output n) hold the same magnitudes and share the exponent.
  int32_t ew[2][D];
  // digits j = 0..6 of W (0) and V (1): BF16 bits, K-major core-matrix layout
  alignas(16) uint16_t sl[2][kTc64Slices][R * R];
};

template <int K>
struct TcDesc {
  static constexpr int D = 1 << K, R = 2 * D;
  PassHeader h;  // tile geometry, g = 7 - K (128 columns per step)
  // slices of W (0) and V (1): row n of W = sum_j sl[0][j][n][.], slice j on
  // the grid 2^(e_n - 7 - 8j) with |W[n][.]| < 2^e_n (BF16 bits at true
  // scale, K-major core-matrix layout).  For a complex64 state, slices 0..2
  // hold each entry's own BF16 x 3 split (hi, mid, lo) instead.
  alignas(16) uint16_t sl[2][kTcSlices][R * R];
};

}  // namespace dmg
