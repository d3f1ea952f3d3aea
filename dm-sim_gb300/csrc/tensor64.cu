// tensor64.cu -- dense K = 3, 4 qubit passes on the tensor cores for an FP64
// state, at FP64 width, on the tensor cores and the integer/FP32 pipes:
// GB300's FP64 pipe and its conversions run at ~1/60 of the FP32 rate, so it
// does one conversion per output and nothing else.
//
// A pass is two products per tile, as in the double-float tensor pass: the
// ket step multiplies every tile column x (2^K complex entries as R = 2^(K+1)
// reals) by the real embedding W = [[Ur, -Ui], [Ui, Ur]], the bra step the
// result's columns by V.  Here every operand value is an integer times a
// power of two, split into 7 balanced base-256 digits (|digit| <= 128, exact
// in BF16):
//   * a state column (ket step): the FP64 bits are aligned in integer
//     arithmetic to the column's largest exponent, v = |x| 2^(1077 - Ec) <
//     2^55 (55 significant bits for the column's largest value);
//   * an operator row (host, TcDesc64): w = t 2^ew with |t| <= 2^55;
//   * a bra-step column: the ket step's exact integer outputs, aligned to the
//     bra column's own magnitude (54-55 significant bits for its largest).
// Digit pairs of orders i + j = 0..7 are summed by tcgen05.mma into one FP32
// accumulator per order; every partial sum is an integer below 7 R 2^14 <=
// 2^22, so the sums are exact.  The orders are combined in 64-bit integer
// arithmetic (orders 6 and 7 below 2^-40 of order 0 enter through one
// truncating shift) and the bra step's result is rounded once to FP64 from
// the 64-bit integer (one conversion per output on the FP64 pipe, which runs
// beside the integer work).  Each value is held with 55 significant bits
// relative to its column's largest (block floating point per column of 2^K
// entries): the error of an output is below 2^-54 of its operator row's
// 1-norm times its column's largest value, per step.
//
// Threads: 1024 (32 warps, 64 registers each), one block per SM, as two
// independent groups of 16 warps that take alternate tiles of the block, each
// with its own tile buffer, digit operand, tensor-memory accumulator set,
// mbarriers and named barrier: while one group waits at a barrier or on its
// products, the other issues, with eight warps per scheduler to hide the
// integer work's latency.  Every thread holds a quarter of a column: in the
// digit steps thread (warp w, lane l) of a group owns tile column 8 (w & 15)
// + (l & 7) and quarter l >> 3 of it (half l >> 4, values (l >> 3) & 1 of
// that half; the four quarters of a column in one warp); in the accumulator
// steps column m = 32 (w & 3) + l -- the TMEM lane quadrant its warp may read
// -- and quarter ((w & 15) >> 2).  The group's first thread issues its MMAs;
// every thread issues its share of the group's bulk copies.  Per tile:
//   1. wait for the tile (TMA bulk copies of its runs, issued one tile
//      ahead), column maxima, ket digits -> A;  2. the ket MMAs;
//   3. ket accumulators -> exact int64 outputs in place of the tile, bra
//      magnitude keys;  4. bra digits -> A;  5. the bra MMAs, and the group's
//      next tile loaded into the freed buffer;  6. bra accumulators -> FP64
//      -> global stores.
// Three group barriers per tile (after steps 1, 3 and 4); the first two also
// OR the threads' timeout flags.  Every wait is bounded; on expiry the group
// leaves its loop at the next such barrier, waits (bounded) for its own copies
// and MMAs in flight, sets the error flag, and the block releases its TMEM;
// the host reports DMSIM_ERR_TIMEOUT.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "kernels.h"
#include "pass_device.cuh"
#include "tc.cuh"

namespace dmg {

namespace {

constexpr int kT64Threads = 1024;
constexpr int kT64GroupThreads = 512;
constexpr uint32_t kT64WaitPolls = 1u << 24;

template <int K>
struct T64 {
  static constexpr int D = 1 << K, R = 2 * D, G = 128 / D, TILE = 128 * D;
  // entries from a loaded tile's real array to its imaginary array: 16-entry
  // pieces 18 entries apart, and an offset of 8 pieces' banks between the two
  static constexpr int ASTR = TILE / 16 * 18 + 8;
  static constexpr uint32_t SBO = 16 * R;                  // bytes between 8-row groups of an R-wide operand
  static constexpr uint32_t A_BYTES = 128 * R * 2;         // one digit slice of the 128 columns
  static constexpr uint32_t B_BYTES = R * R * 2;           // one digit slice of W or V
  static constexpr uint32_t SET_COLS = kTc64Orders * R;    // accumulators of one group
  static constexpr uint32_t TMEM_COLS = 2 * SET_COLS;      // 512 (K = 4), 256 (K = 3)
  static constexpr uint32_t TX_BYTES = TILE * 8 * 2;       // one tile, re + im, 8 bytes per real
  static constexpr uint32_t BUF_BYTES = 2 * ASTR * 8;      // one group's tile buffer
  static_assert(TMEM_COLS <= 512, "two accumulator sets must fit in tensor memory");
  static_assert(ASTR % 2 == 0 && BUF_BYTES % 16 == 0, "bulk copies need 16-byte aligned destinations");
};

// Layout of a loaded tile in shared memory: local entry e at piece_off(e),
// 16-entry pieces (128 bytes, one bulk copy each) 18 entries apart, so that
// the pieces' banks rotate by two 8-byte words per piece.  Each thread of the
// ket step reads one column of the operator's targets (entries whose indices
// differ in the target bits); with the pieces rotated, the columns a warp
// reads at once fall into different banks even when the targets are the low
// bits.  piece_off is additive over disjoint bit fields.
__device__ __forceinline__ int piece_off(int e) { return e + 2 * (e >> 4); }

template <int K>
struct T64Group {
  static constexpr int D = 1 << K;
  uint64_t full;          // the group's tile loads
  uint64_t mma;           // the group's ket and bra commits, alternating
  uint32_t brmax[128];    // per bra column: magnitude key of the ket outputs
  int colEt[D][128 / D];  // biased exponent of ket column (b, f)'s grid, at [b][f]
};

template <int K>
struct T64Tables {
  static constexpr int D = 1 << K;
  uint64_t hioff[256];
  // output (a, b) of a tile, at [b][a]: bits 0..47 its offset from the tile
  // base minus the free bits, bits 48..55 the bra row exponent ew[1][b] +
  // 128, bit 63 set when its run is stored
  uint64_t outoff[D][D];
  // the offsets split by their disjoint bit fields: output (a, b) at
  // offk[a] + offb[b]; allstored: every run of the tile is stored
  uint64_t offk[D], offb[D];
  int allstored;
  T64Group<K> grp[2];
  int pk[D], pb[D];  // piece_off of the ket / bra index bits
  int ew[2][D];
  int hipos[8];
  uint32_t slot;
};

template <int K>
constexpr size_t t64_smem_bytes() {
  using S = T64<K>;
  return 2 * (size_t)kTc64Slices * S::A_BYTES + 2 * (size_t)kTc64Slices * S::B_BYTES + 2 * (size_t)S::BUF_BYTES +
         sizeof(T64Tables<K>);
}

// Named barrier of group g (ids 1, 2), and the same with an OR of p over the group.
__device__ __forceinline__ void group_bar(int g) { tc::named_bar<kT64GroupThreads>(1 + g); }
__device__ __forceinline__ bool group_bar_or(int g, bool p) { return tc::named_bar_or<kT64GroupThreads>(1 + g, p); }

__device__ __forceinline__ uint64_t shr_u64(uint64_t x, uint32_t s) {  // s >= 64 gives 0
  uint64_t r;
  asm("shr.b64 %0, %1, %2;" : "=l"(r) : "l"(x), "r"(s));
  return r;
}
__device__ __forceinline__ int64_t shr_s64(int64_t x, uint32_t s) {  // s >= 64 gives the sign
  int64_t r;
  asm("shr.s64 %0, %1, %2;" : "=l"(r) : "l"(x), "r"(s));
  return r;
}
__device__ __forceinline__ int64_t shl_s64(int64_t x, uint32_t s) {
  int64_t r;
  asm("shl.b64 %0, %1, %2;" : "=l"(r) : "l"(x), "r"(s));
  return r;
}

// Byte-permute selectors: float bits 0x4B0000bb (= 2^23 + bb) from byte k of
// a word, and 0x4B00hhbb from its bytes 2, 3 (the top digit's 9 bits).
constexpr uint32_t kMagicHi = 0x4B000000u;
__device__ __forceinline__ float byte_float(uint32_t x, uint32_t sel) {
  return __uint_as_float(__byte_perm(x, kMagicHi, sel));
}

__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);  // exact: |digit| <= 128
  return *reinterpret_cast<const uint32_t*>(&v);
}

// Digit j (0 the most significant) of the balanced base-256 representation
// of u - B, B = 0x80 in bytes 0..6, times s (+-1): (byte_{6-j}(u) - 128) s,
// the top one from bits 48..56; float (2^23 + byte) from a byte permute, then
// one FMA with c = -(2^23 + 128) s.
__device__ __forceinline__ float digit_of(uint64_t u, int j, float s, float c) {
  const uint32_t ul = (uint32_t)u, uh = (uint32_t)(u >> 32);
  switch (j) {
    case 0: return fmaf(byte_float(uh, 0x7532), s, c);
    case 1: return fmaf(byte_float(uh, 0x7541), s, c);
    case 2: return fmaf(byte_float(uh, 0x7540), s, c);
    case 3: return fmaf(byte_float(ul, 0x7543), s, c);
    case 4: return fmaf(byte_float(ul, 0x7542), s, c);
    case 5: return fmaf(byte_float(ul, 0x7541), s, c);
    default: return fmaf(byte_float(ul, 0x7540), s, c);
  }
}
constexpr uint64_t kDigitBias = 0x0080808080808080ull;

// An FP64 value (bits lo, hi) on its column's grid, as u = v + B and its sign
// s = +-1: ecm is the column's largest exponent field (hi & 0x7FF00000, at
// least 64 << 20); v = |x| 2^(1077 - Ec) = (mantissa << 2) >> (Ec - E) <
// 2^55.  Zeros and subnormals (exponent field 0) shift out.
__device__ __forceinline__ uint64_t align_fp64(uint32_t lo, uint32_t hi, uint32_t ecm, float& s) {
  const uint32_t d = (ecm - (hi & 0x7FF00000u)) >> 20;
  const uint64_t mant = ((uint64_t)((hi & 0x000FFFFFu) | 0x00100000u) << 32) | lo;
  s = __uint_as_float((hi & 0x80000000u) | 0x3F800000u);  // +-1 (one integer op)
  return shr_u64(mant << 2, d) + kDigitBias;
}

// Store the 7 digit slices of NV consecutive K indices (k0 ..) of operand row
// `row`: per slice, the digits of value pairs packed in BF16 pairs, one
// 16-byte (NV = 8) or 8-byte (NV = 4) store.  u: values + B, s: their signs.
template <int NV>
__device__ __forceinline__ void store_digits(unsigned char* sA, uint32_t a_bytes, uint32_t off,
                                             const uint64_t (&u)[NV], const float (&s)[NV]) {
#pragma unroll
  for (int j = 0; j < kTc64Slices; j++) {
    uint32_t pk[NV / 2];
#pragma unroll
    for (int p = 0; p < NV / 2; p++) {
      const float d0 = digit_of(u[2 * p], j, s[2 * p], s[2 * p] * -8388736.0f);
      const float d1 = digit_of(u[2 * p + 1], j, s[2 * p + 1], s[2 * p + 1] * -8388736.0f);
      pk[p] = pack_bf16x2(d0, d1);
    }
    if constexpr (NV == 8)
      *reinterpret_cast<uint4*>(sA + j * a_bytes + off) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
    else
      *reinterpret_cast<uint2*>(sA + j * a_bytes + off) = make_uint2(pk[0], pk[1]);
  }
}

// Y = sum_o S_o 2^(8(5-o)) for o <= 5, plus floor((S_6 2^8 + S_7) / 2^16),
// from the exact integer order sums S_o (|S_o| < 2^22, held in FP32): S + 1.5
// 2^23 has the bits 0x4B400000 + S.
__device__ __forceinline__ int64_t combine_orders(float s0, float s1, float s2, float s3, float s4, float s5,
                                                  float s6, float s7) {
  constexpr float M = 12582912.0f;
  constexpr uint32_t K257 = 257u * 0x4B400000u;  // mod 2^32
  const uint32_t b0 = __float_as_uint(s0 + M), b1 = __float_as_uint(s1 + M), b2 = __float_as_uint(s2 + M),
                 b3 = __float_as_uint(s3 + M), b4 = __float_as_uint(s4 + M), b5 = __float_as_uint(s5 + M),
                 b6 = __float_as_uint(s6 + M), b7 = __float_as_uint(s7 + M);
  const int32_t p01 = (int32_t)((b0 << 8) + b1 - K257);  // S_0 2^8 + S_1, below 2^31 in magnitude
  const int32_t p23 = (int32_t)((b2 << 8) + b3 - K257);
  const int32_t p45 = (int32_t)((b4 << 8) + b5 - K257);
  const int32_t p67 = (int32_t)((b6 << 8) + b7 - K257) >> 16;
  return ((int64_t)p01 << 32) + ((int64_t)p23 << 16) + (int64_t)(p45 + p67);
}

// The FP64 bits of Y 2^P: one conversion on the FP64 pipe (correctly
// rounded), then P added to the exponent field.  0 for Y = 0 and below the
// normal range.
__device__ __forceinline__ uint64_t to_fp64(int64_t Y, int P) {
  const uint64_t b = (uint64_t)__double_as_longlong(__ll2double_rn((long long)Y));
  const int E = (int)((b >> 52) & 0x7FF) + P;
  return (Y != 0 && E > 0) ? b + ((uint64_t)(int64_t)P << 52) : 0ull;
}


// One thread issues every product of a step: digit slices A_0..A_6 of the
// 128 columns against the operator's slices, slice pairs of orders 0..7, the
// pairs of order o into the accumulator at TMEM column o*R of the set.  The
// operator's slices are consecutive R-row blocks of one K-major operand, so
// A_i against slices j0..j0+nb-1 is one MMA of N = nb*R.
template <int K>
__device__ __forceinline__ void issue_step(const unsigned char* sA, const unsigned char* sBside, uint32_t dset) {
  using S = T64<K>;
  constexpr int R = S::R;
  const uint32_t a0 = tc::smem_u32(sA), b0 = tc::smem_u32(sBside);
  auto issue = [&](int i, int j0, int nb, bool overwrite) {
#pragma unroll
    for (int kk = 0; kk < R / 16; kk++) {
      const uint64_t ad = tc::smem_desc(a0 + i * S::A_BYTES + kk * 256, tc::kLbo, S::SBO);
      const uint64_t bd = tc::smem_desc(b0 + j0 * S::B_BYTES + kk * 256, tc::kLbo, S::SBO);
      tc::mma_bf16(dset + (i + j0) * R, ad, bd, tc::idesc_bf16_f32(128, nb * R), (overwrite && kk == 0) ? 0u : 1u);
    }
  };
  issue(0, 0, 1, true);   // order 0
  issue(1, 0, 7, true);   // (1, 0..6): orders 1..7
  issue(0, 1, 6, false);  // (0, 1..6): orders 1..6
#pragma unroll
  for (int i = 2; i < kTc64Slices; i++) issue(i, 0, kTc64Orders - i, false);  // (i, 0..7-i)
}

}  // namespace

template <int K>
__global__ void __launch_bounds__(kT64Threads, 1)
    k_pass_tc64(uint64_t* __restrict__ re, uint64_t* __restrict__ im, const TcDesc64<K>* __restrict__ dp,
                int* __restrict__ err) {
  using S = T64<K>;
  constexpr int D = S::D, R = S::R, G = S::G, TILE = S::TILE, ASTR = S::ASTR;
  extern __shared__ __align__(1024) unsigned char smem[];
  unsigned char* sB = smem + 2 * kTc64Slices * S::A_BYTES;                          // W digits, then V digits
  uint64_t* bufs = reinterpret_cast<uint64_t*>(sB + 2 * kTc64Slices * S::B_BYTES);  // [group][re, im][ASTR]
  T64Tables<K>& tb = *reinterpret_cast<T64Tables<K>*>(bufs + 4 * ASTR);
  const PassHeader& h = dp->h;
  const int tid = threadIdx.x, w = tid >> 5, l = tid & 31;
  const int g = w >> 4, gtid = tid & (kT64GroupThreads - 1), wg = w & 15;
  constexpr int NV = D / 2;  // values a thread holds: a quarter of a column's 2D reals
  // digit steps: column mc = 8 wg + (l & 7), quarter qc = l >> 3 -- half hc =
  // qc >> 1 (real or imaginary parts), values cc NV .. cc NV + NV - 1 of it,
  // cc = qc & 1 (the four quarters of a column in one warp)
  const int mc = 8 * wg + (l & 7), qc = l >> 3, hc = qc >> 1, cc = qc & 1;
  const int rc = mc / G, fc = mc & (G - 1);
  // accumulator steps: column m = 32 (w & 3) + l -- the TMEM lane quadrant
  // its warp may read -- quarter q = (wg >> 2) & 3: half q >> 1, values
  // chunk NV .. of it, chunk = q & 1
  const int m = 32 * (w & 3) + l, q = (wg >> 2) & 3, half = q >> 1, chunk = q & 1;
  const int r = m / G, f = m & (G - 1);
  unsigned char* sA = smem + g * kTc64Slices * S::A_BYTES;  // the group's digit operand (ket, then bra)
  uint64_t* buf = bufs + (size_t)g * 2 * ASTR;             // the group's tile, then its ket outputs
  T64Group<K>& gp = tb.grp[g];

  // ---- per-pass tables, the operator's digits, tensor memory, barriers
  {
    constexpr int per_slice = S::B_BYTES / 16;
    for (int i = tid; i < 2 * kTc64Slices * per_slice; i += blockDim.x) {
      const int side = i / (kTc64Slices * per_slice), rest = i % (kTc64Slices * per_slice);
      reinterpret_cast<uint4*>(sB)[i] = reinterpret_cast<const uint4*>(&dp->sl[side][0][0])[rest];
    }
  }
  const int mhi = h.mhi, L = h.L;
  for (int run = tid; run < (1 << mhi); run += blockDim.x) {
    uint64_t off = 0;
    for (int j = 0; j < mhi; j++) off |= (uint64_t)((run >> j) & 1) << h.hipos[j];
    tb.hioff[run] = off;
  }
  if (tid < D) {
    int lk = 0, lb = 0;
    for (int i = 0; i < K; i++) {
      lk |= ((tid >> i) & 1) << h.lket[i];
      lb |= ((tid >> i) & 1) << h.lbra[i];
    }
    tb.pk[tid] = piece_off(lk);
    tb.pb[tid] = piece_off(lb);
    tb.ew[0][tid] = dp->ew[0][tid];
    tb.ew[1][tid] = dp->ew[1][tid];
  }
  if (tid < D * D) {
    const int a = tid / D, bb = tid % D;
    int e = 0;
    for (int i = 0; i < K; i++) e |= (((a >> i) & 1) << h.lket[i]) | (((bb >> i) & 1) << h.lbra[i]);
    const int run = e >> L;
    uint64_t off = 0;
    for (int j = 0; j < mhi; j++) off |= (uint64_t)((run >> j) & 1) << h.hipos[j];
    off += (uint64_t)(e & ((1 << L) - 1));
    const uint64_t stored = (h.stmask[run >> 5] >> (run & 31)) & 1;
    tb.outoff[bb][a] = off | ((uint64_t)(dp->ew[1][bb] + 128) << 48) | (stored << 63);
  }
  if (tid < 2 * D) {
    const int i = tid & (D - 1), side = tid / D;  // side 0: ket index i, 1: bra index i
    int e = 0;
    for (int k = 0; k < K; k++) e |= ((i >> k) & 1) << (side ? h.lbra[k] : h.lket[k]);
    const int run = e >> L;
    uint64_t off = 0;
    for (int j = 0; j < mhi; j++) off |= (uint64_t)((run >> j) & 1) << h.hipos[j];
    off += (uint64_t)(e & ((1 << L) - 1));
    (side ? tb.offb : tb.offk)[i] = off;
  }
  if (tid == 0) {
    int all = 1;
    for (int run = 0; run < (1 << mhi); run++) all &= (int)((h.stmask[run >> 5] >> (run & 31)) & 1);
    tb.allstored = all;
  }
  if (tid < 8) tb.hipos[tid] = h.hipos[tid];
  if (tid < 256) tb.grp[tid >> 7].brmax[tid & 127] = 0;
  if (w == 0) {
    tc::tmem_alloc(&tb.slot, S::TMEM_COLS);
    tc::tmem_relinquish();
  }
  if (tid == 0) {
    for (int gi = 0; gi < 2; gi++) {
      tc::mbar_init(&tb.grp[gi].full, 1);
      tc::mbar_init(&tb.grp[gi].mma, 1);
    }
    tc::mbar_fence_init();
  }
  tc::fence_proxy_async_smem();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tb.slot + (uint32_t)g * S::SET_COLS;  // the group's accumulator set
  const uint32_t tlane = (uint32_t)(32 * (w & 3)) << 16;

  auto free_off = [&](int ff) {  // local offset of free group ff
    int o = 0;
    for (int j = 0; j < h.g; j++) o |= ((ff >> j) & 1) << h.freepos[j];
    return o;
  };
  const int lf = free_off(f);  // accumulator steps: free offset of column (., f) in the state
  // digit steps: column (b = rc, fc)'s values a = cc NV + i of half hc at
  // buf[basec + tb.pk[cc NV + i]] (the offsets read from shared memory, a
  // broadcast per 8 lanes, to keep the 64-register budget)
  const int basec = hc * ASTR + tb.pb[rc] + piece_off(free_off(fc));
  const uint64_t ntiles = h.ntiles, gstep = 2 * (uint64_t)gridDim.x;
  const int runlen = 1 << L, lgp = L < 4 ? L : 4, npieces = (2 * TILE) >> lgp;
  // The ket step's exact integer outputs Y(a, b) of column (b, ff) replace
  // the tile in its buffer, at [hh][a][b ^ (a & 1)][ff]: the ket step writes,
  // for one a, 32 consecutive words per warp, and the bra step reads, for one
  // b, columns a of both parities -- both free of bank conflicts.
  auto yoff = [&](int hh, int a, int b, int ff) { return hh * ASTR + (a * D + (b ^ (a & 1))) * G + ff; };
  auto tile_base_s = [&](uint64_t t) {  // tile_base from the staged positions
    uint64_t base = t << L;
    for (int j = 0; j < mhi; j++) {
      const int p = tb.hipos[j];
      base = ((base >> p) << (p + 1)) | (base & ((1ull << p) - 1));
    }
    return base;
  };

  // Loads of a tile into the group's buffer: the group's first thread arms
  // its barrier with the tile's bytes before a group barrier, after which
  // every thread of the group issues its share of the 1-D bulk copies, one
  // per piece (16 entries, or a whole run when runs are shorter) of each
  // array.
  auto copy_tile = [&](uint64_t base) {
    for (int i = gtid; i < npieces; i += kT64GroupThreads) {
      const int arr = i & 1, e0 = (i >> 1) << lgp;
      const int run = e0 >> L, o = e0 & (runlen - 1);
      tc::bulk_g2s(buf + arr * ASTR + piece_off(e0), (arr ? im : re) + base + tb.hioff[run] + o, 8u << lgp,
                   &gp.full);
    }
  };

  // outstanding asynchronous work of this thread's view; a phase that did not
  // complete stays pending (the teardown waits for it again)
  uint32_t phf = 0, phm = 0;
  int pendf = 0, pendm = 0;
  bool bad = false;  // one of this thread's waits expired
  auto wait = [&](uint64_t* bar, uint32_t& ph, int& pend) {
    if (!tc::mbar_wait_bounded(bar, ph, kT64WaitPolls)) {
      bad = true;
      return false;
    }
    ph ^= 1u;
    pend = 0;
    return true;
  };

  // ---- prologue: the group's first tile in flight
  uint64_t t = blockIdx.x + (uint64_t)g * gridDim.x;
  uint64_t tbase = t < ntiles ? tile_base_s(t) : 0;
  if (gtid == 0 && t < ntiles) tc::mbar_arrive_expect_tx(&gp.full, S::TX_BYTES);
  group_bar(g);
  if (t < ntiles) {
    copy_tile(tbase);
    pendf = 1;
  }

  for (; t < ntiles; t += gstep) {
    // ---- 1: the tile's values of column (b = rc, fc), quarter qc, its grid
    // (the largest exponent of the column's four quarters, two shuffles
    // away), its ket digits
    wait(&gp.full, phf, pendf);
    {
      uint64_t u[NV];
      float sg[NV];
      uint32_t emx = 0;
#pragma unroll
      for (int i = 0; i < NV; i++) {
        u[i] = buf[basec + tb.pk[cc * NV + i]];
        emx = max(emx, (uint32_t)(u[i] >> 32) & 0x7FF00000u);
      }
      emx = max(emx, __shfl_xor_sync(0xffffffffu, emx, 8));
      emx = max(emx, __shfl_xor_sync(0xffffffffu, emx, 16));
      const uint32_t ecm = max(emx, 64u << 20);
      if (qc == 0) gp.colEt[rc][fc] = (int)(ecm >> 20);
#pragma unroll
      for (int i = 0; i < NV; i++) u[i] = align_fp64((uint32_t)u[i], (uint32_t)(u[i] >> 32), ecm, sg[i]);
      store_digits<NV>(sA, S::A_BYTES, tc_kmajor_offset(mc, hc * D + cc * NV, S::SBO), u, sg);
    }
    tc::fence_proxy_async_smem();
    tc::fence_before_sync();
    if (group_bar_or(g, bad)) break;
    tc::fence_after_sync();

    // ---- 2: ket products
    if (gtid == 0) {
      issue_step<K>(sA, sB, tmem);
      tc::mma_commit(&gp.mma);
    }
    pendm = 1;

    // ---- 3: ket outputs of column (b = r, f) -> exact integers (in place of
    // the tile), and the bra columns' magnitude keys: Ec + exponent of |S_0| +
    // |S_1|/256 + 65, which bounds |Y| 2^Ec by 2^(key - 86) (1 + 2^-23)
    if (wait(&gp.mma, phm, pendm)) {
      tc::fence_after_sync();
      const uint32_t Ec = (uint32_t)gp.colEt[r][f];
#pragma unroll
      for (int c4 = 0; c4 < NV; c4 += 4) {
        float sv[kTc64Orders][4];
        const uint32_t ta = tmem + tlane + half * D + chunk * NV + c4;
#pragma unroll
        for (int o = 0; o < kTc64Orders; o++) tc::tmem_ld4(ta + o * R, sv[o]);
        tc::tmem_wait_ld();
#pragma unroll
        for (int c = 0; c < 4; c++) {
          const int a = chunk * NV + c4 + c;
          buf[yoff(half, a, r, f)] = (uint64_t)combine_orders(sv[0][c], sv[1][c], sv[2][c], sv[3][c], sv[4][c],
                                                              sv[5][c], sv[6][c], sv[7][c]);
          const float mag = fmaf(fabsf(sv[1][c]), 0.00390625f, fabsf(sv[0][c])) + 65.0f;
          atomicMax(&gp.brmax[a * G + f], Ec + (__float_as_uint(mag) >> 23));
        }
      }
    }
    tc::fence_before_sync();
    if (group_bar_or(g, bad)) break;
    tc::fence_after_sync();

    // ---- 4: bra digits of column (a = rc, fc), quarter qc: values Y_b
    // 2^Ec(b) on the grid 2^(mkey - 141), |v| < 2^55 (1 + 2^-23)
    const uint32_t mkey_out = gp.brmax[m];  // the key of this thread's column in step 6
    {
      const uint32_t mkey = gp.brmax[mc];
      uint64_t u[NV];
      float sg[NV];
#pragma unroll
      for (int i = 0; i < NV; i++) {
        const int b = cc * NV + i;
        const int64_t Y = (int64_t)buf[yoff(hc, rc, b, fc)];
        const int sh = (int)mkey - 141 - gp.colEt[b][fc];
        const int64_t v = sh >= 0 ? shr_s64(Y, (uint32_t)sh) : shl_s64(Y, (uint32_t)(-sh));
        u[i] = (uint64_t)v + kDigitBias;
        sg[i] = 1.0f;
      }
      store_digits<NV>(sA, S::A_BYTES, tc_kmajor_offset(mc, hc * D + cc * NV, S::SBO), u, sg);
    }
    const uint64_t tn = t + gstep;
    if (gtid == 0 && tn < ntiles) tc::mbar_arrive_expect_tx(&gp.full, S::TX_BYTES);  // the group's next tile
    tc::fence_proxy_async_smem();
    tc::fence_before_sync();
    group_bar(g);
    tc::fence_after_sync();

    // ---- 5: bra products; the group's next tile into the freed buffer
    if (gtid == 0) {
      issue_step<K>(sA, sB + kTc64Slices * S::B_BYTES, tmem);
      tc::mma_commit(&gp.mma);
    }
    pendm = 1;
    if (gtid < 128) gp.brmax[gtid] = 0;  // the next tile's magnitude keys
    const uint64_t nbase = tn < ntiles ? tile_base_s(tn) : 0;
    if (tn < ntiles) {
      copy_tile(nbase);
      pendf = 1;
    }

    // ---- 6: bra outputs of column (a = r, f) -> FP64 -> the tile's stored runs
    if (wait(&gp.mma, phm, pendm)) {
      tc::fence_after_sync();
      const int pa = (int)mkey_out + tb.ew[0][r] - 1106 - 128;
      uint64_t* arr = (half ? im : re) + tbase + lf;
      uint64_t* col = arr + tb.offk[r];
#pragma unroll
      for (int c4 = 0; c4 < NV; c4 += 4) {
        float sv[kTc64Orders][4];
        const uint32_t ta = tmem + tlane + half * D + chunk * NV + c4;
#pragma unroll
        for (int o = 0; o < kTc64Orders; o++) tc::tmem_ld4(ta + o * R, sv[o]);
        tc::tmem_wait_ld();
        if (tb.allstored) {  // the common case: one base per thread, one offset per output
#pragma unroll
          for (int c = 0; c < 4; c++) {
            const int b = chunk * NV + c4 + c;
            const int64_t Y =
                combine_orders(sv[0][c], sv[1][c], sv[2][c], sv[3][c], sv[4][c], sv[5][c], sv[6][c], sv[7][c]);
            col[tb.offb[b]] = to_fp64(Y, pa + 128 + tb.ew[1][b]);
          }
        } else {
#pragma unroll
          for (int c = 0; c < 4; c++) {
            const uint64_t T = tb.outoff[chunk * NV + c4 + c][r];
            if (!(T >> 63)) continue;  // a run the pass does not change
            const int64_t Y =
                combine_orders(sv[0][c], sv[1][c], sv[2][c], sv[3][c], sv[4][c], sv[5][c], sv[6][c], sv[7][c]);
            arr[T & 0xFFFFFFFFFFFFull] = to_fp64(Y, pa + (int)((T >> 48) & 0xFF));
          }
        }
      }
    }
    tc::fence_before_sync();  // the next tile's first group barrier orders these reads before its MMAs
    tbase = nbase;
  }

  // ---- teardown: nothing of this group may still be in flight when the
  // block's tensor memory and shared memory are released (bounded, after an
  // expiry)
  if (group_bar_or(g, bad)) {
    if (pendm) tc::mbar_wait_bounded(&gp.mma, phm, kT64WaitPolls << 2);
    if (pendf) tc::mbar_wait_bounded(&gp.full, phf, kT64WaitPolls << 2);
    if (gtid == 0) atomicExch(err, 1);
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (w == 0) tc::tmem_dealloc(tb.slot, S::TMEM_COLS);
}

template <int K>
static cudaError_t configure_tc64() {
  constexpr size_t smem = t64_smem_bytes<K>();
  static_assert(smem <= 227 * 1024, "one block's shared memory");
  cudaError_t e = cudaFuncSetAttribute(k_pass_tc64<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_pass_tc64<K>, cudaFuncAttributePreferredSharedMemoryCarveout,
                             (int)cudaSharedmemCarveoutMaxShared);
  return e;
}

template <int K>
static cudaError_t launch_tc64_k(const LaunchArgs& a, cudaStream_t s) {
  static int configured = 0;
  if (!configured) {
    cudaError_t e = configure_tc64<K>();
    if (e != cudaSuccess) return e;
    configured = 1;
  }
  k_pass_tc64<K><<<a.grid, kT64Threads, t64_smem_bytes<K>(), s>>>(
      static_cast<uint64_t*>(a.re), static_cast<uint64_t*>(a.im), static_cast<const TcDesc64<K>*>(a.desc), a.err);
  return cudaGetLastError();
}

cudaError_t launch_pass_tc64(const LaunchArgs& a, cudaStream_t s) {
  if (!a.err || (a.K != 3 && a.K != 4) || a.arith != AR_FP64) return cudaErrorInvalidValue;
  return a.K == 3 ? launch_tc64_k<3>(a, s) : launch_tc64_k<4>(a, s);
}

}  // namespace dmg
