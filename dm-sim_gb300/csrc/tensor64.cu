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
// Threads: 512 (16 warps), one block per SM.  Thread (warp w, lane l) owns
// tile column m = 32 (w & 3) + l -- the TMEM lane its warp may read -- and
// quarter q = w >> 2 of it: R/4 consecutive values (real parts for q < 2,
// imaginary parts for q >= 2).  Thread 0 issues the MMAs; every thread
// issues its share of the bulk copies.  Per tile:
//   2. ket digits -> A_ket;  3. the ket MMAs (TMEM set t&1)
//   4. the previous tile's bra accumulators -> FP64 -> global stores,
//      overlapping the ket MMAs
//   5. ket accumulators -> exact int64 outputs in the tile buffer
//   6. bra digits -> A_bra; the next tile's values (TMA bulk copies of its
//      runs, issued two tiles ahead) and their column maxima
//   7. the bra MMAs (same set);  8. the loads two tiles ahead into the freed
//      buffer.  The bra MMAs overlap the next tile's steps 2-3.
// Three block barriers per tile (after steps 2, 5 and 6).  Every wait is
// bounded; on expiry the block sets the error flag, waits (bounded) for its
// own copies and MMAs in flight, releases its TMEM and returns, and the host
// reports DMSIM_ERR_TIMEOUT.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "kernels.h"
#include "pass_device.cuh"
#include "tc.cuh"

namespace dmg {

namespace {

constexpr int kT64Threads = 512;
constexpr uint32_t kT64WaitPolls = 1u << 24;

template <int K>
struct T64 {
  static constexpr int D = 1 << K, R = 2 * D, G = 128 / D, TILE = 128 * D;
  static constexpr int Q = R / 4;                          // values of one column per thread
  static constexpr uint32_t SBO = 16 * R;                  // bytes between 8-row groups of an R-wide operand
  static constexpr uint32_t A_BYTES = 128 * R * 2;         // one digit slice of the 128 columns
  static constexpr uint32_t B_BYTES = R * R * 2;           // one digit slice of W or V
  static constexpr uint32_t SET_COLS = kTc64Orders * R;    // accumulators of one step
  static constexpr uint32_t TMEM_COLS = 2 * SET_COLS;      // two sets: 512 (K = 4), 256 (K = 3)
  static constexpr uint32_t BUF_BYTES = TILE * 8 * 2;      // one tile, re + im, 8 bytes per real
  static_assert(TMEM_COLS <= 512, "two accumulator sets must fit in tensor memory");
};

template <int K>
struct T64Tables {
  static constexpr int D = 1 << K;
  uint64_t hioff[256];
  uint64_t full[2];       // tile loads into buffer 0 / 1
  uint64_t mma[2];        // commits of the ket (0) and bra (1) products
  uint32_t stmask[8];
  int lk[D], lb[D];
  int ew[2][D];
  // output (a, b) of a tile: bits 0..47 its offset from the tile base minus
  // the free bits, bits 48..55 the bra row exponent ew[1][b] + 128, bit 63
  // set when its run is stored
  uint64_t outoff[D][D];
  uint32_t colmax[4][128];  // per quarter and column: largest FP64 exponent field
  uint32_t brmax[2][128];   // per tile parity and bra column: magnitude key of the ket outputs
  int colEt[128 / D][D];    // biased exponent of ket column (b, f)'s grid, at [f][b]
  uint32_t slot;
  int abort_;
};

template <int K>
constexpr size_t t64_smem_bytes() {
  using S = T64<K>;
  return 2 * (size_t)kTc64Slices * S::A_BYTES + 2 * (size_t)kTc64Slices * S::B_BYTES + 2 * (size_t)S::BUF_BYTES +
         sizeof(T64Tables<K>);
}

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

// The 7 digits (digit 0 the most significant) of the balanced base-256
// representation of u - B, B = 0x80 in bytes 0..6, each times s and shifted
// by c: digit j = (byte_{6-j}(u) - 128) s, the top one from bits 48..56.
__device__ __forceinline__ void digits_of(uint64_t u, float s, float c, float (&dg)[kTc64Slices]) {
  const uint32_t ul = (uint32_t)u, uh = (uint32_t)(u >> 32);
  dg[6] = fmaf(byte_float(ul, 0x7540), s, c);
  dg[5] = fmaf(byte_float(ul, 0x7541), s, c);
  dg[4] = fmaf(byte_float(ul, 0x7542), s, c);
  dg[3] = fmaf(byte_float(ul, 0x7543), s, c);
  dg[2] = fmaf(byte_float(uh, 0x7540), s, c);
  dg[1] = fmaf(byte_float(uh, 0x7541), s, c);
  dg[0] = fmaf(byte_float(uh, 0x7532), s, c);
}
constexpr uint64_t kDigitBias = 0x0080808080808080ull;

// Digits of an FP64 value (bits lo, hi) on its column's grid: ecm is the
// column's largest exponent field (hi & 0x7FF00000, at least 64 << 20).
// v = |x| 2^(1077 - Ec) = (mantissa << 2) >> (Ec - E) < 2^55; the sign is
// applied to every digit.  Zeros and subnormals (exponent field 0) shift out.
__device__ __forceinline__ void digits_fp64(uint32_t lo, uint32_t hi, uint32_t ecm, float (&dg)[kTc64Slices]) {
  const uint32_t d = (ecm - (hi & 0x7FF00000u)) >> 20;
  const uint64_t mant = ((uint64_t)((hi & 0x000FFFFFu) | 0x00100000u) << 32) | lo;
  const uint64_t u = shr_u64(mant << 2, d) + kDigitBias;
  const uint32_t sgn = hi & 0x80000000u;
  digits_of(u, __uint_as_float(sgn | 0x3F800000u), __uint_as_float(sgn ^ 0xCB000080u), dg);  // +-1, -+(2^23 + 128)
}

// Digits of a signed integer |v| < 2^55.
__device__ __forceinline__ void digits_int(int64_t v, float (&dg)[kTc64Slices]) {
  digits_of((uint64_t)v + kDigitBias, 1.0f, -8388736.0f, dg);  // -(2^23 + 128)
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

__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);  // exact: |digit| <= 128
  return *reinterpret_cast<const uint32_t*>(&v);
}

// Store the packed digits of Q consecutive K indices of row m (pk[i][j]:
// values 2i, 2i+1 of slice j) into the K-major operand, one 16-byte (Q = 8)
// or 8-byte (Q = 4) store per slice.
template <int Q>
__device__ __forceinline__ void store_packed(unsigned char* sA, uint32_t a_bytes, uint32_t off,
                                             const uint32_t (&pk)[Q / 2][kTc64Slices]) {
#pragma unroll
  for (int j = 0; j < kTc64Slices; j++) {
    if constexpr (Q == 8)
      *reinterpret_cast<uint4*>(sA + j * a_bytes + off) = make_uint4(pk[0][j], pk[1][j], pk[2][j], pk[3][j]);
    else
      *reinterpret_cast<uint2*>(sA + j * a_bytes + off) = make_uint2(pk[0][j], pk[1][j]);
  }
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
  constexpr int D = S::D, R = S::R, G = S::G, Q = S::Q, TILE = S::TILE;
  extern __shared__ __align__(1024) unsigned char smem[];
  unsigned char* sAk = smem;
  unsigned char* sAb = sAk + kTc64Slices * S::A_BYTES;
  unsigned char* sB = sAb + kTc64Slices * S::A_BYTES;  // W digits, then V digits
  uint64_t* bufs = reinterpret_cast<uint64_t*>(sB + 2 * kTc64Slices * S::B_BYTES);  // [buffer][re, im][TILE]
  T64Tables<K>& tb = *reinterpret_cast<T64Tables<K>*>(bufs + 4 * TILE);
  const PassHeader& h = dp->h;
  const int tid = threadIdx.x, w = tid >> 5, l = tid & 31;
  const int m = 32 * (w & 3) + l, q = w >> 2;
  const int r = m / G, f = m & (G - 1);
  const int c0 = q * Q;       // first value of this thread's quarter of a column
  const int half = c0 / D;    // 0: real parts, 1: imaginary parts
  const int cb = c0 % D;      // first ket (ket step) or bra (bra step) index of the quarter

  // ---- per-pass tables, the operator's digits, tensor memory, barriers
  {
    constexpr int per_slice = S::B_BYTES / 16;
    for (int i = tid; i < 2 * kTc64Slices * per_slice; i += blockDim.x) {
      const int side = i / (kTc64Slices * per_slice), rest = i % (kTc64Slices * per_slice);
      reinterpret_cast<uint4*>(sB)[i] = reinterpret_cast<const uint4*>(&dp->sl[side][0][0])[rest];
    }
  }
  for (int run = tid; run < (1 << h.mhi); run += blockDim.x) {
    uint64_t off = 0;
    for (int j = 0; j < h.mhi; j++) off |= (uint64_t)((run >> j) & 1) << h.hipos[j];
    tb.hioff[run] = off;
  }
  if (tid < 8) tb.stmask[tid] = h.stmask[tid];
  if (tid < D) {
    int lk = 0, lb = 0;
    for (int i = 0; i < K; i++) {
      lk |= ((tid >> i) & 1) << h.lket[i];
      lb |= ((tid >> i) & 1) << h.lbra[i];
    }
    tb.lk[tid] = lk;
    tb.lb[tid] = lb;
    tb.ew[0][tid] = dp->ew[0][tid];
    tb.ew[1][tid] = dp->ew[1][tid];
  }
  if (tid < D * D) {
    const int a = tid / D, bb = tid % D;
    int e = 0;
    for (int i = 0; i < K; i++) e |= (((a >> i) & 1) << h.lket[i]) | (((bb >> i) & 1) << h.lbra[i]);
    const int run = e >> h.L;
    uint64_t off = 0;
    for (int j = 0; j < h.mhi; j++) off |= (uint64_t)((run >> j) & 1) << h.hipos[j];
    off += (uint64_t)(e & ((1 << h.L) - 1));
    const uint64_t stored = (h.stmask[run >> 5] >> (run & 31)) & 1;
    tb.outoff[a][bb] = off | ((uint64_t)(dp->ew[1][bb] + 128) << 48) | (stored << 63);
  }
  if (tid < 128) tb.brmax[0][tid] = tb.brmax[1][tid] = 0;
  if (tid == 0) tb.abort_ = 0;
  if (w == 0) {
    tc::tmem_alloc(&tb.slot, S::TMEM_COLS);
    tc::tmem_relinquish();
  }
  if (tid == 0) {
    tc::mbar_init(&tb.full[0], 1);
    tc::mbar_init(&tb.full[1], 1);
    tc::mbar_init(&tb.mma[0], 1);
    tc::mbar_init(&tb.mma[1], 1);
    tc::mbar_fence_init();
  }
  tc::fence_proxy_async_smem();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tb.slot;
  const uint32_t tlane = (uint32_t)(32 * (w & 3)) << 16;

  int lf_g = 0;  // free-bit offset of this column's group f (the same in both steps)
  for (int j = 0; j < h.g; j++) lf_g |= ((f >> j) & 1) << h.freepos[j];
  const int L = h.L, runlen = 1 << L, ncopies = 2 << h.mhi;  // runs of the real and imaginary arrays
  const uint64_t ntiles = h.ntiles, step = gridDim.x;
  // this thread's values of the loaded tile (ket step): entries (a = cb + c, r, f) at basek + offk[c]
  int offk[Q];
#pragma unroll
  for (int c = 0; c < Q; c++) offk[c] = tb.lk[cb + c];
  const int basek = tb.lb[r] + lf_g;
  // accumulators are read and digits written 4 values at a time
  constexpr int QH = 4;
  // The ket step's exact integer outputs replace the tile in its buffer, at
  // [half][a][b ^ (a & 1)][f]: the ket step writes, for one a, 32 consecutive
  // words per warp, and the bra step reads, for one b, columns a of both
  // parities -- both free of bank conflicts.
  auto yidx = [&](int a, int b) { return half * TILE + (a * D + (b ^ (a & 1))) * G + f; };

  // Loads of a tile: thread 0 arms the buffer's barrier with the tile's bytes
  // before a block barrier, after which every thread issues its share of the
  // 1-D bulk copies (one per run of each array).
  auto copy_tile = [&](uint64_t t, int b) {
    uint64_t* dst = bufs + (size_t)b * 2 * TILE;
    const uint64_t base = tile_base(h, t);
    for (int i = tid; i < ncopies; i += kT64Threads) {
      const int run = i >> 1, arr = i & 1;
      tc::bulk_g2s(dst + arr * TILE + run * runlen, (arr ? im : re) + base + tb.hioff[run], (uint32_t)runlen * 8u,
                   &tb.full[b]);
    }
  };

  // outstanding asynchronous work, the same on every thread
  uint32_t phf0 = 0, phf1 = 0, phk = 0, phb = 0;
  int pendf0 = 0, pendf1 = 0, pendk = 0, pendb = 0;
  bool timed_out = false;
  // a phase that did not complete stays pending (the teardown waits for it again)
  auto wait = [&](uint64_t* bar, uint32_t& ph, int& pend) {
    if (!tc::mbar_wait_bounded(bar, ph, kT64WaitPolls)) {
      timed_out = true;
      tb.abort_ = 1;
      return;
    }
    ph ^= 1u;
    pend = 0;
  };
  auto wait_full = [&](int b) {
    if (b) wait(&tb.full[1], phf1, pendf1);
    else wait(&tb.full[0], phf0, pendf0);
  };

  // the previous tile's bra outputs -> FP64 -> its stored runs
  auto bra_out = [&](uint32_t set, uint64_t base, uint32_t mkey) {
    const int pa = (int)mkey + tb.ew[0][r] - 1106 - 128;
    uint64_t* arr = (half ? im : re) + base + lf_g;
#pragma unroll
    for (int c4 = 0; c4 < Q; c4 += QH) {
      float sv[kTc64Orders][QH];
      const uint32_t ta = tmem + tlane + set + c0 + c4;
#pragma unroll
      for (int o = 0; o < kTc64Orders; o++) tc::tmem_ld4(ta + o * R, sv[o]);
      tc::tmem_wait_ld();
#pragma unroll
      for (int c = 0; c < QH; c++) {
        const uint64_t T = tb.outoff[r][cb + c4 + c];
        if (!(T >> 63)) continue;  // a run the pass does not change
        const int64_t Y =
            combine_orders(sv[0][c], sv[1][c], sv[2][c], sv[3][c], sv[4][c], sv[5][c], sv[6][c], sv[7][c]);
        arr[T & 0xFFFFFFFFFFFFull] = to_fp64(Y, pa + (int)((T >> 48) & 0xFF));
      }
    }
    tc::fence_before_sync();
  };

  // this thread's values of the tile in buffer b (ket step) and their largest exponent field
  uint32_t xl[Q], xh[Q];
  auto read_tile = [&](int b) {
    const uint64_t* barr = bufs + (size_t)b * 2 * TILE + (half ? TILE : 0);
    uint32_t emx = 0;
#pragma unroll
    for (int c = 0; c < Q; c++) {
      const uint64_t v = barr[basek + offk[c]];
      xl[c] = (uint32_t)v;
      xh[c] = (uint32_t)(v >> 32);
      emx = max(emx, xh[c] & 0x7FF00000u);
    }
    tb.colmax[q][m] = emx;
  };

  // ---- prologue: the first two tiles in flight, the first one's values
  const uint64_t t0 = blockIdx.x;
  if (tid == 0) {
    if (t0 < ntiles) tc::mbar_arrive_expect_tx(&tb.full[0], S::BUF_BYTES);
    if (t0 + step < ntiles) tc::mbar_arrive_expect_tx(&tb.full[1], S::BUF_BYTES);
  }
  __syncthreads();
  if (t0 < ntiles) copy_tile(t0, 0);
  if (t0 + step < ntiles) copy_tile(t0 + step, 1);
  pendf0 = t0 < ntiles;
  pendf1 = t0 + step < ntiles;
  if (t0 < ntiles) {
    wait_full(0);
    read_tile(0);
  }
  __syncthreads();

  bool has_prev = false;
  uint64_t prev_base = 0;
  uint32_t prev_set = 0, prev_mkey = 0;
  int it = 0;
  for (uint64_t t = t0; t < ntiles; t += step, it++) {
    if (tb.abort_) break;
    const int b = it & 1;
    const uint32_t set = (uint32_t)b * S::SET_COLS;
    uint64_t* buf = bufs + (size_t)b * 2 * TILE;
    const uint64_t tn = t + 2 * step;

    // ---- 2: ket digits of column (b = r, f), from the values read before the last barrier
    int Ec = 0;
    {
      uint32_t ecm = max(max(tb.colmax[0][m], tb.colmax[1][m]), max(tb.colmax[2][m], tb.colmax[3][m]));
      ecm = max(ecm, 64u << 20);
      Ec = (int)(ecm >> 20);
      if (q == 0) tb.colEt[f][r] = Ec;
      uint32_t pk[Q / 2][kTc64Slices];
#pragma unroll
      for (int c2 = 0; c2 < Q / 2; c2++) {
        float d0[kTc64Slices], d1[kTc64Slices];
        digits_fp64(xl[2 * c2], xh[2 * c2], ecm, d0);
        digits_fp64(xl[2 * c2 + 1], xh[2 * c2 + 1], ecm, d1);
#pragma unroll
        for (int j = 0; j < kTc64Slices; j++) pk[c2][j] = pack_bf16x2(d0[j], d1[j]);
      }
      store_packed<Q>(sAk, S::A_BYTES, tc_kmajor_offset(m, c0, S::SBO), pk);
      tc::fence_proxy_async_smem();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();

    // ---- 3: ket products
    if (tid == 0) {
      issue_step<K>(sAk, sB, tmem + set);
      tc::mma_commit(&tb.mma[0]);
    }
    {
      pendk = 1;
      // ---- 4: the previous tile's outputs (overlapping the ket products)
      if (has_prev) {
        wait(&tb.mma[1], phb, pendb);
        tc::fence_after_sync();
        if (!timed_out) bra_out(prev_set, prev_base, prev_mkey);
      }
      // ---- 5: ket outputs -> exact integers (in place of the tile), and the
      // bra columns' magnitude keys: Ec + exponent of |S_0| + |S_1|/256 + 65,
      // which bounds |Y| 2^Ec by 2^(key - 86) (1 + 2^-23)
      wait(&tb.mma[0], phk, pendk);
      tc::fence_after_sync();
      if (!timed_out) {
#pragma unroll
        for (int c4 = 0; c4 < Q; c4 += QH) {
          float sv[kTc64Orders][QH];
          const uint32_t ta = tmem + tlane + set + c0 + c4;
#pragma unroll
          for (int o = 0; o < kTc64Orders; o++) tc::tmem_ld4(ta + o * R, sv[o]);
          tc::tmem_wait_ld();
#pragma unroll
          for (int c = 0; c < QH; c++) {
            const int a = cb + c4 + c;
            buf[yidx(a, r)] = (uint64_t)combine_orders(sv[0][c], sv[1][c], sv[2][c], sv[3][c], sv[4][c], sv[5][c],
                                                       sv[6][c], sv[7][c]);
            const float mag = fmaf(fabsf(sv[1][c]), 0.00390625f, fabsf(sv[0][c])) + 65.0f;
            atomicMax(&tb.brmax[b][a * G + f], (uint32_t)Ec + (__float_as_uint(mag) >> 23));
          }
        }
      }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (tb.abort_) break;
    tc::fence_after_sync();

    // ---- 6: bra digits of column (a = r, f): values Y_b 2^Ec(b) on the grid
    // 2^(mkey - 141), |v| < 2^55 (1 + 2^-23)
    const uint32_t mkey = tb.brmax[b][m];
    {
      int ecol[Q];
#pragma unroll
      for (int c = 0; c < Q; c++) ecol[c] = tb.colEt[f][cb + c];
      uint32_t pk[Q / 2][kTc64Slices];
#pragma unroll
      for (int c2 = 0; c2 < Q / 2; c2++) {
        float d[2][kTc64Slices];
#pragma unroll
        for (int u = 0; u < 2; u++) {
          const int c = 2 * c2 + u;
          const int64_t Y = (int64_t)buf[yidx(r, cb + c)];
          const int sh = (int)mkey - 141 - ecol[c];
          const int64_t v = sh >= 0 ? shr_s64(Y, (uint32_t)sh) : shl_s64(Y, (uint32_t)(-sh));
          digits_int(v, d[u]);
        }
#pragma unroll
        for (int j = 0; j < kTc64Slices; j++) pk[c2][j] = pack_bf16x2(d[0][j], d[1][j]);
      }
      store_packed<Q>(sAb, S::A_BYTES, tc_kmajor_offset(m, c0, S::SBO), pk);
      // the next tile's values (its loads were issued two tiles ago)
      if (t + step < ntiles) {
        wait_full(b ^ 1);
        read_tile(b ^ 1);
      }
      if (tid < 128) tb.brmax[b ^ 1][tid] = 0;  // the next tile's magnitude keys
      if (tid == 0 && tn < ntiles) tc::mbar_arrive_expect_tx(&tb.full[b], S::BUF_BYTES);  // this buffer's next loads
      tc::fence_proxy_async_smem();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();

    // ---- 7: bra products; 8: the loads two tiles ahead into this buffer
    if (tid == 0) {
      issue_step<K>(sAb, sB + kTc64Slices * S::B_BYTES, tmem + set);
      tc::mma_commit(&tb.mma[1]);
    }
    pendb = 1;
    if (tn < ntiles) {
      copy_tile(tn, b);
      if (b) pendf1 = 1;
      else pendf0 = 1;
    }
    has_prev = true;
    prev_base = tile_base(h, t);
    prev_set = set;
    prev_mkey = mkey;
  }
  if (has_prev && !tb.abort_) {
    wait(&tb.mma[1], phb, pendb);
    tc::fence_after_sync();
    if (!timed_out) bra_out(prev_set, prev_base, prev_mkey);
  }
  // ---- teardown: nothing of this block may still be in flight when its
  // tensor memory and shared memory are released (bounded, after an expiry)
  __syncthreads();
  if (tb.abort_) {
    if (pendk) tc::mbar_wait_bounded(&tb.mma[0], phk, kT64WaitPolls << 2);
    if (pendb) tc::mbar_wait_bounded(&tb.mma[1], phb, kT64WaitPolls << 2);
    if (pendf0) tc::mbar_wait_bounded(&tb.full[0], phf0, kT64WaitPolls << 2);
    if (pendf1) tc::mbar_wait_bounded(&tb.full[1], phf1, kT64WaitPolls << 2);
    if (tid == 0) atomicExch(err, 1);
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (w == 0) tc::tmem_dealloc(tmem, S::TMEM_COLS);
}

template <int K>
static cudaError_t configure_tc64() {
  constexpr size_t smem = t64_smem_bytes<K>();
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
