// tensor32.cu -- dense K = 3, 4 qubit passes of complex64 (FP32) states on
// the tensor cores: the complex64 counterpart of tensor64.cu's pipeline.
//
// A pass is two products per tile of 128 columns: the ket step multiplies
// every tile column x (2^K complex entries as R = 2^(K+1) reals) by the real
// embedding W = [[Ur, -Ui], [Ui, Ur]], the bra step the result's columns by
// V's.  Every FP32 operand value is the sum of three BF16 values, each
// rounded from the remainder of the ones before it (x = h + m + l to 2^-24
// of |x|; the host split W and V's entries the same way, slices 0..2 of
// TcDesc).  The six products whose size reaches 2^-16 of the leading one --
// (l,h) (m,m) (h,l), then (m,h) (h,m), then (h,h), smallest first --
// accumulate into one FP32 accumulator in tensor memory; the three dropped
// ones are below 2^-24 of it.  Each value keeps its own 24-bit precision
// (no shared exponent per column), so a step's error is FP32 accumulation's,
// the FP32-pipe passes' own level.
//
// Threads, tiles and synchronisation follow tensor64.cu: 512 threads, two
// blocks per SM (64 registers a thread, 107 KB of shared memory and 64 TMEM
// columns a block), two independent groups of 8 warps taking alternate tiles,
// each with its own tile buffer (1-D TMA bulk copies of the tile's runs, issued
// one tile ahead), slice operand, accumulator (R TMEM columns), mbarriers and
// named barrier.  Per tile:
//   1. wait for the tile, ket slices -> A;  2. the ket MMAs;  3. ket
//      accumulator -> FP32 ket outputs in place of the tile;  4. bra slices
//      -> A;  5. the bra MMAs, the group's next tile loaded into the freed
//      buffer;  6. bra accumulator -> global stores.
// Three group barriers per tile (after steps 1, 3 and 4); every wait is
// bounded, and on expiry the group leaves its loop at the next
// barrier, waits (bounded) for its own copies and MMAs in flight, sets the
// error flag, and the block releases its tensor memory; the host reports
// DMSIM_ERR_TIMEOUT with rho undefined.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "kernels.h"
#include "pass.h"
#include "tc.cuh"

namespace dmg {

namespace {

constexpr int kT32Threads = 512;
constexpr int kT32GroupThreads = 256;
constexpr uint32_t kT32WaitPolls = 1u << 24;
constexpr int kT32Slices = 3;  // h, m, l: the first 3 of the descriptor's kTcSlices
static_assert(kT32Slices <= kTcSlices, "the operator descriptor holds the slices");

template <int K>
struct T32 {
  static constexpr int D = 1 << K, R = 2 * D, G = 128 / D, TILE = 128 * D;
  // A loaded tile: 16-entry pieces 20 entries (80 bytes) apart, the imaginary
  // array ASTR entries after the real one; ASTR = 16 mod 32 puts the two
  // halves of a column in opposite halves of the banks.
  static constexpr int ASTR = TILE / 16 * 20 + 16;
  static constexpr uint32_t SBO = 16 * R;                  // bytes between 8-row groups of an R-wide operand
  static constexpr uint32_t A_BYTES = 128 * R * 2;         // one slice of the 128 columns
  static constexpr uint32_t B_BYTES = R * R * 2;           // one slice of W or V
  static constexpr uint32_t SET_COLS = R;                  // the accumulator of one group
  static constexpr uint32_t TMEM_COLS = 2 * SET_COLS;      // 64 (K = 4), 32 (K = 3)
  static constexpr uint32_t TX_BYTES = TILE * 4 * 2;       // one tile, re + im
  static constexpr uint32_t BUF_BYTES = 2 * ASTR * 4;      // one group's tile buffer
  static_assert(ASTR % 32 == 16 && BUF_BYTES % 16 == 0, "tile buffer layout");
  static_assert(TMEM_COLS <= 512, "two accumulator sets must fit in tensor memory");
};

// Shared-memory position of local entry e of a loaded tile: 16-entry pieces
// 20 entries apart (each piece's destination 16-byte aligned for the bulk
// copies).  Additive over disjoint bit fields.
__device__ __forceinline__ int piece_off32(int e) { return e + 4 * (e >> 4); }

struct T32Group {
  uint64_t full;  // the group's tile loads
  uint64_t mma;   // the group's ket and bra commits, alternating
};

template <int K>
struct T32Tables {
  static constexpr int D = 1 << K;
  uint64_t hioff[256];
  // output (a, b) of a tile, at [b][a]: bits 0..47 its offset from the tile
  // base minus the free bits, bit 63 set when its run is stored
  uint64_t outoff[D][D];
  // the same offsets split by their disjoint bit fields: output (a, b) at
  // offk[a] + offb[b]; allstored: every run of the tile is stored
  uint64_t offk[D], offb[D];
  int allstored;
  T32Group grp[2];
  int pk[D], pb[D];  // piece_off32 of the ket / bra index bits
  int hipos[8];
  uint32_t slot;
};

template <int K>
constexpr size_t t32_smem_bytes() {
  using S = T32<K>;
  return 2 * (size_t)kT32Slices * S::A_BYTES + 2 * (size_t)kT32Slices * S::B_BYTES + 2 * (size_t)S::BUF_BYTES +
         sizeof(T32Tables<K>);
}

// Named barrier of group g (ids 1, 2), and the same with an OR of p over the group.
__device__ __forceinline__ void group_bar32(int g) { tc::named_bar<kT32GroupThreads>(1 + g); }
__device__ __forceinline__ bool group_bar_or32(int g, bool p) { return tc::named_bar_or<kT32GroupThreads>(1 + g, p); }

__device__ __forceinline__ uint32_t bf16x2_bits(__nv_bfloat162 v) { return *reinterpret_cast<const uint32_t*>(&v); }

// The three BF16 slices (h, m, l) of two values x0, x1, packed in pairs: each
// remainder is exact in FP32 (a value minus its rounding to 8 significant
// bits).
__device__ __forceinline__ void split3(float x0, float x1, uint32_t (&pk)[kT32Slices]) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(x0, x1);
  const float2 hf = __bfloat1622float2(h);
  const float r0 = __fsub_rn(x0, hf.x), r1 = __fsub_rn(x1, hf.y);
  const __nv_bfloat162 m = __floats2bfloat162_rn(r0, r1);
  const float2 mf = __bfloat1622float2(m);
  const __nv_bfloat162 l = __floats2bfloat162_rn(__fsub_rn(r0, mf.x), __fsub_rn(r1, mf.y));
  pk[0] = bf16x2_bits(h);
  pk[1] = bf16x2_bits(m);
  pk[2] = bf16x2_bits(l);
}

// Split the D values of one column half (K index half*D + c, c = 0..D-1) and
// store the slices into the K-major operand, one 16-byte store per slice per
// 8 values.
template <int D, uint32_t A_BYTES, uint32_t SBO>
__device__ __forceinline__ void slice_column(const float (&v)[D], int row, int half, unsigned char* sA) {
#pragma unroll
  for (int ch = 0; ch < D / 8; ch++) {
    uint32_t pk[4][kT32Slices];
#pragma unroll
    for (int c2 = 0; c2 < 4; c2++) split3(v[8 * ch + 2 * c2], v[8 * ch + 2 * c2 + 1], pk[c2]);
    const uint32_t off = tc_kmajor_offset(row, half * D + 8 * ch, SBO);
#pragma unroll
    for (int j = 0; j < kT32Slices; j++)
      *reinterpret_cast<uint4*>(sA + j * A_BYTES + off) = make_uint4(pk[0][j], pk[1][j], pk[2][j], pk[3][j]);
  }
}

// This warp's D consecutive TMEM columns (32 lanes) in one load.
template <int D>
__device__ __forceinline__ void tmem_ld_row(uint32_t taddr, float (&v)[D]) {
  if constexpr (D == 16) tc::tmem_ld16(taddr, v);
  else tc::tmem_ld8(taddr, v);
}

// One thread issues every product of a step: slice pairs (i of the columns,
// j of the operator) (2,0) (1,1) (0,2) (1,0) (0,1) (0,0), smallest first,
// all into the group's one accumulator (N = R).
template <int K>
__device__ __forceinline__ void issue_step32(const unsigned char* sA, const unsigned char* sBside, uint32_t dset) {
  using S = T32<K>;
  constexpr int R = S::R;
  const uint32_t a0 = tc::smem_u32(sA), b0 = tc::smem_u32(sBside);
  constexpr int kPairs[6][2] = {{2, 0}, {1, 1}, {0, 2}, {1, 0}, {0, 1}, {0, 0}};
#pragma unroll
  for (int q = 0; q < 6; q++) {
#pragma unroll
    for (int kk = 0; kk < R / 16; kk++) {
      const uint64_t ad = tc::smem_desc(a0 + kPairs[q][0] * S::A_BYTES + kk * 256, tc::kLbo, S::SBO);
      const uint64_t bd = tc::smem_desc(b0 + kPairs[q][1] * S::B_BYTES + kk * 256, tc::kLbo, S::SBO);
      tc::mma_bf16(dset, ad, bd, tc::idesc_bf16_f32(128, R), (q == 0 && kk == 0) ? 0u : 1u);
    }
  }
}

}  // namespace

template <int K>
__global__ void __launch_bounds__(kT32Threads, 2)
    k_pass_tc32(float* __restrict__ re, float* __restrict__ im, const TcDesc<K>* __restrict__ dp,
                int* __restrict__ err) {
  using S = T32<K>;
  constexpr int D = S::D, R = S::R, G = S::G, TILE = S::TILE, ASTR = S::ASTR;
  extern __shared__ __align__(1024) unsigned char smem[];
  unsigned char* sB = smem + 2 * kT32Slices * S::A_BYTES;                         // W slices, then V slices
  float* bufs = reinterpret_cast<float*>(sB + 2 * kT32Slices * S::B_BYTES);       // [group][re, im][ASTR]
  T32Tables<K>& tb = *reinterpret_cast<T32Tables<K>*>(bufs + 4 * ASTR);
  const PassHeader& h = dp->h;
  const int tid = threadIdx.x, w = tid >> 5, l = tid & 31;
  const int g = w >> 3, gtid = tid & (kT32GroupThreads - 1);
  // slice steps: column mc = 16 (w & 7) + (l & 15), half hc = l >> 4 (both
  // halves of a column in one warp)
  const int mc = 16 * (w & 7) + (l & 15), hc = l >> 4;
  const int rc = mc / G, fc = mc & (G - 1);
  // accumulator steps: column m = 32 (w & 3) + l -- the TMEM lane its warp
  // may read -- half (w >> 2) & 1
  const int m = 32 * (w & 3) + l, half = (w >> 2) & 1;
  const int r = m / G, f = m & (G - 1);
  unsigned char* sA = smem + g * kT32Slices * S::A_BYTES;  // the group's slice operand (ket, then bra)
  float* buf = bufs + (size_t)g * 2 * ASTR;               // the group's tile, then its ket outputs
  T32Group& gp = tb.grp[g];

  // ---- per-pass tables, the operator's slices, tensor memory, barriers
  {
    constexpr int per_slice = S::B_BYTES / 16;
    for (int i = tid; i < 2 * kT32Slices * per_slice; i += blockDim.x) {
      const int side = i / (kT32Slices * per_slice), rest = i % (kT32Slices * per_slice);
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
    tb.pk[tid] = piece_off32(lk);
    tb.pb[tid] = piece_off32(lb);
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
    tb.outoff[bb][a] = off | (stored << 63);
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
  // slice steps: column (b = rc, fc)'s values a = 0..D-1 of half hc at
  // buf[basec + tb.pk[a]] (the offsets read from shared memory, a broadcast,
  // to keep the register budget of two blocks per SM)
  const int basec = hc * ASTR + tb.pb[rc] + piece_off32(free_off(fc));
  const uint64_t ntiles = h.ntiles, gstep = 2 * (uint64_t)gridDim.x;
  const int runlen = 1 << L, lgp = L < 4 ? L : 4, npieces = (2 * TILE) >> lgp;
  // The ket step's outputs Y(a, b) of column (b, ff) replace the tile in its
  // buffer, at [hh][a][b ^ (a & 1)][ff]: the ket step writes, for one a, 32
  // consecutive words per warp, and the bra step reads, for one b, columns a
  // of both parities in distinct banks.
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
  // array.  Runs are at least 8 entries (32 bytes) long.
  auto copy_tile = [&](uint64_t base) {
    for (int i = gtid; i < npieces; i += kT32GroupThreads) {
      const int arr = i & 1, e0 = (i >> 1) << lgp;
      const int run = e0 >> L, o = e0 & (runlen - 1);
      tc::bulk_g2s(buf + arr * ASTR + piece_off32(e0), (arr ? im : re) + base + tb.hioff[run] + o, 4u << lgp,
                   &gp.full);
    }
  };

  // outstanding asynchronous work of this thread's view; a phase that did not
  // complete stays pending (the teardown waits for it again)
  uint32_t phf = 0, phm = 0;
  int pendf = 0, pendm = 0;
  bool bad = false;  // one of this thread's waits expired
  auto wait = [&](uint64_t* bar, uint32_t& ph, int& pend) {
    if (!tc::mbar_wait_bounded(bar, ph, kT32WaitPolls)) {
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
  group_bar32(g);
  if (t < ntiles) {
    copy_tile(tbase);
    pendf = 1;
  }

  for (; t < ntiles; t += gstep) {
    // ---- 1: the tile's values of column (b = rc, fc), half hc: ket slices
    wait(&gp.full, phf, pendf);
    {
      float v[D];
#pragma unroll
      for (int a = 0; a < D; a++) v[a] = buf[basec + tb.pk[a]];
      slice_column<D, S::A_BYTES, S::SBO>(v, mc, hc, sA);
    }
    tc::fence_proxy_async_smem();
    tc::fence_before_sync();
    if (group_bar_or32(g, bad)) break;
    tc::fence_after_sync();

    // ---- 2: ket products
    if (gtid == 0) {
      issue_step32<K>(sA, sB, tmem);
      tc::mma_commit(&gp.mma);
    }
    pendm = 1;

    // ---- 3: ket outputs of column (b = r, f), in place of the tile
    if (wait(&gp.mma, phm, pendm)) {
      tc::fence_after_sync();
      float sv[D];
      tmem_ld_row<D>(tmem + tlane + half * D, sv);
      tc::tmem_wait_ld();
#pragma unroll
      for (int a = 0; a < D; a++) buf[yoff(half, a, r, f)] = sv[a];
    }
    tc::fence_before_sync();
    if (group_bar_or32(g, bad)) break;
    tc::fence_after_sync();

    // ---- 4: bra slices of column (a = rc, fc)
    {
      float v[D];
#pragma unroll
      for (int b = 0; b < D; b++) v[b] = buf[yoff(hc, rc, b, fc)];
      slice_column<D, S::A_BYTES, S::SBO>(v, mc, hc, sA);
    }
    const uint64_t tn = t + gstep;
    if (gtid == 0 && tn < ntiles) tc::mbar_arrive_expect_tx(&gp.full, S::TX_BYTES);  // the group's next tile
    tc::fence_proxy_async_smem();
    tc::fence_before_sync();
    group_bar32(g);
    tc::fence_after_sync();

    // ---- 5: bra products; the group's next tile into the freed buffer
    if (gtid == 0) {
      issue_step32<K>(sA, sB + kT32Slices * S::B_BYTES, tmem);
      tc::mma_commit(&gp.mma);
    }
    pendm = 1;
    const uint64_t nbase = tn < ntiles ? tile_base_s(tn) : 0;
    if (tn < ntiles) {
      copy_tile(nbase);
      pendf = 1;
    }

    // ---- 6: bra outputs of column (a = r, f) -> the tile's stored runs
    if (wait(&gp.mma, phm, pendm)) {
      tc::fence_after_sync();
      float* arr = (half ? im : re) + tbase + lf;
      float sv[D];
      tmem_ld_row<D>(tmem + tlane + half * D, sv);
      tc::tmem_wait_ld();
      if (tb.allstored) {  // the common case: one base per thread, one offset per output
        float* col = arr + tb.offk[r];
#pragma unroll
        for (int b = 0; b < D; b++) col[tb.offb[b]] = sv[b];
      } else {
#pragma unroll
        for (int b = 0; b < D; b++) {
          const uint64_t T = tb.outoff[b][r];
          if (!(T >> 63)) continue;  // a run the pass does not change
          arr[T & 0xFFFFFFFFFFFFull] = sv[b];
        }
      }
    }
    tc::fence_before_sync();  // the next tile's first group barrier orders these reads before its MMAs
    tbase = nbase;
  }

  // ---- teardown: nothing of this group may still be in flight when the
  // block's tensor memory and shared memory are released (bounded, after an
  // expiry)
  if (group_bar_or32(g, bad)) {
    if (pendm) tc::mbar_wait_bounded(&gp.mma, phm, kT32WaitPolls << 2);
    if (pendf) tc::mbar_wait_bounded(&gp.full, phf, kT32WaitPolls << 2);
    if (gtid == 0) atomicExch(err, 1);
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (w == 0) tc::tmem_dealloc(tb.slot, S::TMEM_COLS);
}

template <int K>
static cudaError_t configure_tc32() {
  constexpr size_t smem = t32_smem_bytes<K>();
  static_assert(smem <= 113 * 1024, "two blocks per SM");
  cudaError_t e = cudaFuncSetAttribute(k_pass_tc32<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_pass_tc32<K>, cudaFuncAttributePreferredSharedMemoryCarveout,
                             (int)cudaSharedmemCarveoutMaxShared);
  return e;
}

template <int K>
static cudaError_t launch_tc32_k(const LaunchArgs& a, cudaStream_t s) {
  static int configured = 0;
  if (!configured) {
    cudaError_t e = configure_tc32<K>();
    if (e != cudaSuccess) return e;
    configured = 1;
  }
  k_pass_tc32<K><<<a.grid, kT32Threads, t32_smem_bytes<K>(), s>>>(
      static_cast<float*>(a.re), static_cast<float*>(a.im), static_cast<const TcDesc<K>*>(a.desc), a.err);
  return cudaGetLastError();
}

cudaError_t launch_pass_tc32(const LaunchArgs& a, cudaStream_t s) {
  if (!a.err || (a.K != 3 && a.K != 4) || a.arith != AR_FP32) return cudaErrorInvalidValue;
  return a.K == 3 ? launch_tc32_k<3>(a, s) : launch_tc32_k<4>(a, s);
}

}  // namespace dmg
