// tensor.cu -- dense K = 3, 4 qubit passes on the tensor cores (tcgen05) for
// a double-float state, with FP64-level accuracy (6 slices).  The kernel is
// written for an FP32 element type as well (3 slices), but complex64 states
// run the per-value BF16 x 3 kernel of tensor32.cu, so only the double-float
// instance is built.
//
// A tile is 128 columns of one step: in the ket step column m = (b, f) holds
// the 2^K entries rho[(., b, f)], in the bra step column m = (a, f) holds
// rho[(a, ., f)].  Each column is split into BF16 slices on its own
// power-of-two grid: with |x| < 2^e over the column, slice i holds the part
// of x on the grid 2^(e - 7 - 8i), an integer multiple |s_i| <= 256 of that
// unit (kept at its true scale, so a slice is exact in BF16); the host did the
// same per row for the operator (|t_j| <= 128 units of 2^(e_row - 7 - 8j)).
// One thread issues, per order o, the MMAs of every slice pair i + j = o into
// the FP32 accumulator D_o (TMEM columns o*R ..): within D_o every product is
// an integer multiple of one unit and the sum stays below 2^22.6 units, so
// the tensor cores add exactly and D_o is the true partial sum.  The threads
// then read the orders back and add them in double-float (FP32 for complex64).
// Error per step (numpy emulation of this arithmetic on random unitaries and
// columns): below 2^-46 of |W row|_2 |x|_2 for double-float, dominated by the
// 48-bit slicing of x and W.
//
// Threads: 256.  Thread (warp w, lane l) owns column m = 32*(w & 3) + l (the
// TMEM lane its warp may read) and half hf = w >> 2 of it: hf = 0 slices and
// produces the real parts, hf = 1 the imaginary parts.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#include "kernels.h"
#include "pass_device.cuh"
#include "tc.cuh"

namespace dmg {

namespace {

// Slices per operand: 6 (48 bits) for a double-float state, 3 (24 bits) for
// a complex64 (FP32) state.
template <typename T> struct TcSlices { static constexpr int value = kTcSlices; };
template <> struct TcSlices<float> { static constexpr int value = 3; };

template <int K, typename T>
struct TcShape {
  static constexpr int D = 1 << K, R = 2 * D, G = 128 / D, TILE = 128 * D, S = TcSlices<T>::value;
  static constexpr uint32_t SBO = 16 * R;           // bytes between 8-row groups of an R-wide K-major operand
  static constexpr uint32_t A_BYTES = 128 * R * 2;  // one slice of the 128 columns
  static constexpr uint32_t B_BYTES = R * R * 2;    // one slice of W or V
  // slice-pair orders kept: 0..S (double-float; the first dropped order is
  // below 2^-48), 0..S (FP32: orders 0..3, below 2^-24 after that)
  static constexpr int ORDERS = S + 1;
  static constexpr uint32_t TMEM_COLS =
      ORDERS * R <= 32 ? 32 : (ORDERS * R <= 64 ? 64 : (ORDERS * R <= 128 ? 128 : 256));
  static_assert(ORDERS * R <= 256, "accumulators exceed the tensor-memory allocation");
};

template <int K>
struct TcTables {
  static constexpr int D = 1 << K, R = 2 * D;
  uint64_t hioff[256];
  uint32_t ldmask[8], stmask[8];
  int lk[D], lb[D];
  float colmax[2][128];
  uint64_t bar;
  uint32_t slot;
};

template <int K, typename T>
constexpr size_t tc_smem_bytes() {
  using S = TcShape<K, T>;
  return (size_t)S::S * S::A_BYTES + 2 * (size_t)S::S * S::B_BYTES + 2 * (size_t)S::TILE * sizeof(T) +
         sizeof(TcTables<K>);
}

// Rounding to the grid of slice i of a column whose largest |entry| has
// biased FP32 exponent eb (|x| < 2^(eb-126)): (v + C_i) - C_i with
// C_i = 1.5 * 2^(eb - 110 - 8i) rounds |v| < 2^22 units 2^(eb - 133 - 8i).
__device__ __forceinline__ float slice_magic(int eb, int i) {
  return __int_as_float(((eb + 17 - 8 * i) << 23) | 0x400000);
}

// The slices of x = h + l (double-float).  Slices 0..2 come from h alone
// (exact); its remainder (below half a unit of slice 2) plus l, whose size is
// at most that, is rounded once to FP32 -- an error of at most one unit of
// slice 5 -- and gives slices 3..5.
template <int S>
__device__ __forceinline__ void slice_df(float h, float l, const float (&C)[S], float (&s)[S]) {
  float v = h;
#pragma unroll
  for (int i = 0; i < 3; i++) {
    const float t = __fsub_rn(__fadd_rn(v, C[i]), C[i]);
    s[i] = t;
    v = __fsub_rn(v, t);
  }
  v = __fadd_rn(v, l);
#pragma unroll
  for (int i = 3; i < S; i++) {
    const float t = __fsub_rn(__fadd_rn(v, C[i]), C[i]);
    s[i] = t;
    v = __fsub_rn(v, t);
  }
}

// The slices of an FP32 value.
template <int S>
__device__ __forceinline__ void slice_f(float x, const float (&C)[S], float (&s)[S]) {
  float v = x;
#pragma unroll
  for (int i = 0; i < S; i++) {
    const float t = __fsub_rn(__fadd_rn(v, C[i]), C[i]);
    s[i] = t;
    v = __fsub_rn(v, t);
  }
}

// Asynchronous global -> shared copies of one entry pair (Ampere-style
// cp.async: 16 bytes through L2 only, 8 bytes through L1).
template <int BYTES>
__device__ __forceinline__ void cp_async_pair(void* smem_dst, const void* gmem_src) {
  if constexpr (BYTES == 16)
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(tc::smem_u32(smem_dst)), "l"(gmem_src) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(tc::smem_u32(smem_dst)), "l"(gmem_src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(a, b);  // exact: at most 8 significant bits each
  return *reinterpret_cast<const uint32_t*>(&v);
}

template <int D>
__device__ __forceinline__ void tmem_ld_row(uint32_t taddr, float (&v)[D]) {
  if constexpr (D == 16) tc::tmem_ld16(taddr, v);
  else tc::tmem_ld8(taddr, v);
}

// One step (ket when !BRA) on the tile in shared memory.  Returns false (the
// same on every thread) if the tensor core did not signal completion in time.
// `after_mma` runs on every thread once the step's MMAs have completed (the
// slice buffers are free again): the bra step starts the next tile's loads
// there.
template <int K, typename T, bool BRA, typename F>
__device__ bool tc_step(T* __restrict__ sre, T* __restrict__ sim, unsigned char* sA, const unsigned char* sB,
                        TcTables<K>& tb, uint32_t tmem, int lf_g, uint32_t& phase, const F& after_mma) {
  using SH = TcShape<K, T>;
  constexpr int D = SH::D, R = SH::R, S = SH::S, G = SH::G;
  constexpr bool DF = std::is_same<T, df64>::value;
  const int tid = threadIdx.x;
  const int w = tid >> 5, l = tid & 31;
  const int m = 32 * (w & 3) + l;
  const int hf = w >> 2;
  const int r = m / G;
  const int base = lf_g + (BRA ? tb.lk[r] : tb.lb[r]);
  const int* lc = BRA ? tb.lb : tb.lk;
  T* arr = hf ? sim : sre;

  // ---- gather this half-column and agree on the column's grid
  float xh[D], xl[DF ? D : 1];
  float mx = 0.f;
#pragma unroll
  for (int c = 0; c < D; c++) {
    const T v = arr[base + lc[c]];
    if constexpr (DF) {
      xh[c] = v.hi;
      xl[c] = v.lo;
    } else {
      xh[c] = v;
    }
    mx = fmaxf(mx, fabsf(xh[c]));
  }
  tb.colmax[hf][m] = mx;
  __syncthreads();
  mx = fmaxf(tb.colmax[0][m], tb.colmax[1][m]);
  // mx < 2^(eb-126).  Columns whose largest entry is below 2^-87 keep the
  // grid of 2^-87 (their slices underflow towards 0; absolute error < 2^-87).
  int eb = (__float_as_int(mx) >> 23) & 0xFF;
  eb = max(eb, 40);
  float C[S];
#pragma unroll
  for (int i = 0; i < S; i++) C[i] = slice_magic(eb, i);

  // ---- slices -> the A operand (row m, K index hf*D + c), 16 bytes per 8 values
#pragma unroll
  for (int c8 = 0; c8 < D; c8 += 8) {
    uint32_t pk[S][4];
#pragma unroll
    for (int c = 0; c < 8; c += 2) {
      float s0[S], s1[S];
      if constexpr (DF) {
        slice_df<S>(xh[c8 + c], xl[c8 + c], C, s0);
        slice_df<S>(xh[c8 + c + 1], xl[c8 + c + 1], C, s1);
      } else {
        slice_f<S>(xh[c8 + c], C, s0);
        slice_f<S>(xh[c8 + c + 1], C, s1);
      }
#pragma unroll
      for (int i = 0; i < S; i++) pk[i][c >> 1] = pack_bf16(s0[i], s1[i]);
    }
    const uint32_t off = tc_kmajor_offset(m, hf * D + c8, SH::SBO);
#pragma unroll
    for (int i = 0; i < S; i++)
      *reinterpret_cast<uint4*>(sA + i * SH::A_BYTES + off) = make_uint4(pk[i][0], pk[i][1], pk[i][2], pk[i][3]);
  }
  tc::fence_proxy_async_smem();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();

  // ---- one thread issues the products.  The operator's slices W_0..W_{S-1}
  // are consecutive R-row blocks of one K-major operand, so A_i against
  // W_j0..W_{j0+nb-1} is one MMA of N = nb*R whose block j lands in the
  // accumulator of order i + j when its destination starts at column i*R.
  // Seven MMAs (per 16-wide K chunk) cover every pair with i + j < ORDERS:
  // A_0 W_0 -> D_0 and A_1 W_* -> D_1.. overwrite; the rest accumulate.
  if (tid == 0) {
    const uint32_t a0 = tc::smem_u32(sA);
    const uint32_t b0 = tc::smem_u32(sB) + (BRA ? S * SH::B_BYTES : 0);
    auto issue = [&](int i, int j0, int nb, bool overwrite) {
#pragma unroll
      for (int kk = 0; kk < R / 16; kk++) {
        const uint64_t ad = tc::smem_desc(a0 + i * SH::A_BYTES + kk * 256, tc::kLbo, SH::SBO);
        const uint64_t bd = tc::smem_desc(b0 + j0 * SH::B_BYTES + kk * 256, tc::kLbo, SH::SBO);
        tc::mma_bf16(tmem + (i + j0) * R, ad, bd, tc::idesc_bf16_f32(128, nb * R), (overwrite && kk == 0) ? 0u : 1u);
      }
    };
    constexpr int O = SH::ORDERS;
    issue(0, 0, 1, true);                            // (0,0)
    issue(1, 0, S < O - 1 ? S : O - 1, true);        // (1,0) .. (1,min(S,O-1)-1)
    issue(0, 1, S - 1, false);                       // (0,1) .. (0,S-1)
#pragma unroll
    for (int i = 2; i < S; i++) issue(i, 0, S < O - i ? S : O - i, false);  // (i,0) .. (i,O-1-i)
    tc::mma_commit(&tb.bar);
  }
  const bool done = tc::mbar_wait_bounded(&tb.bar, phase, 1u << 24);
  if (!__syncthreads_and(done)) {
    // The commit did not arrive in time.  The caller releases the tensor
    // memory next, which the MMAs already issued may still write: give them
    // one more, longer, bounded wait first.  The pass has failed either way
    // (the host reports DMSIM_ERR_TIMEOUT and the state is undefined).
    tc::mbar_wait_bounded(&tb.bar, phase, 1u << 26);
    return false;
  }
  phase ^= 1u;
  tc::fence_after_sync();
  after_mma();

  // ---- recombine the orders of outputs n = hf*D + a (a < D)
  const uint32_t trow = tmem + ((uint32_t)(32 * (w & 3)) << 16) + hf * D;
  if constexpr (DF) {
    static_assert(S == 6, "the double-float recombination is written for orders 0..6");
    float lo[D], p3[D], p2[D], p1[D], p0[D];
    {
      float q[D];
      tmem_ld_row<D>(trow + 6 * R, q);
      tmem_ld_row<D>(trow + 5 * R, lo);
      tc::tmem_wait_ld();
#pragma unroll
      for (int a = 0; a < D; a++) lo[a] = __fadd_rn(q[a], lo[a]);
      tmem_ld_row<D>(trow + 4 * R, q);
      tc::tmem_wait_ld();
#pragma unroll
      for (int a = 0; a < D; a++) lo[a] = __fadd_rn(lo[a], q[a]);
    }
    tmem_ld_row<D>(trow + 3 * R, p3);
    tmem_ld_row<D>(trow + 2 * R, p2);
    tmem_ld_row<D>(trow + 1 * R, p1);
    tmem_ld_row<D>(trow, p0);
    tc::tmem_wait_ld();
#pragma unroll
    for (int a = 0; a < D; a++) {
      // orders 0..3 error-free (their sum spans more than 24 bits), 4..6 in lo
      const df64 s1 = two_sum(p0[a], p1[a]);
      const df64 s2 = two_sum(s1.hi, p2[a]);
      const df64 s3 = two_sum(s2.hi, p3[a]);
      arr[base + lc[a]] = fast_two_sum(s3.hi, __fadd_rn(__fadd_rn(__fadd_rn(s1.lo, s2.lo), s3.lo), lo[a]));
    }
  } else {
    static_assert(S == 3, "the FP32 recombination is written for orders 0..3");
    float p3[D], p2[D], p1[D], p0[D];
    tmem_ld_row<D>(trow + 3 * R, p3);
    tmem_ld_row<D>(trow + 2 * R, p2);
    tmem_ld_row<D>(trow + 1 * R, p1);
    tmem_ld_row<D>(trow, p0);
    tc::tmem_wait_ld();
#pragma unroll
    for (int a = 0; a < D; a++) arr[base + lc[a]] = __fadd_rn(p0[a], __fadd_rn(p1[a], __fadd_rn(p2[a], p3[a])));
  }
  tc::fence_before_sync();
  __syncthreads();
  return true;
}

}  // namespace

// Resident blocks the register budget is sized for: two double-float blocks
// (TMEM: 2 x 256 columns), three complex64 blocks (3 x 128 columns), whose
// per-tile work is light enough that the MMA round trips need more blocks to
// overlap.
template <typename T> struct TcMinBlocks { static constexpr int value = 2; };
template <> struct TcMinBlocks<float> { static constexpr int value = 3; };

template <int K, typename T>
__global__ void __launch_bounds__(kThreads, TcMinBlocks<T>::value) k_pass_tc(T* __restrict__ re, T* __restrict__ im,
                                                         const TcDesc<K>* __restrict__ dp, int* __restrict__ err) {
  using SH = TcShape<K, T>;
  using T2 = typename Vec2<T>::type;
  constexpr int D = SH::D, S = SH::S;
  extern __shared__ __align__(1024) unsigned char smem[];
  unsigned char* sA = smem;
  unsigned char* sB = sA + S * SH::A_BYTES;
  T* sre = reinterpret_cast<T*>(sB + 2 * S * SH::B_BYTES);
  T* sim = sre + SH::TILE;
  TcTables<K>& tb = *reinterpret_cast<TcTables<K>*>(sim + SH::TILE);
  const PassHeader& h = dp->h;
  const int tid = threadIdx.x;

  // ---- per-pass tables and the operator slices this state type uses
  {
    constexpr int per_slice = SH::B_BYTES / 16;
    for (int i = tid; i < 2 * S * per_slice; i += blockDim.x) {
      const int side = i / (S * per_slice), rest = i % (S * per_slice);
      reinterpret_cast<uint4*>(sB)[i] = reinterpret_cast<const uint4*>(&dp->sl[side][0][0])[rest];
    }
  }
  for (int r = tid; r < (1 << h.mhi); r += blockDim.x) {
    uint64_t off = 0;
    for (int j = 0; j < h.mhi; j++) off |= (uint64_t)((r >> j) & 1) << h.hipos[j];
    tb.hioff[r] = off;
  }
  if (tid < 8) {
    tb.ldmask[tid] = h.ldmask[tid];
    tb.stmask[tid] = h.stmask[tid];
  }
  if (tid < D) {
    int lk = 0, lb = 0;
    for (int i = 0; i < K; i++) {
      lk |= ((tid >> i) & 1) << h.lket[i];
      lb |= ((tid >> i) & 1) << h.lbra[i];
    }
    tb.lk[tid] = lk;
    tb.lb[tid] = lb;
  }
  if (tid < 32) {
    tc::tmem_alloc(&tb.slot, SH::TMEM_COLS);
    tc::tmem_relinquish();
  }
  if (tid == 0) {
    tc::mbar_init(&tb.bar, 1);
    tc::mbar_fence_init();
  }
  tc::fence_proxy_async_smem();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tb.slot;

  // free-bit offset of this thread's group f = m mod G (the same in both steps)
  int lf_g = 0;
  {
    const int m = 32 * ((tid >> 5) & 3) + (tid & 31);
    const int f = m & (SH::G - 1);
    for (int j = 0; j < h.g; j++) lf_g |= ((f >> j) & 1) << h.freepos[j];
  }

  const int L = h.L, runlen = 1 << L;
  uint32_t phase = 0;
  bool ok = true;
  // Tile t is loaded directly; every later tile is copied asynchronously
  // into the slice buffers while the previous tile's bra step recombines and
  // its runs are stored, then moved into the tile buffer.  Each thread
  // prefetches, stores and moves the same entry pairs, so those three need no
  // barrier between them.
  static_assert(2 * SH::TILE * sizeof(T) <= S * SH::A_BYTES, "the next tile must fit in the slice buffers");
  T* nre = reinterpret_cast<T*>(sA);
  T* nim = nre + SH::TILE;
  constexpr int PAIRS = SH::TILE / 2 / kThreads;
  uint64_t t = blockIdx.x;
  if (t < h.ntiles) {
    const uint64_t base = tile_base(h, t);
    for (int e2 = tid; e2 < (SH::TILE >> 1); e2 += blockDim.x) {
      const int e = e2 << 1;
      const int run = e >> L;
      const uint64_t ga = base + tb.hioff[run] + (uint64_t)(e & (runlen - 1));
      *reinterpret_cast<T2*>(sre + e) = ld2<T>(re + ga);
      *reinterpret_cast<T2*>(sim + e) = ld2<T>(im + ga);
    }
  }
  for (; t < h.ntiles; t += gridDim.x) {
    __syncthreads();
    const uint64_t base = tile_base(h, t);
    const uint64_t tn = t + gridDim.x;
    const bool has_next = tn < h.ntiles;
    const uint64_t base_n = has_next ? tile_base(h, tn) : 0;
    auto nothing = [] {};
    auto prefetch = [&] {
      if (!has_next) return;
#pragma unroll
      for (int k = 0; k < PAIRS; k++) {
        const int e = (tid + k * kThreads) << 1;
        const int run = e >> L;
        const uint64_t ga = base_n + tb.hioff[run] + (uint64_t)(e & (runlen - 1));
        cp_async_pair<2 * sizeof(T)>(nre + e, re + ga);
        cp_async_pair<2 * sizeof(T)>(nim + e, im + ga);
      }
      cp_async_commit();
    };
    if (!tc_step<K, T, false>(sre, sim, sA, sB, tb, tmem, lf_g, phase, nothing) ||
        !tc_step<K, T, true>(sre, sim, sA, sB, tb, tmem, lf_g, phase, prefetch)) {
      ok = false;
      if (has_next) cp_async_wait_all();  // no copy may still target shared memory
      break;
    }
    // ---- store the runs the pass changes, then move the next tile in
#pragma unroll
    for (int k = 0; k < PAIRS; k++) {
      const int e = (tid + k * kThreads) << 1;
      const int run = e >> L;
      if (!((tb.stmask[run >> 5] >> (run & 31)) & 1)) continue;
      const uint64_t ga = base + tb.hioff[run] + (uint64_t)(e & (runlen - 1));
      st2<T>(re + ga, *reinterpret_cast<const T2*>(sre + e));
      st2<T>(im + ga, *reinterpret_cast<const T2*>(sim + e));
    }
    if (has_next) {
      cp_async_wait_all();
#pragma unroll
      for (int k = 0; k < PAIRS; k++) {
        const int e = (tid + k * kThreads) << 1;
        *reinterpret_cast<T2*>(sre + e) = *reinterpret_cast<const T2*>(nre + e);
        *reinterpret_cast<T2*>(sim + e) = *reinterpret_cast<const T2*>(nim + e);
      }
    }
  }
  if (!ok && tid == 0) atomicExch(err, 1);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (tid < 32) tc::tmem_dealloc(tmem, SH::TMEM_COLS);
}

// Dynamic shared memory and the largest shared-memory carveout: without the
// carveout preference the runtime may configure the SM for one 110 KB block.
template <int K, typename T>
static cudaError_t configure_tc() {
  constexpr size_t smem = tc_smem_bytes<K, T>();
  cudaError_t e = cudaFuncSetAttribute(k_pass_tc<K, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_pass_tc<K, T>, cudaFuncAttributePreferredSharedMemoryCarveout,
                             (int)cudaSharedmemCarveoutMaxShared);
  return e;
}

template <int K, typename T>
static cudaError_t launch_tc_k(const LaunchArgs& a, cudaStream_t s) {
  constexpr size_t smem = tc_smem_bytes<K, T>();
  static int configured = 0;
  if (!configured) {
    cudaError_t e = configure_tc<K, T>();
    if (e != cudaSuccess) return e;
    configured = 1;
  }
  k_pass_tc<K, T><<<a.grid, kThreads, smem, s>>>(static_cast<T*>(a.re), static_cast<T*>(a.im),
                                                  static_cast<const TcDesc<K>*>(a.desc), a.err);
  return cudaGetLastError();
}

cudaError_t launch_pass_tc(const LaunchArgs& a, cudaStream_t s) {
  if (!a.err || (a.K != 3 && a.K != 4)) return cudaErrorInvalidValue;
  if (a.arith == AR_DF64) return a.K == 3 ? launch_tc_k<3, df64>(a, s) : launch_tc_k<4, df64>(a, s);
  return cudaErrorInvalidValue;  // FP64 states: tensor64.cu; complex64 states: tensor32.cu
}

// Resident blocks per SM from the kernel's own resources: shared memory
// (plus the 1 KB the driver reserves per block), registers, threads and the
// 512 TMEM columns.  (The runtime occupancy query reported one block for
// this kernel although two fit; the launch statistics confirm two.)
template <int K, typename T>
static int tc_occ() {
  constexpr size_t smem = tc_smem_bytes<K, T>();
  if (configure_tc<K, T>() != cudaSuccess) return 1;
  cudaFuncAttributes fa;
  int dev = 0, smem_sm = 0, regs_sm = 0, threads_sm = 0;
  if (cudaFuncGetAttributes(&fa, k_pass_tc<K, T>) != cudaSuccess || cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&threads_sm, cudaDevAttrMaxThreadsPerMultiProcessor, dev) != cudaSuccess)
    return 1;
  const int by_smem = smem_sm / (int)(smem + fa.sharedSizeBytes + 1024);
  const int by_regs = regs_sm / (fa.numRegs * kThreads);
  const int by_threads = threads_sm / kThreads;
  const int by_tmem = 512 / (int)TcShape<K, T>::TMEM_COLS;
  int nb = by_smem;
  nb = nb < by_regs ? nb : by_regs;
  nb = nb < by_threads ? nb : by_threads;
  nb = nb < by_tmem ? nb : by_tmem;
  return nb > 0 ? nb : 1;
}

int tc_blocks_per_sm(int K, int arith) {
  if (arith == AR_FP64) return 1;  // the FP64-width kernel: one persistent block per SM (tensor64.cu)
  if (arith == AR_FP32) return 2;  // the complex64 kernel: two persistent blocks per SM (tensor32.cu)
  return K == 3 ? tc_occ<3, df64>() : tc_occ<4, df64>();
}

}  // namespace dmg
