// pass_device.cuh -- the device side of one superoperator pass, shared by the
// per-pass kernel (kernels.cu) and the batched work-queue kernel (batch.cu).
//
// A block owns one tile at a time: it loads the tile's touched runs with
// 16-byte vector loads into shared memory, transforms them, and stores them
// back.  Monomial classes (MOVE/SIGNED/PHASE) fuse the permutation and the
// per-entry factor into the store, so they cost at most one complex multiply
// per entry.  DENSE/SPARSE apply U to the ket bits of each column and V to the
// bra bits of each row; V = conj(U) makes the pass U (x) conj(U) on the 2K
// target bits, V = I makes it a ket-only pass (the reference's forward and
// backward stages).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "pass.h"

namespace dmg {

// ---------------------------------------------------------------- df64
// Double-float: an unevaluated sum hi + lo of two floats (|lo| <= ulp(hi)/2),
// a 48-bit significand held in the 8 bytes of a double.  GB300's FP64 pipe
// runs at 1/58 of the FP32 rate (1.21 vs 70.6 TFLOP/s measured), so fused
// passes compute in df64 on the FP32 pipe.  Every operation is an error-free
// transformation written with the _rn intrinsics, which the compiler never
// contracts or reorders (TwoSum: Knuth; FastTwoSum: Dekker; TwoProd with FMA).
struct __align__(8) df64 {
  float hi, lo;
  df64() = default;
  __device__ __forceinline__ df64(float h, float l) : hi(h), lo(l) {}
  __device__ __forceinline__ df64(int v) : hi((float)v), lo(0.f) {}
  __device__ __forceinline__ explicit df64(double x) {
    hi = __double2float_rn(x);
    lo = __double2float_rn(x - (double)hi);
  }
};
struct __align__(16) df64x2 {
  df64 x, y;
};

__device__ __forceinline__ df64 two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float v = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, v)), __fsub_rn(b, v));
  return df64(s, e);
}
__device__ __forceinline__ df64 fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return df64(s, __fsub_rn(b, __fsub_rn(s, a)));
}
__device__ __forceinline__ df64 operator-(df64 a) { return df64(-a.hi, -a.lo); }
__device__ __forceinline__ df64 operator+(df64 a, df64 b) {
  const df64 s = two_sum(a.hi, b.hi);
  return fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ df64 operator*(df64 a, df64 b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return fast_two_sum(p, e);
}
// a*b + c in double-float
__device__ __forceinline__ df64 df_fma(df64 a, df64 b, df64 c) {
  const float p = __fmul_rn(a.hi, b.hi);
  float pe = __fmaf_rn(a.hi, b.hi, -p);
  pe = __fmaf_rn(a.hi, b.lo, pe);
  pe = __fmaf_rn(a.lo, b.hi, pe);
  const df64 s = two_sum(p, c.hi);
  return fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(pe, c.lo)));
}

// a*b + c in the pass's arithmetic
__device__ __forceinline__ double madd(double a, double b, double c) { return ::fma(a, b, c); }
__device__ __forceinline__ float madd(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ df64 madd(df64 a, df64 b, df64 c) { return df_fma(a, b, c); }

// Dot-product accumulator: plain FMA chains for double/float; for df64 the
// high parts are summed error-free (TwoSum) and every low-order term is
// collected in lo, renormalised once when the value is read (12 FP32
// operations per product instead of 15, same accuracy for the <= 16 terms of
// a pass row).
template <typename T>
struct Acc {
  T v;
  __device__ __forceinline__ Acc() : v(0) {}
  __device__ __forceinline__ void mad(T a, T b) { v = madd(a, b, v); }
  __device__ __forceinline__ T get() const { return v; }
};
template <>
struct Acc<df64> {
  float hi, lo;
  __device__ __forceinline__ Acc() : hi(0.f), lo(0.f) {}
  __device__ __forceinline__ void mad(df64 a, df64 b) {
    const float p = __fmul_rn(a.hi, b.hi);
    float pe = __fmaf_rn(a.hi, b.hi, -p);
    pe = __fmaf_rn(a.hi, b.lo, pe);
    pe = __fmaf_rn(a.lo, b.hi, pe);
    const df64 s = two_sum(hi, p);
    hi = s.hi;
    lo = __fadd_rn(lo, __fadd_rn(s.lo, pe));
  }
  __device__ __forceinline__ df64 get() const { return fast_two_sum(hi, lo); }
};

template <typename T> struct Vec2;
template <> struct Vec2<double> { using type = double2; };
template <> struct Vec2<float> { using type = float2; };
template <> struct Vec2<df64> { using type = df64x2; };

// L2-coherent 16-byte state accesses (in the batched work-queue kernel another
// SM may have written a run earlier in the same launch; L1 is not coherent).
template <typename T>
__device__ __forceinline__ typename Vec2<T>::type ld2(const T* p) {
  return __ldcg(reinterpret_cast<const typename Vec2<T>::type*>(p));
}
template <>
__device__ __forceinline__ df64x2 ld2<df64>(const df64* p) {
  const float4 v = __ldcg(reinterpret_cast<const float4*>(p));
  df64x2 r;
  r.x = df64(v.x, v.y);
  r.y = df64(v.z, v.w);
  return r;
}
template <typename T>
__device__ __forceinline__ void st2(T* p, const typename Vec2<T>::type& v) {
  __stcg(reinterpret_cast<typename Vec2<T>::type*>(p), v);
}
template <>
__device__ __forceinline__ void st2<df64>(df64* p, const df64x2& v) {
  __stcg(reinterpret_cast<float4*>(p), make_float4(v.x.hi, v.x.lo, v.y.hi, v.y.lo));
}

// Single-entry L2-coherent accesses.
template <typename T>
__device__ __forceinline__ T ld1(const T* p) {
  return __ldcg(p);
}
template <>
__device__ __forceinline__ df64 ld1<df64>(const df64* p) {
  const float2 v = __ldcg(reinterpret_cast<const float2*>(p));
  return df64(v.x, v.y);
}
template <typename T>
__device__ __forceinline__ void st1(T* p, T v) {
  __stcg(p, v);
}
template <>
__device__ __forceinline__ void st1<df64>(df64* p, df64 v) {
  __stcg(reinterpret_cast<float2*>(p), make_float2(v.hi, v.lo));
}

// Coefficients from the FP64 descriptor tables.
template <typename T> __device__ __forceinline__ T coef(double x) { return (T)x; }
template <> __device__ __forceinline__ df64 coef<df64>(double x) { return df64(x); }

// Sign flip on the integer pipe (GB300's FP64 pipe is ~1/58 of the FP32 rate).
__device__ __forceinline__ double flip(double x) {
  return __longlong_as_double(__double_as_longlong(x) ^ (long long)0x8000000000000000ull);
}
__device__ __forceinline__ float flip(float x) { return __int_as_float(__float_as_int(x) ^ (int)0x80000000); }
__device__ __forceinline__ df64 flip(df64 x) { return df64(flip(x.hi), flip(x.lo)); }

template <int K>
__device__ __forceinline__ int pext_local(int loc, const int* lpos) {
  int a = 0;
#pragma unroll
  for (int i = 0; i < K; i++) a |= ((loc >> lpos[i]) & 1) << i;
  return a;
}

// Shared-memory layout of a tile: entry e sits at tile_sw(e) = e ^ ((e >> B)
// & (E - 1)), E = 128 / sizeof(T) entries per 128-byte row of banks, B =
// log2 E -- within its row, the entry's bank is XORed with its row's low
// bits.  A column or row of an operator's targets (entries 2^p apart, p >= B)
// then spreads over distinct banks instead of one, and runs of consecutive
// entries stay conflict-free.  tile_sw is linear over GF(2): the offset of a
// sum of disjoint bit fields is the XOR of the fields' offsets, so the ket,
// bra and free offsets are swizzled once and combined with XOR.
template <typename T>
__device__ __forceinline__ int tile_sw(int e) {
  constexpr int E = 128 / (int)sizeof(T);
  constexpr int B = E == 32 ? 5 : 4;
  return e ^ ((e >> B) & (E - 1));
}
// The pair of entries (e, e + 1), e even: one aligned vector slot, the two
// entries in swapped order when the XOR mask is odd.
template <typename T>
__device__ __forceinline__ void st_pair(T* s, int e, typename Vec2<T>::type v) {
  constexpr int E = 128 / (int)sizeof(T);
  constexpr int B = E == 32 ? 5 : 4;
  const int x = (e >> B) & (E - 1);
  if (x & 1) {
    const T t = v.x;
    v.x = v.y;
    v.y = t;
  }
  *reinterpret_cast<typename Vec2<T>::type*>(s + (e ^ (x & ~1))) = v;
}
template <typename T>
__device__ __forceinline__ typename Vec2<T>::type ld_pair(const T* s, int e) {
  constexpr int E = 128 / (int)sizeof(T);
  constexpr int B = E == 32 ? 5 : 4;
  const int x = (e >> B) & (E - 1);
  typename Vec2<T>::type v = *reinterpret_cast<const typename Vec2<T>::type*>(s + (e ^ (x & ~1)));
  if (x & 1) {
    const T t = v.x;
    v.x = v.y;
    v.y = t;
  }
  return v;
}

// V consecutive coefficients of a dense row as one 16-byte shared-memory
// vector load: every thread of the block reads the same address (a
// broadcast), so a row of 2^K complex terms costs 2^K / V loads of each of
// U's real and imaginary parts instead of 2^K.  Rows of 3- and 4-qubit
// operators only (the narrow rows keep scalar loads and their register
// budget).
template <typename T, int D>
struct CoefVec {
  static constexpr int V = D < 8 ? 1 : 16 / (int)sizeof(T);
  struct alignas(V * sizeof(T)) Pack {
    T v[V];
  };
  __device__ __forceinline__ static Pack load(const T* p) { return *reinterpret_cast<const Pack*>(p); }
};

// Per-pass constant tables, staged in shared memory once per block (or once
// per work-queue range).  Arrays a class does not use shrink to one element.
template <typename T, int K, int CLS_>
struct PassTables {
  static constexpr int D = 1 << K;
  static constexpr int CLS = base_class(CLS_);
  static constexpr bool kMat = CLS == CLS_DENSE || CLS == CLS_SPARSE;
  uint64_t hioff[256];
  uint32_t ldmask[8], stmask[8];
  int lk[D], lb[D];  // swizzled shared-memory offsets (tile_sw) of the ket / bra indices
  int lket[4], lbra[4];
  // 16-byte aligned: the dense rows read them as 16-byte broadcast vectors
  alignas(16) T ure[kMat ? D * D : 1];
  alignas(16) T uim[kMat ? D * D : 1];
  alignas(16) T vre[kMat ? D * D : 1];
  alignas(16) T vim[kMat ? D * D : 1];
  T fre[CLS == CLS_PHASE ? D * D : 1], fim[CLS == CLS_PHASE ? D * D : 1];
  T rl[32];
  int8_t fk[D * D];
  int8_t src[D], srcb[D], nnz[D], nnzb[D];
  int8_t col[CLS == CLS_SPARSE ? D * D : 1], colb[CLS == CLS_SPARSE ? D * D : 1];
  int nnzmax, nnzbmax;
  T ssr[CLS == CLS_SUPER && K <= 2 ? D * D * D * D : 1], ssi[CLS == CLS_SUPER && K <= 2 ? D * D * D * D : 1];
};

template <typename T, int K, int CLS>
constexpr size_t pass_smem_bytes(int tile_entries) {
  return (((size_t)2 * tile_entries * sizeof(T) + 15) & ~(size_t)15) + sizeof(PassTables<T, K, CLS>);
}

// All threads of the block; the caller synchronises afterwards.
template <typename T, int K, int CLS_>
__device__ void load_tables(const PassDesc<K>* __restrict__ dp, PassTables<T, K, CLS_>& tb) {
  constexpr int D = 1 << K;
  constexpr int CLS = base_class(CLS_);
  const int tid = threadIdx.x;
  const PassHeader& h = dp->h;
  const int mhi = h.mhi;
  for (int r = tid; r < (1 << mhi); r += blockDim.x) {
    uint64_t off = 0;
    for (int j = 0; j < mhi; j++) off |= (uint64_t)((r >> j) & 1) << h.hipos[j];
    tb.hioff[r] = off;
  }
  if (tid < 8) {
    tb.ldmask[tid] = h.ldmask[tid];
    tb.stmask[tid] = h.stmask[tid];
  }
  if (tid < K) {
    tb.lket[tid] = h.lket[tid];
    tb.lbra[tid] = h.lbra[tid];
  }
  if (tid < D) {
    int lk = 0, lb = 0;
    for (int i = 0; i < K; i++) {
      lk |= ((tid >> i) & 1) << h.lket[i];
      lb |= ((tid >> i) & 1) << h.lbra[i];
    }
    tb.lk[tid] = tile_sw<T>(lk);
    tb.lb[tid] = tile_sw<T>(lb);
    tb.src[tid] = dp->op.src[tid];
    tb.srcb[tid] = dp->op.srcb[tid];
    tb.nnz[tid] = dp->op.nnz[tid];
    tb.nnzb[tid] = dp->op.nnzb[tid];
  }
  if (tid == 0) {
    tb.nnzmax = dp->op.nnzmax;
    tb.nnzbmax = dp->op.nnzbmax;
  }
  for (int i = tid; i < D * D; i += blockDim.x) {
    tb.fk[i] = dp->op.fk[i];
    if (PassTables<T, K, CLS_>::kMat) {
      tb.ure[i] = coef<T>(dp->op.ure[i]);
      tb.uim[i] = coef<T>(dp->op.uim[i]);
      tb.vre[i] = coef<T>(dp->op.vre[i]);
      tb.vim[i] = coef<T>(dp->op.vim[i]);
    }
    if (CLS == CLS_SPARSE) {
      tb.col[i] = dp->op.col[i];
      tb.colb[i] = dp->op.colb[i];
    }
    if (CLS == CLS_PHASE) {
      tb.fre[i] = coef<T>(dp->op.fre[i]);
      tb.fim[i] = coef<T>(dp->op.fim[i]);
    }
  }
  if (CLS == CLS_RLIN && tid < 16) {
    tb.rl[tid] = coef<T>(dp->op.rlin[tid]);
    tb.rl[16 + tid] = coef<T>(dp->op.rlinb[tid]);
  }
  if constexpr (CLS == CLS_SUPER && K <= 2) {
    for (int i = tid; i < D * D * D * D; i += blockDim.x) {
      tb.ssr[i] = coef<T>(dp->op.sre[i]);
      tb.ssi[i] = coef<T>(dp->op.sim[i]);
    }
  }
}

// Global index of local entry 0 of tile t: zero bits inserted at the high
// target positions into (t << L).
__device__ __forceinline__ uint64_t tile_base(const PassHeader& h, uint64_t t) {
  uint64_t base = t << h.L;
  for (int j = 0; j < h.mhi; j++) {
    const int p = h.hipos[j];
    base = ((base >> p) << (p + 1)) | (base & ((1ull << p) - 1));
  }
  return base;
}

// Register staging of one tile's loads: thread tid holds entry pairs
// tid + 256 i (i < P) -- the next tile's loads are issued before the current
// tile is transformed, so their latency hides behind its arithmetic.
template <typename T, int P>
struct TileRegs {
  typename Vec2<T>::type r[P], i[P];
};

template <typename T, int K, int CLS, int P>
__device__ __forceinline__ void load_regs(const T* __restrict__ re, const T* __restrict__ im, const PassHeader& h,
                                          const PassTables<T, K, CLS>& tb, uint64_t base, TileRegs<T, P>& x) {
  const int runlen = 1 << h.L;
#pragma unroll
  for (int k = 0; k < P; k++) {
    const int e = (threadIdx.x + k * kThreads) << 1;
    const int run = e >> h.L;
    if ((tb.ldmask[run >> 5] >> (run & 31)) & 1) {
      const uint64_t ga = base + tb.hioff[run] + (uint64_t)(e & (runlen - 1));
      x.r[k] = ld2<T>(re + ga);
      x.i[k] = ld2<T>(im + ga);
    }
  }
}

template <typename T, int K, int CLS, int P>
__device__ __forceinline__ void regs_to_smem(const PassHeader& h, const PassTables<T, K, CLS>& tb,
                                             const TileRegs<T, P>& x, T* __restrict__ sre, T* __restrict__ sim) {
  using T2 = typename Vec2<T>::type;
#pragma unroll
  for (int k = 0; k < P; k++) {
    const int e = (threadIdx.x + k * kThreads) << 1;
    const int run = e >> h.L;
    if ((tb.ldmask[run >> 5] >> (run & 31)) & 1) {
      st_pair<T>(sre, e, x.r[k]);
      st_pair<T>(sim, e, x.i[k]);
    }
  }
}

template <typename T, int K, int CLS_>
__device__ void tile_body(T* __restrict__ re, T* __restrict__ im, const PassHeader& h,
                          const PassTables<T, K, CLS_>& tb, uint64_t base, T* __restrict__ sre, T* __restrict__ sim,
                          int lf);
__device__ __forceinline__ int free_offset(const PassHeader& h);

// One tile t of the pass on the state (re, im).  All threads of the block;
// sre/sim hold G * 4^K entries each.  Ends synchronised.
template <typename T, int K, int CLS>
__device__ void run_tile(T* __restrict__ re, T* __restrict__ im, const PassHeader& h,
                         const PassTables<T, K, CLS>& tb, uint64_t t, T* __restrict__ sre, T* __restrict__ sim) {
  using T2 = typename Vec2<T>::type;
  const int tid = threadIdx.x;
  const int L = h.L;
  const int tile = (1 << h.g) * (1 << K) * (1 << K);
  const int runlen = 1 << L;
  const uint64_t base = tile_base(h, t);
  // ---- load touched runs (pairs of entries; runs are >= 2 long)
  for (int e2 = tid; e2 < (tile >> 1); e2 += blockDim.x) {
    const int e = e2 << 1;
    const int run = e >> L;
    if (!((tb.ldmask[run >> 5] >> (run & 31)) & 1)) continue;
    const uint64_t ga = base + tb.hioff[run] + (uint64_t)(e & (runlen - 1));
    const T2 vr = ld2<T>(re + ga);
    const T2 vi = ld2<T>(im + ga);
    st_pair<T>(sre, e, vr);
    st_pair<T>(sim, e, vi);
  }
  __syncthreads();
  tile_body<T, K, CLS>(re, im, h, tb, base, sre, sim, free_offset(h));
}

// The transform and the store of one tile whose touched runs are in shared
// memory (after a barrier).  Ends synchronised.
// Local offset of this thread's free group f = tid mod G (the same for every
// tile of a pass).
__device__ __forceinline__ int free_offset(const PassHeader& h) {
  const int f = threadIdx.x & ((1 << h.g) - 1);
  int lf = 0;
  for (int j = 0; j < h.g; j++) lf |= ((f >> j) & 1) << h.freepos[j];
  return lf;
}

template <typename T, int K, int CLS_>
__device__ void tile_body(T* __restrict__ re, T* __restrict__ im, const PassHeader& h,
                          const PassTables<T, K, CLS_>& tb, uint64_t base, T* __restrict__ sre, T* __restrict__ sim,
                          int lf) {
  constexpr int D = 1 << K;
  constexpr int CLS = base_class(CLS_);
  constexpr bool RE = real_class(CLS_);  // U and V real: two multiply-adds per term
  using T2 = typename Vec2<T>::type;
  const int tid = threadIdx.x;
  const int L = h.L, g = h.g;
  const int G = 1 << g;
  const int tile = G * D * D;
  const int runlen = 1 << L;
  const bool has_item = tid < G * D;
  const int r_item = tid >> g;  // b in the ket step, a in the bra step
  const int slf = tile_sw<T>(lf);

  if constexpr (CLS == CLS_SUPER && K <= 2) {
    // ---- channel: each group's 4^K entries (a, b) <- S (4^K x 4^K), one thread per group
    constexpr int DD = D * D;
    if (tid < G) {
      int ls = 0;
      for (int j = 0; j < g; j++) ls |= ((tid >> j) & 1) << h.freepos[j];
      ls = tile_sw<T>(ls);
      T xr[DD], xi[DD];
#pragma unroll
      for (int ab = 0; ab < DD; ab++) {
        const int loc = ls ^ tb.lk[ab / D] ^ tb.lb[ab % D];
        xr[ab] = sre[loc];
        xi[ab] = sim[loc];
      }
#pragma unroll
      for (int o = 0; o < DD; o++) {
        T ar = 0, ai = 0;
#pragma unroll
        for (int j = 0; j < DD; j++) {
          const T mr = tb.ssr[o * DD + j], mi = tb.ssi[o * DD + j];
          ar = madd(mr, xr[j], ar);
          ar = madd(-mi, xi[j], ar);
          ai = madd(mr, xi[j], ai);
          ai = madd(mi, xr[j], ai);
        }
        const int loc = ls ^ tb.lk[o / D] ^ tb.lb[o % D];
        sre[loc] = ar;
        sim[loc] = ai;
      }
    }
    __syncthreads();
    for (int e2 = tid; e2 < (tile >> 1); e2 += blockDim.x) {
      const int e = e2 << 1;
      const int run = e >> L;
      const uint64_t ga = base + tb.hioff[run] + (uint64_t)(e & (runlen - 1));
      st2<T>(re + ga, ld_pair<T>(sre, e));
      st2<T>(im + ga, ld_pair<T>(sim, e));
    }
  } else if (CLS == CLS_DENSE || CLS == CLS_SPARSE || CLS == CLS_RLIN) {
    // ---- ket step: column (., b, f) <- U column
    if (has_item) {
      const int b = r_item;
      const int cb = slf ^ tb.lb[b];
      if (CLS == CLS_RLIN) {
        const int p0 = cb ^ tb.lk[0], p1 = cb ^ tb.lk[1];
        const T v[4] = {sre[p0], sim[p0], sre[p1], sim[p1]};
        T o[4];
#pragma unroll
        for (int i = 0; i < 4; i++)
          o[i] = tb.rl[4 * i] * v[0] + tb.rl[4 * i + 1] * v[1] + tb.rl[4 * i + 2] * v[2] + tb.rl[4 * i + 3] * v[3];
        sre[p0] = o[0]; sim[p0] = o[1]; sre[p1] = o[2]; sim[p1] = o[3];
      } else if (CLS == CLS_DENSE) {
        T xr[D], xi[D];
#pragma unroll
        for (int c = 0; c < D; c++) {
          xr[c] = sre[cb ^ tb.lk[c]];
          xi[c] = sim[cb ^ tb.lk[c]];
        }
#pragma unroll
        for (int a = 0; a < D; a++) {
          Acc<T> ar, ai;
          using CV = CoefVec<T, D>;
#pragma unroll
          for (int c0 = 0; c0 < D; c0 += CV::V) {
            if constexpr (CV::V == 1) {
              const T ur = tb.ure[a * D + c0];
              ar.mad(ur, xr[c0]);
              ai.mad(ur, xi[c0]);
              if constexpr (!RE) {
                const T ui = tb.uim[a * D + c0];
                ar.mad(-ui, xi[c0]);
                ai.mad(ui, xr[c0]);
              }
            } else {
              const typename CV::Pack ur = CV::load(&tb.ure[a * D + c0]);
              typename CV::Pack ui;
              if constexpr (!RE) ui = CV::load(&tb.uim[a * D + c0]);
#pragma unroll
              for (int v = 0; v < CV::V; v++) {
                const int c = c0 + v;
                ar.mad(ur.v[v], xr[c]);
                ai.mad(ur.v[v], xi[c]);
                if constexpr (!RE) {
                  ar.mad(-ui.v[v], xi[c]);
                  ai.mad(ui.v[v], xr[c]);
                }
              }
            }
          }
          sre[cb ^ tb.lk[a]] = ar.get();
          sim[cb ^ tb.lk[a]] = ai.get();
        }
      } else {  // SPARSE: the rows advance together (2^K independent chains)
        Acc<T> yr[D], yi[D];
        for (int j = 0; j < tb.nnzmax; j++) {
#pragma unroll
          for (int a = 0; a < D; a++) {
            if (j < tb.nnz[a]) {
              const int c = tb.col[a * D + j];
              const T ur = tb.ure[a * D + c];
              const T vr = sre[cb ^ tb.lk[c]], vi = sim[cb ^ tb.lk[c]];
              yr[a].mad(ur, vr);
              yi[a].mad(ur, vi);
              if constexpr (!RE) {
                const T ui = tb.uim[a * D + c];
                yr[a].mad(-ui, vi);
                yi[a].mad(ui, vr);
              }
            }
          }
        }
#pragma unroll
        for (int a = 0; a < D; a++) {
          sre[cb ^ tb.lk[a]] = yr[a].get();
          sim[cb ^ tb.lk[a]] = yi[a].get();
        }
      }
    }
    __syncthreads();
    // ---- bra step: row (a, ., f) <- V row (V = conj(U) for a superoperator pass)
    if (has_item) {
      const int a = r_item;
      const int ca = slf ^ tb.lk[a];
      if (CLS == CLS_RLIN) {
        const int p0 = ca ^ tb.lb[0], p1 = ca ^ tb.lb[1];
        const T v[4] = {sre[p0], sim[p0], sre[p1], sim[p1]};
        T o[4];
#pragma unroll
        for (int i = 0; i < 4; i++)
          o[i] = tb.rl[16 + 4 * i] * v[0] + tb.rl[16 + 4 * i + 1] * v[1] + tb.rl[16 + 4 * i + 2] * v[2] +
                 tb.rl[16 + 4 * i + 3] * v[3];
        sre[p0] = o[0]; sim[p0] = o[1]; sre[p1] = o[2]; sim[p1] = o[3];
      } else if (CLS == CLS_DENSE) {
        T xr[D], xi[D];
#pragma unroll
        for (int c = 0; c < D; c++) {
          xr[c] = sre[ca ^ tb.lb[c]];
          xi[c] = sim[ca ^ tb.lb[c]];
        }
#pragma unroll
        for (int b = 0; b < D; b++) {
          Acc<T> ar, ai;
          using CV = CoefVec<T, D>;
#pragma unroll
          for (int c0 = 0; c0 < D; c0 += CV::V) {
            if constexpr (CV::V == 1) {
              const T vr = tb.vre[b * D + c0];
              ar.mad(vr, xr[c0]);
              ai.mad(vr, xi[c0]);
              if constexpr (!RE) {
                const T vi = tb.vim[b * D + c0];
                ar.mad(-vi, xi[c0]);
                ai.mad(vi, xr[c0]);
              }
            } else {
              const typename CV::Pack vr = CV::load(&tb.vre[b * D + c0]);
              typename CV::Pack vi;
              if constexpr (!RE) vi = CV::load(&tb.vim[b * D + c0]);
#pragma unroll
              for (int v = 0; v < CV::V; v++) {
                const int c = c0 + v;
                ar.mad(vr.v[v], xr[c]);
                ai.mad(vr.v[v], xi[c]);
                if constexpr (!RE) {
                  ar.mad(-vi.v[v], xi[c]);
                  ai.mad(vi.v[v], xr[c]);
                }
              }
            }
          }
          sre[ca ^ tb.lb[b]] = ar.get();
          sim[ca ^ tb.lb[b]] = ai.get();
        }
      } else {  // SPARSE: the rows advance together (2^K independent chains)
        Acc<T> yr[D], yi[D];
        for (int j = 0; j < tb.nnzbmax; j++) {
#pragma unroll
          for (int b = 0; b < D; b++) {
            if (j < tb.nnzb[b]) {
              const int c = tb.colb[b * D + j];
              const T mr = tb.vre[b * D + c];
              const T vr = sre[ca ^ tb.lb[c]], vi = sim[ca ^ tb.lb[c]];
              yr[b].mad(mr, vr);
              yi[b].mad(mr, vi);
              if constexpr (!RE) {
                const T mi = tb.vim[b * D + c];
                yr[b].mad(-mi, vi);
                yi[b].mad(mi, vr);
              }
            }
          }
        }
#pragma unroll
        for (int b = 0; b < D; b++) {
          sre[ca ^ tb.lb[b]] = yr[b].get();
          sim[ca ^ tb.lb[b]] = yi[b].get();
        }
      }
    }
    __syncthreads();
    // ---- store touched runs
    for (int e2 = tid; e2 < (tile >> 1); e2 += blockDim.x) {
      const int e = e2 << 1;
      const int run = e >> L;
      if (!((tb.stmask[run >> 5] >> (run & 31)) & 1)) continue;
      const uint64_t ga = base + tb.hioff[run] + (uint64_t)(e & (runlen - 1));
      st2<T>(re + ga, ld_pair<T>(sre, e));
      st2<T>(im + ga, ld_pair<T>(sim, e));
    }
  } else {
    // ---- monomial: out[a][b] = f[a][b] * in[src[a]][srcb[b]], fused into the store
    for (int e2 = tid; e2 < (tile >> 1); e2 += blockDim.x) {
      const int e = e2 << 1;
      const int run = e >> L;
      if (!((tb.stmask[run >> 5] >> (run & 31)) & 1)) continue;
      T outr[2], outi[2];
#pragma unroll
      for (int u = 0; u < 2; u++) {
        const int loc = e + u;
        const int a = pext_local<K>(loc, tb.lket);
        const int b = pext_local<K>(loc, tb.lbra);
        const int sa = tb.src[a], sb = tb.srcb[b];
        const int sl = tile_sw<T>(loc) ^ tb.lk[a] ^ tb.lb[b] ^ tb.lk[sa] ^ tb.lb[sb];
        const T vr = sre[sl], vi = sim[sl];
        if (CLS == CLS_MOVE) {
          outr[u] = vr;
          outi[u] = vi;
        } else {
          const int fk = tb.fk[a * D + b];
          if (CLS == CLS_PHASE && fk == FK_GEN) {
            const T fr = tb.fre[a * D + b], fi = tb.fim[a * D + b];
            outr[u] = madd(fr, vr, -fi * vi);
            outi[u] = madd(fr, vi, fi * vr);
          } else if (fk == FK_ONE) {
            outr[u] = vr;
            outi[u] = vi;
          } else if (fk == FK_NEG) {
            outr[u] = flip(vr);
            outi[u] = flip(vi);
          } else if (fk == FK_PI) {  // i*(vr + i vi) = -vi + i vr
            outr[u] = flip(vi);
            outi[u] = vr;
          } else {  // -i*(vr + i vi) = vi - i vr
            outr[u] = vi;
            outi[u] = flip(vr);
          }
        }
      }
      const uint64_t ga = base + tb.hioff[run] + (uint64_t)(e & (runlen - 1));
      T2 wr, wi;
      wr.x = outr[0];
      wr.y = outr[1];
      wi.x = outi[0];
      wi.y = outi[1];
      st2<T>(re + ga, wr);
      st2<T>(im + ga, wi);
    }
  }
  __syncthreads();
}

}  // namespace dmg
