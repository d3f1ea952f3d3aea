// kernels_k1.cu -- 1-qubit passes without shared memory.  A 1-qubit pass
// touches each group of four entries rho[(a, b)] (a = ket bit q, b = bra bit
// q + n) on its own, so a thread takes whole groups straight from global
// memory -- consecutive threads take consecutive groups, so every load and
// store instruction of a warp is coalesced -- applies U on the ket bit and V
// on the bra bit in registers (the same operation order and accumulator as
// the tiled kernel), and writes back the entries the pass changes.  No tile
// staging, no barriers: these passes (most of the plain gate-by-gate path)
// are bound by HBM or by the arithmetic alone.
#include <cuda_runtime.h>
#include <stdint.h>

#include "kernels.h"
#include "pass_device.cuh"

namespace dmg {

namespace {

template <typename T, int CLS_>
__global__ void __launch_bounds__(256) k_pass1(T* __restrict__ re, T* __restrict__ im,
                                               const PassDesc<1>* __restrict__ dp, int q, int n) {
  constexpr int CLS = base_class(CLS_);
  constexpr bool RE = real_class(CLS_);
  constexpr bool kMono = CLS == CLS_MOVE || CLS == CLS_SIGNED || CLS == CLS_PHASE;
  const PassOp<1>& op = dp->op;
  // the operator, uniform over the grid (a few dozen bytes from L1)
  T ur[4], ui[4], vr[4], vi[4], fr[4], fi[4];
  int src[2], srcb[2], fk[4];
  bool need[4], chg[4];
#pragma unroll
  for (int i = 0; i < 4; i++) {
    ur[i] = coef<T>(op.ure[i]);
    ui[i] = coef<T>(op.uim[i]);
    vr[i] = coef<T>(op.vre[i]);
    vi[i] = coef<T>(op.vim[i]);
    fr[i] = coef<T>(op.fre[i]);
    fi[i] = coef<T>(op.fim[i]);
    fk[i] = op.fk[i];
  }
  src[0] = op.src[0];
  src[1] = op.src[1];
  srcb[0] = op.srcb[0];
  srcb[1] = op.srcb[1];
  // entry e = a + 2b: which change, which are read (unrolled comparisons,
  // so that the small arrays stay in registers)
  int sidx[4];
#pragma unroll
  for (int e = 0; e < 4; e++) {
    const int a = e & 1, b = e >> 1;
    sidx[e] = src[a] + 2 * srcb[b];
    chg[e] = !kMono || sidx[e] != e || fk[a * 2 + b] != FK_ONE;
  }
#pragma unroll
  for (int e = 0; e < 4; e++) {
    bool nd = !kMono;
#pragma unroll
    for (int e2 = 0; e2 < 4; e2++) nd = nd || (chg[e2] && sidx[e2] == e);
    need[e] = nd;
  }

  const uint64_t ngroups = 1ull << (2 * n - 2);
  const uint64_t mq = 1ull << q, mb = 1ull << (q + n);
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; g < ngroups; g += stride) {
    uint64_t i = ((g >> q) << (q + 1)) | (g & (mq - 1));
    i = ((i >> (q + n)) << (q + n + 1)) | (i & (mb - 1));
    uint64_t idx[4];
    idx[0] = i;
    idx[1] = i + mq;
    idx[2] = i + mb;
    idx[3] = i + mq + mb;
    T xr[4], xi[4];
#pragma unroll
    for (int e = 0; e < 4; e++) {
      xr[e] = need[e] ? ld1<T>(re + idx[e]) : T(0);
      xi[e] = need[e] ? ld1<T>(im + idx[e]) : T(0);
    }
    T outr[4], outi[4];
    if constexpr (kMono) {
#pragma unroll
      for (int e = 0; e < 4; e++) {
        const int a = e & 1, b = e >> 1, s = sidx[e], k = a * 2 + b;
        const T r = s == 0 ? xr[0] : s == 1 ? xr[1] : s == 2 ? xr[2] : xr[3];
        const T m = s == 0 ? xi[0] : s == 1 ? xi[1] : s == 2 ? xi[2] : xi[3];
        if (CLS == CLS_MOVE || fk[k] == FK_ONE) {
          outr[e] = r;
          outi[e] = m;
        } else if (CLS == CLS_PHASE && fk[k] == FK_GEN) {
          outr[e] = madd(fr[k], r, -fi[k] * m);
          outi[e] = madd(fr[k], m, fi[k] * r);
        } else if (fk[k] == FK_NEG) {
          outr[e] = flip(r);
          outi[e] = flip(m);
        } else if (fk[k] == FK_PI) {
          outr[e] = flip(m);
          outi[e] = r;
        } else {
          outr[e] = m;
          outi[e] = flip(r);
        }
      }
    } else {
      // ket step: y[a][b] = sum_c U[a][c] x[c][b]
      T yr[4], yi[4];
#pragma unroll
      for (int b = 0; b < 2; b++)
#pragma unroll
        for (int a = 0; a < 2; a++) {
          Acc<T> ar, ai;
#pragma unroll
          for (int c = 0; c < 2; c++) {
            ar.mad(ur[a * 2 + c], xr[c + 2 * b]);
            ai.mad(ur[a * 2 + c], xi[c + 2 * b]);
            if constexpr (!RE) {
              ar.mad(-ui[a * 2 + c], xi[c + 2 * b]);
              ai.mad(ui[a * 2 + c], xr[c + 2 * b]);
            }
          }
          yr[a + 2 * b] = ar.get();
          yi[a + 2 * b] = ai.get();
        }
      // bra step: out[a][b] = sum_d V[b][d] y[a][d]
#pragma unroll
      for (int a = 0; a < 2; a++)
#pragma unroll
        for (int b = 0; b < 2; b++) {
          Acc<T> ar, ai;
#pragma unroll
          for (int d = 0; d < 2; d++) {
            ar.mad(vr[b * 2 + d], yr[a + 2 * d]);
            ai.mad(vr[b * 2 + d], yi[a + 2 * d]);
            if constexpr (!RE) {
              ar.mad(-vi[b * 2 + d], yi[a + 2 * d]);
              ai.mad(vi[b * 2 + d], yr[a + 2 * d]);
            }
          }
          outr[a + 2 * b] = ar.get();
          outi[a + 2 * b] = ai.get();
        }
    }
#pragma unroll
    for (int e = 0; e < 4; e++)
      if (chg[e]) {
        st1<T>(re + idx[e], outr[e]);
        st1<T>(im + idx[e], outi[e]);
      }
  }
}

template <typename T, int CLS_>
cudaError_t launch1(const LaunchArgs& a, cudaStream_t s) {
  k_pass1<T, CLS_><<<a.grid, 256, 0, s>>>(static_cast<T*>(a.re), static_cast<T*>(a.im),
                                          static_cast<const PassDesc<1>*>(a.desc), a.q0, a.n);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch1_t(const LaunchArgs& a, cudaStream_t s) {
  switch (a.cls) {
    case CLS_MOVE: return launch1<T, CLS_MOVE>(a, s);
    case CLS_SIGNED: return launch1<T, CLS_SIGNED>(a, s);
    case CLS_PHASE: return launch1<T, CLS_PHASE>(a, s);
    case CLS_DENSE: return a.real ? launch1<T, CLS_DENSE_REAL>(a, s) : launch1<T, CLS_DENSE>(a, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace

bool direct1_class(int cls) { return cls == CLS_MOVE || cls == CLS_SIGNED || cls == CLS_PHASE || cls == CLS_DENSE; }

cudaError_t launch_pass1(const LaunchArgs& a, cudaStream_t s) {
  if (a.K != 1 || !direct1_class(a.cls)) return cudaErrorInvalidValue;
  if (a.arith == AR_DF64) return launch1_t<df64>(a, s);
  return a.fp32 ? launch1_t<float>(a, s) : launch1_t<double>(a, s);
}

}  // namespace dmg
