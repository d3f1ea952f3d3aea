// kernels.cu -- the superoperator pass kernels of the GB300 density-matrix engine.
//
// One kernel template covers every pass: precision T (double or float), width K
// (1..4 qubits) and arithmetic class (pass.h).  A block owns one tile at a time
// (grid-stride over tiles): it loads the tile's touched runs with 16-byte
// vector loads into shared memory, transforms them, and stores them back.
// Monomial classes (MOVE/SIGNED/PHASE) fuse the permutation and the per-entry
// factor into the store, so they cost no FP64 arithmetic beyond one complex
// multiply (PHASE) and never more than one HBM read and write per entry.
// DENSE/SPARSE apply U to the ket bits of each column and V to the bra bits
// of each row; V = conj(U) makes the pass U (x) conj(U) on the 2K target bits,
// V = I makes it a ket-only pass (the reference's forward/backward stages).
#include <cuda_runtime.h>
#include <stdint.h>

#include "kernels.h"
#include "pass.h"

namespace dmg {

template <typename T> struct Vec2;
template <> struct Vec2<double> { using type = double2; };
template <> struct Vec2<float> { using type = float2; };

// Sign flip on the integer pipe (GB300's FP64 pipe is ~1/58 of the FP32 rate).
__device__ __forceinline__ double flip(double x) {
  return __longlong_as_double(__double_as_longlong(x) ^ (long long)0x8000000000000000ull);
}
__device__ __forceinline__ float flip(float x) { return __int_as_float(__float_as_int(x) ^ (int)0x80000000); }

template <int K>
__device__ __forceinline__ int pext_local(int loc, const int* lpos) {
  int a = 0;
#pragma unroll
  for (int i = 0; i < K; i++) a |= ((loc >> lpos[i]) & 1) << i;
  return a;
}

template <typename T, int K, int CLS>
__global__ void __launch_bounds__(kThreads) k_pass(T* __restrict__ re, T* __restrict__ im,
                                                   const PassDesc<K>* __restrict__ dp) {
  constexpr int D = 1 << K;
  using T2 = typename Vec2<T>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* sre = reinterpret_cast<T*>(smem_raw);

  __shared__ uint64_t s_hioff[256];
  __shared__ uint32_t s_ldmask[8], s_stmask[8];
  __shared__ int s_lk[D], s_lb[D];
  __shared__ int s_lket[4], s_lbra[4];
  __shared__ T s_ure[(CLS == CLS_DENSE || CLS == CLS_SPARSE) ? D * D : 1];
  __shared__ T s_uim[(CLS == CLS_DENSE || CLS == CLS_SPARSE) ? D * D : 1];
  __shared__ T s_vre[(CLS == CLS_DENSE || CLS == CLS_SPARSE) ? D * D : 1];
  __shared__ T s_vim[(CLS == CLS_DENSE || CLS == CLS_SPARSE) ? D * D : 1];
  __shared__ T s_fre[CLS == CLS_PHASE ? D * D : 1];
  __shared__ T s_fim[CLS == CLS_PHASE ? D * D : 1];
  __shared__ int8_t s_fk[D * D];
  __shared__ int8_t s_src[D], s_srcb[D];
  __shared__ int8_t s_nnz[D], s_nnzb[D];
  __shared__ int8_t s_col[CLS == CLS_SPARSE ? D * D : 1];
  __shared__ int8_t s_colb[CLS == CLS_SPARSE ? D * D : 1];
  __shared__ T s_rl[32];

  const int tid = threadIdx.x;
  const PassHeader& h = dp->h;
  const int L = h.L, mhi = h.mhi, g = h.g;
  const int G = 1 << g;
  const int tile = G * D * D;
  const uint64_t ntiles = h.ntiles;
  T* sim = sre + tile;

  // ---- per-block constant tables
  for (int r = tid; r < (1 << mhi); r += kThreads) {
    uint64_t off = 0;
    for (int j = 0; j < mhi; j++) off |= (uint64_t)((r >> j) & 1) << h.hipos[j];
    s_hioff[r] = off;
  }
  if (tid < 8) {
    s_ldmask[tid] = h.ldmask[tid];
    s_stmask[tid] = h.stmask[tid];
  }
  if (tid < K) {
    s_lket[tid] = h.lket[tid];
    s_lbra[tid] = h.lbra[tid];
  }
  if (tid < D) {
    int lk = 0, lb = 0;
    for (int i = 0; i < K; i++) {
      lk |= ((tid >> i) & 1) << h.lket[i];
      lb |= ((tid >> i) & 1) << h.lbra[i];
    }
    s_lk[tid] = lk;
    s_lb[tid] = lb;
    s_src[tid] = dp->op.src[tid];
    s_srcb[tid] = dp->op.srcb[tid];
    s_nnz[tid] = dp->op.nnz[tid];
    s_nnzb[tid] = dp->op.nnzb[tid];
  }
  for (int i = tid; i < D * D; i += kThreads) {
    s_fk[i] = dp->op.fk[i];
    if (CLS == CLS_DENSE || CLS == CLS_SPARSE) {
      s_ure[i] = (T)dp->op.ure[i];
      s_uim[i] = (T)dp->op.uim[i];
      s_vre[i] = (T)dp->op.vre[i];
      s_vim[i] = (T)dp->op.vim[i];
    }
    if (CLS == CLS_SPARSE) {
      s_col[i] = dp->op.col[i];
      s_colb[i] = dp->op.colb[i];
    }
    if (CLS == CLS_PHASE) {
      s_fre[i] = (T)dp->op.fre[i];
      s_fim[i] = (T)dp->op.fim[i];
    }
  }
  if (CLS == CLS_RLIN && tid < 16) {
    s_rl[tid] = (T)dp->op.rlin[tid];
    s_rl[16 + tid] = (T)dp->op.rlinb[tid];
  }
  __syncthreads();

  // free-bit deposit of this thread's group index (fixed over tiles)
  const int w = tid;
  const bool has_item = w < G * D;
  int lf = 0;
  {
    const int f = w & (G - 1);
    for (int j = 0; j < g; j++) lf |= ((f >> j) & 1) << h.freepos[j];
  }
  const int r_item = w >> g;  // b in the ket step, a in the bra step
  __syncthreads();

  const int runlen = 1 << L;

  for (uint64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    // tile base: insert zero bits at the high target positions into (t << L)
    uint64_t base = t << L;
    for (int j = 0; j < mhi; j++) {
      const int p = h.hipos[j];
      base = ((base >> p) << (p + 1)) | (base & ((1ull << p) - 1));
    }
    // ---- load touched runs (pairs of entries; runs are >= 2 long)
    for (int e2 = tid; e2 < (tile >> 1); e2 += kThreads) {
      const int e = e2 << 1;
      const int run = e >> L;
      if (!((s_ldmask[run >> 5] >> (run & 31)) & 1)) continue;
      const uint64_t ga = base + s_hioff[run] + (uint64_t)(e & (runlen - 1));
      const T2 vr = *reinterpret_cast<const T2*>(re + ga);
      const T2 vi = *reinterpret_cast<const T2*>(im + ga);
      *reinterpret_cast<T2*>(sre + e) = vr;
      *reinterpret_cast<T2*>(sim + e) = vi;
    }
    __syncthreads();

    if (CLS == CLS_DENSE || CLS == CLS_SPARSE || CLS == CLS_RLIN) {
      // ---- ket step: column (., b, f) <- U column
      if (has_item) {
        const int b = r_item;
        const int cb = lf + s_lb[b];
        if (CLS == CLS_RLIN) {
          const int p0 = cb + s_lk[0], p1 = cb + s_lk[1];
          const T v[4] = {sre[p0], sim[p0], sre[p1], sim[p1]};
          T o[4];
#pragma unroll
          for (int i = 0; i < 4; i++) o[i] = s_rl[4 * i] * v[0] + s_rl[4 * i + 1] * v[1] + s_rl[4 * i + 2] * v[2] + s_rl[4 * i + 3] * v[3];
          sre[p0] = o[0]; sim[p0] = o[1]; sre[p1] = o[2]; sim[p1] = o[3];
        } else if (CLS == CLS_DENSE) {
          T xr[D], xi[D];
#pragma unroll
          for (int c = 0; c < D; c++) {
            xr[c] = sre[cb + s_lk[c]];
            xi[c] = sim[cb + s_lk[c]];
          }
#pragma unroll
          for (int a = 0; a < D; a++) {
            T ar = 0, ai = 0;
#pragma unroll
            for (int c = 0; c < D; c++) {
              const T ur = s_ure[a * D + c], ui = s_uim[a * D + c];
              ar = fma(ur, xr[c], ar);
              ar = fma(-ui, xi[c], ar);
              ai = fma(ur, xi[c], ai);
              ai = fma(ui, xr[c], ai);
            }
            sre[cb + s_lk[a]] = ar;
            sim[cb + s_lk[a]] = ai;
          }
        } else {  // SPARSE
          T yr[D], yi[D];
#pragma unroll
          for (int a = 0; a < D; a++) {
            T ar = 0, ai = 0;
            const int nz = s_nnz[a];
            for (int j = 0; j < nz; j++) {
              const int c = s_col[a * D + j];
              const T ur = s_ure[a * D + c], ui = s_uim[a * D + c];
              const T vr = sre[cb + s_lk[c]], vi = sim[cb + s_lk[c]];
              ar = fma(ur, vr, ar);
              ar = fma(-ui, vi, ar);
              ai = fma(ur, vi, ai);
              ai = fma(ui, vr, ai);
            }
            yr[a] = ar;
            yi[a] = ai;
          }
#pragma unroll
          for (int a = 0; a < D; a++) {
            sre[cb + s_lk[a]] = yr[a];
            sim[cb + s_lk[a]] = yi[a];
          }
        }
      }
      __syncthreads();
      // ---- bra step: row (a, ., f) <- V row (V = conj(U) for a superoperator pass)
      if (has_item) {
        const int a = r_item;
        const int ca = lf + s_lk[a];
        if (CLS == CLS_RLIN) {
          const int p0 = ca + s_lb[0], p1 = ca + s_lb[1];
          const T v[4] = {sre[p0], sim[p0], sre[p1], sim[p1]};
          T o[4];
#pragma unroll
          for (int i = 0; i < 4; i++) o[i] = s_rl[16 + 4 * i] * v[0] + s_rl[16 + 4 * i + 1] * v[1] + s_rl[16 + 4 * i + 2] * v[2] + s_rl[16 + 4 * i + 3] * v[3];
          sre[p0] = o[0]; sim[p0] = o[1]; sre[p1] = o[2]; sim[p1] = o[3];
        } else if (CLS == CLS_DENSE) {
          T xr[D], xi[D];
#pragma unroll
          for (int c = 0; c < D; c++) {
            xr[c] = sre[ca + s_lb[c]];
            xi[c] = sim[ca + s_lb[c]];
          }
#pragma unroll
          for (int b = 0; b < D; b++) {
            T ar = 0, ai = 0;
#pragma unroll
            for (int c = 0; c < D; c++) {
              const T vr = s_vre[b * D + c], vi = s_vim[b * D + c];
              ar = fma(vr, xr[c], ar);
              ar = fma(-vi, xi[c], ar);
              ai = fma(vr, xi[c], ai);
              ai = fma(vi, xr[c], ai);
            }
            sre[ca + s_lb[b]] = ar;
            sim[ca + s_lb[b]] = ai;
          }
        } else {  // SPARSE
          T yr[D], yi[D];
#pragma unroll
          for (int b = 0; b < D; b++) {
            T ar = 0, ai = 0;
            const int nz = s_nnzb[b];
            for (int j = 0; j < nz; j++) {
              const int c = s_colb[b * D + j];
              const T mr = s_vre[b * D + c], mi = s_vim[b * D + c];
              const T vr = sre[ca + s_lb[c]], vi = sim[ca + s_lb[c]];
              ar = fma(mr, vr, ar);
              ar = fma(-mi, vi, ar);
              ai = fma(mr, vi, ai);
              ai = fma(mi, vr, ai);
            }
            yr[b] = ar;
            yi[b] = ai;
          }
#pragma unroll
          for (int b = 0; b < D; b++) {
            sre[ca + s_lb[b]] = yr[b];
            sim[ca + s_lb[b]] = yi[b];
          }
        }
      }
      __syncthreads();
      // ---- store touched runs
      for (int e2 = tid; e2 < (tile >> 1); e2 += kThreads) {
        const int e = e2 << 1;
        const int run = e >> L;
        if (!((s_stmask[run >> 5] >> (run & 31)) & 1)) continue;
        const uint64_t ga = base + s_hioff[run] + (uint64_t)(e & (runlen - 1));
        *reinterpret_cast<T2*>(re + ga) = *reinterpret_cast<const T2*>(sre + e);
        *reinterpret_cast<T2*>(im + ga) = *reinterpret_cast<const T2*>(sim + e);
      }
    } else {
      // ---- monomial: out[a][b] = f[a][b] * in[src[a]][src[b]], fused into the store
      for (int e2 = tid; e2 < (tile >> 1); e2 += kThreads) {
        const int e = e2 << 1;
        const int run = e >> L;
        if (!((s_stmask[run >> 5] >> (run & 31)) & 1)) continue;
        T outr[2], outi[2];
#pragma unroll
        for (int u = 0; u < 2; u++) {
          const int loc = e + u;
          const int a = pext_local<K>(loc, s_lket);
          const int b = pext_local<K>(loc, s_lbra);
          const int sa = s_src[a], sb = s_srcb[b];
          const int sl = loc - s_lk[a] - s_lb[b] + s_lk[sa] + s_lb[sb];
          const T vr = sre[sl], vi = sim[sl];
          if (CLS == CLS_MOVE) {
            outr[u] = vr;
            outi[u] = vi;
          } else {
            const int fk = s_fk[a * D + b];
            if (CLS == CLS_PHASE && fk == FK_GEN) {
              const T fr = s_fre[a * D + b], fi = s_fim[a * D + b];
              outr[u] = fma(fr, vr, -fi * vi);
              outi[u] = fma(fr, vi, fi * vr);
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
        const uint64_t ga = base + s_hioff[run] + (uint64_t)(e & (runlen - 1));
        T2 wr, wi;
        wr.x = outr[0]; wr.y = outr[1];
        wi.x = outi[0]; wi.y = outi[1];
        *reinterpret_cast<T2*>(re + ga) = wr;
        *reinterpret_cast<T2*>(im + ga) = wi;
      }
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------- launchers
template <typename T, int K, int CLS>
static cudaError_t launch_one(const LaunchArgs& a, cudaStream_t s) {
  constexpr int D = 1 << K;
  const size_t smem = (size_t)2 * a.tile_entries * sizeof(T);
  static int configured = 0;  // per instance; attribute set once per process
  if (!configured) {
    cudaError_t e = cudaFuncSetAttribute(k_pass<T, K, CLS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)(2 * kThreads * D * sizeof(T)));
    if (e != cudaSuccess) return e;
    configured = 1;
  }
  k_pass<T, K, CLS><<<a.grid, kThreads, smem, s>>>(static_cast<T*>(a.re), static_cast<T*>(a.im),
                                                   static_cast<const PassDesc<K>*>(a.desc));
  return cudaGetLastError();
}

template <typename T, int K>
static cudaError_t launch_k(const LaunchArgs& a, cudaStream_t s) {
  switch (a.cls) {
    case CLS_MOVE: return launch_one<T, K, CLS_MOVE>(a, s);
    case CLS_SIGNED: return launch_one<T, K, CLS_SIGNED>(a, s);
    case CLS_PHASE: return launch_one<T, K, CLS_PHASE>(a, s);
    case CLS_DENSE: return launch_one<T, K, CLS_DENSE>(a, s);
    case CLS_SPARSE: return launch_one<T, K, CLS_SPARSE>(a, s);
    case CLS_RLIN:
      if (K == 1) return launch_one<T, 1, CLS_RLIN>(a, s);
      return cudaErrorInvalidValue;
    default: return cudaErrorInvalidValue;
  }
}

template <typename T>
static cudaError_t launch_t(const LaunchArgs& a, cudaStream_t s) {
  switch (a.K) {
    case 1: return launch_k<T, 1>(a, s);
    case 2: return launch_k<T, 2>(a, s);
    case 3: return launch_k<T, 3>(a, s);
    case 4: return launch_k<T, 4>(a, s);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_pass(const LaunchArgs& a, cudaStream_t s) {
  return a.fp32 ? launch_t<float>(a, s) : launch_t<double>(a, s);
}

template <typename T, int K, int CLS>
static int occ_one() {
  constexpr int D = 1 << K;
  int nb = 0;
  const size_t smem = (size_t)2 * kThreads * D * sizeof(T);
  cudaFuncSetAttribute(k_pass<T, K, CLS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_pass<T, K, CLS>, kThreads, smem) != cudaSuccess) return 1;
  return nb > 0 ? nb : 1;
}

template <typename T, int K>
static int occ_k(int cls) {
  switch (cls) {
    case CLS_MOVE: return occ_one<T, K, CLS_MOVE>();
    case CLS_SIGNED: return occ_one<T, K, CLS_SIGNED>();
    case CLS_PHASE: return occ_one<T, K, CLS_PHASE>();
    case CLS_DENSE: return occ_one<T, K, CLS_DENSE>();
    case CLS_SPARSE: return occ_one<T, K, CLS_SPARSE>();
    default: return occ_one<T, 1, CLS_RLIN>();
  }
}

int pass_blocks_per_sm(int K, int cls, bool fp32) {
  if (fp32) {
    switch (K) { case 1: return occ_k<float, 1>(cls); case 2: return occ_k<float, 2>(cls); case 3: return occ_k<float, 3>(cls); default: return occ_k<float, 4>(cls); }
  }
  switch (K) { case 1: return occ_k<double, 1>(cls); case 2: return occ_k<double, 2>(cls); case 3: return occ_k<double, 3>(cls); default: return occ_k<double, 4>(cls); }
}

// ---------------------------------------------------------------- conj transpose
// In place A'[x*dim + y] = conj(A[y*dim + x]): the reference's adjoint stage
// between its forward and backward passes (block_transpose,
// src/dmsim_nvgpu_omp.cuh:825-855), done as swaps of tile pairs (I, J), I <= J,
// staged in shared memory so both the loads and the stores are coalesced.
template <typename T>
__global__ void __launch_bounds__(256) k_conj_transpose(T* __restrict__ re, T* __restrict__ im, int n) {
  constexpr int TS = 32;
  __shared__ T a_re[TS][TS + 1], a_im[TS][TS + 1], b_re[TS][TS + 1], b_im[TS][TS + 1];
  const uint64_t dim = 1ull << n;
  const int ts = dim < TS ? (int)dim : TS;
  const uint64_t nt = dim / ts;
  const int tx = threadIdx.x & 31, ty0 = threadIdx.x >> 5;  // 32 x 8 threads
  for (uint64_t p = blockIdx.x; p < nt * nt; p += gridDim.x) {
    const uint64_t I = p / nt, J = p % nt;
    if (I > J) continue;  // uniform over the block
    if (tx < ts)
      for (int ty = ty0; ty < ts; ty += 8) {
        const uint64_t ia = (I * ts + ty) * dim + J * ts + tx;  // tile (I,J)
        const uint64_t ib = (J * ts + ty) * dim + I * ts + tx;  // tile (J,I)
        a_re[ty][tx] = re[ia];
        a_im[ty][tx] = im[ia];
        b_re[ty][tx] = re[ib];
        b_im[ty][tx] = im[ib];
      }
    __syncthreads();
    if (tx < ts)
      for (int ty = ty0; ty < ts; ty += 8) {
        const uint64_t ia = (I * ts + ty) * dim + J * ts + tx;
        const uint64_t ib = (J * ts + ty) * dim + I * ts + tx;
        re[ia] = b_re[tx][ty];
        im[ia] = flip(b_im[tx][ty]);
        re[ib] = a_re[tx][ty];
        im[ib] = flip(a_im[tx][ty]);
      }
    __syncthreads();
  }
}

cudaError_t launch_conj_transpose(void* re, void* im, int n, bool fp32, unsigned grid, cudaStream_t s) {
  if (fp32) k_conj_transpose<float><<<grid, 256, 0, s>>>((float*)re, (float*)im, n);
  else k_conj_transpose<double><<<grid, 256, 0, s>>>((double*)re, (double*)im, n);
  return cudaGetLastError();
}

// ---------------------------------------------------------------- utilities
template <typename T>
__global__ void k_set_basis(T* re, T* im, uint64_t idx) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    re[idx] = (T)1;
    im[idx] = (T)0;
  }
}

template <typename T>
__global__ void k_get_diag(const T* __restrict__ re, uint64_t dim, double* __restrict__ out) {
  const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i < dim) out[i] = (double)re[i * dim + i];
}

cudaError_t launch_set_zero_state(void* re, void* im, uint64_t N, bool fp32, cudaStream_t s) {
  const size_t es = fp32 ? 4 : 8;
  cudaError_t e = cudaMemsetAsync(re, 0, N * es, s);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(im, 0, N * es, s);
  if (e != cudaSuccess) return e;
  if (fp32) k_set_basis<float><<<1, 32, 0, s>>>((float*)re, (float*)im, 0);
  else k_set_basis<double><<<1, 32, 0, s>>>((double*)re, (double*)im, 0);
  return cudaGetLastError();
}

cudaError_t launch_get_diag(const void* re, uint64_t dim, bool fp32, double* d_out, cudaStream_t s) {
  const unsigned blocks = (unsigned)((dim + 255) / 256);
  if (fp32) k_get_diag<float><<<blocks, 256, 0, s>>>((const float*)re, dim, d_out);
  else k_get_diag<double><<<blocks, 256, 0, s>>>((const double*)re, dim, d_out);
  return cudaGetLastError();
}

}  // namespace dmg
