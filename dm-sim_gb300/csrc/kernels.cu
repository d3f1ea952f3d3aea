// kernels.cu -- the superoperator pass kernels of the GB300 density-matrix engine.
//
// One kernel template (pass_kernel.cuh) covers every FP32-pipe / FP64 pass:
// element type T (double, float, or double-float pairs), width K (1..4 qubits)
// and arithmetic class (pass.h); the real-operator instances live in
// kernels_real.cu and the tensor-core passes in tensor.cu.  A block owns one tile at a time
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

#include <algorithm>
#include <type_traits>

#include "kernels.h"
#include "pass.h"
#include "pass_device.cuh"
#include "pass_kernel.cuh"

namespace dmg {

// 3- and 4-qubit SPARSE passes of complex64 states run as dense ones: on the
// FP32 pipe a dense row is 4 * 2^K multiply-adds fed by 16-byte broadcast
// coefficient loads, where the sparse row walk costs several dependent
// shared-memory loads per nonzero and runs slower at every density these
// fused blocks have.  (FP64 and double-float keep the sparse walk: their
// multiply-adds, not the loads, bound them.)
template <typename T, int K>
constexpr bool sparse_as_dense() {
  return std::is_same<T, float>::value && K >= 3;
}

template <typename T, int K>
static cudaError_t launch_k(const LaunchArgs& a, cudaStream_t s) {
  switch (a.cls) {
    case CLS_MOVE: return launch_one<T, K, CLS_MOVE>(a, s);
    case CLS_SIGNED: return launch_one<T, K, CLS_SIGNED>(a, s);
    case CLS_PHASE: return launch_one<T, K, CLS_PHASE>(a, s);
    case CLS_DENSE:
      if (a.real && K <= 2) return launch_pass_real(a, s);
      return launch_one<T, K, CLS_DENSE>(a, s);
    case CLS_SPARSE:
      if (a.real && K <= 2) return launch_pass_real(a, s);
      if (sparse_as_dense<T, K>()) return launch_one<T, K, CLS_DENSE>(a, s);
      return launch_one<T, K, CLS_SPARSE>(a, s);
    case CLS_RLIN:
      if (K == 1) return launch_one<T, 1, CLS_RLIN>(a, s);
      return cudaErrorInvalidValue;
    case CLS_SUPER:
      if (K == 1) return launch_one<T, 1, CLS_SUPER>(a, s);
      if (K == 2) return launch_one<T, 2, CLS_SUPER>(a, s);
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
  if (a.tc) {
    if (a.arith == AR_FP64) return launch_pass_tc64(a, s);
    if (a.arith == AR_FP32) return launch_pass_tc32(a, s);
    return launch_pass_tc(a, s);
  }
  if (a.direct1) return launch_pass1(a, s);
  if (a.arith == AR_DF64) return launch_t<df64>(a, s);
  return a.fp32 ? launch_t<float>(a, s) : launch_t<double>(a, s);
}

template <typename T, int K, int CLS>
static int occ_one() {
  constexpr int D = 1 << K;
  int nb = 0;
  const size_t smem = pass_smem_bytes<T, K, CLS>(kThreads * D);
  if (configure_pass<T, K, CLS>() != cudaSuccess) return 1;
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
    case CLS_SPARSE: return sparse_as_dense<T, K>() ? occ_one<T, K, CLS_DENSE>() : occ_one<T, K, CLS_SPARSE>();
    case CLS_SUPER: return K <= 1 ? occ_one<T, 1, CLS_SUPER>() : occ_one<T, 2, CLS_SUPER>();
    default: return occ_one<T, 1, CLS_RLIN>();
  }
}

int pass_blocks_per_sm(int K, int cls, int arith) {
  if (arith == AR_FP32) {
    switch (K) { case 1: return occ_k<float, 1>(cls); case 2: return occ_k<float, 2>(cls); case 3: return occ_k<float, 3>(cls); default: return occ_k<float, 4>(cls); }
  }
  if (arith == AR_DF64) {
    switch (K) { case 1: return occ_k<df64, 1>(cls); case 2: return occ_k<df64, 2>(cls); case 3: return occ_k<df64, 3>(cls); default: return occ_k<df64, 4>(cls); }
  }
  switch (K) { case 1: return occ_k<double, 1>(cls); case 2: return occ_k<double, 2>(cls); case 3: return occ_k<double, 3>(cls); default: return occ_k<double, 4>(cls); }
}

// ---------------------------------------------------------------- df64 format
// In place, once per fused run: each FP64 entry becomes the double-float pair
// (hi, lo) = (round(x), round(x - hi)) in the same 8 bytes, and back.  These
// run on the FP64 pipe, but only twice per run.
__global__ void k_to_df64(double* __restrict__ re, double* __restrict__ im, uint64_t N) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < N; i += (uint64_t)gridDim.x * blockDim.x) {
    const df64 a(re[i]), b(im[i]);
    reinterpret_cast<df64*>(re)[i] = a;
    reinterpret_cast<df64*>(im)[i] = b;
  }
}
__global__ void k_from_df64(double* __restrict__ re, double* __restrict__ im, uint64_t N) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < N; i += (uint64_t)gridDim.x * blockDim.x) {
    const df64 a = reinterpret_cast<const df64*>(re)[i], b = reinterpret_cast<const df64*>(im)[i];
    re[i] = (double)a.hi + (double)a.lo;
    im[i] = (double)b.hi + (double)b.lo;
  }
}
cudaError_t launch_to_df64(void* re, void* im, uint64_t N, unsigned grid, cudaStream_t s) {
  k_to_df64<<<grid, 256, 0, s>>>((double*)re, (double*)im, N);
  return cudaGetLastError();
}
cudaError_t launch_from_df64(void* re, void* im, uint64_t N, unsigned grid, cudaStream_t s) {
  k_from_df64<<<grid, 256, 0, s>>>((double*)re, (double*)im, N);
  return cudaGetLastError();
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

// ---------------------------------------------------------------- renormalisation
// complex64 mode: every R passes, trace(rho) is summed in FP64 and rho is made
// Hermitian with unit trace, A <- (A + A^dagger) / (2 tr), each entry in the
// state's precision scaled by the FP64 trace (tile pairs as in
// k_conj_transpose).
template <typename T>
__global__ void __launch_bounds__(256) k_trace(const T* __restrict__ re, int n, double* __restrict__ out) {
  const uint64_t dim = 1ull << n;
  double acc = 0;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < dim; i += (uint64_t)gridDim.x * blockDim.x)
    acc += (double)re[i * dim + i];
  __shared__ double sh[256];
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int st = 128; st > 0; st >>= 1) {
    if (threadIdx.x < st) sh[threadIdx.x] += sh[threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x == 0) atomicAdd(out, sh[0]);
}

template <typename T>
__global__ void __launch_bounds__(256) k_hermitise(T* __restrict__ re, T* __restrict__ im, int n,
                                                   const double* __restrict__ trace) {
  constexpr int TS = 32;
  __shared__ T a_re[TS][TS + 1], a_im[TS][TS + 1], b_re[TS][TS + 1], b_im[TS][TS + 1];
  const uint64_t dim = 1ull << n;
  const int ts = dim < TS ? (int)dim : TS;
  const uint64_t nt = dim / ts;
  const double inv = 1.0 / *trace;
  const int tx = threadIdx.x & 31, ty0 = threadIdx.x >> 5;
  for (uint64_t p = blockIdx.x; p < nt * nt; p += gridDim.x) {
    const uint64_t I = p / nt, J = p % nt;
    if (I > J) continue;
    if (tx < ts)
      for (int ty = ty0; ty < ts; ty += 8) {
        const uint64_t ia = (I * ts + ty) * dim + J * ts + tx, ib = (J * ts + ty) * dim + I * ts + tx;
        a_re[ty][tx] = re[ia];
        a_im[ty][tx] = im[ia];
        b_re[ty][tx] = re[ib];
        b_im[ty][tx] = im[ib];
      }
    __syncthreads();
    if (tx < ts)
      for (int ty = ty0; ty < ts; ty += 8) {
        const uint64_t ia = (I * ts + ty) * dim + J * ts + tx, ib = (J * ts + ty) * dim + I * ts + tx;
        // new A[x][y] = (A[x][y] + conj(A[y][x])) / 2 / tr, in the state's
        // precision with the FP64 trace's scale (FP64 arithmetic on FP32
        // entries would be bound by the f32 <-> f64 conversion rate)
        const T h = (T)(0.5 * inv);
        re[ia] = (a_re[ty][tx] + b_re[tx][ty]) * h;
        im[ia] = (a_im[ty][tx] - b_im[tx][ty]) * h;
        re[ib] = (b_re[ty][tx] + a_re[tx][ty]) * h;
        im[ib] = (b_im[ty][tx] - a_im[tx][ty]) * h;
      }
    __syncthreads();
  }
}

cudaError_t launch_renormalise(void* re, void* im, int n, bool fp32, double* d_trace, unsigned grid, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(d_trace, 0, sizeof(double), s);
  if (e != cudaSuccess) return e;
  const unsigned tg = (unsigned)std::min<uint64_t>((1ull << n) / 256 + 1, 1024);
  if (fp32) {
    k_trace<float><<<tg, 256, 0, s>>>((const float*)re, n, d_trace);
    k_hermitise<float><<<grid, 256, 0, s>>>((float*)re, (float*)im, n, d_trace);
  } else {
    k_trace<double><<<tg, 256, 0, s>>>((const double*)re, n, d_trace);
    k_hermitise<double><<<grid, 256, 0, s>>>((double*)re, (double*)im, n, d_trace);
  }
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
