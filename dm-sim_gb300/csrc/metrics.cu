// metrics.cu -- comparison of the device density matrix with a pure state.
//
// For rho held as A[c*2^n + r] = rho[r][c] and a pure state psi, one pass
// over A gives the fidelity <psi|rho|psi> = sum_{r,c} conj(psi_r) rho[r][c]
// psi_c, the trace, the largest |rho[r][c] - psi_r conj(psi_c)| and the
// Frobenius norm of the difference.  These back the full-size parity checks,
// where the CPU density-matrix oracle cannot run, with the statevector oracle.
#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>
#include <mutex>

#include "metrics.h"

namespace dmg {

// Scratch of the no-allocation metrics entry point (dmsim_pure_metrics_noalloc):
// the pure state's real parts, its imaginary parts (kNoAllocMaxDim each) and
// four accumulators -- 1 MiB + 64 B, held by every GPU that loads the library
// until the process exits.  Host code must not use this name as a device
// address; it asks the runtime for the address (noalloc_scratch below).
static __device__ __align__(256) double g_noalloc_scratch[2 * kNoAllocMaxDim + 8];

__device__ __forceinline__ void atomic_max_nonneg(double* addr, double v) {
  // non-negative doubles order like their bit patterns
  atomicMax(reinterpret_cast<unsigned long long*>(addr), (unsigned long long)__double_as_longlong(v));
}

template <typename T>
__global__ void __launch_bounds__(256) k_pure_metrics(const T* __restrict__ re, const T* __restrict__ im,
                                                      const double* __restrict__ pr, const double* __restrict__ pi,
                                                      int n, double* acc) {
  const uint64_t dim = 1ull << n, N = dim * dim;
  double fid = 0, tr = 0, mx = 0, fro = 0;
  for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < N; v += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t r = v & (dim - 1), c = v >> n;
    const double ar = (double)re[v], ai = (double)im[v];
    // psi_r conj(psi_c)
    const double er = pr[r] * pr[c] + pi[r] * pi[c];
    const double ei = pi[r] * pr[c] - pr[r] * pi[c];
    const double dr = ar - er, di = ai - ei;
    const double d2 = dr * dr + di * di;
    fro += d2;
    mx = fmax(mx, d2);
    // conj(psi_r) * A * psi_c, real part
    const double tr_ = pr[r] * ar + pi[r] * ai;  // conj(psi_r) * A
    const double ti_ = pr[r] * ai - pi[r] * ar;
    fid += tr_ * pr[c] - ti_ * pi[c];
    if (r == c) tr += ar;
  }
  __shared__ double s[4][256];
  s[0][threadIdx.x] = fid;
  s[1][threadIdx.x] = tr;
  s[2][threadIdx.x] = mx;
  s[3][threadIdx.x] = fro;
  __syncthreads();
  for (int st = 128; st > 0; st >>= 1) {
    if (threadIdx.x < st) {
      s[0][threadIdx.x] += s[0][threadIdx.x + st];
      s[1][threadIdx.x] += s[1][threadIdx.x + st];
      s[2][threadIdx.x] = fmax(s[2][threadIdx.x], s[2][threadIdx.x + st]);
      s[3][threadIdx.x] += s[3][threadIdx.x + st];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    atomicAdd(&acc[0], s[0][0]);
    atomicAdd(&acc[1], s[1][0]);
    atomic_max_nonneg(&acc[2], s[2][0]);
    atomicAdd(&acc[3], s[3][0]);
  }
}

template <typename T, typename U>
__global__ void __launch_bounds__(256) k_compare(const T* __restrict__ ar, const T* __restrict__ ai,
                                                 const U* __restrict__ br, const U* __restrict__ bi, uint64_t N,
                                                 double* acc) {
  double mx = 0, fro = 0;
  for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < N; v += (uint64_t)gridDim.x * blockDim.x) {
    const double dr = (double)ar[v] - (double)br[v], di = (double)ai[v] - (double)bi[v];
    const double d2 = dr * dr + di * di;
    fro += d2;
    mx = fmax(mx, d2);
  }
  __shared__ double s[2][256];
  s[0][threadIdx.x] = mx;
  s[1][threadIdx.x] = fro;
  __syncthreads();
  for (int st = 128; st > 0; st >>= 1) {
    if (threadIdx.x < st) {
      s[0][threadIdx.x] = fmax(s[0][threadIdx.x], s[0][threadIdx.x + st]);
      s[1][threadIdx.x] += s[1][threadIdx.x + st];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    atomic_max_nonneg(&acc[0], s[0][0]);
    atomicAdd(&acc[1], s[1][0]);
  }
}

cudaError_t launch_compare(const void* ar, const void* ai, const void* br, const void* bi, bool a_fp32, bool b_fp32,
                           uint64_t N, double* d_acc, int sms, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(d_acc, 0, 2 * sizeof(double), s);
  if (e != cudaSuccess) return e;
  const unsigned grid = (unsigned)(sms * 4);
  if (a_fp32 && b_fp32)
    k_compare<float, float><<<grid, 256, 0, s>>>((const float*)ar, (const float*)ai, (const float*)br, (const float*)bi, N, d_acc);
  else if (a_fp32)
    k_compare<float, double><<<grid, 256, 0, s>>>((const float*)ar, (const float*)ai, (const double*)br, (const double*)bi, N, d_acc);
  else if (b_fp32)
    k_compare<double, float><<<grid, 256, 0, s>>>((const double*)ar, (const double*)ai, (const float*)br, (const float*)bi, N, d_acc);
  else
    k_compare<double, double><<<grid, 256, 0, s>>>((const double*)ar, (const double*)ai, (const double*)br, (const double*)bi, N, d_acc);
  return cudaGetLastError();
}

cudaError_t launch_pure_metrics(const void* re, const void* im, bool fp32, const double* psi_re, const double* psi_im,
                                int n, double* d_acc, int sms, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(d_acc, 0, 4 * sizeof(double), s);
  if (e != cudaSuccess) return e;
  const unsigned grid = (unsigned)(sms * 4);
  if (fp32)
    k_pure_metrics<float><<<grid, 256, 0, s>>>((const float*)re, (const float*)im, psi_re, psi_im, n, d_acc);
  else
    k_pure_metrics<double><<<grid, 256, 0, s>>>((const double*)re, (const double*)im, psi_re, psi_im, n, d_acc);
  return cudaGetLastError();
}

namespace {
std::mutex g_noalloc_mu;
double* g_noalloc_addr[256] = {};  // device address of the scratch, per device ordinal
}  // namespace

// Once per device, with that device current: look up the scratch's device
// address.  Later calls on the device reuse it (for the life of the process:
// a device reset in between would leave the cached address stale, which the
// header tells callers not to do).
static cudaError_t noalloc_scratch(double** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 256) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_noalloc_addr[dev] = static_cast<double*>(p);
  }
  *out = g_noalloc_addr[dev];
  return cudaSuccess;
}

cudaError_t pure_metrics_noalloc(const void* re, const void* im, bool fp32, const double* psi_re, const double* psi_im,
                                 int n, int sms, cudaStream_t s, double out[4]) {
  if (n < 1 || n > kNoAllocMaxQubits) return cudaErrorInvalidValue;
  double* scratch = nullptr;
  cudaError_t e = noalloc_scratch(&scratch);
  if (e != cudaSuccess) return e;
  const size_t dim = (size_t)1 << n;
  double* d_pr = scratch;
  double* d_pi = scratch + kNoAllocMaxDim;
  double* d_acc = scratch + 2 * kNoAllocMaxDim;
  e = cudaMemcpyAsync(d_pr, psi_re, dim * sizeof(double), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_pi, psi_im, dim * sizeof(double), cudaMemcpyHostToDevice, s);
  // launch_pure_metrics zeroes the accumulators before the kernel
  if (e == cudaSuccess) e = launch_pure_metrics(re, im, fp32, d_pr, d_pi, n, d_acc, sms, s);
  double acc[4] = {0, 0, 0, 0};
  if (e == cudaSuccess) e = cudaMemcpyAsync(acc, d_acc, 4 * sizeof(double), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return e;
  out[0] = acc[0];
  out[1] = acc[1];
  out[2] = std::sqrt(acc[2]);
  out[3] = std::sqrt(acc[3]);
  return cudaSuccess;
}

}  // namespace dmg
