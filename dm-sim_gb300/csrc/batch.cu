// batch.cu -- many small circuits (uneven qubit counts) in one persistent
// work-queue kernel, the batched parameter-sweep path.
//
// Work items are tiles of passes, ordered layer-major: every circuit's pass 0
// tiles, then every circuit's pass 1 tiles, and so on.  A block takes the next
// item with one atomic, waits (bounded) until the previous pass of the same
// circuit has all of its tiles done, runs the tile with the same device code as
// the per-pass kernel, and counts it done.  Items are taken in increasing order,
// so every item a block waits for was taken earlier by a running block: the
// queue cannot deadlock whatever the grid size.  A wait that runs out sets an
// error flag and the item is skipped, so a fault can never hang the GPU; the
// host reports DMSIM_ERR_TIMEOUT.
#include <cuda_runtime.h>
#include <stdint.h>

#include "batch.h"
#include "pass_device.cuh"

namespace dmg {

namespace {

template <typename T, int K, int CLS>
__device__ void batch_tile(T* re, T* im, const unsigned char* __restrict__ blob, const BatchRange& R, int range,
                           uint64_t t, unsigned char* smem, int* s_loaded) {
  constexpr int D = 1 << K;
  const PassDesc<K>* dp = reinterpret_cast<const PassDesc<K>*>(blob + R.desc_off);
  const int tile = (1 << dp->h.g) * D * D;
  T* sre = reinterpret_cast<T*>(smem);
  T* sim = sre + tile;
  auto& tb = *reinterpret_cast<PassTables<T, K, CLS>*>(smem + ((2 * (size_t)tile * sizeof(T) + 15) & ~(size_t)15));
  if (*s_loaded != range) {  // uniform: every thread read s_loaded after the same barrier
    load_tables<T, K, CLS>(dp, tb);
    __syncthreads();
    if (threadIdx.x == 0) *s_loaded = range;
  }
  run_tile<T, K, CLS>(re + R.state_off, im + R.state_off, dp->h, tb, t, sre, sim);
}

template <typename T, int K>
__device__ void batch_dispatch_k(int cls, T* re, T* im, const unsigned char* blob, const BatchRange& R, int range,
                                 uint64_t t, unsigned char* smem, int* s_loaded) {
  switch (cls) {
    case CLS_MOVE: batch_tile<T, K, CLS_MOVE>(re, im, blob, R, range, t, smem, s_loaded); break;
    case CLS_SIGNED: batch_tile<T, K, CLS_SIGNED>(re, im, blob, R, range, t, smem, s_loaded); break;
    case CLS_PHASE: batch_tile<T, K, CLS_PHASE>(re, im, blob, R, range, t, smem, s_loaded); break;
    case CLS_DENSE: batch_tile<T, K, CLS_DENSE>(re, im, blob, R, range, t, smem, s_loaded); break;
    case CLS_SPARSE: batch_tile<T, K, CLS_SPARSE>(re, im, blob, R, range, t, smem, s_loaded); break;
    default:
      if (K == 1) batch_tile<T, 1, CLS_RLIN>(re, im, blob, R, range, t, smem, s_loaded);
      break;
  }
}

}  // namespace

template <typename T>
__global__ void __launch_bounds__(kThreads) k_batch(T* re, T* im, const unsigned char* __restrict__ blob,
                                                    const BatchRange* __restrict__ ranges, int nranges,
                                                    unsigned long long nitems, unsigned long long* next,
                                                    unsigned* done, int* err, unsigned spin_limit) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ unsigned long long s_item;
  __shared__ int s_range, s_skip, s_loaded;
  if (threadIdx.x == 0) s_loaded = -1;
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) {
      s_item = atomicAdd(next, 1ull);
      s_skip = 0;
      if (s_item < nitems) {
        // the range holding the item: largest r with item_begin <= item
        int lo = 0, hi = nranges - 1;
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (ranges[mid].item_begin <= s_item) lo = mid;
          else hi = mid - 1;
        }
        s_range = lo;
        const int dep = ranges[lo].dep;
        if (dep >= 0) {
          const unsigned want = ranges[lo].dep_expected;
          volatile unsigned* vd = done;
          unsigned spins = 0;
          while (vd[dep] < want) {
            __nanosleep(128);
            if (++spins > spin_limit) {
              atomicExch(err, 1);
              s_skip = 1;
              break;
            }
          }
          __threadfence();
        }
      }
    }
    __syncthreads();
    if (s_item >= nitems) break;
    const int r = s_range;
    const BatchRange R = ranges[r];
    if (!s_skip) {
      const uint64_t t = s_item - R.item_begin;
      switch (R.K) {
        case 1: batch_dispatch_k<T, 1>(R.cls, re, im, blob, R, r, t, smem_raw, &s_loaded); break;
        case 2: batch_dispatch_k<T, 2>(R.cls, re, im, blob, R, r, t, smem_raw, &s_loaded); break;
        case 3: batch_dispatch_k<T, 3>(R.cls, re, im, blob, R, r, t, smem_raw, &s_loaded); break;
        default: batch_dispatch_k<T, 4>(R.cls, re, im, blob, R, r, t, smem_raw, &s_loaded); break;
      }
    }
    // publish the tile: every writer fences, then one count per tile
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) atomicAdd(&done[r], 1u);
  }
}

template <typename T>
__global__ void k_batch_init(T* re, const BatchCircuit* __restrict__ circs, int ncirc) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < ncirc) re[circs[c].state_off] = T(1);
}

__device__ __forceinline__ double to_double(double x) { return x; }
__device__ __forceinline__ double to_double(df64 x) { return (double)x.hi + (double)x.lo; }

// Per circuit (one block each): the diagonal of rho and <Z_i Z_{i+1}>.
template <typename T>
__global__ void __launch_bounds__(256) k_batch_epilogue(const T* __restrict__ re,
                                                        const BatchCircuit* __restrict__ circs, double* __restrict__ diag,
                                                        double* __restrict__ zz) {
  const BatchCircuit C = circs[blockIdx.x];
  const int n = C.n;
  const uint64_t dim = 1ull << n;
  const T* A = re + C.state_off;
  double acc[kBatchMaxQubits];
#pragma unroll
  for (int i = 0; i < kBatchMaxQubits; i++) acc[i] = 0;
  for (uint64_t r = threadIdx.x; r < dim; r += blockDim.x) {
    const double d = to_double(A[r * dim + r]);
    diag[C.diag_off + r] = d;
#pragma unroll
    for (int i = 0; i < kBatchMaxQubits - 1; i++)
      if (i < n - 1) acc[i] += (((r >> i) ^ (r >> (i + 1))) & 1) ? -d : d;
  }
  __shared__ double s[256];
  for (int i = 0; i < n - 1; i++) {
    s[threadIdx.x] = acc[i];
    __syncthreads();
    for (int st = 128; st > 0; st >>= 1) {
      if (threadIdx.x < st) s[threadIdx.x] += s[threadIdx.x + st];
      __syncthreads();
    }
    if (threadIdx.x == 0) zz[C.zz_off + i] = s[0];
    __syncthreads();
  }
}

// One circuit held outside the batch arrays (a wide circuit, run by the
// engine's own pass kernels): its diagonal and <Z_i Z_{i+1}>, one block.
__global__ void __launch_bounds__(256) k_circuit_epilogue(const double* __restrict__ re, int n, double* __restrict__ diag,
                                                          double* __restrict__ zz) {
  const uint64_t dim = 1ull << n;
  double acc[kBatchMaxQubits];
#pragma unroll
  for (int i = 0; i < kBatchMaxQubits; i++) acc[i] = 0;
  for (uint64_t r = threadIdx.x; r < dim; r += blockDim.x) {
    const double d = re[r * dim + r];
    diag[r] = d;
#pragma unroll
    for (int i = 0; i < kBatchMaxQubits - 1; i++)
      if (i < n - 1) acc[i] += (((r >> i) ^ (r >> (i + 1))) & 1) ? -d : d;
  }
  __shared__ double s[256];
  for (int i = 0; i < n - 1; i++) {
    s[threadIdx.x] = acc[i];
    __syncthreads();
    for (int st = 128; st > 0; st >>= 1) {
      if (threadIdx.x < st) s[threadIdx.x] += s[threadIdx.x + st];
      __syncthreads();
    }
    if (threadIdx.x == 0) zz[i] = s[0];
    __syncthreads();
  }
}

cudaError_t launch_circuit_epilogue(const double* re, int n, double* diag, double* zz, cudaStream_t s) {
  k_circuit_epilogue<<<1, 256, 0, s>>>(re, n, diag, zz);
  return cudaGetLastError();
}

template <typename T, int K>
static size_t smem_k() {
  size_t m = 0;
  m = m > pass_smem_bytes<T, K, CLS_MOVE>(kThreads << K) ? m : pass_smem_bytes<T, K, CLS_MOVE>(kThreads << K);
  m = m > pass_smem_bytes<T, K, CLS_SIGNED>(kThreads << K) ? m : pass_smem_bytes<T, K, CLS_SIGNED>(kThreads << K);
  m = m > pass_smem_bytes<T, K, CLS_PHASE>(kThreads << K) ? m : pass_smem_bytes<T, K, CLS_PHASE>(kThreads << K);
  m = m > pass_smem_bytes<T, K, CLS_DENSE>(kThreads << K) ? m : pass_smem_bytes<T, K, CLS_DENSE>(kThreads << K);
  m = m > pass_smem_bytes<T, K, CLS_SPARSE>(kThreads << K) ? m : pass_smem_bytes<T, K, CLS_SPARSE>(kThreads << K);
  return m;
}

size_t batch_smem_bytes() {
  size_t m = pass_smem_bytes<double, 1, CLS_RLIN>(kThreads << 1);
  const size_t k[4] = {smem_k<double, 1>(), smem_k<double, 2>(), smem_k<double, 3>(), smem_k<double, 4>()};
  for (size_t v : k) m = m > v ? m : v;
  return m;
}

template <typename T>
static int blocks_t() {
  const size_t smem = batch_smem_bytes();
  cudaFuncSetAttribute(k_batch<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  cudaFuncSetAttribute(k_batch<T>, cudaFuncAttributePreferredSharedMemoryCarveout, (int)cudaSharedmemCarveoutMaxShared);
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_batch<T>, kThreads, smem) != cudaSuccess) return 1;
  return nb > 0 ? nb : 1;
}

int batch_blocks_per_sm(bool df64_arith) { return df64_arith ? blocks_t<df64>() : blocks_t<double>(); }

template <typename T>
static cudaError_t launch_t(const BatchLaunch& a, cudaStream_t s) {
  const size_t smem = batch_smem_bytes();
  cudaError_t e = cudaFuncSetAttribute(k_batch<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_batch<T>, cudaFuncAttributePreferredSharedMemoryCarveout,
                             (int)cudaSharedmemCarveoutMaxShared);
  if (e != cudaSuccess) return e;
  // all-zero bytes are 0 in both FP64 and double-float
  if (a.ncirc == 0) return cudaSuccess;  // every circuit is a wide one
  e = cudaMemsetAsync(a.re, 0, a.total_entries * sizeof(double), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(a.im, 0, a.total_entries * sizeof(double), s);
  if (e != cudaSuccess) return e;
  T* re = reinterpret_cast<T*>(a.re);
  T* im = reinterpret_cast<T*>(a.im);
  k_batch_init<T><<<(a.ncirc + 255) / 256, 256, 0, s>>>(re, a.circs, a.ncirc);
  e = cudaMemsetAsync(a.next, 0, sizeof(unsigned long long), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(a.done, 0, (size_t)a.nranges * sizeof(unsigned), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(a.err, 0, sizeof(int), s);
  if (e != cudaSuccess) return e;
  k_batch<T><<<a.grid, kThreads, smem, s>>>(re, im, a.blob, a.ranges, a.nranges, a.nitems, a.next, a.done, a.err,
                                            a.spin_limit);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_batch_epilogue<T><<<a.ncirc, 256, 0, s>>>(re, a.circs, a.diag, a.zz);
  return cudaGetLastError();
}

cudaError_t launch_batch(const BatchLaunch& a, cudaStream_t s) {
  return a.df64_arith ? launch_t<df64>(a, s) : launch_t<double>(a, s);
}

}  // namespace dmg
