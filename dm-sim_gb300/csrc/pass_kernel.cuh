// pass_kernel.cuh -- the per-pass kernel template and its launcher, shared by
// kernels.cu (complex operators) and kernels_real.cu (real operators).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#include "kernels.h"
#include "pass.h"
#include "pass_device.cuh"

namespace dmg {

// One pass over the whole state: the block stages the pass's tables once,
// then grid-strides over the tiles.
template <typename T, int K, int CLS>
__global__ void __launch_bounds__(kThreads) k_pass(T* __restrict__ re, T* __restrict__ im,
                                                   const PassDesc<K>* __restrict__ dp) {
  constexpr int D = 1 << K;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const PassHeader& h = dp->h;
  const int tile = (1 << h.g) * D * D;
  T* sre = reinterpret_cast<T*>(smem_raw);
  T* sim = sre + tile;
  auto& tb = *reinterpret_cast<PassTables<T, K, CLS>*>(smem_raw + ((2 * (size_t)tile * sizeof(T) + 15) & ~(size_t)15));
  load_tables<T, K, CLS>(dp, tb);
  __syncthreads();
  // Full-size tiles of narrow passes (2^(K-1) entry pairs per thread): the
  // next tile's loads go out before the current tile is transformed.
  constexpr int P = K >= 1 ? 1 << (K - 1) : 1;
  if constexpr ((K >= 1 && K <= 2) || (std::is_same<T, float>::value && base_class(CLS) == CLS_DENSE)) {
    if (tile == 2 * kThreads * P) {
      uint64_t t = blockIdx.x;
      if (t >= h.ntiles) return;
      TileRegs<T, P> x;
      const int lf = free_offset(h);
      uint64_t base = tile_base(h, t);
      load_regs<T, K, CLS, P>(re, im, h, tb, base, x);
      for (; t < h.ntiles; t += gridDim.x) {
        regs_to_smem<T, K, CLS, P>(h, tb, x, sre, sim);
        __syncthreads();
        const uint64_t tn = t + gridDim.x;
        const uint64_t base_n = tn < h.ntiles ? tile_base(h, tn) : 0;
        if (tn < h.ntiles) load_regs<T, K, CLS, P>(re, im, h, tb, base_n, x);
        tile_body<T, K, CLS>(re, im, h, tb, base, sre, sim, lf);
        base = base_n;
      }
      return;
    }
  }
  for (uint64_t t = blockIdx.x; t < h.ntiles; t += gridDim.x) run_tile<T, K, CLS>(re, im, h, tb, t, sre, sim);
}

// ---------------------------------------------------------------- launchers
// Dynamic shared memory for the largest tile, and the largest shared-memory
// carveout so that the resident-block count the occupancy query reports is
// the one the launches get.
template <typename T, int K, int CLS>
inline cudaError_t configure_pass() {
  constexpr int D = 1 << K;
  cudaError_t e = cudaFuncSetAttribute(k_pass<T, K, CLS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)pass_smem_bytes<T, K, CLS>(kThreads * D));
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_pass<T, K, CLS>, cudaFuncAttributePreferredSharedMemoryCarveout,
                             (int)cudaSharedmemCarveoutMaxShared);
  return e;
}

template <typename T, int K, int CLS>
inline cudaError_t launch_one(const LaunchArgs& a, cudaStream_t s) {
  constexpr int D = 1 << K;
  const size_t smem = pass_smem_bytes<T, K, CLS>(a.tile_entries);
  static int configured = 0;  // per instance; attribute set once per process
  if (!configured) {
    cudaError_t e = configure_pass<T, K, CLS>();
    if (e != cudaSuccess) return e;
    configured = 1;
  }
  k_pass<T, K, CLS><<<a.grid, kThreads, smem, s>>>(static_cast<T*>(a.re), static_cast<T*>(a.im),
                                                   static_cast<const PassDesc<K>*>(a.desc));
  return cudaGetLastError();
}

}  // namespace dmg
