// peaks.cu -- throughput probes of the execution units the pass kernels are
// designed around: FP64 FMA, the FP64 tensor-core MMA (mma.sync m8n8k4),
// FP32 FMA, the 32-bit integer ALU (lop3, add, funnel shift, byte permute,
// multiply-add), and the conversions between FP64, FP32 and 64-bit integers.
//
// Each probe runs a fixed number of independent dependency chains per thread
// (8 chains, enough to cover the latency of every unit probed) on 8 blocks of
// 256 threads per SM, and reports operations per second: PTX instructions of
// the probed kind, or FLOPs for the MMA.  The chains end in a global store so
// the work cannot be removed.  No probe waits on anything: each launch ends
// after its fixed loop.
#include <cuda_runtime.h>
#include <stdint.h>

#include "dmsim_gb300.h"

namespace dmg {
namespace {

constexpr int kChains = 8;
constexpr int kIters = 2048;
constexpr int kProbeThreads = 256;

template <int WHICH>
__global__ void __launch_bounds__(kProbeThreads) k_probe(uint64_t* sink, uint32_t seed) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  uint64_t out = 0;
  if constexpr (WHICH == DMSIM_PROBE_FP64_FMA) {
    double a[kChains];
    const double b = 1.0 + 1e-9 * (seed & 7), c = 1e-12 * (t & 15);
#pragma unroll
    for (int i = 0; i < kChains; i++) a[i] = 1.0 + i * 1e-3;
    for (int it = 0; it < kIters; it++) {
#pragma unroll
      for (int i = 0; i < kChains; i++) asm volatile("fma.rn.f64 %0, %0, %1, %2;" : "+d"(a[i]) : "d"(b), "d"(c));
    }
#pragma unroll
    for (int i = 0; i < kChains; i++) out += (uint64_t)__double_as_longlong(a[i]);
  } else if constexpr (WHICH == DMSIM_PROBE_FP32_FMA) {
    float a[kChains];
    const float b = 1.0f + 1e-6f * (seed & 7), c = 1e-9f * (t & 15);
#pragma unroll
    for (int i = 0; i < kChains; i++) a[i] = 1.0f + i * 1e-3f;
    for (int it = 0; it < kIters; it++) {
#pragma unroll
      for (int i = 0; i < kChains; i++) asm volatile("fma.rn.f32 %0, %0, %1, %2;" : "+f"(a[i]) : "f"(b), "f"(c));
    }
#pragma unroll
    for (int i = 0; i < kChains; i++) out += __float_as_uint(a[i]);
  } else if constexpr (WHICH == DMSIM_PROBE_DMMA) {
    // D (8x8) += A (8x4) * B (4x8) per warp: 512 FLOPs per instruction
    double acc[kChains][2];
    const double av = 1.0 + 1e-9 * (t & 7), bv = 1.0 - 1e-9 * (seed & 7);
#pragma unroll
    for (int i = 0; i < kChains; i++) acc[i][0] = acc[i][1] = 0.0;
    for (int it = 0; it < kIters / 4; it++) {
#pragma unroll
      for (int i = 0; i < kChains; i++)
        asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
                     : "+d"(acc[i][0]), "+d"(acc[i][1])
                     : "d"(av), "d"(bv));
    }
#pragma unroll
    for (int i = 0; i < kChains; i++) out += (uint64_t)__double_as_longlong(acc[i][0] + acc[i][1]);
  } else if constexpr (WHICH == DMSIM_PROBE_INT_LOP3) {
    uint32_t a[kChains];
    const uint32_t b = seed * 2654435761u, c = t * 40503u;
#pragma unroll
    for (int i = 0; i < kChains; i++) a[i] = t + i;
    for (int it = 0; it < kIters; it++) {
#pragma unroll
      for (int i = 0; i < kChains; i++)
        asm volatile("lop3.b32 %0, %0, %1, %2, 0x96;" : "+r"(a[i]) : "r"(b), "r"(c));
    }
#pragma unroll
    for (int i = 0; i < kChains; i++) out += a[i];
  } else if constexpr (WHICH == DMSIM_PROBE_INT_ADD) {
    uint32_t a[kChains];
    const uint32_t b = seed * 2654435761u;
#pragma unroll
    for (int i = 0; i < kChains; i++) a[i] = t + i;
    for (int it = 0; it < kIters; it++) {
#pragma unroll
      for (int i = 0; i < kChains; i++) asm volatile("add.u32 %0, %0, %1;" : "+r"(a[i]) : "r"(b));
    }
#pragma unroll
    for (int i = 0; i < kChains; i++) out += a[i];
  } else if constexpr (WHICH == DMSIM_PROBE_INT_SHF) {
    uint32_t a[kChains];
    const uint32_t b = seed * 2654435761u, s = (seed & 15) + 1;
#pragma unroll
    for (int i = 0; i < kChains; i++) a[i] = t + i;
    for (int it = 0; it < kIters; it++) {
#pragma unroll
      for (int i = 0; i < kChains; i++) asm volatile("shf.r.clamp.b32 %0, %0, %1, %2;" : "+r"(a[i]) : "r"(b), "r"(s));
    }
#pragma unroll
    for (int i = 0; i < kChains; i++) out += a[i];
  } else if constexpr (WHICH == DMSIM_PROBE_INT_PRMT) {
    uint32_t a[kChains];
    const uint32_t b = seed * 2654435761u;
#pragma unroll
    for (int i = 0; i < kChains; i++) a[i] = t + i;
    for (int it = 0; it < kIters; it++) {
#pragma unroll
      for (int i = 0; i < kChains; i++) asm volatile("prmt.b32 %0, %0, %1, 0x6521;" : "+r"(a[i]) : "r"(b));
    }
#pragma unroll
    for (int i = 0; i < kChains; i++) out += a[i];
  } else if constexpr (WHICH == DMSIM_PROBE_INT_MAD) {
    uint32_t a[kChains];
    const uint32_t b = seed * 2654435761u | 1u, c = t;
#pragma unroll
    for (int i = 0; i < kChains; i++) a[i] = t + i;
    for (int it = 0; it < kIters; it++) {
#pragma unroll
      for (int i = 0; i < kChains; i++) asm volatile("mad.lo.u32 %0, %0, %1, %2;" : "+r"(a[i]) : "r"(b), "r"(c));
    }
#pragma unroll
    for (int i = 0; i < kChains; i++) out += a[i];
  } else if constexpr (WHICH == DMSIM_PROBE_CVT_S64_F64) {
    // int64 -> FP64 and back through the bits: one conversion per step, the
    // rest of the chain is a single integer xor
    uint64_t a[kChains];
#pragma unroll
    for (int i = 0; i < kChains; i++) a[i] = ((uint64_t)t << 20) + i + seed;
    for (int it = 0; it < kIters; it++) {
#pragma unroll
      for (int i = 0; i < kChains; i++) {
        double d;
        asm volatile("cvt.rn.f64.s64 %0, %1;" : "=d"(d) : "l"(a[i]));
        a[i] = (uint64_t)__double_as_longlong(d) >> 12;
      }
    }
#pragma unroll
    for (int i = 0; i < kChains; i++) out += a[i];
  } else if constexpr (WHICH == DMSIM_PROBE_CVT_F32_F64) {
    float a[kChains];
#pragma unroll
    for (int i = 0; i < kChains; i++) a[i] = 1.0f + i + (t & 7);
    for (int it = 0; it < kIters; it++) {
#pragma unroll
      for (int i = 0; i < kChains; i++) {
        double d;
        asm volatile("cvt.f64.f32 %0, %1;" : "=d"(d) : "f"(a[i]));
        asm volatile("cvt.rn.f32.f64 %0, %1;" : "=f"(a[i]) : "d"(d));
      }
    }
#pragma unroll
    for (int i = 0; i < kChains; i++) out += __float_as_uint(a[i]);
  } else if constexpr (WHICH == DMSIM_PROBE_CVT_F32_S32) {
    float a[kChains];
#pragma unroll
    for (int i = 0; i < kChains; i++) a[i] = 1.0f + i + (t & 7);
    for (int it = 0; it < kIters; it++) {
#pragma unroll
      for (int i = 0; i < kChains; i++) {
        int32_t k;
        asm volatile("cvt.rni.s32.f32 %0, %1;" : "=r"(k) : "f"(a[i]));
        asm volatile("cvt.rn.f32.s32 %0, %1;" : "=f"(a[i]) : "r"(k));
      }
    }
#pragma unroll
    for (int i = 0; i < kChains; i++) out += __float_as_uint(a[i]);
  } else if constexpr (WHICH == DMSIM_PROBE_MIX_FADD_LOP3) {
    // one FP32 add and one lop3 per chain step: can the two pipes overlap
    float f[kChains];
    uint32_t u[kChains];
    const uint32_t b = seed * 2654435761u, c = t * 40503u;
    const float fb = 1e-7f * (seed & 7);
#pragma unroll
    for (int i = 0; i < kChains; i++) {
      f[i] = 1.0f + i;
      u[i] = t + i;
    }
    for (int it = 0; it < kIters; it++) {
#pragma unroll
      for (int i = 0; i < kChains; i++) {
        asm volatile("add.rn.f32 %0, %0, %1;" : "+f"(f[i]) : "f"(fb));
        asm volatile("lop3.b32 %0, %0, %1, %2, 0x96;" : "+r"(u[i]) : "r"(b), "r"(c));
      }
    }
#pragma unroll
    for (int i = 0; i < kChains; i++) out += __float_as_uint(f[i]) + u[i];
  }
  sink[t] = out;
}

// operations counted per chain step, per thread (DMMA: FLOPs per warp / 32)
template <int WHICH>
constexpr double ops_per_step() {
  if (WHICH == DMSIM_PROBE_DMMA) return 512.0 / 32.0 / 4.0;  // one MMA every 4 steps (kIters / 4 iterations)
  if (WHICH == DMSIM_PROBE_CVT_F32_F64 || WHICH == DMSIM_PROBE_CVT_F32_S32 || WHICH == DMSIM_PROBE_MIX_FADD_LOP3)
    return 2.0;
  return 1.0;
}

template <int WHICH>
cudaError_t run_probe(int sms, uint64_t* sink, double* ops_per_s) {
  const unsigned grid = (unsigned)sms * 8u;
  cudaEvent_t e0, e1;
  cudaError_t e = cudaEventCreate(&e0);
  if (e != cudaSuccess) return e;
  e = cudaEventCreate(&e1);
  if (e != cudaSuccess) {
    cudaEventDestroy(e0);
    return e;
  }
  k_probe<WHICH><<<grid, kProbeThreads>>>(sink, 1u);  // warm-up
  cudaEventRecord(e0);
  constexpr int kReps = 5;
  for (int r = 0; r < kReps; r++) k_probe<WHICH><<<grid, kProbeThreads>>>(sink, (uint32_t)r + 2u);
  cudaEventRecord(e1);
  e = cudaEventSynchronize(e1);
  float ms = 0.f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
  if (e == cudaSuccess) e = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (e != cudaSuccess) return e;
  const double ops = (double)kReps * grid * kProbeThreads * kIters * kChains * ops_per_step<WHICH>();
  *ops_per_s = ops / (ms * 1e-3);
  return cudaSuccess;
}

}  // namespace
}  // namespace dmg

extern "C" int dmsim_probe_rate(int which, double* ops_per_s) {
  using namespace dmg;
  if (!ops_per_s || which < 0 || which >= DMSIM_PROBE_COUNT) return DMSIM_ERR_ARG;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return DMSIM_ERR_CUDA;
  uint64_t* sink = nullptr;
  if (cudaMalloc(&sink, (size_t)sms * 8 * kProbeThreads * sizeof(uint64_t)) != cudaSuccess) return DMSIM_ERR_OOM;
  cudaError_t e = cudaErrorInvalidValue;
  switch (which) {
    case DMSIM_PROBE_FP64_FMA: e = run_probe<DMSIM_PROBE_FP64_FMA>(sms, sink, ops_per_s); break;
    case DMSIM_PROBE_FP32_FMA: e = run_probe<DMSIM_PROBE_FP32_FMA>(sms, sink, ops_per_s); break;
    case DMSIM_PROBE_DMMA: e = run_probe<DMSIM_PROBE_DMMA>(sms, sink, ops_per_s); break;
    case DMSIM_PROBE_INT_LOP3: e = run_probe<DMSIM_PROBE_INT_LOP3>(sms, sink, ops_per_s); break;
    case DMSIM_PROBE_INT_ADD: e = run_probe<DMSIM_PROBE_INT_ADD>(sms, sink, ops_per_s); break;
    case DMSIM_PROBE_INT_SHF: e = run_probe<DMSIM_PROBE_INT_SHF>(sms, sink, ops_per_s); break;
    case DMSIM_PROBE_INT_PRMT: e = run_probe<DMSIM_PROBE_INT_PRMT>(sms, sink, ops_per_s); break;
    case DMSIM_PROBE_INT_MAD: e = run_probe<DMSIM_PROBE_INT_MAD>(sms, sink, ops_per_s); break;
    case DMSIM_PROBE_CVT_S64_F64: e = run_probe<DMSIM_PROBE_CVT_S64_F64>(sms, sink, ops_per_s); break;
    case DMSIM_PROBE_CVT_F32_F64: e = run_probe<DMSIM_PROBE_CVT_F32_F64>(sms, sink, ops_per_s); break;
    case DMSIM_PROBE_CVT_F32_S32: e = run_probe<DMSIM_PROBE_CVT_F32_S32>(sms, sink, ops_per_s); break;
    case DMSIM_PROBE_MIX_FADD_LOP3: e = run_probe<DMSIM_PROBE_MIX_FADD_LOP3>(sms, sink, ops_per_s); break;
    default: break;
  }
  cudaFree(sink);
  return e == cudaSuccess ? DMSIM_OK : DMSIM_ERR_CUDA;
}
