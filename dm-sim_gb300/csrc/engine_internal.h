// engine_internal.h -- per-pass bookkeeping shared inside the engine.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/dmsim_gb300.h"
#include "plan.h"

namespace dmg {

struct PassInfo {
  int K, cls;
  bool transpose;       // the in-place conjugate transpose (reference-order plans)
  int conv;             // 1: FP64 -> double-float before a fused run, 2: back after it
  bool renorm;          // complex64: FP64 trace + Hermitian renormalisation
  size_t desc_off;      // byte offset of the descriptor in the device blob
  int tile_entries;
  unsigned grid;
  double bytes;         // algorithmic bytes moved (reads + writes)
  int nbasic;
  bool tc;              // runs on the tensor cores (tensor.cu)
  bool real;            // real operator (kernels_real.cu for K <= 2)
  bool direct1;         // 1-qubit pass on the register kernel (kernels_k1.cu)
  int q0;               // first target qubit
  PassFeatures feat;
  cudaEvent_t ev0, ev1; // per-pass timing (record mode)
};

// Passes that apply no gates (K = 0) report these class codes.
constexpr int kRecConvert = 16, kRecTranspose = 17, kRecRenorm = 18;

struct PassRecord {
  PassFeatures feat;
  double ms;
  double bytes;
  unsigned grid;
};

// For the batched sweep (batch.cpp): enqueue |0..0><0..0| and every pass of
// s's uploaded plan on stream st (e.g. inside another stream's capture), and
// read-and-clear s's device error flag (set by an expired bounded wait).
cudaError_t sim_enqueue(dmsim_handle s, cudaStream_t st, std::string& err);
cudaError_t sim_take_error(dmsim_handle s, int* flag);
// algorithmic bytes of s's uploaded plan (reads + writes of every pass)
double sim_plan_bytes(dmsim_handle s);

}  // namespace dmg
