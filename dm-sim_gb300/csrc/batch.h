// batch.h -- device-side records of the batched sweep (batch.cu / batch.cpp).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace dmg {

constexpr int kBatchMaxQubits = 16;

// One (circuit, pass): its descriptor, its circuit's state and its tiles.
struct BatchRange {
  uint64_t desc_off;      // byte offset of the pass descriptor in the blob
  uint64_t state_off;     // entry offset of the circuit's rho in the batch arrays
  uint64_t item_begin;    // first work item of this range (layer-major order)
  uint32_t ntiles;
  int32_t K, cls;
  int32_t dep;            // range of the previous pass of the same circuit, -1 if none
  uint32_t dep_expected;  // its tile count
  int32_t pad;
};

struct BatchCircuit {
  uint64_t state_off, diag_off, zz_off;
  int32_t n, pad;
};

struct BatchLaunch {
  double *re, *im;
  uint64_t total_entries;
  const unsigned char* blob;
  const BatchRange* ranges;
  int nranges;
  unsigned long long nitems;
  const BatchCircuit* circs;
  int ncirc;
  unsigned long long* next;
  unsigned* done;
  int* err;
  double *diag, *zz;
  unsigned grid;
  unsigned spin_limit;
  bool df64_arith;  // the states hold double-float pairs (fused batches)
};

size_t batch_smem_bytes();
int batch_blocks_per_sm(bool df64_arith);
// memset states, rho_c = |0><0|, reset the queue, the work-queue kernel, the epilogue
// (circs: the circuits held in the batch arrays; nothing when ncirc is 0)
cudaError_t launch_batch(const BatchLaunch& a, cudaStream_t s);
// diag[0..2^n) and zz[0..n-1) of one FP64 state held elsewhere (one block)
cudaError_t launch_circuit_epilogue(const double* re, int n, double* diag, double* zz, cudaStream_t s);

}  // namespace dmg
