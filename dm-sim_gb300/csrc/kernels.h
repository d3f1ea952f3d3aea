// kernels.h -- host-side entry points of the pass kernels (kernels.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace dmg {

// Arithmetic of a pass: the state's element type.
enum Arith : int { AR_FP64 = 0, AR_FP32 = 1, AR_DF64 = 2 };

struct LaunchArgs {
  void* re;            // device real parts (double, float, or double-float pairs)
  void* im;            // device imaginary parts
  const void* desc;    // device PassDesc<K>
  int K, cls;
  bool fp32;           // complex64 state
  int arith;           // Arith
  unsigned grid;       // blocks
  int tile_entries;    // G * 4^K
  bool real;           // DENSE/SPARSE pass whose U and V are real (pass.h kPassRealOperator)
  bool tc;             // tensor-core pass, K = 3, 4: desc is a TcDesc<K> (double-float or FP32 state) or,
                       // for an FP64 state, a TcDesc64<K>
  int* err;            // device flag set to 1 when a bounded wait of a tensor pass runs out
  bool direct1;        // 1-qubit pass run by the register kernel (kernels_k1.cu)
  int q0, n;           // its qubit and the state's qubit count
};

// Launch one pass on stream s.
cudaError_t launch_pass(const LaunchArgs& a, cudaStream_t s);
// Resident blocks per SM of the kernel instance for (K, cls, arithmetic).
int pass_blocks_per_sm(int K, int cls, int arith);
// 1-qubit MOVE / SIGNED / PHASE / DENSE passes without shared memory (kernels_k1.cu).
bool direct1_class(int cls);
cudaError_t launch_pass1(const LaunchArgs& a, cudaStream_t s);
// Real-operator instances of the 1- and 2-qubit DENSE/SPARSE kernels (kernels_real.cu).
cudaError_t launch_pass_real(const LaunchArgs& a, cudaStream_t s);
// Tensor-core passes (tensor.cu): launch, and resident blocks per SM.
cudaError_t launch_pass_tc(const LaunchArgs& a, cudaStream_t s);
int tc_blocks_per_sm(int K, int arith);
// Tensor-core passes on a complex64 (FP32) state (tensor32.cu): two
// persistent 512-thread blocks per SM.
cudaError_t launch_pass_tc32(const LaunchArgs& a, cudaStream_t s);
// FP64-width tensor-core passes on an FP64 state (tensor64.cu): one
// persistent 1024-thread block per SM.
cudaError_t launch_pass_tc64(const LaunchArgs& a, cudaStream_t s);
// In place: FP64 entries <-> double-float pairs (the fused path's working format)
cudaError_t launch_to_df64(void* re, void* im, uint64_t N, unsigned grid, cudaStream_t s);
cudaError_t launch_from_df64(void* re, void* im, uint64_t N, unsigned grid, cudaStream_t s);
// In place A'[x*2^n + y] = conj(A[y*2^n + x]) (the reference's adjoint stage)
cudaError_t launch_conj_transpose(void* re, void* im, int n, bool fp32, unsigned grid, cudaStream_t s);
// rho <- (rho + rho^dagger) / (2 trace), trace summed in FP64 into d_trace
cudaError_t launch_renormalise(void* re, void* im, int n, bool fp32, double* d_trace, unsigned grid, cudaStream_t s);
// rho <- |0..0><0..0|
cudaError_t launch_set_zero_state(void* re, void* im, uint64_t N, bool fp32, cudaStream_t s);
// d_out[i] = Re rho[i][i] (FP64 whatever the state precision)
cudaError_t launch_get_diag(const void* re, uint64_t dim, bool fp32, double* d_out, cudaStream_t s);

}  // namespace dmg
