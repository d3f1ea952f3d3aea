// metrics.h -- device comparison of rho with a pure state (metrics.cu).
#pragma once
#include <cuda_runtime.h>

namespace dmg {
// d_acc[0] = <psi|rho|psi>, d_acc[1] = trace, d_acc[2] = max |rho - psi psi^+|^2,
// d_acc[3] = ||rho - psi psi^+||_F^2 (the caller takes square roots).
cudaError_t launch_pure_metrics(const void* re, const void* im, bool fp32, const double* psi_re, const double* psi_im,
                                int n, double* d_acc, int sms, cudaStream_t s);
// d_acc[0] = max |A - B|^2, d_acc[1] = ||A - B||_F^2 over two states of N entries.
cudaError_t launch_compare(const void* ar, const void* ai, const void* br, const void* bi, bool a_fp32, bool b_fp32,
                           uint64_t N, double* d_acc, int sms, cudaStream_t s);
// The no-allocation variant of the pure-state metrics: psi is staged in a
// file-scope device array instead of a cudaMalloc'd buffer.  States of at most
// kNoAllocMaxQubits qubits (2^16 amplitudes); calls share the array.
constexpr int kNoAllocMaxQubits = 16;
constexpr size_t kNoAllocMaxDim = (size_t)1 << kNoAllocMaxQubits;
// out = {fidelity, trace, max |rho - psi psi^+|, ||rho - psi psi^+||_F};
// cudaErrorInvalidValue when n is beyond the limit.  Synchronises s.
cudaError_t pure_metrics_noalloc(const void* re, const void* im, bool fp32, const double* psi_re, const double* psi_im,
                                 int n, int sms, cudaStream_t s, double out[4]);
}  // namespace dmg
