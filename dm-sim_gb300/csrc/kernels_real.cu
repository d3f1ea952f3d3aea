// kernels_real.cu -- the 1- and 2-qubit DENSE / SPARSE pass kernels for real
// operators (U and V with vanishing imaginary parts): two multiply-adds per
// complex term instead of four.  Most single-qubit dense gates of the
// reference's decompositions are real (H, RY and the U3(theta, 0, 0) parts of
// the controlled gates), so the plain path runs these for most of its dense
// passes.  A separate translation unit so that the build compiles it in
// parallel with kernels.cu.
#include "pass_kernel.cuh"

namespace dmg {

template <typename T, int K>
static cudaError_t launch_real_k(const LaunchArgs& a, cudaStream_t s) {
  if (a.cls == CLS_DENSE) return launch_one<T, K, CLS_DENSE_REAL>(a, s);
  if (a.cls == CLS_SPARSE) return launch_one<T, K, CLS_SPARSE_REAL>(a, s);
  return cudaErrorInvalidValue;
}

template <typename T>
static cudaError_t launch_real_t(const LaunchArgs& a, cudaStream_t s) {
  if (a.K == 1) return launch_real_k<T, 1>(a, s);
  if (a.K == 2) return launch_real_k<T, 2>(a, s);
  return cudaErrorInvalidValue;
}

cudaError_t launch_pass_real(const LaunchArgs& a, cudaStream_t s) {
  if (a.arith == AR_DF64) return launch_real_t<df64>(a, s);
  return a.fp32 ? launch_real_t<float>(a, s) : launch_real_t<double>(a, s);
}

}  // namespace dmg
