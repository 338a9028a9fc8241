// Robust window statistics for float64 inputs (the kernels of robust.cuh,
// instantiated apart from the float32 ones so the two compile in parallel).
#include "robust.cuh"

namespace ndf {

cudaError_t launch_robust_f64(const Plan& p, const double* in, double* out, cudaStream_t s) {
  return launch_robust_t<double>(p, in, out, s);
}

}  // namespace ndf
