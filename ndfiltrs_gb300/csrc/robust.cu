// Robust window statistics for float32 inputs, the plan hooks and the
// dispatch (float64 inputs instantiate in robust_f64.cu).
#include "robust.cuh"

namespace ndf {

cudaError_t launch_robust_f64(const Plan& p, const double* in, double* out, cudaStream_t s);

// Windows beyond 256 samples take per-thread slices of a scratch buffer of
// at most 1 GiB (three float64 arrays per thread): the thread count is the
// largest multiple of the block size within that, capped at 16 blocks per
// SM. Returns false when the scratch cannot be allocated.
bool robust_configure(Plan& p) {
  p.robust_threads = 0;
  if (p.r.count <= 256) return true;
  const size_t per_thread = (size_t)p.r.count * 3 * sizeof(double);
  long long threads = (long long)((1ull << 30) / per_thread) / kRThreads * kRThreads;
  threads = std::min(threads, (long long)std::max(1, p.sm_count) * 16 * kRThreads);
  if (threads < kRThreads) threads = kRThreads;
  p.robust_threads = threads;
  p.scratch_bytes = (size_t)threads * per_thread;
  return cudaMalloc(&p.d_scratch, p.scratch_bytes) == cudaSuccess;
}

cudaError_t launch_robust(const Plan& p, const void* in, void* out, cudaStream_t s) {
  if (p.dtype == 0) return launch_robust_t<float>(p, (const float*)in, (float*)out, s);
  return launch_robust_f64(p, (const double*)in, (double*)out, s);
}

}  // namespace ndf
