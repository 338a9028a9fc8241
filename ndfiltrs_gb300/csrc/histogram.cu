// Sliding-window histogram median and rank for rectangular 1-D/2-D windows.
// (Kernel under construction: plans fall back to the tile kernels.)
#include "common.cuh"
#include "plan.h"

namespace ndf {

bool histogram_supported(const Plan&) { return false; }
void histogram_configure(Plan&) {}
size_t histogram_smem(const Plan&) { return 0; }
cudaError_t launch_histogram(const Plan&, const void*, void*, cudaStream_t) {
  return cudaErrorNotSupported;
}

}  // namespace ndf
