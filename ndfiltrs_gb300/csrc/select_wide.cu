// Tile network kernels of widths 80 to 128 (float32 keys), compiled apart
// from select.cu so the two translation units build in parallel.
#include "select_launch.cuh"

namespace ndf {

cudaError_t launch_network_wide(const Plan& p, const void* in, void* out, cudaStream_t s) {
  using namespace netlaunch;
  const float* fin = (const float*)in;
  float* fout = (float*)out;
  switch (p.network) {
    case 80:
      return dispatch_network_mode<float, 80>(p, fin, fout, s);
    case 96:
      return dispatch_network_mode<float, 96>(p, fin, fout, s);
    case 112:
      return dispatch_network_mode<float, 112>(p, fin, fout, s);
    case 128:
      return dispatch_network_mode<float, 128>(p, fin, fout, s);
    default:
      return cudaErrorInvalidValue;
  }
}

}  // namespace ndf
