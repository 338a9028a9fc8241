// Window moments: mean, variance and standard deviation.
//
// Two arithmetic paths:
//  * NDF_MOMENTS_FP64 restates the reference's float64 algorithms operation
//    for operation: the streaming Neumaier mean in tap order with infinity
//    flags and the scaled overflow retry (src/filter_nd.rs:142-158,
//    src/mean.rs:28-113), and dispersion_valid (src/dispersion.rs:5-61).
//    Results are bit-identical to the reference.
//  * NDF_MOMENTS_FP32C (default) sums exactly: per tile, every sample's
//    deviation from the tile's pivot becomes an exact integer in units of
//    the tile's lowest set bit (fixed_moments.cuh); each window sums X and
//    X^2 in 64- / 128-bit integers, the mean is the exact n P + S1 divided
//    once, the variance's numerator n S2 - S1^2 is exact in 192 bits, and
//    FP64 runs only for the conversion, the division, the scaling and the
//    square root (float32 outputs finish in float-float on the FP32 pipe).
//    Results are the exact moments rounded to within about an ulp. Tiles
//    whose span does not fit the integers take the FP64 path.
#include "moments.cuh"

namespace ndf {
namespace {
using namespace mom;
constexpr int kThreads = 256;

template <typename T, int PREC>
__global__ void __launch_bounds__(kThreads)
    tile_moments_kernel(const T* __restrict__ in, T* __restrict__ out,
                        const __grid_constant__ TileArgs a, const int32_t* __restrict__ taps,
                        const __grid_constant__ CUtensorMap tmap) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  tile_moments_body<T, PREC>(in, out, a, blockIdx.x, smem_raw, taps, &tmap);
}

// Generic N-D gather (rank > 3 or supports beyond shared memory): the FP64
// path, taps mapped per axis as in Window::visit (src/window.rs:232-294).
template <typename T>
__global__ void __launch_bounds__(kThreads)
    generic_moments_kernel(const T* __restrict__ in, T* __restrict__ out,
                           const __grid_constant__ GenericArgs a,
                           const long long* __restrict__ taps) {
  const int rank = a.rank;
  const long long* flat = taps + (long long)a.r.count * rank;
  const double cval = a.r.cval;
  for (long long o = blockIdx.x * (long long)blockDim.x + threadIdx.x; o < a.n_out;
       o += (long long)gridDim.x * blockDim.x) {
    long long coord[kMaxGenericRank];
    long long rem = o;
    bool interior = true;
    for (int d = 0; d < rank; ++d) {
      coord[d] = rem / a.stride[d];
      rem -= coord[d] * a.stride[d];
      interior = interior && coord[d] + a.low[d] >= 0 && coord[d] + a.high[d] < a.shape[d];
    }
    auto fetch = [&](int i) -> double {
      if (interior) return (double)__ldg(in + o + flat[i]);
      const long long* tap = taps + (long long)i * rank;
      long long src = 0;
      for (int d = 0; d < rank; ++d) {
        long long m;
        if (!map_index(coord[d] + tap[d], a.shape[d], a.mode[d], &m)) return cval;
        src += m * a.stride[d];
      }
      return (double)__ldg(in + src);
    };
    out[o] = canonical(from_f64<T>(moments_exact(fetch, a.r)));
  }
}

template <typename T, int PREC>
cudaError_t launch_tile_t(const Plan& p, const T* in, T* out, cudaStream_t s) {
  auto kernel = tile_moments_kernel<T, PREC>;
  cudaError_t e =
      allow_max_smem((const void*)kernel);
  if (e != cudaSuccess) return e;
  TileArgs args = p.tile;
  CUtensorMap map{};
  size_t smem = p.smem_bytes;
  tma_prepare(p, p.tile.t, in, &map, &args, &smem);
  kernel<<<(unsigned)p.tile.t.tiles, kThreads, smem, s>>>(in, out, args, p.d_tile_taps, map);
  return cudaGetLastError();
}

}  // namespace

size_t tile_moments_smem(const Plan& p, const Tile& t) {
  size_t elem = p.dtype == 0 ? 4 : 8;
  size_t support = (size_t)p.tile.g.kd * t.SH * t.SW;
  // Remap tables | staged values | (FP32C: deviations and count increments,
  // 8 bytes each per sample) | tap offsets, laid out as tile_moments_body
  // does.
  size_t staged = (support * elem + 15) / 16 * 16;
  if (p.r.moments == 0) staged += support * 16;
  return (size_t)(t.SW + t.SH + p.tile.g.kd) * 8 + staged + (size_t)p.r.count * sizeof(int32_t);
}

cudaError_t launch_tile_moments(const Plan& p, const void* in, void* out, cudaStream_t s) {
  const bool fp64 = p.r.moments == 1;
  if (p.dtype == 0)
    return fp64 ? launch_tile_t<float, 1>(p, (const float*)in, (float*)out, s)
                : launch_tile_t<float, 0>(p, (const float*)in, (float*)out, s);
  return fp64 ? launch_tile_t<double, 1>(p, (const double*)in, (double*)out, s)
              : launch_tile_t<double, 0>(p, (const double*)in, (double*)out, s);
}

cudaError_t launch_generic_moments(const Plan& p, const void* in, void* out, cudaStream_t s) {
  long long blocks = (p.n_out + kThreads - 1) / kThreads;
  long long cap = (long long)p.sm_count * 8;
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  if (p.dtype == 0)
    generic_moments_kernel<float><<<(unsigned)blocks, kThreads, 0, s>>>(
        (const float*)in, (float*)out, p.generic, p.d_gen_taps);
  else
    generic_moments_kernel<double><<<(unsigned)blocks, kThreads, 0, s>>>(
        (const double*)in, (double*)out, p.generic, p.d_gen_taps);
  return cudaGetLastError();
}

}  // namespace ndf
