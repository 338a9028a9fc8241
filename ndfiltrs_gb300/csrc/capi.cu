// C-ABI of the GB300 windowed-statistics library: plan validation and
// dispatch, host-buffer runs, and the one-shot entry points that replace the
// reference's `_core.window_filter` / `_core.robust_filter`.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <mutex>
#include <new>
#include <string>

#include "../../include/ndfiltrs_gb300.h"
#include "common.cuh"
#include "plan.h"
#include "tma.cuh"
#include "hostpool.h"

struct ndf_plan {
  ndf::Plan p;
};

namespace ndf {

thread_local std::string g_error;

int fail(int code, const std::string& message) {
  g_error = message;
  return code;
}

int cuda_fail(cudaError_t e, const char* what) {
  return fail(NDF_ERR_CUDA, std::string("CUDA error in ") + what + ": " + cudaGetErrorString(e));
}

const char* algo_name(Algo a) {
  switch (a) {
    case Algo::kEmpty:
      return "empty";
    case Algo::kTileNetwork:
      return "tile_network";
    case Algo::kTileBox:
      return "tile_box";
    case Algo::kTileRadix:
      return "tile_radix";
    case Algo::kGenericSelect:
      return "generic_select";
    case Algo::kHistogram:
      return "histogram";
    case Algo::kMomentsTile:
      return "moments_tile";
    case Algo::kMomentsGeneric:
      return "moments_generic";
    case Algo::kBoxcarTile:
      return "boxcar_tile";
    case Algo::kBoxcarDirect:
      return "boxcar_direct";
    case Algo::kBoxcarBand:
      return "boxcar_band";
    case Algo::kExtremaPasses:
      return "extrema_passes";
    case Algo::kRobust:
      return "robust";
    case Algo::kMomentsSlide:
      return "moments_slide";
    case Algo::kTileRank:
      return "rank_network";
    case Algo::kExtremaTile:
      return "extrema_tile";
  }
  return "unknown";
}

cudaError_t allow_max_smem(const void* kernel) {
  static std::mutex lock;
  static std::vector<const void*> done;
  std::lock_guard<std::mutex> guard(lock);
  for (const void* k : done)
    if (k == kernel) return cudaSuccess;
  int dev = 0, optin = 0;
  cudaGetDevice(&dev);
  cudaError_t e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (e != cudaSuccess) return e;
  cudaFuncAttributes attr;
  e = cudaFuncGetAttributes(&attr, kernel);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           optin - (int)attr.sharedSizeBytes);
  if (e == cudaSuccess) done.push_back(kernel);
  return e;
}

namespace {

struct DeviceState {
  std::once_flag once;
  int status = NDF_ERR_NO_DEVICE;
  std::string message;
  int sm_count = 0;
  int smem_optin = 0;
};

DeviceState& device_state() {
  static DeviceState s;
  return s;
}

// Reads the current device's properties once; every compute entry point
// fails with NDF_ERR_NO_DEVICE when no CUDA device can be used.
int ensure_device(int* device, int* sm_count, int* smem_optin) {
  DeviceState& s = device_state();
  std::call_once(s.once, [&] {
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) {
      s.status = NDF_ERR_NO_DEVICE;
      s.message = std::string("no usable CUDA device: ") +
                  (e != cudaSuccess ? cudaGetErrorString(e) : "device count is zero");
      cudaGetLastError();
      return;
    }
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&s.sm_count, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&s.smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    s.status = NDF_OK;
  });
  if (s.status != NDF_OK) return fail(s.status, s.message);
  cudaGetDevice(device);
  *sm_count = s.sm_count;
  *smem_optin = s.smem_optin;
  return NDF_OK;
}

bool checked_mul(unsigned long long a, unsigned long long b, unsigned long long* out) {
  if (a != 0 && b > std::numeric_limits<unsigned long long>::max() / a) return false;
  *out = a * b;
  return true;
}

bool is_selection(int kind) {
  switch (kind) {
    case kMedian:
    case kMedianNetwork:
    case kMedianHistogram:
    case kMin:
    case kMax:
    case kRank:
    case kRankHistogram:
    case kPercentile:
      return true;
    default:
      return false;
  }
}

bool is_moment(int kind) { return kind == kMean || kind == kVar || kind == kStd; }

bool is_robust(int kind) { return kind >= kMad && kind <= kSigmaMode; }

// RobustReduction::validate (src/robust.rs:187-240) for the robust kinds,
// then their parameters as the kernels read them.
int validate_robust(const ndf_filter_desc* d, size_t count, Plan& p) {
  const ndf_robust_params* rp = d->robust;
  if (!rp) return fail(NDF_ERR_INVALID_CONFIGURATION, "missing robust filter parameters");
  const int kind = d->kind;
  const bool clip = kind >= kSigmaMean;
  auto pearson_ok = [&]() { return std::isfinite(rp->pearson) && rp->pearson >= 1.0; };
  if (kind == kMad && (!std::isfinite(rp->parameter) || rp->parameter < 0.0))
    return fail(NDF_ERR_INVALID_CONFIGURATION, "MAD scale must be finite and nonnegative");
  if (kind == kMode && !pearson_ok())
    return fail(NDF_ERR_INVALID_CONFIGURATION, "pearson must be finite and at least one");
  if ((kind == kBiweightLocation || kind == kBiweightScale) &&
      (!std::isfinite(rp->parameter) || rp->parameter <= 0.0))
    return fail(NDF_ERR_INVALID_CONFIGURATION, "biweight tuning constant must be finite and positive");
  if (clip) {
    if (!std::isfinite(rp->sigma_lower) || !std::isfinite(rp->sigma_upper) || rp->sigma_lower < 0.0 ||
        rp->sigma_upper < 0.0)
      return fail(NDF_ERR_INVALID_CONFIGURATION, "clipping limits must be finite and nonnegative");
    if (kind == kSigmaMode && !pearson_ok())
      return fail(NDF_ERR_INVALID_CONFIGURATION, "pearson must be finite and at least one");
  }
  const uint64_t min_count = clip || d->omit_nan ? d->min_count : 1;
  if (min_count == 0 || min_count > count)
    return fail(NDF_ERR_INVALID_CONFIGURATION,
                "min_count must be between one and the number of window elements");
  if ((rp->center != 0 && rp->center != 1) || (rp->spread != 0 && rp->spread != 1) || rp->estimator < 0 ||
      rp->estimator > 2)
    return fail(NDF_ERR_INVALID_CONFIGURATION, "unsupported clipping or mode option");
  RobustArgs& a = p.robust;
  a.kind = kind - kPercentile;
  a.parameter = rp->parameter;
  a.lower = rp->sigma_lower;
  a.upper = rp->sigma_upper;
  a.maxiters = rp->maxiters < 0 ? -1 : rp->maxiters;
  a.center = rp->center;
  a.spread = rp->spread;
  a.estimator = rp->estimator;
  a.modify_sample_size = rp->modify_sample_size != 0;
  a.pearson = rp->pearson;
  a.clip_min_count = (long long)min_count;
  return NDF_OK;
}

// Canonical 3-D tile geometry for rank 1-3 arrays.
void setup_tile(Plan& p) {
  int pad = 3 - p.ndim;
  long long shape3[3], size3[3], anchor3[3];
  int mode3[3];
  for (int a = 0; a < 3; ++a) {
    int src = a - pad;
    if (src < 0) {
      shape3[a] = 1;
      size3[a] = 1;
      anchor3[a] = 0;
      mode3[a] = kNearest;
    } else {
      shape3[a] = p.shape[src];
      size3[a] = p.size[src];
      anchor3[a] = p.size[src] / 2 + p.origin[src];
      mode3[a] = p.modes[src];
    }
  }
  Geom3& g = p.tile.g;
  g.D = shape3[0];
  g.H = shape3[1];
  g.W = shape3[2];
  g.kd = (int)size3[0];
  g.kh = (int)size3[1];
  g.kw = (int)size3[2];
  g.az = (int)anchor3[0];
  g.ay = (int)anchor3[1];
  g.ax = (int)anchor3[2];
  g.mz = mode3[0];
  g.my = mode3[1];
  g.mx = mode3[2];
  Tile& t = p.tile.t;
  if (g.H == 1) {
    t.TW = 256;
    t.TH = 1;
  } else {
    t.TW = 32;
    t.TH = 8;
  }
  t.SW = t.TW + g.kw - 1;
  t.SH = t.TH + g.kh - 1;
  t.tiles_x = (g.W + t.TW - 1) / t.TW;
  t.tiles_y = (g.H + t.TH - 1) / t.TH;
  t.tiles = t.tiles_x * t.tiles_y * g.D;
  p.tile.r = p.r;
  // Box positions of the taps in the canonical (z, y, x) box.
  p.box_taps.clear();
  long long volume = (long long)g.kd * g.kh * g.kw;
  for (long long e = 0; e < volume; ++e) {
    if (!p.footprint.empty() && !p.footprint[e]) continue;
    int kx = (int)(e % g.kw);
    int ky = (int)((e / g.kw) % g.kh);
    int kz = (int)(e / ((long long)g.kw * g.kh));
    p.box_taps.push_back(kz);
    p.box_taps.push_back(ky);
    p.box_taps.push_back(kx);
  }
}

int setup_generic(Plan& p) {
  if (p.ndim > kMaxGenericRank)
    return fail(NDF_ERR_UNSUPPORTED, "arrays with more than 32 dimensions are not supported");
  GenericArgs& a = p.generic;
  a.rank = p.ndim;
  a.n_out = p.n_out;
  long long stride = 1;
  for (int d = p.ndim - 1; d >= 0; --d) {
    a.shape[d] = p.shape[d];
    a.stride[d] = stride;
    stride *= p.shape[d];
    a.mode[d] = p.modes[d];
    a.low[d] = std::numeric_limits<long long>::max();
    a.high[d] = std::numeric_limits<long long>::min();
  }
  a.r = p.r;
  std::vector<long long> table(p.taps);
  size_t count = (size_t)p.r.count;
  for (size_t t = 0; t < count; ++t) {
    long long flat = 0;
    for (int d = 0; d < p.ndim; ++d) {
      long long off = p.taps[t * p.ndim + d];
      flat += off * a.stride[d];
      a.low[d] = std::min(a.low[d], off);
      a.high[d] = std::max(a.high[d], off);
    }
    table.push_back(flat);
  }
  cudaError_t e = cudaMalloc(&p.d_gen_taps, table.size() * sizeof(long long));
  if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(taps)");
  e = cudaMemcpy(p.d_gen_taps, table.data(), table.size() * sizeof(long long), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpy(taps)");
  return NDF_OK;
}

int upload_tile_taps(Plan& p) {
  const Tile& t = p.tile.t;
  std::vector<int32_t> offs((size_t)p.r.count);
  for (int i = 0; i < p.r.count; ++i) {
    const int* bt = &p.box_taps[(size_t)i * 3];
    offs[i] = (bt[0] * t.SH + bt[1]) * t.SW + bt[2];
  }
  cudaError_t e = cudaMalloc(&p.d_tile_taps, offs.size() * sizeof(int32_t));
  if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(tile taps)");
  e = cudaMemcpy(p.d_tile_taps, offs.data(), offs.size() * sizeof(int32_t), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpy(tile taps)");
  return NDF_OK;
}

void release(Plan& p) {
  p.strips.reset();
  p.strips_tried = false;
  if (p.d_tile_taps) cudaFree(p.d_tile_taps);
  if (p.d_gen_taps) cudaFree(p.d_gen_taps);
  if (p.d_in) cudaFree(p.d_in);
  if (p.d_out) cudaFree(p.d_out);
  if (p.d_scratch) cudaFree(p.d_scratch);
  if (p.d_status) cudaFree(p.d_status);
  if (p.d_hist_lists) cudaFree(p.d_hist_lists);
  if (p.d_pct) cudaFree(p.d_pct);
  p.d_hist_lists = nullptr;
  p.d_pct = nullptr;
  p.r.pct = nullptr;
  p.d_tile_taps = nullptr;
  p.d_gen_taps = nullptr;
  p.d_in = p.d_out = p.d_scratch = nullptr;
  p.d_status = nullptr;
}

// Validation in the reference's order: Window::new (src/window.rs:44-137),
// FilterConfig::from_window (src/filter_nd.rs:35-51), WindowFilter::new
// (src/plan.rs:260-324), RobustReduction::validate (src/robust.rs:187-240).
int build_plan(const ndf_filter_desc* d, Plan& p) {
  if (!d) return fail(NDF_ERR_INVALID_CONFIGURATION, "missing filter description");
  if (d->dtype != NDF_FLOAT32 && d->dtype != NDF_FLOAT64)
    return fail(NDF_ERR_INVALID_CONFIGURATION, "array dtype must be float32 or float64");
  if (d->ndim <= 0)
    return fail(NDF_ERR_INVALID_CONFIGURATION, "filtering requires at least one dimension");
  if (!d->shape || !d->size || !d->origin || !d->modes)
    return fail(NDF_ERR_INVALID_CONFIGURATION, "missing shape, size, origin or mode");
  p.dtype = d->dtype;
  p.ndim = d->ndim;
  p.shape.assign(d->ndim, 0);
  p.size.assign(d->ndim, 0);
  p.origin.assign(d->ndim, 0);
  p.modes.assign(d->ndim, 0);
  for (int a = 0; a < d->ndim; ++a) {
    if (d->shape[a] > (uint64_t)std::numeric_limits<long long>::max() ||
        d->size[a] > (uint64_t)std::numeric_limits<int32_t>::max())
      return fail(NDF_ERR_OVERFLOW, "shape or index arithmetic overflowed");
    p.shape[a] = (long long)d->shape[a];
    p.size[a] = (long long)d->size[a];
    p.origin[a] = d->origin[a];
    p.modes[a] = d->modes[a];
    if (d->modes[a] < 0 || d->modes[a] > 4)
      return fail(NDF_ERR_INVALID_CONFIGURATION, "unsupported boundary mode");
  }
  for (int a = 0; a < d->ndim; ++a)
    if (p.size[a] == 0) return fail(NDF_ERR_INVALID_CONFIGURATION, "window sizes must be positive");
  unsigned long long volume = 1;
  for (int a = 0; a < d->ndim; ++a)
    if (!checked_mul(volume, (unsigned long long)p.size[a], &volume))
      return fail(NDF_ERR_OVERFLOW, "shape or index arithmetic overflowed");
  for (int a = 0; a < d->ndim; ++a) {
    long long length = p.size[a];
    if (p.origin[a] < -(length / 2) || p.origin[a] > (length - 1) / 2)
      return fail(NDF_ERR_INVALID_CONFIGURATION,
                  "origin must satisfy -(size // 2) <= origin <= (size - 1) // 2");
  }
  unsigned long long n_out = 1;
  for (int a = 0; a < d->ndim; ++a)
    if (!checked_mul(n_out, (unsigned long long)p.shape[a], &n_out) ||
        n_out > (unsigned long long)std::numeric_limits<long long>::max())
      return fail(NDF_ERR_OVERFLOW, "shape or index arithmetic overflowed");
  p.n_out = (long long)n_out;
  if (volume > (1ull << 31)) return fail(NDF_ERR_MEMORY, "unable to allocate filtering workspace");
  const int kind = d->kind;
  // RollingMean plans reject footprints before anything else about them
  // (src/plan.rs:280-285).
  if (kind == kMeanRolling && d->footprint)
    return fail(NDF_ERR_INVALID_CONFIGURATION, "rolling means require rectangular size, not footprint");
  size_t count = 0;
  if (d->footprint) {
    p.footprint.assign(d->footprint, d->footprint + volume);
    for (auto v : p.footprint) count += v != 0;
  } else {
    count = (size_t)volume;
  }
  if (count == 0)
    return fail(NDF_ERR_INVALID_CONFIGURATION, "footprint must select at least one element");
  if (!is_selection(kind) && !is_moment(kind) && kind != kMeanRolling && !is_robust(kind))
    return fail(NDF_ERR_INVALID_CONFIGURATION, "unsupported window filter kind");
  Reduce& r = p.r;
  r.kind = kind;
  r.omit = d->omit_nan != 0;
  r.drop_inf = r.omit && d->ignore_inf != 0;
  r.count = (int)count;
  r.min_count = r.omit ? (long long)d->min_count : 1;
  r.param = (long long)std::min<uint64_t>(d->parameter, (uint64_t)std::numeric_limits<long long>::max());
  r.q = d->percentile;
  r.q_fraction = d->percentile / 100.0;
  r.q_is_max = d->percentile == 100.0;
  r.pct = nullptr;
  r.cval = d->dtype == NDF_FLOAT32 ? (double)(float)d->cval : d->cval;
  r.moments = d->moments == NDF_MOMENTS_FP64 ? 1 : 0;
  if (is_robust(kind)) {
    int rc = validate_robust(d, count, p);
    if (rc != NDF_OK) return rc;
    if (kind >= kSigmaMean) {
      // Clipping always drops NaN and infinite samples (src/robust.rs:260-263).
      r.omit = 1;
      r.drop_inf = 1;
    }
    r.min_count = p.robust.clip_min_count;
  } else if (kind == kPercentile) {
    if (!std::isfinite(r.q) || r.q < 0.0 || r.q > 100.0)
      return fail(NDF_ERR_INVALID_CONFIGURATION,
                  "percentile must be finite and between zero and 100");
    if (r.omit && (d->min_count == 0 || d->min_count > count))
      return fail(NDF_ERR_INVALID_CONFIGURATION,
                  "min_count must be between one and the number of window elements");
  } else if (r.omit && (d->min_count == 0 || d->min_count > count)) {
    return fail(NDF_ERR_INVALID_CONFIGURATION,
                "min_count must be between 1 and the number of window elements");
  }
  const bool hist_kind = kind == kMedianHistogram || kind == kRankHistogram;
  if (hist_kind && !p.footprint.empty())
    return fail(NDF_ERR_INVALID_CONFIGURATION,
                "histogram reductions require rectangular size, not footprint");
  // Taps in C order over the footprint (src/window.rs:96-125).
  p.taps.clear();
  p.taps.reserve(count * d->ndim);
  std::vector<long long> index(d->ndim, 0);
  for (unsigned long long e = 0; e < volume; ++e) {
    if (p.footprint.empty() || p.footprint[e]) {
      for (int a = 0; a < d->ndim; ++a)
        p.taps.push_back(index[a] - (p.size[a] / 2 + p.origin[a]));
    }
    for (int a = d->ndim - 1; a >= 0; --a) {
      if (++index[a] < p.size[a]) break;
      index[a] = 0;
    }
  }
  return NDF_OK;
}

// The percentile rank split per retained count n = 0..count, in the float64
// arithmetic of src/robust.rs:343-352 (the library's host code is compiled
// without floating-point contraction, so each operation rounds once).
int upload_percentile_table(Plan& p) {
  std::vector<PctEntry> table((size_t)p.r.count + 1);
  for (int n = 1; n <= p.r.count; ++n) {
    const double rank = p.r.q_fraction * (double)(n - 1);
    const double lower = std::floor(rank);
    const double fraction = rank - lower;
    PctEntry& e = table[(size_t)n];
    e.fraction = fraction;
    e.lower = (int)lower;
    const bool low = fraction <= 0.5;
    e.w = low ? fraction : 1.0 - fraction;
    e.flags = (fraction == 0.0 ? kPctFracZero : 0) | (low ? kPctLowSide : 0) |
              (fraction == 1.0 ? kPctFracOne : 0);
  }
  cudaError_t e = cudaMalloc(&p.d_pct, table.size() * sizeof(PctEntry));
  if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(percentile table)");
  e = cudaMemcpy(p.d_pct, table.data(), table.size() * sizeof(PctEntry), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpy(percentile table)");
  p.r.pct = p.d_pct;
  return NDF_OK;
}

// Output tile of the one-thread-per-output tile kernels.
void set_tile(Plan& p, int tw, int th) {
  const Geom3& g = p.tile.g;
  Tile& t = p.tile.t;
  t.TW = tw;
  t.TH = th;
  t.SW = t.TW + g.kw - 1;
  t.SH = t.TH + g.kh - 1;
  t.tiles_x = (g.W + t.TW - 1) / t.TW;
  t.tiles_y = (g.H + t.TH - 1) / t.TH;
  t.tiles = t.tiles_x * t.tiles_y * g.D;
}

// Kernel candidates of a tileable plan whose shared memory fits, in the
// default preference order (the first is used unless the autotuner knows
// better). Every candidate gives bit-identical order statistics; the
// moments candidates differ only in the output tile.
std::vector<Candidate> plan_candidates_impl(Plan& p, int smem_limit) {
  std::vector<Candidate> out;
  const Geom3& g = p.tile.g;
  const bool line = g.H == 1;
  const std::vector<std::pair<int, int>> tiles =
      line ? std::vector<std::pair<int, int>>{{256, 1}}
           : std::vector<std::pair<int, int>>{{32, 8}, {16, 16}, {64, 4}};
  auto fits_tile = [&](int tw, int th, bool moments) {
    Tile t = p.tile.t;
    t.TW = tw;
    t.TH = th;
    t.SW = tw + g.kw - 1;
    t.SH = th + g.kh - 1;
    return (moments ? tile_moments_smem(p, t) : tile_select_smem(p, t)) <= (size_t)smem_limit;
  };
  if (p.r.kind == kMeanRolling) {
    // Exact rolling means: the band kernel (its cost does not grow with the
    // window) and the tiled kernel; the direct kernel when neither fits.
    Plan probe = p;
    if (boxcar_band_configure(probe, smem_limit)) out.push_back({Algo::kBoxcarBand, 0, 0});
    probe = p;
    if (boxcar_configure(probe, smem_limit)) out.push_back({Algo::kBoxcarTile, 0, 0});
    return out;
  }
  if (is_moment(p.r.kind)) {
    // FP32C boxes: sliding exact sums first; the FP64 mode keeps the
    // reference's per-window arithmetic.
    if (p.r.moments == 0) {
      Plan probe = p;
      if (moments_slide_configure(probe, smem_limit)) out.push_back({Algo::kMomentsSlide, 0, 0});
    }
    for (auto [tw, th] : tiles)
      if (fits_tile(tw, th, true)) out.push_back({Algo::kMomentsTile, tw, th});
    return out;
  }
  const bool hist_kind = p.r.kind == kMedianHistogram || p.r.kind == kRankHistogram;
  const int width = network_width_for(p.dtype, p.r.count);
  bool hist_ok = false;
  if (histogram_supported(p)) {
    Plan probe = p;  // configuration only, no device resources
    histogram_configure(probe);
    hist_ok = histogram_smem(probe) <= (size_t)smem_limit;
  }
  // Rectangular minima / maxima: the separable kernel (its cost does not grow
  // with the window) ahead of everything for windows wider than 5 x 5.
  bool extrema_ok = false, passes_ok = false;
  if (p.r.kind == kMin || p.r.kind == kMax) {
    Plan probe = p;
    extrema_ok = extrema_configure(probe, smem_limit);
    probe = p;
    passes_ok = extrema_passes_configure(probe, smem_limit);
  }
  if (passes_ok && p.r.count > 25) out.push_back({Algo::kExtremaPasses, 0, 0});
  if (extrema_ok && p.r.count > 25) out.push_back({Algo::kExtremaTile, 0, 0});
  // Sliding-histogram tiles besides the cost model's for windows of up to
  // 2,048 samples, whose sparse bitsets favour other tile shapes (measured
  // by the autotuner; every tile gives the same result).
  std::vector<Candidate> hist_tiles;
  if (hist_ok) {
    hist_tiles.push_back({Algo::kHistogram, 0, 0});
    if (p.r.count <= 2048 && g.kd == 1 && !line) {
      Plan probe = p;
      histogram_configure(probe);
      const int dw = probe.hist_block_w, dh = probe.hist_block_h;
      for (auto [tw, th] : {std::pair<int, int>{32, 128}, {128, 64}, {64, 64}}) {
        if (tw == dw && th == dh) continue;
        Plan q = p;
        histogram_configure(q, tw, th);
        if (q.hist_block_w == tw && histogram_smem(q) <= (size_t)smem_limit) hist_tiles.push_back({Algo::kHistogram, tw, th});
      }
    }
  }
  if (hist_ok && (hist_kind || width == 0)) out.insert(out.end(), hist_tiles.begin(), hist_tiles.end());
  if (p.footprint.empty() && g.kd == 1 && !line && box_supported(p.dtype, g.kh, g.kw)) {
    Tile bt = box_tile(g);
    if (tile_select_smem(p, bt) <= (size_t)smem_limit) out.push_back({Algo::kTileBox, bt.TW, bt.TH});
  }
  if (width >= 48 && !line) {
    // Float32 networks of 48 wires or more: rank codes, two windows per thread.
    Plan probe = p;
    if (rank_network_configure(probe, smem_limit))
      out.push_back({Algo::kTileRank, probe.tile.t.TW, probe.tile.t.TH});
  }
  for (auto [tw, th] : tiles) {
    if (!fits_tile(tw, th, false)) continue;
    if (width > 0)
      out.push_back({Algo::kTileNetwork, tw, th});
    else if (!hist_ok)
      out.push_back({Algo::kTileRadix, tw, th});
  }
  if (hist_ok && !(hist_kind || width == 0)) out.insert(out.end(), hist_tiles.begin(), hist_tiles.end());
  if (passes_ok && p.r.count <= 25) out.push_back({Algo::kExtremaPasses, 0, 0});
  if (extrema_ok && p.r.count <= 25) out.push_back({Algo::kExtremaTile, 0, 0});
  if (out.empty() && fits_tile(tiles[0].first, tiles[0].second, false))
    out.push_back({Algo::kTileRadix, tiles[0].first, tiles[0].second});
  return out;
}

int apply_candidate_impl(Plan& p, const Candidate& c, int smem_limit) {
  p.algo = c.algo;
  switch (c.algo) {
    case Algo::kHistogram: {
      histogram_configure(p, c.tw, c.th);
      p.smem_bytes = histogram_smem(p);
      if (p.smem_bytes > (size_t)smem_limit) return fail(NDF_ERR_UNSUPPORTED, "window too large");
      cudaError_t e = histogram_allocate(p);
      if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(NDF_ERR_MEMORY, "unable to allocate filtering workspace");
      }
      return NDF_OK;
    }
    case Algo::kTileBox:
      p.tile.t = box_tile(p.tile.g);
      p.smem_bytes = tile_select_smem(p, p.tile.t);
      return NDF_OK;
    case Algo::kTileNetwork:
      set_tile(p, c.tw, c.th);
      p.smem_bytes = tile_select_smem(p, p.tile.t);
      p.network = network_width_for(p.dtype, p.r.count);
      return NDF_OK;
    case Algo::kTileRank:
      if (!rank_network_configure(p, smem_limit)) return fail(NDF_ERR_UNSUPPORTED, "window too large");
      return NDF_OK;
    case Algo::kTileRadix:
      set_tile(p, c.tw, c.th);
      p.smem_bytes = tile_select_smem(p, p.tile.t);
      return upload_tile_taps(p);
    case Algo::kMomentsTile:
      set_tile(p, c.tw, c.th);
      p.smem_bytes = tile_moments_smem(p, p.tile.t);
      return upload_tile_taps(p);
    case Algo::kMomentsSlide:
      if (!moments_slide_configure(p, smem_limit)) return fail(NDF_ERR_UNSUPPORTED, "window too large");
      return NDF_OK;
    case Algo::kExtremaTile:
      if (!extrema_configure(p, smem_limit)) return fail(NDF_ERR_UNSUPPORTED, "window too large");
      return NDF_OK;
    case Algo::kExtremaPasses: {
      if (!extrema_passes_configure(p, smem_limit)) return fail(NDF_ERR_UNSUPPORTED, "window too large");
      cudaError_t e = cudaMalloc(&p.d_scratch, p.scratch_bytes);
      if (e != cudaSuccess) {
        cudaGetLastError();
        p.d_scratch = nullptr;
        return fail(NDF_ERR_MEMORY, "unable to allocate filtering workspace");
      }
      return NDF_OK;
    }
    case Algo::kBoxcarBand:
    case Algo::kBoxcarTile: {
      // Both finish over-wide spans with the direct kernel's taps.
      if (!p.d_gen_taps) {
        int rc = setup_generic(p);
        if (rc != NDF_OK) return rc;
      }
      const bool band = c.algo == Algo::kBoxcarBand;
      if (!(band ? boxcar_band_configure(p, smem_limit) : boxcar_configure(p, smem_limit)))
        return fail(NDF_ERR_UNSUPPORTED, "window too large");
      p.scratch_bytes = ((size_t)p.tile.t.tiles * (band ? 2 : 1) + 2) * sizeof(unsigned int);
      cudaError_t e = cudaMalloc(&p.d_scratch, p.scratch_bytes);
      if (e != cudaSuccess) {
        cudaGetLastError();
        p.d_scratch = nullptr;
        return fail(NDF_ERR_MEMORY, "unable to allocate filtering workspace");
      }
      return NDF_OK;
    }
    default:
      return fail(NDF_ERR_UNSUPPORTED, "not a tile kernel");
  }
}

int choose_algorithm(Plan& p, int smem_limit) {
  if (p.n_out == 0) {
    p.algo = Algo::kEmpty;
    return NDF_OK;
  }
  if (p.r.kind == kPercentile && !p.r.q_is_max) {
    int rc = upload_percentile_table(p);
    if (rc != NDF_OK) return rc;
  }
  const bool tileable = p.ndim <= 3 && p.r.count <= (1 << 24);
  if (is_robust(p.r.kind)) {
    int rc = setup_generic(p);
    if (rc != NDF_OK) return rc;
    if (!robust_configure(p)) {
      cudaGetLastError();
      p.d_scratch = nullptr;
      return fail(NDF_ERR_MEMORY, "unable to allocate filtering workspace");
    }
    p.algo = Algo::kRobust;
    return NDF_OK;
  }
  if (p.r.kind == kMeanRolling) {
    // Exact rolling mean: the band or tiled kernel when one fits, with the
    // direct kernel for spans too wide for them (or for the whole array).
    int rc = setup_generic(p);
    if (rc != NDF_OK) return rc;
    if (tileable) {
      setup_tile(p);
      std::vector<Candidate> cands = plan_candidates_impl(p, smem_limit);
      if (!cands.empty()) {
        Candidate pick = cands.size() > 1 ? autotune_pick(p, cands, smem_limit) : cands[0];
        return apply_candidate_impl(p, pick, smem_limit);
      }
    }
    p.algo = Algo::kBoxcarDirect;
    return NDF_OK;
  }
  if (tileable) {
    setup_tile(p);
    std::vector<Candidate> cands = plan_candidates_impl(p, smem_limit);
    if (!cands.empty()) {
      Candidate pick = cands[0];
      if (cands.size() > 1) pick = autotune_pick(p, cands, smem_limit);
      return apply_candidate_impl(p, pick, smem_limit);
    }
  }
  if (is_moment(p.r.kind)) {
    p.algo = Algo::kMomentsGeneric;
    return setup_generic(p);
  }
  p.algo = Algo::kGenericSelect;
  return setup_generic(p);
}

int run_plan(const Plan& p, const void* in, void* out, cudaStream_t s) {
  cudaError_t e = cudaSuccess;
  switch (p.algo) {
    case Algo::kEmpty:
      return NDF_OK;
    case Algo::kTileNetwork:
    case Algo::kTileBox:
    case Algo::kTileRadix:
      e = launch_tile_select(p, in, out, s);
      break;
    case Algo::kGenericSelect:
      e = launch_generic_select(p, in, out, s);
      break;
    case Algo::kHistogram:
      e = launch_histogram(p, in, out, s);
      break;
    case Algo::kMomentsTile:
      e = launch_tile_moments(p, in, out, s);
      break;
    case Algo::kMomentsGeneric:
      e = launch_generic_moments(p, in, out, s);
      break;
    case Algo::kBoxcarTile:
    case Algo::kBoxcarBand:
    case Algo::kBoxcarDirect:
      e = launch_boxcar(p, in, out, s);
      break;
    case Algo::kMomentsSlide:
      e = launch_moments_slide(p, in, out, s);
      break;
    case Algo::kTileRank:
      e = launch_rank_network(p, in, out, s);
      break;
    case Algo::kExtremaTile:
    case Algo::kExtremaPasses:
      e = launch_extrema(p, in, out, s);
      break;
    case Algo::kRobust:
      e = launch_robust(p, in, out, s);
      break;
  }
  if (e != cudaSuccess) return cuda_fail(e, algo_name(p.algo));
  return NDF_OK;
}

size_t element_bytes(const Plan& p) { return p.dtype == NDF_FLOAT32 ? 4 : 8; }

// A pageable output that the host has not touched yet faults its pages in
// during the device-to-host copy, one 64 KB page at a time on one thread;
// touching them first on the host thread pool is several times faster.
// Pinned (registered) buffers are resident already.
void prefault_output(void* h_out, size_t bytes) {
  cudaPointerAttributes attr{};
  if (cudaPointerGetAttributes(&attr, h_out) != cudaSuccess) {
    cudaGetLastError();
    return;
  }
  if (attr.type == cudaMemoryTypeUnregistered) prefault_pages(h_out, bytes);
}

// After a synchronization: a device wait that timed out fails the call.
int check_status() {
  return status_take() ? fail(NDF_ERR_TIMEOUT, "a bounded device wait gave up") : NDF_OK;
}

int ensure_buffers(Plan& p) {
  size_t bytes = (size_t)p.n_out * element_bytes(p);
  if (bytes == 0 || (p.d_in && p.buffer_bytes >= bytes)) return NDF_OK;
  if (p.d_in) cudaFree(p.d_in);
  if (p.d_out) cudaFree(p.d_out);
  p.d_in = p.d_out = nullptr;
  cudaError_t e = cudaMalloc(&p.d_in, bytes);
  if (e == cudaSuccess) e = cudaMalloc(&p.d_out, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    if (p.d_in) cudaFree(p.d_in);
    p.d_in = nullptr;
    return fail(NDF_ERR_MEMORY, "unable to allocate filtering workspace");
  }
  p.buffer_bytes = bytes;
  return NDF_OK;
}

int parse_mode(const char* name, int32_t* out) {
  static const char* names[] = {"reflect", "constant", "nearest", "mirror", "wrap"};
  for (int i = 0; i < 5; ++i)
    if (name && std::strcmp(name, names[i]) == 0) {
      *out = i;
      return NDF_OK;
    }
  return fail(NDF_ERR_INVALID_CONFIGURATION, "unsupported boundary mode");
}

int parse_window_kind(const char* kind, int32_t* out) {
  static const struct {
    const char* name;
    int32_t kind;
  } table[] = {{"median", kMedian},         {"median_network", kMedianNetwork},
               {"median_histogram", kMedianHistogram}, {"mean", kMean},
               {"mean_rolling", kMeanRolling}, {"min", kMin},
               {"max", kMax},               {"var", kVar},
               {"std", kStd},               {"rank", kRank},
               {"rank_histogram", kRankHistogram}};
  for (const auto& e : table)
    if (kind && std::strcmp(kind, e.name) == 0) {
      *out = e.kind;
      return NDF_OK;
    }
  return fail(NDF_ERR_INVALID_CONFIGURATION, "unsupported window filter kind");
}

int moments_default() {
  const char* env = std::getenv("NDF_MOMENTS");
  if (env && std::strcmp(env, "fp64") == 0) return NDF_MOMENTS_FP64;
  return NDF_MOMENTS_FP32C;
}

int one_shot(const ndf_filter_desc& d, const void* h_in, void* h_out) {
  ndf_plan* plan = nullptr;
  int rc = ndf_plan_create(&d, &plan);
  if (rc != NDF_OK) return rc;
  rc = ndf_plan_run_host(plan, h_in, h_out, nullptr);
  std::string message = g_error;
  ndf_plan_destroy(plan);
  if (rc != NDF_OK) g_error = message;
  return rc;
}

}  // namespace

// Device check for translation units without plans (mesh.cu).
int device_ready(int* device, int* sm_count, int* smem_optin) { return ensure_device(device, sm_count, smem_optin); }

// Plan construction for the batched path (batch.cu).
int batch_build_plan(const ndf_filter_desc* d, Plan& p, int* smem_limit) {
  int rc = build_plan(d, p);
  if (rc != NDF_OK) return rc;
  if (p.n_out == 0) {
    p.algo = Algo::kEmpty;
    return NDF_OK;
  }
  rc = ensure_device(&p.device, &p.sm_count, smem_limit);
  if (rc != NDF_OK) return rc;
  p.may_tune = true;  // batches measure kernel choices they have not seen
  return choose_algorithm(p, *smem_limit);
}

void batch_release_plan(Plan& p) { release(p); }

// Plan internals used by the autotuner (autotune.cu).
void plan_setup_tile(Plan& p) { setup_tile(p); }
void plan_release(Plan& p) { release(p); }
int plan_run(const Plan& p, const void* in, void* out, cudaStream_t s) { return run_plan(p, in, out, s); }
int plan_apply(Plan& p, const Candidate& c, int smem_limit) { return apply_candidate_impl(p, c, smem_limit); }

// ---------------------------------------------------------------------------
// Host-buffer runs in row bands.
//
// A host-buffer run copies the array in, filters it and copies the result
// out; done in that order the host link idles during the kernel and carries
// one direction at a time. Split along the first axis into overlapping bands
// (each band's input reaches as far as its kept outputs' windows), each band
// filtered by a plan of its own over the band, the uploads of later bands,
// the kernels and the downloads of earlier bands overlap on three streams,
// and both directions of the link run at once. Every kept output's window
// lies inside its band's real rows except at the array's own first and last
// rows, where the band's edge is the array's edge, so boundary modes behave
// as for the whole array. Not used for the wrap mode along the first axis
// (its windows reach the far edge), for float32-compensated moments other
// than the sliding kernel's float32 outputs (elsewhere the last bits depend
// on the tiling), for robust
// windows beyond 256 samples (their per-plan scratch), or for small arrays.
// Bands pay for recomputing their overlaps and for smaller launches, which
// costs more than it saves for kernels slower than the copies (wide
// histograms, the rolling-mean band kernel): a plan times its second
// host-buffer run (whole array) and its third (bands) and keeps the bands
// when they were at least 5% faster.
struct StripSet {
  struct Band {
    Plan plan;
    long long in_row0 = 0, in_rows = 0;    // rows the band's plan filters
    long long out_row0 = 0, out_rows = 0;  // rows it keeps
    long long upload_end = 0;              // rows uploaded before it runs
    size_t out_offset = 0;                 // its outputs in `out` (elements)
  };
  std::vector<Band> bands;
  void* out = nullptr;
  cudaStream_t up = nullptr, down = nullptr;
  std::vector<cudaEvent_t> uploaded, filtered;
  cudaEvent_t start = nullptr, done = nullptr;
  ~StripSet() {
    for (Band& b : bands) release(b.plan);
    if (out) cudaFree(out);
    for (cudaEvent_t e : uploaded) cudaEventDestroy(e);
    for (cudaEvent_t e : filtered) cudaEventDestroy(e);
    if (start) cudaEventDestroy(start);
    if (done) cudaEventDestroy(done);
    if (up) cudaStreamDestroy(up);
    if (down) cudaStreamDestroy(down);
  }
};

constexpr int kMaxBands = 8;
constexpr size_t kBandMinBytes = 16u << 20;

// Bands for `p`, or none (an empty set) when banding does not apply.
int build_strips(Plan& p) {
  p.strips_tried = true;
  if (p.algo == Algo::kEmpty || p.ndim < 1 || p.modes[0] == NDF_MODE_WRAP) return NDF_OK;
  // Float32-compensated moments: only the sliding kernel with float32
  // output, whose exact-integer combine depends on the window's samples
  // alone (not on its tile's pivot or lowest bit), so bands give the whole
  // array's bits; float64 outputs convert the exact numerator word by word,
  // and the footprint kernel is not banded either.
  const bool fp32c = is_moment(p.r.kind) && p.r.moments == 0;
  if (fp32c && !(p.algo == Algo::kMomentsSlide && p.dtype == 0)) return NDF_OK;
  if (p.robust_threads > 0) return NDF_OK;  // per-thread scratch of up to 1 GiB per plan
  const size_t bytes = (size_t)p.n_out * element_bytes(p);
  if (bytes < kBandMinBytes) return NDF_OK;
  long long low = 0, high = 0;  // input rows reached above / below an output
  for (size_t t = 0; t < p.taps.size(); t += (size_t)p.ndim) {
    low = std::min(low, p.taps[t]);
    high = std::max(high, p.taps[t]);
  }
  const long long rows = p.shape[0];
  const long long min_rows = std::max(256ll, 8 * (high - low + 1));
  const long long count = std::min<long long>(kMaxBands, rows / min_rows);
  if (count < 2) return NDF_OK;
  int device = 0, sm_count = 0, smem_limit = 0;
  int rc = ensure_device(&device, &sm_count, &smem_limit);
  if (rc != NDF_OK) return rc;
  auto set = std::make_shared<StripSet>();
  set->bands.resize((size_t)count);
  size_t total = 0;
  long long uploaded = 0;
  for (long long i = 0; i < count; ++i) {
    StripSet::Band& b = set->bands[(size_t)i];
    b.out_row0 = rows * i / count;
    b.out_rows = rows * (i + 1) / count - b.out_row0;
    b.in_row0 = std::max(0ll, b.out_row0 + low);
    const long long end = std::min(rows, b.out_row0 + b.out_rows + high);
    b.in_rows = end - b.in_row0;
    uploaded = std::max(uploaded, end);
    b.upload_end = uploaded;
    // The band's plan: the array's configuration over the band's rows.
    b.plan = p;
    Plan& q = b.plan;
    q.strips.reset();
    q.strips_tried = true;
    q.d_tile_taps = nullptr;
    q.d_gen_taps = nullptr;
    q.d_in = q.d_out = q.d_scratch = nullptr;
    q.buffer_bytes = q.scratch_bytes = 0;
    q.d_status = nullptr;
    q.d_hist_lists = nullptr;
    q.d_pct = nullptr;
    q.r.pct = nullptr;
    q.shape[0] = b.in_rows;
    q.n_out = p.n_out / rows * b.in_rows;
    q.device = device;
    q.sm_count = sm_count;
    rc = choose_algorithm(q, smem_limit);
    if (rc != NDF_OK) return rc;
    if (fp32c && q.algo != Algo::kMomentsSlide) return NDF_OK;
    b.out_offset = total;
    total += (size_t)q.n_out;
  }
  cudaError_t e = cudaMalloc(&set->out, total * element_bytes(p));
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&set->up, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&set->down, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&set->start, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&set->done, cudaEventDisableTiming);
  for (long long i = 0; i < count && e == cudaSuccess; ++i) {
    cudaEvent_t a = nullptr, b = nullptr;
    e = cudaEventCreateWithFlags(&a, cudaEventDisableTiming);
    if (e == cudaSuccess) set->uploaded.push_back(a);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b, cudaEventDisableTiming);
    if (e == cudaSuccess) set->filtered.push_back(b);
  }
  if (e != cudaSuccess) {
    cudaGetLastError();
    return NDF_OK;  // the whole-array path runs instead
  }
  p.strips = std::move(set);
  return NDF_OK;
}

int run_host_strips(Plan& p, const void* h_in, void* h_out, cudaStream_t s) {
  StripSet& set = *p.strips;
  const size_t row_bytes = (size_t)(p.n_out / p.shape[0]) * element_bytes(p);
  const char* src = static_cast<const char*>(h_in);
  char* dst = static_cast<char*>(h_out);
  char* d_in = static_cast<char*>(p.d_in);
  char* d_out = static_cast<char*>(set.out);
  cudaError_t e = cudaEventRecord(set.start, s);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(set.up, set.start, 0);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(set.down, set.start, 0);
  long long uploaded = 0;
  for (size_t i = 0; i < set.bands.size() && e == cudaSuccess; ++i) {
    const StripSet::Band& b = set.bands[i];
    if (b.upload_end > uploaded) {
      e = cudaMemcpyAsync(d_in + uploaded * row_bytes, src + uploaded * row_bytes,
                          (size_t)(b.upload_end - uploaded) * row_bytes, cudaMemcpyHostToDevice, set.up);
      uploaded = b.upload_end;
    }
    if (e == cudaSuccess) e = cudaEventRecord(set.uploaded[i], set.up);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s, set.uploaded[i], 0);
    if (e != cudaSuccess) break;
    const int rc = run_plan(b.plan, d_in + b.in_row0 * row_bytes, d_out + b.out_offset * element_bytes(p), s);
    if (rc != NDF_OK) return rc;
    e = cudaEventRecord(set.filtered[i], s);
  }
  if (e != cudaSuccess) return cuda_fail(e, "band upload");
  prefault_output(h_out, (size_t)p.n_out * element_bytes(p));  // overlaps the uploads and kernels
  for (size_t i = 0; i < set.bands.size() && e == cudaSuccess; ++i) {
    const StripSet::Band& b = set.bands[i];
    e = cudaStreamWaitEvent(set.down, set.filtered[i], 0);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(dst + b.out_row0 * row_bytes,
                          d_out + b.out_offset * element_bytes(p) + (b.out_row0 - b.in_row0) * row_bytes,
                          (size_t)b.out_rows * row_bytes, cudaMemcpyDeviceToHost, set.down);
  }
  if (e == cudaSuccess) e = cudaEventRecord(set.done, set.down);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(s, set.done, 0);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(e, "band download");
  return check_status();
}

}  // namespace ndf

using namespace ndf;

extern "C" {

const char* ndf_last_error(void) { return g_error.c_str(); }

int ndf_device_info(int32_t* sm_count, int32_t* major, int32_t* minor, char* name,
                    size_t name_capacity) {
  int dev, sms, smem;
  int rc = ensure_device(&dev, &sms, &smem);
  if (rc != NDF_OK) return rc;
  cudaDeviceProp prop;
  cudaError_t e = cudaGetDeviceProperties(&prop, dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDeviceProperties");
  if (sm_count) *sm_count = prop.multiProcessorCount;
  if (major) *major = prop.major;
  if (minor) *minor = prop.minor;
  if (name && name_capacity) {
    std::strncpy(name, prop.name, name_capacity - 1);
    name[name_capacity - 1] = 0;
  }
  return NDF_OK;
}

int32_t ndf_get_num_threads(void) { return (int32_t)ndf::host_thread_count(); }

int ndf_plan_create(const ndf_filter_desc* desc, ndf_plan** out) {
  if (!out) return fail(NDF_ERR_INVALID_CONFIGURATION, "missing plan output pointer");
  *out = nullptr;
  ndf_plan* plan = new (std::nothrow) ndf_plan();
  if (!plan) return fail(NDF_ERR_MEMORY, "unable to allocate filtering workspace");
  int rc = build_plan(desc, plan->p);
  if (rc == NDF_OK && plan->p.n_out > 0) {
    int smem_limit = 0;
    rc = ensure_device(&plan->p.device, &plan->p.sm_count, &smem_limit);
    if (rc == NDF_OK) rc = choose_algorithm(plan->p, smem_limit);
  } else if (rc == NDF_OK) {
    plan->p.algo = Algo::kEmpty;
  }
  if (rc != NDF_OK) {
    release(plan->p);
    delete plan;
    return rc;
  }
  *out = plan;
  return NDF_OK;
}

int ndf_plan_destroy(ndf_plan* plan) {
  if (!plan) return NDF_OK;
  release(plan->p);
  delete plan;
  return NDF_OK;
}

const char* ndf_plan_algorithm(const ndf_plan* plan) {
  return plan ? algo_name(plan->p.algo) : "none";
}

int32_t ndf_plan_host_bands(const ndf_plan* plan) {
  return plan && plan->p.strips ? (int32_t)plan->p.strips->bands.size() : 0;
}

int ndf_plan_set_host_bands(ndf_plan* plan, int32_t mode) {
  if (!plan) return fail(NDF_ERR_INVALID_CONFIGURATION, "missing plan");
  if (mode < 0 || mode > 2) return fail(NDF_ERR_INVALID_CONFIGURATION, "band mode must be 0, 1 or 2");
  Plan& p = plan->p;
  p.band_mode = mode;
  p.strips.reset();
  p.strips_tried = false;
  p.strips_decided = false;
  p.host_runs = 0;
  return NDF_OK;
}

int ndf_plan_run(ndf_plan* plan, const void* d_in, void* d_out, void* stream) {
  if (!plan) return fail(NDF_ERR_INVALID_CONFIGURATION, "missing plan");
  if (plan->p.n_out == 0) return NDF_OK;
  if (!d_in || !d_out) return fail(NDF_ERR_LENGTH_MISMATCH, "missing input or output buffer");
  if (d_in == d_out) return fail(NDF_ERR_INVALID_CONFIGURATION, "input and output must not overlap");
  return run_plan(plan->p, d_in, d_out, (cudaStream_t)stream);
}

int ndf_plan_upload(ndf_plan* plan, const void* h_in) {
  if (!plan) return fail(NDF_ERR_INVALID_CONFIGURATION, "missing plan");
  Plan& p = plan->p;
  if (p.n_out == 0) return NDF_OK;
  int rc = ensure_buffers(p);
  if (rc != NDF_OK) return rc;
  cudaError_t e = cudaMemcpy(p.d_in, h_in, (size_t)p.n_out * element_bytes(p), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpy(input)");
  return NDF_OK;
}

int ndf_plan_compute_download(ndf_plan* plan, void* h_out) {
  if (!plan) return fail(NDF_ERR_INVALID_CONFIGURATION, "missing plan");
  Plan& p = plan->p;
  if (p.n_out == 0) return NDF_OK;
  if (!p.d_in) return fail(NDF_ERR_INVALID_CONFIGURATION, "no input was uploaded");
  int rc = run_plan(p, p.d_in, p.d_out, nullptr);
  if (rc != NDF_OK) return rc;
  const size_t bytes = (size_t)p.n_out * element_bytes(p);
  prefault_output(h_out, bytes);  // overlaps the kernel
  cudaError_t e = cudaMemcpy(h_out, p.d_out, bytes, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpy(output)");
  return check_status();
}

int ndf_plan_run_host(ndf_plan* plan, const void* h_in, void* h_out, void* stream) {
  if (!plan) return fail(NDF_ERR_INVALID_CONFIGURATION, "missing plan");
  Plan& p = plan->p;
  if (p.n_out == 0) return NDF_OK;
  int rc = ensure_buffers(p);
  if (rc != NDF_OK) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  ++p.host_runs;
  if (!p.strips_tried && p.band_mode != 0 && (p.host_runs >= 3 || p.band_mode == 2)) {
    rc = build_strips(p);
    if (rc != NDF_OK) return rc;
  }
  const auto begin = std::chrono::steady_clock::now();
  auto elapsed_ms = [&] {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - begin).count();
  };
  if (p.strips) {
    rc = run_host_strips(p, h_in, h_out, s);
    if (rc == NDF_OK && !p.strips_decided && p.band_mode == 1) {
      p.strips_decided = true;
      // Kept when at least 5% faster than the whole-array run (a single
      // timing each; kernel-bound plans gain little and lose to noise).
      if (elapsed_ms() >= 0.95 * p.whole_ms) p.strips.reset();
    }
    return rc;
  }
  size_t bytes = (size_t)p.n_out * element_bytes(p);
  cudaError_t e = cudaMemcpyAsync(p.d_in, h_in, bytes, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync(input)");
  rc = run_plan(p, p.d_in, p.d_out, s);
  if (rc != NDF_OK) return rc;
  prefault_output(h_out, bytes);  // overlaps the upload and the kernel
  e = cudaMemcpyAsync(h_out, p.d_out, bytes, cudaMemcpyDeviceToHost, s);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync(output)");
  e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamSynchronize");
  if (p.host_runs == 2) p.whole_ms = elapsed_ms();
  return check_status();
}

int ndf_window_filter(const void* h_in, void* h_out, int32_t dtype, int32_t ndim,
                      const uint64_t* shape, const char* kind, const uint64_t* size,
                      const uint8_t* footprint, const int64_t* origin,
                      const char* const* modes, double cval, int32_t omit_nan,
                      int32_t ignore_inf, uint64_t min_count, uint64_t parameter) {
  int32_t k;
  int rc = parse_window_kind(kind, &k);
  if (rc != NDF_OK) return rc;
  if (ndim <= 0) return fail(NDF_ERR_INVALID_CONFIGURATION, "filtering requires at least one dimension");
  std::vector<int32_t> m(ndim);
  for (int a = 0; a < ndim; ++a) {
    rc = parse_mode(modes ? modes[a] : nullptr, &m[a]);
    if (rc != NDF_OK) return rc;
  }
  ndf_filter_desc d{};
  d.dtype = dtype;
  d.ndim = ndim;
  d.shape = shape;
  d.size = size;
  d.footprint = footprint;
  d.origin = origin;
  d.modes = m.data();
  d.cval = cval;
  d.kind = k;
  d.omit_nan = omit_nan;
  d.ignore_inf = ignore_inf;
  d.min_count = min_count;
  d.parameter = parameter;
  d.percentile = 50.0;
  d.moments = moments_default();
  return one_shot(d, h_in, h_out);
}

int ndf_robust_filter(const void* h_in, void* h_out, int32_t dtype, int32_t ndim,
                      const uint64_t* shape, const uint64_t* size, const uint8_t* footprint,
                      const int64_t* origin, const char* const* modes, double cval,
                      const char* kind, double parameter, int32_t omit_nan,
                      int32_t ignore_inf, uint64_t min_count, double sigma_lower,
                      double sigma_upper, int64_t maxiters, const char* center,
                      const char* spread, const char* estimator, int32_t modify_sample_size,
                      double pearson) {
  static const std::pair<const char*, int> kinds[] = {
      {"percentile", kPercentile},      {"mad", kMad},
      {"mode", kMode},                  {"biweight_location", kBiweightLocation},
      {"biweight_scale", kBiweightScale}, {"sigma_mean", kSigmaMean},
      {"sigma_median", kSigmaMedian},   {"sigma_mode", kSigmaMode}};
  int k = -1;
  for (const auto& entry : kinds)
    if (kind && std::strcmp(kind, entry.first) == 0) k = entry.second;
  if (k < 0) return fail(NDF_ERR_INVALID_CONFIGURATION, "unsupported robust filter kind");
  const bool clip = k >= kSigmaMean;
  // src/pyapi/robust.rs:104-116 (non-clipping kinds), then the clipping and
  // mode options in the order the reference parses them.
  if (!clip && !omit_nan && (ignore_inf || min_count != 1))
    return fail(NDF_ERR_INVALID_CONFIGURATION, "ignore_inf and min_count require NaN omission");
  ndf_robust_params rp{};
  rp.parameter = parameter;
  rp.sigma_lower = sigma_lower;
  rp.sigma_upper = sigma_upper;
  rp.maxiters = maxiters;
  rp.modify_sample_size = modify_sample_size;
  rp.pearson = pearson;
  rp.center = NDF_CLIP_CENTER_MEDIAN;
  rp.spread = NDF_CLIP_SPREAD_STD;
  rp.estimator = NDF_MODE_ESTIMATOR_SEX;
  auto parse_estimator = [&]() {
    const char* e = estimator ? estimator : "sex";
    if (std::strcmp(e, "sex") == 0) rp.estimator = NDF_MODE_ESTIMATOR_SEX;
    else if (std::strcmp(e, "mmm") == 0) rp.estimator = NDF_MODE_ESTIMATOR_MMM;
    else if (std::strcmp(e, "iraf") == 0) rp.estimator = NDF_MODE_ESTIMATOR_IRAF;
    else return fail(NDF_ERR_INVALID_CONFIGURATION, "mode estimator must be 'sex', 'mmm', or 'iraf'");
    return NDF_OK;
  };
  if (k == kMode) {
    int rc = parse_estimator();
    if (rc != NDF_OK) return rc;
  }
  if (clip) {
    const char* c = center ? center : "median";
    if (std::strcmp(c, "mean") == 0) rp.center = NDF_CLIP_CENTER_MEAN;
    else if (std::strcmp(c, "median") == 0) rp.center = NDF_CLIP_CENTER_MEDIAN;
    else return fail(NDF_ERR_INVALID_CONFIGURATION, "center must be 'mean' or 'median'");
    const char* sp = spread ? spread : "std";
    if (std::strcmp(sp, "std") == 0) rp.spread = NDF_CLIP_SPREAD_STD;
    else if (std::strcmp(sp, "mad") == 0) rp.spread = NDF_CLIP_SPREAD_MAD;
    else return fail(NDF_ERR_INVALID_CONFIGURATION, "spread must be 'std' or 'mad'");
    if (k == kSigmaMode) {
      int rc = parse_estimator();
      if (rc != NDF_OK) return rc;
    }
  }
  if (ndim <= 0) return fail(NDF_ERR_INVALID_CONFIGURATION, "filtering requires at least one dimension");
  std::vector<int32_t> m(ndim);
  for (int a = 0; a < ndim; ++a) {
    int rc = parse_mode(modes ? modes[a] : nullptr, &m[a]);
    if (rc != NDF_OK) return rc;
  }
  ndf_filter_desc d{};
  d.dtype = dtype;
  d.ndim = ndim;
  d.shape = shape;
  d.size = size;
  d.footprint = footprint;
  d.origin = origin;
  d.modes = m.data();
  d.cval = cval;
  d.kind = k;
  d.omit_nan = clip ? 1 : omit_nan;
  d.ignore_inf = clip ? 1 : ignore_inf;
  d.min_count = min_count;
  d.percentile = parameter;
  d.moments = NDF_MOMENTS_FP32C;
  d.robust = k == kPercentile ? nullptr : &rp;
  return one_shot(d, h_in, h_out);
}

}  // extern "C"
