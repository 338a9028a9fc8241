// Host-side plan and kernel argument structures shared by the translation
// units of the GB300 library.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <memory>
#include <string>
#include <vector>

namespace ndf {

constexpr int kMaxNetwork32 = 128;  // largest register network for float32 keys
constexpr int kMaxNetwork64 = 64;   // largest register network for float64 keys
constexpr int kMaxGenericRank = 32; // largest array rank of the generic kernels

// Canonical 3-D view of a rank 1-3 array: axes (z, y, x), x contiguous.
struct Geom3 {
  long long D, H, W;  // array extent per axis
  int kd, kh, kw;     // window box per axis
  int az, ay, ax;     // anchors: size / 2 + origin
  int mz, my, mx;     // boundary modes
};

// Reduction parameters every kernel reads.
// Percentile rank split for a window of n retained samples (src/robust.rs:
// 343-352), tabulated per n on the host: rank = (q / 100) * (n - 1),
// lower = floor(rank), fraction f = rank - lower, w = f (f <= 0.5) or 1 - f.
struct PctEntry {
  double fraction;
  double w;
  int lower;
  int flags;  // kPctFracZero | kPctLowSide | kPctFracOne
};
constexpr int kPctFracZero = 1;
constexpr int kPctLowSide = 2;
constexpr int kPctFracOne = 4;

struct Reduce {
  int kind;            // NDF_KIND_*
  int omit;            // InvalidPolicy::Omit
  int drop_inf;        // Omit { ignore_inf: true }
  int count;           // taps per window (V)
  long long min_count; // Omit { min_count }
  long long param;     // rank or ddof
  double q;            // percentile
  double q_fraction;   // q / 100.0 (src/robust.rs:348 computes it the same way)
  double cval;         // constant boundary value, already cast to the dtype
  int moments;         // NDF_MOMENTS_* for mean/var/std
  int q_is_max;        // q == 100 (the maximum)
  const PctEntry* pct; // device table indexed by n (count + 1 entries), or nullptr
};

// Robust reductions: estimator kinds as the kernels number them (kind - 11
// of the C-ABI kinds) and their parameters (RobustReduction and ClipConfig,
// src/robust.rs:52-185; ModeEstimator, src/location.rs:13-25).
enum RobustKind {
  kRobustPercentile = 0,
  kRobustMad = 1,
  kRobustMode = 2,
  kRobustBiweightLocation = 3,
  kRobustBiweightScale = 4,
  kRobustSigmaMean = 5,
  kRobustSigmaMedian = 6,
  kRobustSigmaMode = 7,
};
enum ModeRule { kModeSex = 0, kModeMmm = 1, kModeIraf = 2 };

struct RobustArgs {
  int kind;                  // RobustKind
  double parameter;          // MAD scale or biweight c
  double lower, upper;       // clipping multipliers
  long long maxiters;        // < 0: clip until stable
  int center;                // 0 mean, 1 median
  int spread;                // 0 std, 1 MAD
  int estimator;             // ModeRule
  int modify_sample_size;    // biweight scale
  double pearson;            // mode rule factor
  long long clip_min_count;  // ClipConfig::min_count
};

// Halo tile of one thread block: TW x TH outputs of one z slice. The block
// stages kd x SH x SW samples (SH = TH + kh - 1, SW = TW + kw - 1).
struct Tile {
  int TW, TH, SH, SW;
  long long tiles_x, tiles_y, tiles;  // tiles per row, per slice, total
};

struct TileArgs {
  Geom3 g;
  Tile t;
  Reduce r;
  // TMA staging of interior tiles, set per launch (0 in plans and batch
  // tasks): box width in elements (a multiple of 16 bytes; 0 = off), tensor
  // rank (2 or 3), byte offset of the staging area in dynamic shared memory,
  // and the host-mapped status word a timed-out wait writes.
  int tma_bw;
  int tma_rank;
  int tma_offset;
  unsigned int* status;
};

// Generic N-D gather (any rank): one thread per output.
struct GenericArgs {
  int rank;
  long long n_out;
  long long shape[kMaxGenericRank];
  long long stride[kMaxGenericRank];
  int mode[kMaxGenericRank];
  long long low[kMaxGenericRank], high[kMaxGenericRank];
  Reduce r;
};

enum class Algo {
  kEmpty,
  kTileNetwork,
  kTileBox,
  kTileRadix,
  kGenericSelect,
  kHistogram,
  kMomentsTile,
  kMomentsGeneric,
  kBoxcarTile,    // exact rolling mean, tiled sliding integer sums
  kBoxcarDirect,  // exact rolling mean, full-width direct sums
  kMomentsSlide,  // mean / var / std, sliding exact integer sums (boxes)
  kExtremaTile,   // separable min / max (van Herk / Gil-Werman) over boxes
  kBoxcarBand,    // exact rolling mean, column sums sliding down bands
  kExtremaPasses, // separable min / max, two transposing column passes
  kRobust,        // MAD, sigma clipping, mode, biweight: per-window float64
  kTileRank,      // float32 register networks on 16-bit rank codes, two windows per thread
};

struct StripSet;  // row bands of host-buffer runs (capi.cu)

struct Plan {
  // Validated description.
  int dtype = 0;
  int ndim = 0;
  std::vector<long long> shape, size, origin;
  std::vector<int> modes;
  std::vector<uint8_t> footprint;  // empty for a rectangular window
  Reduce r{};
  long long n_out = 0;

  // Window taps in C order over the footprint: per-axis offsets
  // (count x ndim, k - anchor) and, for the tile kernels, (kz, ky, kx) box
  // positions.
  std::vector<long long> taps;
  std::vector<int> box_taps;  // count x 3 (canonical z, y, x), tile kernels

  Algo algo = Algo::kEmpty;
  int network = 0;  // register-network width (power of two) for kTileNetwork
  TileArgs tile{};
  size_t smem_bytes = 0;
  GenericArgs generic{};

  // Device resources.
  int device = 0;
  int sm_count = 0;
  int32_t* d_tile_taps = nullptr;   // smem offsets of the taps (tile kernels)
  long long* d_gen_taps = nullptr;  // count x rank offsets + count flat offsets
  void* d_in = nullptr;             // buffers for host-buffer runs
  void* d_out = nullptr;
  size_t buffer_bytes = 0;
  void* d_scratch = nullptr;        // kernel scratch (histogram ranks, ...)
  size_t scratch_bytes = 0;
  unsigned int* d_status = nullptr; // device error flags

  // Histogram kernel geometry (1-D/2-D windows).
  int hist_block_w = 0, hist_block_h = 0;
  bool hist_sdec = false;  // sorted keys staged in shared memory
  long long hist_blocks_x = 0, hist_blocks_y = 0;
  // Footprint windows: tap and run-end offsets in the tile's support
  // (taps | top | bottom | left | right ends) and their counts.
  bool hist_footprint = false;
  int hist_nf = 0, hist_nv = 0, hist_nh = 0;
  std::vector<uint16_t> hist_lists;
  uint16_t* d_hist_lists = nullptr;
  PctEntry* d_pct = nullptr;  // percentile rank table (kPercentile, q < 100)

  // Kernel choice: measure candidates not in the autotune cache (batches).
  bool may_tune = false;
  int ext_rows[2] = {0, 0};  // rows per block of the two extrema column passes
  int slide_rows = 0;        // output rows per chunk of the sliding moments kernel
  RobustArgs robust{};       // robust estimator parameters
  long long robust_threads = 0;  // threads of the scratch-backed robust kernel

  // Host-buffer runs in overlapping row bands: built on a plan's third
  // host-buffer run (one-shot calls skip the setup), timed against the
  // second (whole-array) run, and kept only when 5% faster.
  std::shared_ptr<StripSet> strips;
  bool strips_tried = false;
  bool strips_decided = false;
  int band_mode = 1;  // 0: never, 1: timed choice, 2: always (where they apply)
  int host_runs = 0;
  double whole_ms = 0.0;
};

const char* algo_name(Algo a);

// A kernel choice for a tileable plan: the algorithm and, for the tile
// kernels, the output tile (tw x th outputs, one thread per output; 0 for
// the histogram, whose block comes from its cost model).
struct Candidate {
  Algo algo = Algo::kEmpty;
  int tw = 0, th = 0;
};

// Plan internals (capi.cu) used by the autotuner.
void plan_setup_tile(Plan& p);
void plan_release(Plan& p);
int plan_run(const Plan& p, const void* in, void* out, cudaStream_t s);
int plan_apply(Plan& p, const Candidate& c, int smem_limit);

// The autotuner (autotune.cu): picks one of `cands` (two or more) by the
// cached or, when the plan may tune, freshly measured timings of the plan's
// (device, dtype, statistic, window, footprint class) key.
Candidate autotune_pick(const Plan& p, const std::vector<Candidate>& cands, int smem_limit);

// Raise a kernel's dynamic shared-memory limit to the device maximum, once.
// The attribute belongs to the function, not to a plan, so it is never
// lowered after one plan set it.
cudaError_t allow_max_smem(const void* kernel);

// Launchers (one per translation unit). Return a cudaError_t.
cudaError_t launch_tile_select(const Plan& p, const void* in, void* out, cudaStream_t s);
cudaError_t launch_tile_box(const Plan& p, const void* in, void* out, cudaStream_t s);
cudaError_t launch_generic_select(const Plan& p, const void* in, void* out, cudaStream_t s);
cudaError_t launch_tile_moments(const Plan& p, const void* in, void* out, cudaStream_t s);
cudaError_t launch_generic_moments(const Plan& p, const void* in, void* out, cudaStream_t s);
cudaError_t launch_histogram(const Plan& p, const void* in, void* out, cudaStream_t s);
cudaError_t launch_boxcar(const Plan& p, const void* in, void* out, cudaStream_t s);
cudaError_t launch_moments_slide(const Plan& p, const void* in, void* out, cudaStream_t s);
bool moments_slide_configure(Plan& p, int smem_limit);
cudaError_t launch_rank_network(const Plan& p, const void* in, void* out, cudaStream_t s);
bool rank_network_configure(Plan& p, int smem_limit);
cudaError_t launch_extrema(const Plan& p, const void* in, void* out, cudaStream_t s);
bool extrema_configure(Plan& p, int smem_limit);
bool extrema_passes_configure(Plan& p, int smem_limit);
bool robust_configure(Plan& p);
int device_ready(int* device, int* sm_count, int* smem_optin);
int fail(int code, const std::string& message);
int cuda_fail(cudaError_t e, const char* what);
cudaError_t launch_robust(const Plan& p, const void* in, void* out, cudaStream_t s);
bool boxcar_configure(Plan& p, int smem_limit);
bool boxcar_band_configure(Plan& p, int smem_limit);

// Shared-memory bytes a tile kernel needs for `t` (0 when it does not fit).
size_t tile_select_smem(const Plan& p, const Tile& t);
size_t tile_moments_smem(const Plan& p, const Tile& t);
size_t histogram_smem(const Plan& p);
bool histogram_supported(const Plan& p);
// The cost model's tile, or tw x th (an autotuner candidate) when given.
void histogram_configure(Plan& p, int tw = 0, int th = 0);
cudaError_t histogram_allocate(Plan& p);
int network_width_for(int dtype, int count);
bool box_supported(int dtype, int kh, int kw);
Tile box_tile(const Geom3& g);

// A kernel family of the batched path (float32 images): one persistent
// launch walks the concatenated tile lists of several images, each described
// by a task of `task_bytes` (written by write_task with the image's buffers
// and its first tile in the family's list). `variant` picks the kernel
// instantiation a plan needs (-1: the plan's kernel is not of this family).
struct FamilyOps {
  size_t task_bytes;
  int (*variant)(const Plan& p);
  long long (*tiles)(const Plan& p);
  long long (*slot_bytes)(const Plan& p);  // per-block scratch bytes (0: none)
  void (*write_task)(const Plan& p, const void* in, void* out, long long first_tile, void* task);
  const void* (*kernel)(int variant);
  cudaError_t (*launch)(int variant, const void* d_tasks, int ntasks, long long tiles, unsigned char* scratch,
                        long long slot_bytes, size_t smem, int grid, cudaStream_t s);
};
const FamilyOps& histogram_family_ops();  // sliding histogram (histogram.cu), 4 variants
const FamilyOps& box_family_ops();        // box pair 3x3 / 5x5 / 7x7 (box.cu), 6 variants
const FamilyOps& slide_family_ops();      // sliding exact moments (moments_slide.cu), 1 variant
const FamilyOps& rank_family_ops();       // ranked networks (rank_network.cu), 13 variants

}  // namespace ndf
