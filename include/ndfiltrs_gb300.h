/*
 * ndfiltrs_gb300 — C-ABI of the GB300 (sm_103a) windowed-statistics library.
 *
 * This is the drop-in boundary for ndfiltrs' native module `ndfiltrs._core`
 * (ysBach/ndfiltrs v0.2.0, a PyO3 extension of a Rust crate). The reference's
 * Python layer calls three native functions on this path; the first three
 * entry points below take the same arguments with the same meaning (the
 * Python objects flattened to plain pointers and sizes) and return the same
 * error classes as status codes. The plan entry points expose the reference's
 * Rust plan API (`WindowFilter::new` / `apply_into`) for device-resident and
 * batched use.
 *
 * Conventions
 *   - Arrays are C-contiguous float32 (dtype 0) or float64 (dtype 1).
 *   - `shape`, `size` and `origin` have `ndim` entries; `footprint` is NULL
 *     (rectangular window) or prod(size) bytes, nonzero = selected, C order.
 *   - Mode names are "reflect", "constant", "nearest", "mirror", "wrap".
 *   - Every function returns NDF_OK or an error code; ndf_last_error() gives
 *     the calling thread's message. No exception crosses the ABI.
 *   - There is no CPU fallback: without a usable CUDA device every compute
 *     entry point returns NDF_ERR_NO_DEVICE.
 *   - Host entry points copy the input to the device before computing (the
 *     snapshot of src/pyapi/filter.rs:219-229) and write a new result into
 *     `h_out`; input and output never alias.
 */
#ifndef NDFILTRS_GB300_H
#define NDFILTRS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. 1-5 mirror `Error` in src/error.rs:6-18 and map to the same
 * Python exceptions (src/pyapi/filter.rs:37-44): 1-3 ValueError,
 * 4 MemoryError, 5 OverflowError. */
#define NDF_OK 0
#define NDF_ERR_EMPTY_AXIS 1
#define NDF_ERR_INVALID_CONFIGURATION 2
#define NDF_ERR_LENGTH_MISMATCH 3
#define NDF_ERR_MEMORY 4
#define NDF_ERR_OVERFLOW 5
#define NDF_ERR_CUDA 6        /* a CUDA runtime call failed */
#define NDF_ERR_TIMEOUT 7     /* a bounded device wait gave up */
#define NDF_ERR_UNSUPPORTED 8 /* a reduction outside this library's scope */
#define NDF_ERR_NO_DEVICE 9   /* no CUDA device could be used */

#define NDF_FLOAT32 0
#define NDF_FLOAT64 1

/* Reduction kinds: the `kind` strings of src/pyapi/filter.rs:286-300 plus
 * the percentile kind of src/pyapi/robust.rs:118-121. */
#define NDF_KIND_MEDIAN 0
#define NDF_KIND_MEDIAN_NETWORK 1
#define NDF_KIND_MEDIAN_HISTOGRAM 2
#define NDF_KIND_MEAN 3
#define NDF_KIND_MEAN_ROLLING 4 /* exact boxcar mean (method="boxcar"), rectangular windows */
#define NDF_KIND_MIN 5
#define NDF_KIND_MAX 6
#define NDF_KIND_VAR 7
#define NDF_KIND_STD 8
#define NDF_KIND_RANK 9
#define NDF_KIND_RANK_HISTOGRAM 10
#define NDF_KIND_PERCENTILE 11
/* The other robust kinds of src/pyapi/robust.rs:117-154 ("mad", "mode",
 * "biweight_location", "biweight_scale", "sigma_mean", "sigma_median",
 * "sigma_mode"); their parameters travel in ndf_robust_params. */
#define NDF_KIND_MAD 12
#define NDF_KIND_MODE 13
#define NDF_KIND_BIWEIGHT_LOCATION 14
#define NDF_KIND_BIWEIGHT_SCALE 15
#define NDF_KIND_SIGMA_MEAN 16
#define NDF_KIND_SIGMA_MEDIAN 17
#define NDF_KIND_SIGMA_MODE 18

/* ClipCenter, ClipSpread (src/robust.rs:16-35) and ModeEstimator
 * (src/location.rs:13-25). */
#define NDF_CLIP_CENTER_MEAN 0
#define NDF_CLIP_CENTER_MEDIAN 1
#define NDF_CLIP_SPREAD_STD 0
#define NDF_CLIP_SPREAD_MAD 1
#define NDF_MODE_ESTIMATOR_SEX 0
#define NDF_MODE_ESTIMATOR_MMM 1
#define NDF_MODE_ESTIMATOR_IRAF 2

/* Boundary modes, src/boundary.rs:16-27. */
#define NDF_MODE_REFLECT 0
#define NDF_MODE_CONSTANT 1
#define NDF_MODE_NEAREST 2
#define NDF_MODE_MIRROR 3
#define NDF_MODE_WRAP 4

/* Arithmetic of the mean/var/std reductions. */
#define NDF_MOMENTS_FP32C 0 /* pivot-shifted FP32 compensated sums, FP64 combine */
#define NDF_MOMENTS_FP64 1  /* the reference's float64 algorithm, bit for bit */

/* Replaces `_core.window_filter(array, kind, size, footprint, origin, mode,
 * cval, omit_nan, ignore_inf, min_count, parameter)`,
 * src/pyapi/filter.rs:261-314 (plan: src/plan.rs:260-324, run:
 * src/plan.rs:370-428). `kind` is one of "median", "median_network",
 * "median_histogram", "mean", "mean_rolling", "min", "max", "var", "std",
 * "rank", "rank_histogram"; `parameter` is ddof for var/std and the rank for
 * the rank kinds. `cval` is cast to the array dtype (src/pyapi/filter.rs:308). */
int ndf_window_filter(const void* h_in, void* h_out, int32_t dtype, int32_t ndim,
                      const uint64_t* shape, const char* kind, const uint64_t* size,
                      const uint8_t* footprint, const int64_t* origin,
                      const char* const* modes, double cval, int32_t omit_nan,
                      int32_t ignore_inf, uint64_t min_count, uint64_t parameter);

/* Replaces `_core.robust_filter(array, size, footprint, origin, mode, cval,
 * kind, parameter, omit_nan, ignore_inf, min_count, sigma_lower,
 * sigma_upper, maxiters, center, spread, estimator, modify_sample_size,
 * pearson)`, src/pyapi/robust.rs:78-171 (plan: src/robust_plan.rs:55-67,
 * run: src/robust.rs:725-785). `kind` is one of "percentile", "mad", "mode",
 * "biweight_location", "biweight_scale", "sigma_mean", "sigma_median",
 * "sigma_mode"; `parameter` is the percentile q, the MAD scale or the
 * biweight c; `maxiters` < 0 stands for None (clip until stable); `center`
 * is "mean" or "median", `spread` "std" or "mad", `estimator` "sex", "mmm"
 * or "iraf". */
int ndf_robust_filter(const void* h_in, void* h_out, int32_t dtype, int32_t ndim,
                      const uint64_t* shape, const uint64_t* size, const uint8_t* footprint,
                      const int64_t* origin, const char* const* modes, double cval,
                      const char* kind, double parameter, int32_t omit_nan,
                      int32_t ignore_inf, uint64_t min_count, double sigma_lower,
                      double sigma_upper, int64_t maxiters, const char* center,
                      const char* spread, const char* estimator, int32_t modify_sample_size,
                      double pearson);

/* ---- Mesh background: MeshBackground (src/background.rs:31-923) and
 * `_core.mesh_background` (src/pyapi/background.rs:225-280). The rule set of
 * MeshConfig (src/background.rs:144-289), numbered as below. */
#define NDF_MESH_ESTIMATOR_SEXTRACTOR 0
#define NDF_MESH_ESTIMATOR_SIGMA_CLIP 1
#define NDF_MESH_STATISTIC_MEAN 0
#define NDF_MESH_STATISTIC_MEDIAN 1
#define NDF_MESH_STATISTIC_MODE 2
#define NDF_MESH_RMS_STD 0
#define NDF_MESH_RMS_MAD_STD 1
#define NDF_MESH_VALID_FINITE 0
#define NDF_MESH_VALID_RETAINED 1
#define NDF_MESH_BASE_MESH 0
#define NDF_MESH_BASE_BOX 1
#define NDF_MESH_FILL_NEAREST 0
#define NDF_MESH_FILL_IDW 1
#define NDF_MESH_EDGE_SHRINK 0
#define NDF_MESH_EDGE_TRUNCATE 1
#define NDF_MESH_THRESHOLD_ALL 0
#define NDF_MESH_THRESHOLD_DEVIATION 1
#define NDF_MESH_THRESHOLD_ABOVE 2
#define NDF_MESH_INTERP_SPLINE 0
#define NDF_MESH_INTERP_SEXTRACTOR 1

typedef struct ndf_mesh_config {
  int32_t estimator;          /* NDF_MESH_ESTIMATOR_* */
  double pearson;             /* mode rule factor (>= 1) */
  double sigma_lower;         /* sigma clip: multipliers (>= 0) */
  double sigma_upper;
  int64_t maxiters;           /* sigma clip: passes; < 0: until stable */
  int32_t center;             /* NDF_CLIP_CENTER_* */
  int32_t spread;             /* NDF_CLIP_SPREAD_* */
  int32_t statistic;          /* NDF_MESH_STATISTIC_* */
  int32_t mode_estimator;     /* NDF_MODE_ESTIMATOR_* */
  int32_t rms;                /* NDF_MESH_RMS_* */
  double min_valid_fraction;  /* [0, 1] */
  int32_t valid_count;        /* NDF_MESH_VALID_* */
  int32_t valid_base;         /* NDF_MESH_BASE_* */
  int32_t fill;               /* NDF_MESH_FILL_* */
  uint64_t idw_neighbors;     /* >= 1 */
  double idw_power;           /* finite, >= 0 */
  int32_t filter_edge;        /* NDF_MESH_EDGE_* */
  int32_t threshold_kind;     /* NDF_MESH_THRESHOLD_* */
  double threshold;           /* finite unless NDF_MESH_THRESHOLD_ALL */
  int32_t interpolation;      /* NDF_MESH_INTERP_* */
} ndf_mesh_config;

/* Replaces `_core.mesh_background(array, mask, box_size, filter_size, ...)`:
 * per-mesh statistics on the GPU, fill and median filter of the mesh grid,
 * and the full-resolution background and RMS maps (dtype of the input) on the
 * GPU. `h_mask` is NULL or prod(shape) bytes (nonzero excludes the sample).
 * Mesh outputs have prod(ceil(shape / box_size)) entries; `globals` receives
 * the global background and RMS. */
int ndf_mesh_background(const void* h_in, const uint8_t* h_mask, int32_t dtype, int32_t ndim,
                        const uint64_t* shape, const uint64_t* box_size, const uint64_t* filter_size,
                        const ndf_mesh_config* config, void* h_background, void* h_rms,
                        double* mesh_background, double* mesh_rms, uint8_t* mesh_valid,
                        int64_t* mesh_finite_count, int64_t* mesh_retained_count, double* globals);

/* The same pipeline over device buffers (`d_mask` may be NULL), enqueued on
 * `stream`; the call synchronizes once between the mesh statistics and the
 * host-side fill / filter and returns after enqueuing the interpolation. */
int ndf_mesh_background_device(const void* d_in, const uint8_t* d_mask, int32_t dtype, int32_t ndim,
                               const uint64_t* shape, const uint64_t* box_size,
                               const uint64_t* filter_size, const ndf_mesh_config* config,
                               void* d_background, void* d_rms, double* mesh_background,
                               double* mesh_rms, uint8_t* mesh_valid, int64_t* mesh_finite_count,
                               int64_t* mesh_retained_count, double* globals, void* stream);

/* Replaces `_core.get_num_threads()`, src/pyapi/filter.rs:378-380. Returns
 * the number of host threads of the library's host-side pools (pageable
 * copies, page prefaulting, mesh fill): RAYON_NUM_THREADS when it is set to a
 * positive integer, else the hardware thread count capped at 16; fixed at
 * the first call of the process, like the reference's global Rayon pool.
 * Needs no device. */
int32_t ndf_get_num_threads(void);

/* Thread-local message of the last error on the calling thread. */
const char* ndf_last_error(void);

/* ---- Plans: WindowFilter::new / RobustFilter::new, src/plan.rs:260-324,
 * src/robust_plan.rs:55-67. A plan validates the geometry once and applies it
 * to any number of arrays of its shape. */

typedef struct ndf_plan ndf_plan;

/* Parameters of the robust kinds other than the percentile (RobustReduction
 * and ClipConfig, src/robust.rs:52-185). */
typedef struct ndf_robust_params {
  double parameter;           /* MAD scale (>= 0) or biweight c (> 0) */
  double sigma_lower;         /* clipping multipliers (>= 0) */
  double sigma_upper;
  int64_t maxiters;           /* clipping passes; < 0: until stable */
  int32_t center;             /* NDF_CLIP_CENTER_* */
  int32_t spread;             /* NDF_CLIP_SPREAD_* */
  int32_t estimator;          /* NDF_MODE_ESTIMATOR_* */
  int32_t modify_sample_size; /* biweight scale: count only |u| < 1 */
  double pearson;             /* mode rule factor (>= 1) */
} ndf_robust_params;

typedef struct ndf_filter_desc {
  int32_t dtype;             /* NDF_FLOAT32 / NDF_FLOAT64 */
  int32_t ndim;              /* >= 1 */
  const uint64_t* shape;     /* ndim */
  const uint64_t* size;      /* ndim: window box */
  const uint8_t* footprint;  /* NULL or prod(size) bytes */
  const int64_t* origin;     /* ndim */
  const int32_t* modes;      /* ndim: NDF_MODE_* */
  double cval;               /* cast to dtype by the plan */
  int32_t kind;              /* NDF_KIND_* */
  int32_t omit_nan;          /* InvalidPolicy::Omit when nonzero */
  int32_t ignore_inf;        /* Omit{ignore_inf} */
  uint64_t min_count;        /* Omit{min_count} */
  uint64_t parameter;        /* rank or ddof */
  double percentile;         /* q for NDF_KIND_PERCENTILE */
  int32_t moments;           /* NDF_MOMENTS_* for mean/var/std */
  const ndf_robust_params* robust; /* NDF_KIND_MAD .. NDF_KIND_SIGMA_MODE; else NULL */
} ndf_filter_desc;

int ndf_plan_create(const ndf_filter_desc* desc, ndf_plan** plan);
int ndf_plan_destroy(ndf_plan* plan);

/* apply_into over device buffers, src/plan.rs:403-428. Enqueues on `stream`
 * (a cudaStream_t, NULL = the legacy default stream) and returns without
 * synchronizing. */
int ndf_plan_run(ndf_plan* plan, const void* d_in, void* d_out, void* stream);

/* apply_into over host buffers: copies h_in to the device, filters, copies
 * the result to h_out and synchronizes `stream`. Device buffers are owned by
 * the plan and reused across calls. Pinned host memory gives the fastest
 * copies. */
int ndf_plan_run_host(ndf_plan* plan, const void* h_in, void* h_out, void* stream);

/* Split form of ndf_plan_run_host for callers that must take the input
 * snapshot before releasing a lock (the reference snapshots under the GIL,
 * src/pyapi/filter.rs:219-242): upload copies h_in to the plan's device
 * input synchronously; compute filters it and copies the result to h_out. */
int ndf_plan_upload(ndf_plan* plan, const void* h_in);
int ndf_plan_compute_download(ndf_plan* plan, void* h_out);

/* Name of the kernel family the plan dispatches to ("tile_network",
 * "tile_radix", "histogram", "moments_tile", "generic", ...). */
const char* ndf_plan_algorithm(const ndf_plan* plan);

/* Number of row bands ndf_plan_run_host pipelines (uploads, kernels and
 * downloads of successive bands overlap); 0 while it runs the whole array in
 * one piece. A plan tries bands on its third host-buffer run and keeps them
 * when that run was at least 5% faster than the second (whole-array) one;
 * they apply to arrays of at least 16 MiB with 256 or more rows per band,
 * exact statistics (not the float32-compensated moments) and a first-axis
 * mode other than wrap. No counterpart in the reference. */
int32_t ndf_plan_host_bands(const ndf_plan* plan);

/* Band policy of ndf_plan_run_host: 0 never, 1 the timed choice above
 * (default), 2 always where bands apply (from the next run on). */
int ndf_plan_set_host_bands(ndf_plan* plan, int32_t mode);

/* ---- Batched persistent path. Many images of uneven sizes, each with its
 * own window, footprint and reduction, run as one persistent launch per
 * kernel family (register networks, radix select, moments) plus one launch
 * per image for the specialized kernels (box pair, sliding histogram); the
 * launches are captured once into a CUDA graph as concurrent branches and
 * replayed. No counterpart in the reference (its Python callers loop). */

typedef struct ndf_batch ndf_batch;

/* `descs[i]` describes image i (shape, window, reduction; dtype must be
 * float32). `d_in[i]` / `d_out[i]` are device buffers of image i. */
int ndf_batch_create(const ndf_filter_desc* descs, int32_t count, ndf_batch** batch);
int ndf_batch_destroy(ndf_batch* batch);
int ndf_batch_run(ndf_batch* batch, const void* const* d_in, void* const* d_out, void* stream);
/* Host-buffer run of a batch: `h_in[i]` / `h_out[i]` are host buffers
 * (pageable or pinned) of image i. Copies every image to batch-owned device
 * buffers, filters, copies the results back and returns after synchronizing.
 * Images are processed in groups so that host copies, uploads, kernels and
 * downloads of different groups overlap; the first call allocates the device
 * buffers and two pinned staging slots per direction. Starts after the work
 * already enqueued on `stream`; runs of one batch must not overlap. */
int ndf_batch_run_host(ndf_batch* batch, const void* const* h_in, void* const* h_out, void* stream);
/* Number of launches (persistent family launches plus per-image launches)
 * one ndf_batch_run replays; valid after the first run. */
int32_t ndf_batch_launches(const ndf_batch* batch);

/* Allocation-free histogram filter over caller-owned device buffers. No
 * counterpart in the reference. For callers that cannot let a library
 * allocate device memory (code running during stream capture, frameworks
 * that own all device memory, real-time pipelines that cannot absorb an
 * allocation's implicit synchronization): the sliding rank-histogram kernel's
 * sort scratch lives in a static 16 MiB device array of the library, so this
 * call never runs cudaMalloc, cudaFree or any allocating routine. 1-D and 2-D
 * rectangular windows; `kind` is an order statistic (median, rank, min, max,
 * percentile; histogram or not); arguments mean what they mean in
 * ndf_filter_desc. Enqueues on `stream` and returns. The array is shared by
 * every call and keeps the last call's contents (the kernel overwrites what
 * it reads, nothing needs clearing); calls that overlap on the GPU race on
 * it. The first call on a device looks up the array's address with that
 * device current: make it before any stream capture. The address is kept
 * for the process, so the call must not be used on a device after
 * cudaDeviceReset. A window whose sort slot does not fit in the array returns
 * NDF_ERR_MEMORY. */
int ndf_histogram_filter_noalloc(const void* d_in, void* d_out, int32_t dtype, int32_t ndim,
                                 const uint64_t* shape, const uint64_t* size, const int64_t* origin,
                                 const int32_t* modes, double cval, int32_t kind, int32_t omit_nan,
                                 int32_t ignore_inf, uint64_t min_count, uint64_t parameter,
                                 double percentile, void* stream);

/* ---- Autotuner. A plan whose window can run on several kernels (sliding
 * histogram, box pair kernel, register network, radix select; output tile
 * shapes) takes the choice measured for its (device, dtype, statistic,
 * policy, window box, tap count, footprint class); every choice gives the
 * same results. Modes: 0 = off (built-in preference order), 1 = plans use
 * measured choices and batches measure the keys they miss (the default),
 * 2 = every plan measures the keys it misses. Measured choices persist in a
 * text file: `cache_path` NULL keeps the current file, "" keeps choices in
 * memory only. The initial mode comes from the environment variable
 * NDF_AUTOTUNE and the initial file from NDF_AUTOTUNE_CACHE (default
 * $XDG_CACHE_HOME or ~/.cache, then ndfiltrs_gb300/autotune.txt). No
 * counterpart in the reference. */
int ndf_set_autotune(int32_t mode, const char* cache_path);
/* Number of measured choices known (loading the file first). */
int32_t ndf_autotune_entries(void);
/* Pin the kernel family ("histogram", "box", "network", "radix", "moments",
 * "slide", "extrema", "passes", "boxcar", "band") that plans take whenever
 * it is one of their candidates, ahead of the autotuner; NULL or "" unpins.
 * For A/B comparisons and tests: every family gives the same results. No
 * counterpart in the reference. */
int ndf_pin_kernel(const char* family);

/* ---- TMA staging and bounded waits. Interior halo tiles of the tile
 * kernels are staged by one TMA (cp.async.bulk.tensor) copy each; every
 * device wait is bounded and a wait that runs out is reported as
 * NDF_ERR_TIMEOUT by the next synchronizing call. No counterpart in the
 * reference. */
/* Turn TMA staging on (default; NDF_TMA=0 in the environment turns it off)
 * or off. Results are identical either way. */
int ndf_set_tma(int32_t enabled);
/* Synchronize the device and read (and clear) the status flags; returns
 * NDF_ERR_TIMEOUT when a device wait gave up since the last check. */
int ndf_device_status(uint32_t* flags);
/* Self-test of the bounded wait: runs a kernel whose barrier wait can never
 * complete; returns NDF_ERR_TIMEOUT when the wait gave up and reported it,
 * as it must. */
int ndf_selftest_wait_timeout(void);

/* Number of SMs, device name and compute capability of device 0. */
int ndf_device_info(int32_t* sm_count, int32_t* major, int32_t* minor, char* name,
                    size_t name_capacity);

#ifdef __cplusplus
}
#endif

#endif /* NDFILTRS_GB300_H */
