// Batched persistent path: many float32 images of uneven sizes, each with its
// own window, footprint and reduction.
//
// Images are grouped into kernel families (register-network width 8..128,
// radix select, FP32C / FP64 moments). Each family runs as ONE persistent
// launch whose thread blocks walk the concatenated tile list of all images in
// the family (grid-stride over tiles; a block finds its image by binary search
// over the per-image first-tile prefix). Images a family cannot take (rank > 3
// or supports beyond shared memory) run their own plan's launch. The whole
// sequence (task-table upload + launches) is captured once into a CUDA graph
// and replayed; it is re-captured only when the caller's buffer pointers
// change.
//
// The reference has no counterpart: its callers loop over images, which is
// what the plain per-call path here measures against.
#include <algorithm>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/ndfiltrs_gb300.h"
#include "moments.cuh"
#include "network.cuh"
#include "plan.h"

struct ndf_plan {
  ndf::Plan p;
};

namespace ndf {

int fail(int code, const std::string& message);
int cuda_fail(cudaError_t e, const char* what);

namespace {

constexpr int kThreads = 256;
constexpr int kMaxTaps = 128;

// One image of a family (device table entry).
struct BatchTask {
  const float* in;
  float* out;
  TileArgs tile;
  long long first_tile;  // first tile of this image in the family's tile list
  int taps_offset;       // into the family's tap pool (shared-memory offsets)
  int count;
};

enum Family : int {
  kNet8 = 0,
  kNet16,
  kNet32,
  kNet64,
  kNet128,
  kRadix,
  kMomentsFP32C,
  kMomentsFP64,
  kFamilies,
};

__device__ __forceinline__ int find_task(const BatchTask* tasks, int ntasks, long long tile) {
  int lo = 0, hi = ntasks - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (tasks[mid].first_tile <= tile)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

// Block-shared copy of the current task, refreshed only when the image
// changes between two tiles of the block.
struct SharedTask {
  BatchTask task;
  int index;
};

__device__ __forceinline__ bool load_task(SharedTask& st, const BatchTask* tasks, int ntasks,
                                          long long tile, const int32_t* pool, int32_t* taps_s,
                                          int max_taps) {
  __shared__ int s_index;
  if (threadIdx.x == 0) s_index = find_task(tasks, ntasks, tile);
  __syncthreads();
  const int index = s_index;
  const bool changed = index != st.index;
  if (changed) {
    // Copy the task as 8-byte words (the struct is 8-byte aligned).
    const long long* src = reinterpret_cast<const long long*>(tasks + index);
    long long* dst = reinterpret_cast<long long*>(&st.task);
    for (int i = threadIdx.x; i < (int)(sizeof(BatchTask) / 8); i += blockDim.x) dst[i] = src[i];
    __syncthreads();
    if (taps_s) {
      const int count = min(st.task.count, max_taps);
      for (int i = threadIdx.x; i < count; i += blockDim.x) taps_s[i] = pool[st.task.taps_offset + i];
    }
    if (threadIdx.x == 0) st.index = index;
  }
  __syncthreads();
  return changed;
}

template <int N>
__global__ void __launch_bounds__(kThreads, 1)
    batch_network_kernel(const BatchTask* __restrict__ tasks, int ntasks, long long total_tiles,
                         const int32_t* __restrict__ pool) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ SharedTask st;
  __shared__ int32_t taps_s[N];
  if (threadIdx.x == 0) st.index = -1;
  __syncthreads();
  for (long long tile = blockIdx.x; tile < total_tiles; tile += gridDim.x) {
    load_task(st, tasks, ntasks, tile, pool, taps_s, N);
    const BatchTask& t = st.task;
    net::tile_network_body<float, N, 0, 0>(t.in, t.out, t.tile, tile - t.first_tile, smem_raw,
                                           [&](int i) { return taps_s[i]; });
    __syncthreads();
  }
}

__global__ void __launch_bounds__(kThreads)
    batch_radix_kernel(const BatchTask* __restrict__ tasks, int ntasks, long long total_tiles,
                       const int32_t* __restrict__ pool) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ SharedTask st;
  if (threadIdx.x == 0) st.index = -1;
  __syncthreads();
  for (long long tile = blockIdx.x; tile < total_tiles; tile += gridDim.x) {
    load_task(st, tasks, ntasks, tile, pool, nullptr, 0);
    const BatchTask& t = st.task;
    net::tile_radix_body<float>(t.in, t.out, t.tile, tile - t.first_tile, smem_raw,
                                pool + t.taps_offset);
    __syncthreads();
  }
}

template <int PREC>
__global__ void __launch_bounds__(kThreads)
    batch_moments_kernel(const BatchTask* __restrict__ tasks, int ntasks, long long total_tiles,
                         const int32_t* __restrict__ pool) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ SharedTask st;
  if (threadIdx.x == 0) st.index = -1;
  __syncthreads();
  for (long long tile = blockIdx.x; tile < total_tiles; tile += gridDim.x) {
    load_task(st, tasks, ntasks, tile, pool, nullptr, 0);
    const BatchTask& t = st.task;
    mom::tile_moments_body<float, PREC>(t.in, t.out, t.tile, tile - t.first_tile, smem_raw,
                                        pool + t.taps_offset);
    __syncthreads();
  }
}

const void* family_kernel(int family) {
  switch (family) {
    case kNet8:
      return (const void*)batch_network_kernel<8>;
    case kNet16:
      return (const void*)batch_network_kernel<16>;
    case kNet32:
      return (const void*)batch_network_kernel<32>;
    case kNet64:
      return (const void*)batch_network_kernel<64>;
    case kNet128:
      return (const void*)batch_network_kernel<128>;
    case kRadix:
      return (const void*)batch_radix_kernel;
    case kMomentsFP32C:
      return (const void*)batch_moments_kernel<0>;
    default:
      return (const void*)batch_moments_kernel<1>;
  }
}

struct FamilyState {
  std::vector<int> images;       // image indices in this family
  std::vector<BatchTask> tasks;  // host copy (pointers filled at run)
  std::vector<int32_t> pool;     // tap offsets of every image
  long long tiles = 0;
  size_t smem = 0;
  int grid = 0;
  BatchTask* d_tasks = nullptr;
  BatchTask* h_tasks = nullptr;  // pinned staging read by the graph's copy node
  int32_t* d_pool = nullptr;
};

}  // namespace

// Plan-level helpers shared with capi.cu.
int batch_build_plan(const ndf_filter_desc* d, Plan& p, int* smem_limit);
void batch_release_plan(Plan& p);

}  // namespace ndf

struct ndf_batch {
  std::vector<std::unique_ptr<ndf_plan>> plans;
  std::vector<int> family_of;  // per image: family, or -1 for its own plan launch
  ndf::FamilyState families[ndf::kFamilies];
  std::vector<const void*> in_ptrs;
  std::vector<void*> out_ptrs;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaStream_t capture = nullptr;
  int launches = 0;
  std::mutex lock;
};

using namespace ndf;

namespace {

int family_for(const Plan& p) {
  if (p.algo == Algo::kMomentsTile) return p.r.moments == NDF_MOMENTS_FP64 ? kMomentsFP64 : kMomentsFP32C;
  if (p.algo == Algo::kTileNetwork || p.algo == Algo::kTileBox) {
    int width = network_width_for(0, p.r.count);
    switch (width) {
      case 8:
        return kNet8;
      case 16:
        return kNet16;
      case 32:
        return kNet32;
      case 64:
        return kNet64;
      case 128:
        return kNet128;
      default:
        return -1;
    }
  }
  if (p.algo == Algo::kTileRadix) return kRadix;
  return -1;
}

void destroy_batch(ndf_batch* b) {
  if (!b) return;
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  if (b->capture) cudaStreamDestroy(b->capture);
  for (auto& f : b->families) {
    if (f.d_tasks) cudaFree(f.d_tasks);
    if (f.d_pool) cudaFree(f.d_pool);
    if (f.h_tasks) cudaFreeHost(f.h_tasks);
  }
  for (auto& p : b->plans)
    if (p) batch_release_plan(p->p);
  delete b;
}

}  // namespace

extern "C" {

int ndf_batch_create(const ndf_filter_desc* descs, int32_t count, ndf_batch** out) {
  if (!out) return fail(NDF_ERR_INVALID_CONFIGURATION, "missing batch output pointer");
  *out = nullptr;
  if (!descs || count <= 0) return fail(NDF_ERR_INVALID_CONFIGURATION, "a batch needs at least one image");
  ndf_batch* b = new (std::nothrow) ndf_batch();
  if (!b) return fail(NDF_ERR_MEMORY, "unable to allocate filtering workspace");
  int smem_limit = 0;
  int sm_count = 0;
  for (int i = 0; i < count; ++i) {
    if (descs[i].dtype != NDF_FLOAT32) {
      destroy_batch(b);
      return fail(NDF_ERR_UNSUPPORTED, "batched images must be float32");
    }
    auto plan = std::make_unique<ndf_plan>();
    int rc = batch_build_plan(&descs[i], plan->p, &smem_limit);
    if (rc != NDF_OK) {
      destroy_batch(b);
      return rc;
    }
    sm_count = plan->p.sm_count;
    int fam = plan->p.n_out > 0 ? family_for(plan->p) : -1;
    if (fam >= 0) {
      // Network images use the generic tile (32 x 8 or 256 x 1), not the
      // box-pair tile, inside a family kernel.
      Plan& p = plan->p;
      if (p.algo == Algo::kTileBox || p.algo == Algo::kTileNetwork) {
        Geom3 g = p.tile.g;
        Tile& t = p.tile.t;
        t.TW = g.H == 1 ? 256 : 32;
        t.TH = g.H == 1 ? 1 : 8;
        t.SW = t.TW + g.kw - 1;
        t.SH = t.TH + g.kh - 1;
        t.tiles_x = (g.W + t.TW - 1) / t.TW;
        t.tiles_y = (g.H + t.TH - 1) / t.TH;
        t.tiles = t.tiles_x * t.tiles_y * g.D;
        p.smem_bytes = tile_select_smem(p, t);
        if (p.smem_bytes > (size_t)smem_limit) fam = -1;
      }
    }
    b->family_of.push_back(fam);
    b->plans.push_back(std::move(plan));
  }
  b->in_ptrs.assign(count, nullptr);
  b->out_ptrs.assign(count, nullptr);
  // Build each family's task table and tap pool.
  for (int i = 0; i < count; ++i) {
    int fam = b->family_of[i];
    if (fam < 0) continue;
    FamilyState& f = b->families[fam];
    const Plan& p = b->plans[i]->p;
    BatchTask task{};
    task.tile = p.tile;
    task.tile.r = p.r;
    task.first_tile = f.tiles;
    task.taps_offset = (int)f.pool.size();
    task.count = p.r.count;
    const Tile& t = p.tile.t;
    for (int k = 0; k < p.r.count; ++k) {
      const int* bt = &p.box_taps[(size_t)k * 3];
      f.pool.push_back((bt[0] * t.SH + bt[1]) * t.SW + bt[2]);
    }
    f.tiles += t.tiles;
    f.smem = std::max(f.smem, p.smem_bytes);
    f.images.push_back(i);
    f.tasks.push_back(task);
  }
  for (int fam = 0; fam < kFamilies; ++fam) {
    FamilyState& f = b->families[fam];
    if (f.images.empty()) continue;
    const void* kernel = family_kernel(fam);
    cudaError_t e = allow_max_smem(kernel);
    int per_sm = 1;
    if (e == cudaSuccess)
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kThreads, f.smem);
    size_t task_bytes = f.tasks.size() * sizeof(BatchTask);
    if (e == cudaSuccess) e = cudaMalloc(&f.d_tasks, task_bytes);
    if (e == cudaSuccess) e = cudaMallocHost(&f.h_tasks, task_bytes);
    if (e == cudaSuccess) e = cudaMalloc(&f.d_pool, std::max<size_t>(f.pool.size(), 1) * sizeof(int32_t));
    if (e == cudaSuccess && !f.pool.empty())
      e = cudaMemcpy(f.d_pool, f.pool.data(), f.pool.size() * sizeof(int32_t), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
      destroy_batch(b);
      return cuda_fail(e, "batch setup");
    }
    std::memcpy(f.h_tasks, f.tasks.data(), task_bytes);
    f.grid = (int)std::min<long long>(f.tiles, (long long)std::max(per_sm, 1) * sm_count);
  }
  *out = b;
  return NDF_OK;
}

int ndf_batch_destroy(ndf_batch* batch) {
  destroy_batch(batch);
  return NDF_OK;
}

int32_t ndf_batch_launches(const ndf_batch* batch) { return batch ? batch->launches : 0; }

int ndf_batch_run(ndf_batch* b, const void* const* d_in, void* const* d_out, void* stream) {
  if (!b) return fail(NDF_ERR_INVALID_CONFIGURATION, "missing batch");
  if (!d_in || !d_out) return fail(NDF_ERR_LENGTH_MISMATCH, "missing input or output buffers");
  std::lock_guard<std::mutex> guard(b->lock);
  const int count = (int)b->plans.size();
  bool changed = b->exec == nullptr;
  for (int i = 0; i < count; ++i)
    if (b->in_ptrs[i] != d_in[i] || b->out_ptrs[i] != d_out[i]) changed = true;
  cudaStream_t user = (cudaStream_t)stream;
  if (changed) {
    // Wait for replays still reading the staging tables, then rebuild.
    cudaError_t e = cudaStreamSynchronize(user);
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamSynchronize");
    for (int i = 0; i < count; ++i) {
      b->in_ptrs[i] = d_in[i];
      b->out_ptrs[i] = d_out[i];
    }
    for (auto& f : b->families) {
      for (size_t k = 0; k < f.images.size(); ++k) {
        f.h_tasks[k].in = (const float*)d_in[f.images[k]];
        f.h_tasks[k].out = (float*)d_out[f.images[k]];
      }
    }
    if (b->exec) {
      cudaGraphExecDestroy(b->exec);
      b->exec = nullptr;
    }
    if (b->graph) {
      cudaGraphDestroy(b->graph);
      b->graph = nullptr;
    }
    if (!b->capture) {
      e = cudaStreamCreateWithFlags(&b->capture, cudaStreamNonBlocking);
      if (e != cudaSuccess) return cuda_fail(e, "cudaStreamCreate");
    }
    e = cudaStreamBeginCapture(b->capture, cudaStreamCaptureModeRelaxed);
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamBeginCapture");
    int launches = 0;
    int rc = NDF_OK;
    for (int fam = 0; fam < kFamilies && rc == NDF_OK; ++fam) {
      FamilyState& f = b->families[fam];
      if (f.images.empty()) continue;
      e = cudaMemcpyAsync(f.d_tasks, f.h_tasks, f.tasks.size() * sizeof(BatchTask),
                          cudaMemcpyHostToDevice, b->capture);
      if (e != cudaSuccess) {
        rc = cuda_fail(e, "batch task upload");
        break;
      }
      const int ntasks = (int)f.tasks.size();
      dim3 grid(f.grid), block(kThreads);
      switch (fam) {
        case kNet8:
          batch_network_kernel<8><<<grid, block, f.smem, b->capture>>>(f.d_tasks, ntasks, f.tiles, f.d_pool);
          break;
        case kNet16:
          batch_network_kernel<16><<<grid, block, f.smem, b->capture>>>(f.d_tasks, ntasks, f.tiles, f.d_pool);
          break;
        case kNet32:
          batch_network_kernel<32><<<grid, block, f.smem, b->capture>>>(f.d_tasks, ntasks, f.tiles, f.d_pool);
          break;
        case kNet64:
          batch_network_kernel<64><<<grid, block, f.smem, b->capture>>>(f.d_tasks, ntasks, f.tiles, f.d_pool);
          break;
        case kNet128:
          batch_network_kernel<128><<<grid, block, f.smem, b->capture>>>(f.d_tasks, ntasks, f.tiles, f.d_pool);
          break;
        case kRadix:
          batch_radix_kernel<<<grid, block, f.smem, b->capture>>>(f.d_tasks, ntasks, f.tiles, f.d_pool);
          break;
        case kMomentsFP32C:
          batch_moments_kernel<0><<<grid, block, f.smem, b->capture>>>(f.d_tasks, ntasks, f.tiles, f.d_pool);
          break;
        default:
          batch_moments_kernel<1><<<grid, block, f.smem, b->capture>>>(f.d_tasks, ntasks, f.tiles, f.d_pool);
          break;
      }
      e = cudaGetLastError();
      if (e != cudaSuccess) rc = cuda_fail(e, "batch family launch");
      ++launches;
    }
    for (int i = 0; i < count && rc == NDF_OK; ++i) {
      if (b->family_of[i] >= 0 || b->plans[i]->p.n_out == 0) continue;
      rc = ndf_plan_run(b->plans[i].get(), d_in[i], d_out[i], b->capture);
      ++launches;
    }
    cudaGraph_t graph = nullptr;
    cudaError_t end = cudaStreamEndCapture(b->capture, &graph);
    if (rc != NDF_OK) {
      if (graph) cudaGraphDestroy(graph);
      return rc;
    }
    if (end != cudaSuccess) return cuda_fail(end, "cudaStreamEndCapture");
    b->graph = graph;
    e = cudaGraphInstantiate(&b->exec, b->graph, 0);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
    b->launches = launches;
  }
  cudaError_t e = cudaGraphLaunch(b->exec, user);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGraphLaunch");
  return NDF_OK;
}

}  // extern "C"
