// Batched persistent path: many float32 images of uneven sizes, each with its
// own window, footprint and reduction.
//
// Images whose plan uses a register network, radix select or the moments
// tile kernel are grouped into kernel families (network width 8..128, radix,
// FP32C / FP64 moments); each family runs as ONE persistent launch whose
// thread blocks walk the concatenated tile list of its images (grid-stride
// over tiles; a block finds its image by binary search over the per-image
// first-tile prefix). Images whose plan uses a specialized kernel (box pair,
// sliding histogram) or the generic kernels run their own plan's launch. All
// launches are captured once into a CUDA graph as independent branches and
// replayed; the graph is re-captured only when the caller's buffer pointers
// change.
//
// Host buffers go through a pipeline over groups of images: pageable ->
// pinned copies on a pool of host threads, one upload per group, the group's
// graph, one download per group and pinned -> pageable copies, with the
// uploads, kernels and downloads of different groups overlapping.
//
// The reference has no counterpart: its callers loop over images, which is
// what the plain per-call path measures.
#include <algorithm>
#include <condition_variable>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <utility>
#include <vector>

#include "../../include/ndfiltrs_gb300.h"
#include "moments.cuh"
#include "network.cuh"
#include "plan.h"
#include "tma.cuh"
#include "hostpool.h"

struct ndf_plan {
  ndf::Plan p;
};

namespace ndf {

int fail(int code, const std::string& message);
int cuda_fail(cudaError_t e, const char* what);

namespace {

constexpr int kThreads = 256;

// One image of a family (device table entry).
struct BatchTask {
  const float* in;
  float* out;
  TileArgs tile;
  long long first_tile;  // first tile of this image in the family's tile list
  int taps_offset;       // into the family's tap pool (shared-memory offsets)
  int count;
};

// Kernel families: a register network per (width, epilogue) pair (the
// widths of network_width_for; epilogue 0 = any selection kind, 1 = medians
// only), the radix select and the two moments precisions.
constexpr int kNetWidths[] = {8, 16, 32, 48, 64, 80, 96, 112, 128};
constexpr int kNumNetWidths = sizeof(kNetWidths) / sizeof(kNetWidths[0]);
constexpr int kRadix = 2 * kNumNetWidths;
constexpr int kMomentsFP32C = kRadix + 1;
constexpr int kMomentsFP64 = kRadix + 2;
constexpr int kFamilies = kRadix + 3;

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

template <int N, int MODE>
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
    net::tile_network_body<float, N, 0, MODE>(t.in, t.out, t.tile, tile - t.first_tile, smem_raw,
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

template <int... I>
const void* network_kernel_at(int family, std::integer_sequence<int, I...>) {
  static const void* const table[] = {(const void*)batch_network_kernel<kNetWidths[I / 2], I % 2>...};
  return table[family];
}

const void* family_kernel(int family) {
  if (family < kRadix)
    return network_kernel_at(family, std::make_integer_sequence<int, 2 * kNumNetWidths>{});
  if (family == kRadix) return (const void*)batch_radix_kernel;
  if (family == kMomentsFP32C) return (const void*)batch_moments_kernel<0>;
  return (const void*)batch_moments_kernel<1>;
}


// One image group's launches: a persistent launch per kernel family over the
// group's images of that family, plus the images that run their own plan's
// kernel (box pair, histogram, generic). The launches are captured into one
// CUDA graph as independent branches on kBranches streams, so kernels of
// different images overlap and fill the GPU.
struct FamilyState {
  std::vector<int> images;       // image indices in this family
  std::vector<BatchTask> tasks;  // host copy (pointers filled at capture)
  std::vector<int32_t> pool;     // tap offsets of every image
  long long tiles = 0;
  size_t smem = 0;
  int grid = 0;
  BatchTask* d_tasks = nullptr;
  BatchTask* h_tasks = nullptr;  // pinned staging read by the graph's copy node
  int32_t* d_pool = nullptr;
};

// A family of a specialised kernel reached through FamilyOps (box pair,
// sliding histogram, sliding moments, ranked networks): one (kind, variant)
// pair.
constexpr int kOpsKinds = 4;

const FamilyOps& ops_of(int kind) {
  return kind == 0 ? box_family_ops()
         : kind == 1 ? histogram_family_ops()
         : kind == 2 ? slide_family_ops()
                     : rank_family_ops();
}

struct OpsFamily {
  int kind = 0, variant = 0;
  std::vector<int> images;
  std::vector<long long> first;     // first tile of each image in the family's list
  long long tiles = 0, slot_bytes = 0;
  size_t smem = 0;
  int grid = 0;
  unsigned char* d_tasks = nullptr;
  unsigned char* h_tasks = nullptr;  // pinned staging read by the graph's copy node
  unsigned char* d_scratch = nullptr;
};

struct Segment {
  std::vector<int> images;  // batch image indices, ascending
  FamilyState families[kFamilies];
  std::vector<OpsFamily> ops;  // box pair, histogram, sliding moments and ranked network families
  std::vector<int> own;     // images launched through their own plan
  std::vector<const void*> in_ptrs;
  std::vector<void*> out_ptrs;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int launches = 0;
};

constexpr int kBranches = 8;
constexpr int kChunks = 8;             // image groups of the host pipeline

}  // namespace

// Plan-level helpers shared with capi.cu.
int batch_build_plan(const ndf_filter_desc* d, Plan& p, int* smem_limit);
void batch_release_plan(Plan& p);

}  // namespace ndf

// Host pipeline of ndf_batch_run_host: batch-owned device buffers, two
// pinned staging slots per direction and the copy/compute streams.
struct HostPipeline {
  std::vector<ndf::Segment> chunks;
  std::vector<size_t> offset;      // per image: byte offset in each device region
  std::vector<size_t> bytes;       // per image: buffer bytes
  unsigned char* d_in = nullptr;   // inputs of every image, then outputs
  unsigned char* d_out = nullptr;
  unsigned char* h_in[2] = {nullptr, nullptr};
  unsigned char* h_out[2] = {nullptr, nullptr};
  size_t slot_bytes = 0;
  cudaStream_t up = nullptr, compute = nullptr, down = nullptr;
  cudaEvent_t start = nullptr, uploaded[2] = {nullptr, nullptr}, downloaded[2] = {nullptr, nullptr};
  std::vector<cudaEvent_t> computed;
  std::unique_ptr<ndf::CopyPool> pool;
};

struct ndf_batch {
  std::vector<std::unique_ptr<ndf_plan>> plans;
  std::vector<int> family_of;  // per image: family, or -1 for its own plan launch
  std::vector<long long> pixels;
  ndf::Segment whole;
  cudaStream_t capture = nullptr;
  cudaStream_t branch[ndf::kBranches] = {};
  cudaEvent_t fork = nullptr;
  cudaEvent_t join[ndf::kBranches] = {};
  int sm_count = 0;
  HostPipeline host;
  bool host_ready = false;
  std::mutex lock;
};

using namespace ndf;

namespace {

int family_for(const Plan& p) {
  if (p.algo == Algo::kMomentsTile) return p.r.moments == NDF_MOMENTS_FP64 ? kMomentsFP64 : kMomentsFP32C;
  if (p.algo == Algo::kTileNetwork) {
    const bool median = p.r.kind == kMedian || p.r.kind == kMedianNetwork || p.r.kind == kMedianHistogram;
    for (int w = 0; w < kNumNetWidths; ++w)
      if (kNetWidths[w] == p.network) return 2 * w + (median ? 1 : 0);
    return -1;
  }
  if (p.algo == Algo::kTileRadix) return kRadix;
  return -1;  // box pair, histogram and generic kernels keep their own launch
}

void release_segment(Segment& s) {
  if (s.exec) cudaGraphExecDestroy(s.exec);
  if (s.graph) cudaGraphDestroy(s.graph);
  s.exec = nullptr;
  s.graph = nullptr;
  for (auto& f : s.families) {
    if (f.d_tasks) cudaFree(f.d_tasks);
    if (f.d_pool) cudaFree(f.d_pool);
    if (f.h_tasks) cudaFreeHost(f.h_tasks);
    f.d_tasks = nullptr;
    f.d_pool = nullptr;
    f.h_tasks = nullptr;
  }
  for (auto& f : s.ops) {
    if (f.d_tasks) cudaFree(f.d_tasks);
    if (f.h_tasks) cudaFreeHost(f.h_tasks);
    if (f.d_scratch) cudaFree(f.d_scratch);
    f.d_tasks = f.h_tasks = f.d_scratch = nullptr;
  }
}

void destroy_batch(ndf_batch* b) {
  if (!b) return;
  release_segment(b->whole);
  HostPipeline& h = b->host;
  for (auto& c : h.chunks) release_segment(c);
  if (h.d_in) cudaFree(h.d_in);
  for (int s = 0; s < 2; ++s) {
    if (h.h_in[s]) cudaFreeHost(h.h_in[s]);
    if (h.h_out[s]) cudaFreeHost(h.h_out[s]);
    if (h.uploaded[s]) cudaEventDestroy(h.uploaded[s]);
    if (h.downloaded[s]) cudaEventDestroy(h.downloaded[s]);
  }
  for (cudaEvent_t e : h.computed)
    if (e) cudaEventDestroy(e);
  if (h.start) cudaEventDestroy(h.start);
  for (cudaStream_t s : {h.up, h.compute, h.down})
    if (s) cudaStreamDestroy(s);
  h.pool.reset();
  if (b->fork) cudaEventDestroy(b->fork);
  for (int i = 0; i < kBranches; ++i) {
    if (b->join[i]) cudaEventDestroy(b->join[i]);
    if (b->branch[i]) cudaStreamDestroy(b->branch[i]);
  }
  if (b->capture) cudaStreamDestroy(b->capture);
  for (auto& p : b->plans)
    if (p) batch_release_plan(p->p);
  delete b;
}

// Family tables of a segment's images.
int build_segment(ndf_batch* b, Segment& s, const std::vector<int>& images) {
  s.images = images;
  s.in_ptrs.assign(images.size(), nullptr);
  s.out_ptrs.assign(images.size(), nullptr);
  for (int i : images) {
    const Plan& p = b->plans[i]->p;
    if (p.n_out == 0) continue;
    const int fam = b->family_of[i];
    if (fam < 0) {
      int kind = 0, variant = -1;
      for (; kind < kOpsKinds && variant < 0; ++kind) variant = ops_of(kind).variant(p);
      if (variant < 0) {
        s.own.push_back(i);
        continue;
      }
      --kind;
      OpsFamily* f = nullptr;
      for (auto& o : s.ops)
        if (o.kind == kind && o.variant == variant) f = &o;
      if (!f) {
        s.ops.emplace_back();
        f = &s.ops.back();
        f->kind = kind;
        f->variant = variant;
      }
      const FamilyOps& ops = ops_of(kind);
      f->images.push_back(i);
      f->first.push_back(f->tiles);
      f->tiles += ops.tiles(p);
      f->smem = std::max(f->smem, p.smem_bytes);
      f->slot_bytes = std::max(f->slot_bytes, ops.slot_bytes(p));
      continue;
    }
    FamilyState& f = s.families[fam];
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
    FamilyState& f = s.families[fam];
    if (f.images.empty()) continue;
    const void* kernel = family_kernel(fam);
    cudaError_t e = allow_max_smem(kernel);
    int per_sm = 1;
    if (e == cudaSuccess)
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kThreads, f.smem);
    const size_t task_bytes = f.tasks.size() * sizeof(BatchTask);
    if (e == cudaSuccess) e = cudaMalloc(&f.d_tasks, task_bytes);
    if (e == cudaSuccess) e = cudaMallocHost(&f.h_tasks, task_bytes);
    if (e == cudaSuccess) e = cudaMalloc(&f.d_pool, std::max<size_t>(f.pool.size(), 1) * sizeof(int32_t));
    if (e == cudaSuccess && !f.pool.empty())
      e = cudaMemcpy(f.d_pool, f.pool.data(), f.pool.size() * sizeof(int32_t), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(e, "batch setup");
    std::memcpy(f.h_tasks, f.tasks.data(), task_bytes);
    f.grid = (int)std::min<long long>(f.tiles, (long long)std::max(per_sm, 1) * b->sm_count);
  }
  for (auto& f : s.ops) {
    const FamilyOps& ops = ops_of(f.kind);
    const void* kernel = ops.kernel(f.variant);
    cudaError_t e = allow_max_smem(kernel);
    int per_sm = 1;
    const int threads = f.kind == 1 ? 512 : kThreads;
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, f.smem);
    f.grid = (int)std::min<long long>(f.tiles, (long long)std::max(per_sm, 1) * b->sm_count);
    const size_t bytes = f.images.size() * ops.task_bytes;
    if (e == cudaSuccess) e = cudaMalloc(&f.d_tasks, bytes);
    if (e == cudaSuccess) e = cudaMallocHost(&f.h_tasks, bytes);
    if (e == cudaSuccess && f.slot_bytes > 0) e = cudaMalloc(&f.d_scratch, (size_t)f.grid * (size_t)f.slot_bytes);
    if (e != cudaSuccess) return cuda_fail(e, "batch setup");
  }
  return NDF_OK;
}

cudaError_t launch_family(int fam, FamilyState& f, cudaStream_t s) {
  int ntasks = (int)f.tasks.size();
  void* args[] = {&f.d_tasks, &ntasks, &f.tiles, &f.d_pool};
  return cudaLaunchKernel(family_kernel(fam), dim3(f.grid), dim3(kThreads), args, f.smem, s);
}

// (Re)capture a segment's graph for the given buffers when they changed.
// The caller has synchronized every earlier replay of the segment.
int capture_segment(ndf_batch* b, Segment& s, const void* const* d_in, void* const* d_out) {
  bool changed = s.exec == nullptr;
  for (size_t k = 0; k < s.images.size(); ++k)
    if (s.in_ptrs[k] != d_in[s.images[k]] || s.out_ptrs[k] != d_out[s.images[k]]) changed = true;
  if (!changed) return NDF_OK;
  for (size_t k = 0; k < s.images.size(); ++k) {
    s.in_ptrs[k] = d_in[s.images[k]];
    s.out_ptrs[k] = d_out[s.images[k]];
  }
  for (auto& f : s.families)
    for (size_t k = 0; k < f.images.size(); ++k) {
      f.h_tasks[k].in = (const float*)d_in[f.images[k]];
      f.h_tasks[k].out = (float*)d_out[f.images[k]];
    }
  for (auto& f : s.ops) {
    const FamilyOps& ops = ops_of(f.kind);
    for (size_t k = 0; k < f.images.size(); ++k) {
      const int i = f.images[k];
      ops.write_task(b->plans[i]->p, d_in[i], d_out[i], f.first[k], f.h_tasks + k * ops.task_bytes);
    }
  }
  if (s.exec) cudaGraphExecDestroy(s.exec);
  if (s.graph) cudaGraphDestroy(s.graph);
  s.exec = nullptr;
  s.graph = nullptr;
  cudaError_t e = cudaStreamBeginCapture(b->capture, cudaStreamCaptureModeRelaxed);
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamBeginCapture");
  int rc = NDF_OK;
  int launches = 0;
  bool used[kBranches] = {};
  int next = 0;
  e = cudaEventRecord(b->fork, b->capture);
  auto branch = [&]() -> cudaStream_t {
    const int i = next++ % kBranches;
    if (!used[i]) {
      used[i] = true;
      cudaError_t w = cudaStreamWaitEvent(b->branch[i], b->fork, 0);
      if (w != cudaSuccess && e == cudaSuccess) e = w;
    }
    return b->branch[i];
  };
  for (int fam = 0; fam < kFamilies && e == cudaSuccess; ++fam) {
    FamilyState& f = s.families[fam];
    if (f.images.empty()) continue;
    cudaStream_t st = branch();
    e = cudaMemcpyAsync(f.d_tasks, f.h_tasks, f.tasks.size() * sizeof(BatchTask), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) break;
    e = launch_family(fam, f, st);
    ++launches;
  }
  for (auto& f : s.ops) {
    if (e != cudaSuccess) break;
    const FamilyOps& ops = ops_of(f.kind);
    cudaStream_t st = branch();
    e = cudaMemcpyAsync(f.d_tasks, f.h_tasks, f.images.size() * ops.task_bytes, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) break;
    e = ops.launch(f.variant, f.d_tasks, (int)f.images.size(), f.tiles, f.d_scratch, f.slot_bytes, f.smem, f.grid,
                   st);
    ++launches;
  }
  for (size_t k = 0; k < s.own.size() && e == cudaSuccess && rc == NDF_OK; ++k) {
    const int i = s.own[k];
    rc = ndf_plan_run(b->plans[i].get(), d_in[i], d_out[i], branch());
    ++launches;
  }
  for (int i = 0; i < kBranches && e == cudaSuccess; ++i) {
    if (!used[i]) continue;
    e = cudaEventRecord(b->join[i], b->branch[i]);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(b->capture, b->join[i], 0);
  }
  cudaGraph_t graph = nullptr;
  cudaError_t end = cudaStreamEndCapture(b->capture, &graph);
  if (rc != NDF_OK || e != cudaSuccess || end != cudaSuccess) {
    if (graph) cudaGraphDestroy(graph);
    if (rc != NDF_OK) return rc;
    return cuda_fail(e != cudaSuccess ? e : end, "batch graph capture");
  }
  s.graph = graph;
  e = cudaGraphInstantiate(&s.exec, s.graph, 0);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
  s.launches = launches;
  return NDF_OK;
}

// Device buffers, pinned staging, streams and the image groups of the host
// pipeline (set up on the first host run).
int setup_host(ndf_batch* b) {
  HostPipeline& h = b->host;
  const int count = (int)b->plans.size();
  h.offset.resize(count);
  h.bytes.resize(count);
  size_t total = 0;
  long long pixels = 0;
  for (int i = 0; i < count; ++i) {
    h.offset[i] = total;
    h.bytes[i] = (size_t)b->pixels[i] * sizeof(float);
    total += (h.bytes[i] + 255) & ~(size_t)255;
    pixels += b->pixels[i];
  }
  // Groups of consecutive images with about equal pixel counts.
  const int groups = std::min(count, kChunks);
  std::vector<std::vector<int>> members(1);
  long long acc = 0;
  for (int i = 0; i < count; ++i) {
    members.back().push_back(i);
    acc += b->pixels[i];
    if ((int)members.size() < groups && acc * groups >= pixels * (long long)members.size() && i + 1 < count)
      members.emplace_back();
  }
  h.chunks.resize(members.size());
  for (size_t c = 0; c < members.size(); ++c) {
    int rc = build_segment(b, h.chunks[c], members[c]);
    if (rc != NDF_OK) return rc;
    const int first = members[c].front(), last = members[c].back();
    h.slot_bytes = std::max(h.slot_bytes, h.offset[last] + h.bytes[last] - h.offset[first]);
  }
  cudaError_t e = cudaMalloc(&h.d_in, std::max<size_t>(2 * total, 256));
  if (e != cudaSuccess) return fail(NDF_ERR_MEMORY, "unable to allocate filtering workspace");
  h.d_out = h.d_in + total;
  for (int s = 0; s < 2 && e == cudaSuccess; ++s) {
    e = cudaMallocHost(&h.h_in[s], std::max<size_t>(h.slot_bytes, 256));
    if (e == cudaSuccess) e = cudaMallocHost(&h.h_out[s], std::max<size_t>(h.slot_bytes, 256));
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h.uploaded[s], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h.downloaded[s], cudaEventDisableTiming);
  }
  h.computed.assign(h.chunks.size(), nullptr);
  for (auto& ev : h.computed)
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h.start, cudaEventDisableTiming);
  for (cudaStream_t* s : {&h.up, &h.compute, &h.down})
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(s, cudaStreamNonBlocking);
  if (e != cudaSuccess) return cuda_fail(e, "batch host pipeline setup");
  h.pool = std::make_unique<CopyPool>(host_thread_count() - 1);
  b->host_ready = true;
  return NDF_OK;
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
    b->sm_count = plan->p.sm_count;
    int fam = plan->p.n_out > 0 ? family_for(plan->p) : -1;
    b->family_of.push_back(fam);
    b->pixels.push_back(plan->p.n_out);
    b->plans.push_back(std::move(plan));
  }
  cudaError_t e = cudaStreamCreateWithFlags(&b->capture, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
  for (int i = 0; i < kBranches && e == cudaSuccess; ++i) {
    e = cudaStreamCreateWithFlags(&b->branch[i], cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->join[i], cudaEventDisableTiming);
  }
  if (e != cudaSuccess) {
    destroy_batch(b);
    return cuda_fail(e, "batch streams");
  }
  std::vector<int> all(count);
  for (int i = 0; i < count; ++i) all[i] = i;
  int rc = build_segment(b, b->whole, all);
  if (rc != NDF_OK) {
    destroy_batch(b);
    return rc;
  }
  *out = b;
  return NDF_OK;
}

int ndf_batch_destroy(ndf_batch* batch) {
  destroy_batch(batch);
  return NDF_OK;
}

int32_t ndf_batch_launches(const ndf_batch* batch) { return batch ? batch->whole.launches : 0; }

int ndf_batch_run(ndf_batch* b, const void* const* d_in, void* const* d_out, void* stream) {
  if (!b) return fail(NDF_ERR_INVALID_CONFIGURATION, "missing batch");
  if (!d_in || !d_out) return fail(NDF_ERR_LENGTH_MISMATCH, "missing input or output buffers");
  std::lock_guard<std::mutex> guard(b->lock);
  cudaStream_t user = (cudaStream_t)stream;
  Segment& s = b->whole;
  bool changed = s.exec == nullptr;
  for (size_t k = 0; k < s.images.size(); ++k)
    if (s.in_ptrs[k] != d_in[s.images[k]] || s.out_ptrs[k] != d_out[s.images[k]]) changed = true;
  if (changed) {
    // Earlier replays may still read the task staging tables.
    cudaError_t e = cudaStreamSynchronize(user);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->capture);
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamSynchronize");
    int rc = capture_segment(b, s, d_in, d_out);
    if (rc != NDF_OK) return rc;
  }
  cudaError_t e = cudaGraphLaunch(s.exec, user);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGraphLaunch");
  return NDF_OK;
}

int ndf_batch_run_host(ndf_batch* b, const void* const* h_in, void* const* h_out, void* stream) {
  if (!b) return fail(NDF_ERR_INVALID_CONFIGURATION, "missing batch");
  if (!h_in || !h_out) return fail(NDF_ERR_LENGTH_MISMATCH, "missing input or output buffers");
  std::lock_guard<std::mutex> guard(b->lock);
  const int count = (int)b->plans.size();
  for (int i = 0; i < count; ++i)
    if (b->pixels[i] > 0 && (!h_in[i] || !h_out[i]))
      return fail(NDF_ERR_LENGTH_MISMATCH, "missing input or output buffers");
  if (!b->host_ready) {
    int rc = setup_host(b);
    if (rc != NDF_OK) return rc;
  }
  HostPipeline& h = b->host;
  std::vector<const void*> d_in(count);
  std::vector<void*> d_out(count);
  for (int i = 0; i < count; ++i) {
    d_in[i] = h.d_in + h.offset[i];
    d_out[i] = h.d_out + h.offset[i];
  }
  cudaError_t e = cudaSuccess;
  for (auto& c : h.chunks) {
    int rc = capture_segment(b, c, d_in.data(), d_out.data());
    if (rc != NDF_OK) return rc;
  }
  // Start after the caller's earlier work on `stream`.
  e = cudaEventRecord(h.start, (cudaStream_t)stream);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(h.up, h.start, 0);
  if (e != cudaSuccess) return cuda_fail(e, "batch host run");
  const int groups = (int)h.chunks.size();
  auto span = [&](int c, size_t* base, size_t* bytes) {
    const int first = h.chunks[c].images.front(), last = h.chunks[c].images.back();
    *base = h.offset[first];
    *bytes = h.offset[last] + h.bytes[last] - h.offset[first];
  };
  auto download_to_user = [&](int c) -> cudaError_t {
    cudaError_t w = cudaEventSynchronize(h.downloaded[c & 1]);
    if (w != cudaSuccess) return w;
    size_t base, bytes;
    span(c, &base, &bytes);
    std::vector<CopyPool::Piece> pieces;
    for (int i : h.chunks[c].images)
      if (h.bytes[i]) add_pieces(pieces, h_out[i], h.h_out[c & 1] + (h.offset[i] - base), h.bytes[i]);
    h.pool->run(pieces);
    return cudaSuccess;
  };
  for (int c = 0; c < groups && e == cudaSuccess; ++c) {
    const int slot = c & 1;
    size_t base, bytes;
    span(c, &base, &bytes);
    // Pageable -> pinned slot (free once the upload of group c - 2 is done).
    if (c >= 2) e = cudaEventSynchronize(h.uploaded[slot]);
    if (e != cudaSuccess) break;
    std::vector<CopyPool::Piece> pieces;
    for (int i : h.chunks[c].images)
      if (h.bytes[i]) add_pieces(pieces, h.h_in[slot] + (h.offset[i] - base), h_in[i], h.bytes[i]);
    h.pool->run(pieces);
    e = cudaMemcpyAsync(h.d_in + base, h.h_in[slot], bytes, cudaMemcpyHostToDevice, h.up);
    if (e == cudaSuccess) e = cudaEventRecord(h.uploaded[slot], h.up);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(h.compute, h.uploaded[slot], 0);
    if (e == cudaSuccess) e = cudaGraphLaunch(h.chunks[c].exec, h.compute);
    if (e == cudaSuccess) e = cudaEventRecord(h.computed[c], h.compute);
    // Group c - 2's results leave the pinned slot before group c reuses it.
    if (e == cudaSuccess && c >= 2) e = download_to_user(c - 2);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(h.down, h.computed[c], 0);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(h.h_out[slot], h.d_out + base, bytes, cudaMemcpyDeviceToHost, h.down);
    if (e == cudaSuccess) e = cudaEventRecord(h.downloaded[slot], h.down);
  }
  for (int c = std::max(0, groups - 2); c < groups && e == cudaSuccess; ++c) e = download_to_user(c);
  if (e != cudaSuccess) {
    cudaDeviceSynchronize();
    return cuda_fail(e, "batch host run");
  }
  return status_take() ? fail(NDF_ERR_TIMEOUT, "a bounded device wait gave up") : NDF_OK;
}

}  // extern "C"
