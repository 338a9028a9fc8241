// Host side of TMA staging (tensor maps) and of the device status word, plus
// the self-test of the bounded mbarrier wait.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <cstdlib>
#include <mutex>
#include <string>

#include "../../include/ndfiltrs_gb300.h"
#include "plan.h"
#include "tma.cuh"

namespace ndf {

int fail(int code, const std::string& message);
int cuda_fail(cudaError_t e, const char* what);

namespace {

struct TmaState {
  std::once_flag once;
  PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
  int smem_optin = 0;
  int enabled = -1;  // -1: from the environment (NDF_TMA, default on)
  std::mutex lock;
};

TmaState& tma_state() {
  static TmaState s;
  return s;
}

void tma_init(TmaState& s) {
  std::call_once(s.once, [&] {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult found = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &found) ==
            cudaSuccess &&
        found == cudaDriverEntryPointSuccess)
      s.encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    int dev = 0;
    if (cudaGetDevice(&dev) == cudaSuccess)
      cudaDeviceGetAttribute(&s.smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaGetLastError();
  });
}

bool tma_enabled(TmaState& s) {
  std::lock_guard<std::mutex> g(s.lock);
  if (s.enabled < 0) {
    const char* env = std::getenv("NDF_TMA");
    s.enabled = (env && *env == '0') ? 0 : 1;
  }
  return s.enabled != 0;
}

struct StatusWord {
  std::once_flag once;
  unsigned int* host = nullptr;
  unsigned int* device = nullptr;
};

StatusWord& status_state() {
  static StatusWord w;
  return w;
}

// A wait that nothing completes: thread 0 arms the barrier for two arrivals
// and arrives once, so every thread's bounded wait runs out.
__global__ void wait_selftest_kernel(unsigned int* status, unsigned long long limit_ns) {
  __shared__ __align__(8) unsigned long long bar;
  if (threadIdx.x == 0) {
    tma::mbar_init(&bar, 2);
    tma::fence_barrier_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) tma::mbar_arrive(&bar);
  tma::mbar_wait(&bar, 0, limit_ns, status);
}

}  // namespace

unsigned int* status_word_device() {
  StatusWord& w = status_state();
  std::call_once(w.once, [&] {
    void* h = nullptr;
    if (cudaHostAlloc(&h, sizeof(unsigned int), cudaHostAllocMapped) == cudaSuccess) {
      void* d = nullptr;
      if (cudaHostGetDevicePointer(&d, h, 0) == cudaSuccess) {
        w.host = static_cast<unsigned int*>(h);
        w.device = static_cast<unsigned int*>(d);
        *w.host = 0;
      } else {
        cudaFreeHost(h);
      }
    }
    cudaGetLastError();
  });
  return w.device;
}

unsigned int status_take() {
  StatusWord& w = status_state();
  if (!w.host) return 0;
  volatile unsigned int* word = w.host;
  const unsigned int v = *word;
  if (v) *word = 0;
  return v;
}

bool tma_prepare(const Plan& p, const Tile& t, const void* in, CUtensorMap* map, TileArgs* a, size_t* smem) {
  a->tma_bw = 0;
  a->status = status_word_device();
  TmaState& s = tma_state();
  if (!tma_enabled(s)) return false;
  tma_init(s);
  const Geom3& g = p.tile.g;
  if (!s.encode || g.H == 1 || !in) return false;
  const size_t elem = p.dtype == 0 ? 4 : 8;
  const int align = (int)(16 / elem);
  const int rank = g.D > 1 ? 3 : 2;
  if (((uintptr_t)in & 15) != 0 || ((size_t)g.W * elem) % 16 != 0) return false;
  if (g.W >= (1ll << 31) || g.H >= (1ll << 31) || g.D >= (1ll << 31)) return false;
  const int bw = (t.SW + align - 1 + align - 1) / align * align;
  if (bw > 256 || t.SH > 256 || g.kd > 256) return false;
  const size_t offset = (*smem + 15) / 16 * 16;
  const size_t raw = (size_t)bw * t.SH * g.kd * elem;
  const size_t total = offset + 127 + raw;
  if (total > (size_t)s.smem_optin || raw >= (1u << 20)) return false;
  cuuint64_t dims[3] = {(cuuint64_t)g.W, (cuuint64_t)g.H, (cuuint64_t)g.D};
  cuuint64_t strides[2] = {(cuuint64_t)(g.W * elem), (cuuint64_t)(g.W * g.H * elem)};
  cuuint32_t box[3] = {(cuuint32_t)bw, (cuuint32_t)t.SH, (cuuint32_t)g.kd};
  cuuint32_t estride[3] = {1, 1, 1};
  CUresult r = s.encode(map, p.dtype == 0 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64,
                        (cuuint32_t)rank, const_cast<void*>(in), dims, strides, box, estride,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return false;
  a->tma_bw = bw;
  a->tma_rank = rank;
  a->tma_offset = (int)offset;
  *smem = total;
  return true;
}

}  // namespace ndf

extern "C" {

int ndf_set_tma(int32_t enabled) {
  ndf::TmaState& s = ndf::tma_state();
  std::lock_guard<std::mutex> g(s.lock);
  s.enabled = enabled ? 1 : 0;
  return NDF_OK;
}

int ndf_device_status(uint32_t* flags) {
  cudaError_t e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return ndf::cuda_fail(e, "cudaDeviceSynchronize");
  const unsigned int v = ndf::status_take();
  if (flags) *flags = v;
  return v ? ndf::fail(NDF_ERR_TIMEOUT, "a bounded device wait gave up") : NDF_OK;
}

int ndf_selftest_wait_timeout(void) {
  unsigned int* status = ndf::status_word_device();
  if (!status) return ndf::fail(NDF_ERR_NO_DEVICE, "no usable CUDA device");
  cudaStream_t s = nullptr;
  cudaError_t e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  if (e != cudaSuccess) return ndf::cuda_fail(e, "cudaStreamCreate");
  ndf::wait_selftest_kernel<<<1, 64, 0, s>>>(status, 2000000ull);  // 2 ms
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaStreamDestroy(s);
  if (e != cudaSuccess) return ndf::cuda_fail(e, "wait self-test");
  return ndf::status_take() ? ndf::fail(NDF_ERR_TIMEOUT, "a bounded device wait gave up") : NDF_OK;
}

}  // extern "C"
