// Autotuner: the kernel choice of a tileable plan (sliding histogram, box
// pair kernel, register network or radix select, and their output tiles;
// the moments tile) measured on the device and cached per (device, dtype,
// statistic, invalid-value policy, window box, tap count, footprint class).
//
// Every candidate computes bit-identical order statistics (and the moments
// candidates differ only in their tiles), so a cached choice changes speed,
// never results. A key is measured once: each candidate filters a seeded
// synthetic image of a fixed shape (1-D 1M samples, 2-D 1024 x 1024, 3-D
// 8 x 256 x 512; N(1000, 10)-like values, 1% NaN, 0.2% outliers) once to
// warm up and three times under CUDA events; the fastest wins. Choices live
// in memory and, unless disabled, in a text file (one "key algo tw th ms"
// line per choice) so that later processes reuse them.
#include <sys/stat.h>

#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <limits>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/ndfiltrs_gb300.h"
#include "common.cuh"
#include "plan.h"

namespace ndf {

int fail(int code, const std::string& message);

namespace {

struct TuneEntry {
  Candidate c;
  double ms = 0.0;
};

struct TuneCache {
  std::mutex lock;
  int mode = -1;  // -1: not read from the environment yet
  bool path_set = false;
  std::string path;  // "" keeps choices in memory only
  bool loaded = false;
  std::map<std::string, TuneEntry> entries;
  std::string pinned;  // kernel family every choice takes when offered
};

TuneCache& cache() {
  static TuneCache c;
  return c;
}

int mode_locked(TuneCache& c) {
  if (c.mode < 0) {
    const char* env = std::getenv("NDF_AUTOTUNE");
    int m = env && *env ? std::atoi(env) : 1;
    c.mode = m < 0 ? 0 : (m > 2 ? 2 : m);
  }
  return c.mode;
}

std::string default_path() {
  if (const char* env = std::getenv("NDF_AUTOTUNE_CACHE")) return env;
  std::string base;
  if (const char* xdg = std::getenv("XDG_CACHE_HOME"); xdg && *xdg)
    base = xdg;
  else if (const char* home = std::getenv("HOME"); home && *home)
    base = std::string(home) + "/.cache";
  else
    return "";
  return base + "/ndfiltrs_gb300/autotune.txt";
}

const char* algo_token(Algo a) {
  switch (a) {
    case Algo::kHistogram:
      return "histogram";
    case Algo::kTileBox:
      return "box";
    case Algo::kTileNetwork:
      return "network";
    case Algo::kTileRank:
      return "ranked";
    case Algo::kTileRadix:
      return "radix";
    case Algo::kMomentsTile:
      return "moments";
    case Algo::kMomentsSlide:
      return "slide";
    case Algo::kExtremaTile:
      return "extrema";
    case Algo::kBoxcarTile:
      return "boxcar";
    case Algo::kBoxcarBand:
      return "band";
    case Algo::kExtremaPasses:
      return "passes";
    default:
      return "other";
  }
}

bool parse_algo(const std::string& t, Algo* a) {
  static const std::pair<const char*, Algo> names[] = {{"histogram", Algo::kHistogram},
                                                       {"box", Algo::kTileBox},
                                                       {"network", Algo::kTileNetwork},
                                                       {"ranked", Algo::kTileRank},
                                                       {"radix", Algo::kTileRadix},
                                                       {"moments", Algo::kMomentsTile},
                                                       {"slide", Algo::kMomentsSlide},
                                                       {"extrema", Algo::kExtremaTile},
                                                       {"boxcar", Algo::kBoxcarTile},
                                                       {"band", Algo::kBoxcarBand},
                                                       {"passes", Algo::kExtremaPasses}};
  for (const auto& n : names)
    if (t == n.first) {
      *a = n.second;
      return true;
    }
  return false;
}

void load_locked(TuneCache& c) {
  if (c.loaded) return;
  c.loaded = true;
  if (!c.path_set) {
    c.path = default_path();
    c.path_set = true;
  }
  if (c.path.empty()) return;
  std::ifstream in(c.path);
  std::string line;
  while (std::getline(in, line)) {
    std::istringstream fields(line);
    std::string key, algo;
    TuneEntry e;
    if (!(fields >> key >> algo >> e.c.tw >> e.c.th >> e.ms)) continue;
    if (!parse_algo(algo, &e.c.algo)) continue;
    c.entries[key] = e;
  }
}

void make_dirs(const std::string& path) {
  for (size_t i = 1; i < path.size(); ++i)
    if (path[i] == '/') {
      std::string dir = path.substr(0, i);
      if (mkdir(dir.c_str(), 0755) != 0 && errno != EEXIST) return;
    }
}

void append_locked(TuneCache& c, const std::string& key, const TuneEntry& e) {
  if (c.path.empty()) return;
  make_dirs(c.path);
  std::ofstream out(c.path, std::ios::app);
  if (!out) return;  // an unwritable cache only costs re-measuring later
  out << key << ' ' << algo_token(e.c.algo) << ' ' << e.c.tw << ' ' << e.c.th << ' ' << e.ms << '\n';
}

const char* statistic_class(const Reduce& r) {
  switch (r.kind) {
    case kMedian:
    case kMedianNetwork:
    case kMedianHistogram:
      return "median";
    case kRank:
    case kRankHistogram:
      return "rank";
    case kMin:
    case kMax:
      return "extremum";
    case kPercentile:
      return r.q_is_max ? "extremum" : "percentile";
    case kMean:
    case kVar:
    case kStd:
      return r.moments ? "moments64" : "moments32c";
    case kMeanRolling:
      return "boxcar";
    default:
      return "other";
  }
}

std::string key_of(const Plan& p) {
  static std::once_flag once;
  static int major = 0, minor = 0;
  std::call_once(once, [] {
    int dev = 0;
    if (cudaGetDevice(&dev) == cudaSuccess) {
      cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
      cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
    }
    cudaGetLastError();
  });
  const Geom3& g = p.tile.g;
  char buf[256];
  std::snprintf(buf, sizeof(buf), "sm%d%d-%d/%s/%s/%s/d%d%s/%dx%dx%d/V%d/%s", major, minor, p.sm_count,
                p.dtype == 0 ? "f32" : "f64", statistic_class(p.r), p.r.omit ? "omit" : "propagate",
                p.ndim, g.H == 1 ? "line" : "", g.kd, g.kh, g.kw, p.r.count,
                p.footprint.empty() ? "box" : "footprint");
  return buf;
}

bool same(const Candidate& a, const Candidate& b) {
  return a.algo == b.algo && a.tw == b.tw && a.th == b.th;
}

// Seeded N(1000, 10)-like samples (sum of four uniforms) with 1% NaN and
// 0.2% outliers in [2000, 60000).
template <typename T>
std::vector<T> synthetic(size_t n) {
  std::vector<T> v(n);
  unsigned long long state = 0x9E3779B97F4A7C15ull;
  auto next = [&]() {
    state ^= state << 13;
    state ^= state >> 7;
    state ^= state << 17;
    return (double)(state >> 11) * (1.0 / 9007199254740992.0);
  };
  for (size_t i = 0; i < n; ++i) {
    const double u = next();
    if (u < 0.01) {
      v[i] = std::numeric_limits<T>::quiet_NaN();
    } else if (u < 0.012) {
      v[i] = (T)(2000.0 + 58000.0 * next());
    } else {
      const double s = next() + next() + next() + next() - 2.0;
      v[i] = (T)(1000.0 + 10.0 * 1.7320508075688772 * s);
    }
  }
  return v;
}

// The tuning image keeps the plan's rank and, for 2-D plans of single-row
// images, their single row.
std::vector<long long> tuning_shape(const Plan& p) {
  if (p.ndim == 1) return {1ll << 20};
  if (p.ndim == 2) return p.tile.g.H == 1 ? std::vector<long long>{1, 1ll << 20}
                                          : std::vector<long long>{1024, 1024};
  return {8, 256, 512};
}

// Median of three timed runs of candidate `c` on the tuning image, in ms
// (infinity when the candidate cannot be set up).
double time_candidate(const Plan& p, const Candidate& c, int smem_limit, const std::vector<long long>& shape,
                      const void* d_in, void* d_out, cudaStream_t s, cudaEvent_t e0, cudaEvent_t e1) {
  Plan t;
  t.dtype = p.dtype;
  t.ndim = p.ndim;
  t.shape = shape;
  t.size = p.size;
  t.origin = p.origin;
  t.modes = p.modes;
  t.footprint = p.footprint;
  t.r = p.r;  // the percentile table stays owned by `p`
  t.taps = p.taps;
  t.device = p.device;
  t.sm_count = p.sm_count;
  t.n_out = 1;
  for (long long v : shape) t.n_out *= v;
  plan_setup_tile(t);
  double best = std::numeric_limits<double>::infinity();
  if (plan_apply(t, c, smem_limit) == NDF_OK && plan_run(t, d_in, d_out, s) == NDF_OK) {
    double runs[3];
    bool ok = true;
    for (int k = 0; k < 3 && ok; ++k) {
      ok = cudaEventRecord(e0, s) == cudaSuccess && plan_run(t, d_in, d_out, s) == NDF_OK &&
           cudaEventRecord(e1, s) == cudaSuccess && cudaEventSynchronize(e1) == cudaSuccess;
      float ms = 0.0f;
      if (ok) ok = cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess;
      runs[k] = ms;
    }
    if (ok) {
      std::sort(runs, runs + 3);
      best = runs[1];
    }
  }
  cudaStreamSynchronize(s);
  cudaGetLastError();
  plan_release(t);
  return best;
}

TuneEntry measure(const Plan& p, const std::vector<Candidate>& cands, int smem_limit) {
  TuneEntry pick{cands[0], std::numeric_limits<double>::infinity()};
  const std::vector<long long> shape = tuning_shape(p);
  size_t n = 1;
  for (long long v : shape) n *= (size_t)v;
  const size_t bytes = n * (p.dtype == 0 ? 4 : 8);
  void* d_in = nullptr;
  void* d_out = nullptr;
  cudaStream_t s = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t e = cudaMalloc(&d_in, bytes);
  if (e == cudaSuccess) e = cudaMalloc(&d_out, bytes);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  if (e == cudaSuccess) {
    if (p.dtype == 0) {
      std::vector<float> host = synthetic<float>(n);
      e = cudaMemcpy(d_in, host.data(), bytes, cudaMemcpyHostToDevice);
    } else {
      std::vector<double> host = synthetic<double>(n);
      e = cudaMemcpy(d_in, host.data(), bytes, cudaMemcpyHostToDevice);
    }
  }
  if (e == cudaSuccess) {
    for (const Candidate& c : cands) {
      const double ms = time_candidate(p, c, smem_limit, shape, d_in, d_out, s, e0, e1);
      if (ms < pick.ms) pick = TuneEntry{c, ms};
    }
  }
  cudaGetLastError();
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (s) cudaStreamDestroy(s);
  if (d_in) cudaFree(d_in);
  if (d_out) cudaFree(d_out);
  return pick;
}

}  // namespace

Candidate autotune_pick(const Plan& p, const std::vector<Candidate>& cands, int smem_limit) {
  TuneCache& c = cache();
  std::lock_guard<std::mutex> guard(c.lock);
  if (!c.pinned.empty())
    for (const Candidate& k : cands)
      if (c.pinned == algo_token(k.algo)) return k;
  const int mode = mode_locked(c);
  if (mode == 0) return cands[0];
  load_locked(c);
  const std::string key = key_of(p);
  auto it = c.entries.find(key);
  if (it != c.entries.end()) {
    for (const Candidate& k : cands)
      if (same(k, it->second.c)) return k;
  }
  if (!(mode == 2 || p.may_tune)) return cands[0];
  TuneEntry e = measure(p, cands, smem_limit);
  if (!std::isfinite(e.ms)) return cands[0];
  c.entries[key] = e;
  append_locked(c, key, e);
  return e.c;
}

}  // namespace ndf

extern "C" {

int ndf_set_autotune(int32_t mode, const char* cache_path) {
  using namespace ndf;
  if (mode < 0 || mode > 2) return fail(NDF_ERR_INVALID_CONFIGURATION, "autotune mode must be 0, 1 or 2");
  TuneCache& c = cache();
  std::lock_guard<std::mutex> guard(c.lock);
  c.mode = mode;
  if (cache_path) {
    c.path = cache_path;
    c.path_set = true;
    c.loaded = false;
    c.entries.clear();
  }
  return NDF_OK;
}

int ndf_pin_kernel(const char* family) {
  using namespace ndf;
  Algo a;
  if (family && *family && !parse_algo(family, &a))
    return fail(NDF_ERR_INVALID_CONFIGURATION, "unknown kernel family");
  TuneCache& c = cache();
  std::lock_guard<std::mutex> guard(c.lock);
  c.pinned = family ? family : "";
  return NDF_OK;
}

int32_t ndf_autotune_entries(void) {
  using namespace ndf;
  TuneCache& c = cache();
  std::lock_guard<std::mutex> guard(c.lock);
  load_locked(c);
  return (int32_t)c.entries.size();
}

}  // extern "C"
