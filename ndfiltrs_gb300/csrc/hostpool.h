// A fixed pool of host threads for host-memory work that is bound by page
// faults and memory bandwidth: pageable <-> pinned copies, and first-touch of
// fresh output pages before a device-to-host copy (the kernel zero-fills a
// 64 KB page per fault; faulting in parallel threads instead of inside one
// copy is several times faster on the Grace host).
#pragma once

#include <algorithm>
#include <condition_variable>
#include <cstddef>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <thread>
#include <vector>

namespace ndf {

class CopyPool {
 public:
  // Copy `bytes` from src to dst, or (src == nullptr) touch every page of
  // dst so that it is resident.
  struct Piece {
    void* dst;
    const void* src;
    size_t bytes;
  };

  explicit CopyPool(int threads) {
    for (int i = 0; i < threads; ++i) workers_.emplace_back([this] { loop(); });
  }
  ~CopyPool() {
    {
      std::lock_guard<std::mutex> g(m_);
      stop_ = true;
    }
    cv_.notify_all();
    for (auto& t : workers_) t.join();
  }
  // Copies every piece and returns when all are done.
  void run(const std::vector<Piece>& pieces) {
    if (pieces.empty()) return;
    {
      std::lock_guard<std::mutex> g(m_);
      job_ = &pieces;
      next_ = 0;
      done_ = 0;
      ++generation_;
    }
    cv_.notify_all();
    work();
    std::unique_lock<std::mutex> g(m_);
    done_cv_.wait(g, [&] { return done_ == pieces.size(); });
    job_ = nullptr;
  }

 private:
  void work() {
    for (;;) {
      const Piece* p = nullptr;
      {
        std::lock_guard<std::mutex> g(m_);
        if (!job_ || next_ >= job_->size()) return;
        p = &(*job_)[next_++];
      }
      if (p->src) {
        std::memcpy(p->dst, p->src, p->bytes);
      } else {
        volatile unsigned char* c = static_cast<unsigned char*>(p->dst);
        for (size_t off = 0; off < p->bytes; off += 4096) c[off] = 0;
      }
      std::lock_guard<std::mutex> g(m_);
      if (++done_ == job_->size()) done_cv_.notify_all();
    }
  }
  void loop() {
    unsigned long long seen = 0;
    for (;;) {
      {
        std::unique_lock<std::mutex> g(m_);
        cv_.wait(g, [&] { return stop_ || (generation_ != seen && job_ && next_ < job_->size()); });
        if (stop_) return;
        seen = generation_;
      }
      work();
    }
  }

  std::vector<std::thread> workers_;
  std::mutex m_;
  std::condition_variable cv_, done_cv_;
  const std::vector<Piece>* job_ = nullptr;
  size_t next_ = 0, done_ = 0;
  unsigned long long generation_ = 0;
  bool stop_ = false;
};

// Split a copy into pieces of `piece` bytes.
inline void add_pieces(std::vector<CopyPool::Piece>& out, void* dst, const void* src, size_t bytes,
                       size_t piece = 4u << 20) {
  for (size_t off = 0; off < bytes; off += piece)
    out.push_back({(unsigned char*)dst + off, (const unsigned char*)src + off, std::min(piece, bytes - off)});
}

// Number of host threads the library works with (the calling thread plus
// the workers of a pool), fixed at the first call of the process: the value
// of RAYON_NUM_THREADS when it is a positive integer (the variable the
// reference's thread pool reads, so one setting sizes either library), else
// the hardware thread count capped at 16. get_num_threads() reports it.
inline int host_thread_count() {
  static const int count = [] {
    const char* env = std::getenv("RAYON_NUM_THREADS");
    if (env && *env) {
      char* end = nullptr;
      const long v = std::strtol(env, &end, 10);
      if (end && *end == '\0' && v > 0) return (int)std::min<long>(v, 1024);
    }
    const unsigned hc = std::thread::hardware_concurrency();
    return (int)std::max(1u, std::min(hc == 0 ? 4u : hc, 16u));
  }();
  return count;
}

// The process-wide pool used by plans (one job at a time; callers serialize
// through `lock`).
struct SharedHostPool {
  std::mutex lock;
  CopyPool* pool = nullptr;
};

inline SharedHostPool& shared_host_pool() {
  static SharedHostPool p;
  return p;
}

// Make every page of [p, p + bytes) resident using the shared pool; small
// buffers are left to the copy itself.
inline void prefault_pages(void* p, size_t bytes) {
  constexpr size_t kMin = 2u << 20, kPiece = 1u << 20;
  if (!p || bytes < kMin) return;
  SharedHostPool& s = shared_host_pool();
  std::lock_guard<std::mutex> guard(s.lock);
  if (!s.pool) s.pool = new CopyPool(host_thread_count() - 1);
  std::vector<CopyPool::Piece> pieces;
  for (size_t off = 0; off < bytes; off += kPiece)
    pieces.push_back({static_cast<unsigned char*>(p) + off, nullptr, std::min(kPiece, bytes - off)});
  s.pool->run(pieces);
}

}  // namespace ndf
