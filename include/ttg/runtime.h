// The single-process task runtime behind the TTG API on GB300.
//
// Replaces the PaRSEC backend's task core and device hooks (ttg/ttg/parsec/ttg.h:1203-1672,
// 2397-2727, 3828-3883): worker threads take ready tasks from a priority queue (priorities from
// each TT's priomap, the DPLASMA rules in examples/potrf/potrf.h:742-752); device tasks run on a
// pool of CUDA streams of the one local GPU and are resumed by stream callbacks; `fence` waits
// until no task is ready, running or in flight on the GPU. There is no MPI: rank 0 of 1.
#pragma once
#include <cuda_runtime_api.h>

#include <atomic>
#include <condition_variable>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <deque>
#include <exception>
#include <functional>
#include <iostream>
#include <memory>
#include <mutex>
#include <queue>
#include <sstream>
#include <stdexcept>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

namespace ttg {

enum class ExecutionSpace { Host, CUDA, HIP, L0 };
enum class scope { Allocate = 0x1, SyncIn = 0x2 };
enum class Runtime { PaRSEC, MADNESS, GB300 };
inline constexpr Runtime ttg_runtime = Runtime::GB300;

struct Void {};

// ---- tracing / printing (ttg/util/trace.h, ttg/util/print.h) -----------------------------------
namespace detail {
inline std::atomic<bool>& tracing_flag() {
  static std::atomic<bool> f{false};
  return f;
}
inline std::mutex& print_mutex() {
  static std::mutex m;
  return m;
}
}  // namespace detail

inline bool tracing() { return detail::tracing_flag().load(std::memory_order_relaxed); }
inline void trace_on() { detail::tracing_flag() = true; }
inline void trace_off() { detail::tracing_flag() = false; }

template <typename... Ts>
void print(const Ts&... ts) {
  std::ostringstream os;
  ((os << ts), ...);
  std::lock_guard<std::mutex> lk(detail::print_mutex());
  std::cout << os.str() << std::endl;
}
template <typename... Ts>
void print_error(const Ts&... ts) {
  std::ostringstream os;
  ((os << ts), ...);
  std::lock_guard<std::mutex> lk(detail::print_mutex());
  std::cerr << os.str() << std::endl;
}
template <typename... Ts>
void trace(const Ts&... ts) {
  if (tracing()) print(ts...);
}

// ---- device identity -----------------------------------------------------------------------------
namespace device {
class Device {
  int m_id = -1;  // -1: host
 public:
  Device() = default;
  explicit Device(int id) : m_id(id) {}
  int id() const { return m_id; }
  operator int() const { return m_id; }
  bool is_device() const { return m_id >= 0; }
  bool is_host() const { return m_id < 0; }
  static Device host() { return Device(); }
};

namespace detail {
inline Device& tl_device() {
  thread_local Device d;
  return d;
}
inline cudaStream_t& tl_stream() {
  thread_local cudaStream_t s = nullptr;
  return s;
}
}  // namespace detail

/// The device selected for the running device task (host outside of one).
inline Device current_device() { return detail::tl_device(); }
/// The CUDA stream of the running device task: launch its kernels here.
inline cudaStream_t current_stream() { return detail::tl_stream(); }
inline int num_devices() {
  static int n = [] {
    int c = 0;
    if (cudaGetDeviceCount(&c) != cudaSuccess) {
      cudaGetLastError();
      c = 0;
    }
    return c > 1 ? 1 : c;  // one GPU per process
  }();
  return n;
}
}  // namespace device

// ---- the runtime -------------------------------------------------------------------------------------
namespace rt {

inline void cuda_check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw std::runtime_error(std::string("ttg: ") + what + ": " + cudaGetErrorString(e));
}

struct Job {
  int64_t prio;
  uint64_t seq;
  std::function<void()> fn;
};
struct JobCmp {
  bool operator()(const Job& a, const Job& b) const {
    return a.prio < b.prio || (a.prio == b.prio && a.seq > b.seq);  // max priority, then FIFO
  }
};

// Caching device allocator: freed blocks are kept per size and reused.
class DevicePool {
  std::mutex m;
  std::unordered_map<size_t, std::vector<void*>> free_;
  size_t bytes_live = 0;

 public:
  void* alloc(size_t bytes) {
    bytes = (bytes + 255) & ~size_t(255);
    {
      std::lock_guard<std::mutex> lk(m);
      auto it = free_.find(bytes);
      if (it != free_.end() && !it->second.empty()) {
        void* p = it->second.back();
        it->second.pop_back();
        return p;
      }
    }
    void* p = nullptr;
    cuda_check(cudaMalloc(&p, bytes ? bytes : 256), "cudaMalloc");
    std::lock_guard<std::mutex> lk(m);
    bytes_live += bytes;
    return p;
  }
  void release(void* p, size_t bytes) {
    if (!p) return;
    bytes = (bytes + 255) & ~size_t(255);
    std::lock_guard<std::mutex> lk(m);
    free_[bytes].push_back(p);
  }
  void trim() {
    std::lock_guard<std::mutex> lk(m);
    for (auto& kv : free_)
      for (void* p : kv.second) cudaFree(p);
    free_.clear();
  }
};

class Runtime {
 public:
  static Runtime& get() {
    static Runtime* r = new Runtime();  // intentionally leaked: lives until exit
    return *r;
  }

  void initialize(int nthreads) {
    std::lock_guard<std::mutex> lk(m_);
    if (!workers_.empty()) return;
    if (nthreads <= 0) {
      const char* env = std::getenv("TTG_NUM_THREADS");
      nthreads = env ? std::atoi(env) : (int)std::thread::hardware_concurrency();
      if (nthreads <= 0) nthreads = 1;
    }
    stop_ = false;
    for (int i = 0; i < nthreads; ++i) workers_.emplace_back([this] { worker_loop(); });
  }

  void finalize() {
    {
      std::lock_guard<std::mutex> lk(m_);
      stop_ = true;
    }
    cv_.notify_all();
    for (auto& t : workers_) t.join();
    workers_.clear();
    {
      std::lock_guard<std::mutex> lk(m_);
      executing_ = false;  // a re-initialised runtime waits for execute() again
      stop_ = false;
    }
    if (dev_ready_) {
      for (auto s : streams_) cudaStreamDestroy(s);
      streams_.clear();
      pool_.trim();
      dev_ready_ = false;
    }
  }

  void execute() {
    {
      std::lock_guard<std::mutex> lk(m_);
      executing_ = true;
    }
    cv_.notify_all();
  }

  /// Waits until no task is ready, running or in flight on the GPU; rethrows the first task error.
  void fence() {
    execute();
    std::unique_lock<std::mutex> lk(m_);
    idle_cv_.wait(lk, [this] { return active_ == 0 && q_.empty(); });
    if (error_) {
      auto e = error_;
      error_ = nullptr;
      std::rethrow_exception(e);
    }
  }

  /// Queues a job. `active` counts it until it (and any continuation it registers) completes.
  void submit(int64_t prio, std::function<void()> fn) {
    {
      std::lock_guard<std::mutex> lk(m_);
      ++active_;
      q_.push(Job{prio, seq_++, std::move(fn)});
    }
    cv_.notify_one();
  }

  /// Re-queues a continuation of an already counted job (no new `active` count).
  void resubmit(int64_t prio, std::function<void()> fn) {
    {
      std::lock_guard<std::mutex> lk(m_);
      q_.push(Job{prio, seq_++, std::move(fn)});
    }
    cv_.notify_one();
  }

  /// Marks one counted job finished.
  void done() {
    std::lock_guard<std::mutex> lk(m_);
    if (--active_ == 0 && q_.empty()) idle_cv_.notify_all();
  }

  void hold() {  // an extra count (e.g. a device task waiting on its stream)
    std::lock_guard<std::mutex> lk(m_);
    ++active_;
  }

  void record_error(std::exception_ptr e) {
    std::lock_guard<std::mutex> lk(m_);
    if (!error_) error_ = e;
  }

  // ---- device side ----
  void ensure_device() {
    std::lock_guard<std::mutex> lk(dev_m_);
    if (dev_ready_) return;
    if (device::num_devices() < 1) throw std::runtime_error("ttg: a device task needs a CUDA device");
    cuda_check(cudaSetDevice(0), "cudaSetDevice");
    const char* env = std::getenv("TTG_NUM_STREAMS");
    const int ns = env ? std::max(1, std::atoi(env)) : 16;
    for (int i = 0; i < ns; ++i) {
      cudaStream_t s;
      cuda_check(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "cudaStreamCreate");
      streams_.push_back(s);
    }
    cuda_check(cudaStreamCreateWithFlags(&copy_stream_, cudaStreamNonBlocking), "cudaStreamCreate");
    dev_ready_ = true;
  }
  cudaStream_t pick_stream(int hint) {
    ensure_device();
    const size_t i = hint >= 0 ? (size_t)hint : (size_t)next_stream_.fetch_add(1);
    return streams_[i % streams_.size()];
  }
  cudaStream_t copy_stream() {
    ensure_device();
    return copy_stream_;
  }
  DevicePool& pool() { return pool_; }

  /// Runs `fn` on a worker (priority `prio`) once all work queued so far on `s` has finished.
  void when_stream_done(cudaStream_t s, int64_t prio, std::function<void()> fn) {
    auto* payload = new std::pair<int64_t, std::function<void()>>(prio, std::move(fn));
    cuda_check(cudaLaunchHostFunc(
                   s,
                   [](void* p) {
                     // no CUDA calls here: hand the continuation to a worker
                     auto* pl = static_cast<std::pair<int64_t, std::function<void()>>*>(p);
                     Runtime::get().resubmit(pl->first, std::move(pl->second));
                     delete pl;
                   },
                   payload),
               "cudaLaunchHostFunc");
  }

  bool executing() {
    std::lock_guard<std::mutex> lk(m_);
    return executing_;
  }

 private:
  Runtime() = default;

  void worker_loop() {
    for (;;) {
      Job j;
      {
        std::unique_lock<std::mutex> lk(m_);
        cv_.wait(lk, [this] { return stop_ || (executing_ && !q_.empty()); });
        if (stop_ && (q_.empty() || !executing_)) return;
        j = std::move(const_cast<Job&>(q_.top()));
        q_.pop();
      }
      try {
        j.fn();
      } catch (...) {
        // task wrappers settle their own accounting; anything escaping here is recorded
        record_error(std::current_exception());
      }
    }
  }

  std::mutex m_;
  std::condition_variable cv_, idle_cv_;
  std::priority_queue<Job, std::vector<Job>, JobCmp> q_;
  std::vector<std::thread> workers_;
  uint64_t seq_ = 0;
  int64_t active_ = 0;
  bool stop_ = false, executing_ = false;
  std::exception_ptr error_;

  std::mutex dev_m_;
  bool dev_ready_ = false;
  std::vector<cudaStream_t> streams_;
  cudaStream_t copy_stream_ = nullptr;
  std::atomic<uint64_t> next_stream_{0};
  DevicePool pool_;
};

}  // namespace rt

// ---- world / lifecycle (ttg/run.h:30-118, ttg/base/world.h) -----------------------------------------
class World {
 public:
  int rank() const { return 0; }
  int size() const { return 1; }
  void profile_on() {}
  void profile_off() {}
  bool profiling() const { return false; }
  void dag_on(const std::string&) {}
  void dag_off() {}
  void fence() { rt::Runtime::get().fence(); }
  void execute() { rt::Runtime::get().execute(); }
  World& impl() { return *this; }
};

inline World& default_execution_context() {
  static World w;
  return w;
}
inline World& ttg_default_execution_context() { return default_execution_context(); }

inline void initialize(int /*argc*/, char** /*argv*/, int num_threads = -1) {
  rt::Runtime::get().initialize(num_threads);
}
inline void finalize() { rt::Runtime::get().finalize(); }
inline void execute(World& = default_execution_context()) { rt::Runtime::get().execute(); }
inline void fence(World& = default_execution_context()) { rt::Runtime::get().fence(); }
inline void ttg_initialize(int argc, char** argv, int n = -1) { initialize(argc, argv, n); }
inline void ttg_finalize() { finalize(); }
inline void ttg_execute(World& w) { execute(w); }
inline void ttg_fence(World& w) { fence(w); }

/// The reference aborts the whole job here (MPI_Abort). By default a library cannot, so this
/// throws (the error then surfaces from ttg::fence). Opt-in, reference-faithful mode:
/// set_abort_terminates(true), or the environment variable TTG_ABORT_TERMINATES=1, makes it end
/// the process with std::abort().
inline bool& abort_terminates_flag() {
  static bool flag = [] {
    const char* e = std::getenv("TTG_ABORT_TERMINATES");
    return e != nullptr && e[0] == '1';
  }();
  return flag;
}
inline void set_abort_terminates(bool on) { abort_terminates_flag() = on; }
inline bool abort_terminates() { return abort_terminates_flag(); }
[[noreturn]] inline void abort() {
  if (abort_terminates()) {
    std::fputs("ttg::abort() called\n", stderr);
    std::abort();
  }
  throw std::runtime_error("ttg::abort() called");
}
[[noreturn]] inline void ttg_abort() { abort(); }

}  // namespace ttg

#define TTGUNUSED(x) ((void)(x))
