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
#include <shared_mutex>
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
/// Set while a host job that waited for a device-queue batch brings its inputs to the host: the
/// batch has completed, so no further run is needed before the copies.
inline bool& tl_after_flush() {
  thread_local bool f = false;
  return f;
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

/// A device task queue behind the device tasks (include/ttg/device/gbx_queue.h wires in the GB300
/// library's): while a queue is set, device task bodies see its recording stream as their current
/// stream, so the kernels they call append tile operations to it instead of launching, and the
/// runtime runs what was recorded in batches, one persistent launch per batch, on a stream of its
/// own. A batch runs when a device task waits for its buffers (`co_await wait(...)`), when the
/// workers fall idle with host tasks waiting for device data, and at `fence`.
struct DeviceQueue {
  virtual ~DeviceQueue() = default;
  virtual cudaStream_t record_stream() = 0;  // what device task bodies see as current_stream()
  virtual long long pending() = 0;           // operations recorded and not yet run
  virtual void run(cudaStream_t s) = 0;      // runs them on s (asynchronous)
  virtual void check(cudaStream_t s) = 0;    // synchronises s; throws if a run failed on the device
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
    if (dq_) {  // the device queue's last runs finish before the memory goes
      flush();
      reclaim(true);
      dq_.reset();
    }
    if (dev_ready_) {
      for (auto s : streams_) cudaStreamDestroy(s);
      streams_.clear();
      if (exec_stream_) cudaStreamDestroy(exec_stream_);
      exec_stream_ = nullptr;
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
  /// With a device queue, the operations still recorded are run and waited for.
  void fence() {
    execute();
    {
      std::unique_lock<std::mutex> lk(m_);
      idle_cv_.wait(lk, [this] { return active_ == 0 && q_.empty(); });
    }
    if (dq_) {
      flush();
      try {
        dq_->check(exec_stream_);
      } catch (...) {
        record_error(std::current_exception());
      }
      reclaim(true);
    }
    std::lock_guard<std::mutex> lk(m_);
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

  // ---- device queue ----
  /// Sets (or, with nullptr, clears) the device task queue. Call between executions, not while
  /// tasks run.
  void set_device_queue(std::shared_ptr<DeviceQueue> q) {
    ensure_device();
    if (q && !exec_stream_) cuda_check(cudaStreamCreateWithFlags(&exec_stream_, cudaStreamNonBlocking), "stream");
    if (!q && dq_) {
      flush();
      reclaim(true);
    }
    dq_ = std::move(q);
  }
  DeviceQueue* device_queue() { return dq_.get(); }

  /// Device memory a buffer gives back: with a device queue, kept until the runs that may still
  /// read it (everything recorded so far) have completed.
  void release_device(void* p, size_t bytes) {
    if (!p) return;
    if (!dq_) {
      pool_.release(p, bytes);
      return;
    }
    std::lock_guard<std::mutex> lk(frees_m_);
    pending_frees_.emplace_back(p, bytes);
  }

  /// Runs everything recorded so far (after the stage-in copies issued so far) on the queue's
  /// stream; the host tasks waiting for device data run once it has completed. Returns the stream.
  cudaStream_t flush() {
    std::lock_guard<std::mutex> lk(flush_m_);
    reclaim(false);
    // Taken BEFORE the queue's snapshot of its operations: a buffer freed, or a host job deferred,
    // before this point was read or produced by operations recorded before it, so by this run or
    // an earlier one; anything later belongs to a later run.
    std::vector<std::pair<void*, size_t>> frees;
    std::vector<Job> later;
    {
      std::lock_guard<std::mutex> fl(frees_m_);
      frees.swap(pending_frees_);
    }
    {
      std::lock_guard<std::mutex> ql(m_);
      later.swap(deferred_host_);
    }
    {
      // no task is between its stage-in copies and the recording of its operations here, so every
      // recorded operation's copies are before this event
      std::unique_lock<std::shared_mutex> st(stage_m_);
      cudaEvent_t staged;
      cuda_check(cudaEventCreateWithFlags(&staged, cudaEventDisableTiming), "event");
      cuda_check(cudaEventRecord(staged, copy_stream()), "event record");
      cuda_check(cudaStreamWaitEvent(exec_stream_, staged, 0), "stream wait");
      cuda_check(cudaEventDestroy(staged), "event destroy");
      dq_->run(exec_stream_);
    }
    cudaEvent_t done;
    cuda_check(cudaEventCreateWithFlags(&done, cudaEventDisableTiming), "event");
    cuda_check(cudaEventRecord(done, exec_stream_), "event record");
    {
      std::lock_guard<std::mutex> fl(frees_m_);
      inflight_frees_.emplace_back(done, std::move(frees));
    }
    for (auto& j : later) when_stream_done(exec_stream_, j.prio, std::move(j.fn));
    return exec_stream_;
  }
  cudaStream_t exec_stream() { return exec_stream_; }
  /// Held (shared) by a device task from its stage-in copies through the recording of its operations.
  std::shared_mutex& stage_mutex() { return stage_m_; }

  /// A counted host job that reads device data: runs after the next batch has completed.
  void defer_host(int64_t prio, std::function<void()> fn) {
    std::lock_guard<std::mutex> lk(m_);
    deferred_host_.push_back(Job{prio, seq_++, std::move(fn)});
  }

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
        ++busy_;
      }
      try {
        j.fn();
      } catch (...) {
        // task wrappers settle their own accounting; anything escaping here is recorded
        record_error(std::current_exception());
      }
      bool flush_now = false;
      {
        std::lock_guard<std::mutex> lk(m_);
        --busy_;
        // every worker idle, nothing ready, host tasks waiting for device data: run the batch
        flush_now = dq_ && busy_ == 0 && q_.empty() && !deferred_host_.empty();
      }
      if (flush_now) {
        try {
          flush();
        } catch (...) {
          record_error(std::current_exception());
        }
      }
    }
  }

  // gives the memory of completed runs back to the pool (all runs when `wait`)
  void reclaim(bool wait) {
    std::lock_guard<std::mutex> lk(frees_m_);
    size_t i = 0;
    for (; i < inflight_frees_.size(); ++i) {
      auto& f = inflight_frees_[i];
      if (wait) cuda_check(cudaEventSynchronize(f.first), "event sync");
      else if (cudaEventQuery(f.first) != cudaSuccess) break;
      for (auto& p : f.second) pool_.release(p.first, p.second);
      cudaEventDestroy(f.first);
    }
    inflight_frees_.erase(inflight_frees_.begin(), inflight_frees_.begin() + i);
    if (wait) {
      for (auto& p : pending_frees_) pool_.release(p.first, p.second);
      pending_frees_.clear();
    }
  }

  std::mutex m_;
  std::condition_variable cv_, idle_cv_;
  std::priority_queue<Job, std::vector<Job>, JobCmp> q_;
  std::vector<std::thread> workers_;
  uint64_t seq_ = 0;
  int64_t active_ = 0;
  int busy_ = 0;                    // workers running a job
  std::vector<Job> deferred_host_;  // host jobs waiting for the next device-queue batch
  bool stop_ = false, executing_ = false;
  std::exception_ptr error_;

  std::mutex dev_m_;
  bool dev_ready_ = false;
  std::vector<cudaStream_t> streams_;
  cudaStream_t copy_stream_ = nullptr;
  std::atomic<uint64_t> next_stream_{0};
  DevicePool pool_;

  std::shared_ptr<DeviceQueue> dq_;
  cudaStream_t exec_stream_ = nullptr;  // the device queue's runs and the copies that follow them
  std::mutex flush_m_, frees_m_;
  std::shared_mutex stage_m_;
  std::vector<std::pair<void*, size_t>> pending_frees_;
  std::vector<std::pair<cudaEvent_t, std::vector<std::pair<void*, size_t>>>> inflight_frees_;
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
