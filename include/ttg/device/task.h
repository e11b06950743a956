// ttg::device::Task — the C++20 coroutine protocol of device task bodies (ttg/ttg/device/task.h),
// driven by the GB300 runtime.
//
//   co_await ttg::device::select(buffers...)   stage buffers into HBM on the task's stream
//   <launch kernels on ttg::device::current_stream()>
//   co_await ttg::device::wait(buffers...)     (optional) copy buffers back, resume when done
//   co_await ttg::device::forward(send...)     sends that run once the stream has drained
//
// The runtime resumes the coroutine on a worker thread with current_device()/current_stream()
// set (ttg/ttg/device/device.h:119-146 semantics). Stage-in is stream-ordered, so the body
// continues right after `select` without a host round trip; `wait` and the final sends resume
// from a stream callback (the states INIT -> WAIT_TRANSFER -> WAIT_KERNEL -> SENDOUT -> COMPLETE
// of device/task.h:102-109).
#pragma once
#include <coroutine>
#include <exception>
#include <functional>
#include <tuple>
#include <utility>
#include <vector>

#include "ttg/buffer.h"
#include "ttg/tt.h"

namespace ttg::device {

namespace detail {

enum class State { None, Init, WaitTransfer, WaitKernel, SendOut, Complete };

struct BufRef {
  ttg::detail::BufferState* st;
  bool is_const;
  bool is_scratch;
};

template <typename T>
BufRef make_ref(T& b) {
  using U = std::remove_reference_t<T>;
  constexpr bool is_scratch = ttg::meta::is_devicescratch_v<U>;
  constexpr bool is_const = std::is_const_v<U> || std::is_const_v<typename std::decay_t<U>::element_type>;
  return BufRef{b.state(), is_const, is_scratch};
}

struct select_t {
  std::vector<BufRef> refs;
};
struct wait_t {
  std::vector<BufRef> refs;
};
/// A deferred send: runs once the task's kernels have completed.
struct send_t {
  std::function<void()> fn;
};

}  // namespace detail

/// Input list assembled at run time (ttg::device::Input of the reference).
struct Input {
  std::vector<detail::BufRef> refs;
  Input() = default;
  template <typename... Args>
  Input(Args&&... args) : refs{detail::make_ref(args)...} {}
  template <typename T>
  void add(T&& v) {
    refs.push_back(detail::make_ref(v));
  }
};

template <typename... Args>
[[nodiscard]] inline detail::select_t select(Args&&... args) {
  return detail::select_t{{detail::make_ref(args)...}};
}
[[nodiscard]] inline detail::select_t select(Input& in) { return detail::select_t{in.refs}; }

template <typename... Buffers>
[[nodiscard]] inline detail::wait_t wait(Buffers&&... args) {
  static_assert(((ttg::meta::is_buffer_v<std::decay_t<Buffers>> ||
                  ttg::meta::is_devicescratch_v<std::decay_t<Buffers>>) &&
                 ...),
                "Only ttg::Buffer and ttg::devicescratch can be waited on!");
  return detail::wait_t{{detail::make_ref(args)...}};
}

// ---- deferred sends (device/task.h:244-545) ------------------------------------------------------
template <size_t i, typename keyT, typename valueT, typename... out_keysT, typename... out_valuesT>
inline detail::send_t send(const keyT& key, valueT&& value, std::tuple<ttg::Out<out_keysT, out_valuesT>...>& t) {
  using V = std::decay_t<valueT>;
  auto holder = std::make_shared<V>(std::forward<valueT>(value));
  auto* term = &std::get<i>(t);
  return {[term, key, holder]() { term->send(key, std::move(*holder)); }};
}
template <size_t i, typename keyT, typename valueT>
inline detail::send_t send(const keyT& key, valueT&& value) {
  using V = std::decay_t<valueT>;
  auto* term = ttg::detail::get_out_terminal<std::decay_t<keyT>, V>(i, "ttg::device::send");
  auto holder = std::make_shared<V>(std::forward<valueT>(value));
  return {[term, key, holder]() { term->send(key, std::move(*holder)); }};
}
template <size_t i, typename keyT, typename... out_keysT, typename... out_valuesT>
inline detail::send_t sendk(const keyT& key, std::tuple<ttg::Out<out_keysT, out_valuesT>...>& t) {
  auto* term = &std::get<i>(t);
  return {[term, key]() { term->sendk(key); }};
}
template <size_t i, typename keyT>
inline detail::send_t sendk(const keyT& key) {
  auto* term = ttg::detail::get_out_terminal<std::decay_t<keyT>, void>(i, "ttg::device::sendk");
  return {[term, key]() { term->sendk(key); }};
}
template <size_t i, typename valueT, typename... out_keysT, typename... out_valuesT>
inline detail::send_t sendv(valueT&& value, std::tuple<ttg::Out<out_keysT, out_valuesT>...>& t) {
  using V = std::decay_t<valueT>;
  auto holder = std::make_shared<V>(std::forward<valueT>(value));
  auto* term = &std::get<i>(t);
  return {[term, holder]() { term->sendv(std::move(*holder)); }};
}

template <size_t I, size_t... Is, typename rangeT, typename valueT, typename... out_keysT, typename... out_valuesT>
[[nodiscard]] inline detail::send_t broadcast(rangeT&& keylists, valueT&& value,
                                              std::tuple<ttg::Out<out_keysT, out_valuesT>...>& t) {
  using V = std::decay_t<valueT>;
  using KL = std::decay_t<rangeT>;
  auto holder = std::make_shared<V>(std::forward<valueT>(value));
  auto kl = std::make_shared<KL>(std::forward<rangeT>(keylists));
  auto* tp = &t;
  return {[tp, kl, holder]() { ttg::broadcast<I, Is...>(*kl, std::move(*holder), *tp); }};
}
template <size_t I, size_t... Is, typename rangeT, typename... out_keysT, typename... out_valuesT>
[[nodiscard]] inline detail::send_t broadcastk(rangeT&& keylists, std::tuple<ttg::Out<out_keysT, out_valuesT>...>& t) {
  using KL = std::decay_t<rangeT>;
  auto kl = std::make_shared<KL>(std::forward<rangeT>(keylists));
  auto* tp = &t;
  return {[tp, kl]() { ttg::broadcastk<I, Is...>(*kl, *tp); }};
}

template <typename... Args>
[[nodiscard]] std::vector<detail::send_t> forward(Args&&... args) {
  return std::vector<detail::send_t>{std::forward<Args>(args)...};
}

// ---- the coroutine type ---------------------------------------------------------------------------
struct Task;

namespace detail {
struct promise_type {
  State state = State::None;
  std::vector<BufRef> select_refs, wait_refs;
  std::vector<send_t> sends;
  std::exception_ptr error;

  std::suspend_never initial_suspend() noexcept {
    state = State::Init;
    return {};
  }
  std::suspend_always final_suspend() noexcept {
    state = State::Complete;
    return {};
  }
  std::suspend_always await_transform(select_t&& s) {
    select_refs = std::move(s.refs);
    state = State::WaitTransfer;
    return {};
  }
  struct wait_awaiter {
    promise_type* p;
    bool await_ready() const noexcept { return false; }
    void await_suspend(std::coroutine_handle<>) const noexcept {}
    void await_resume() const noexcept {
      // the copies completed: the host holds the newest data of every waited buffer
    }
  };
  wait_awaiter await_transform(wait_t&& w) {
    wait_refs = std::move(w.refs);
    state = State::WaitKernel;
    return wait_awaiter{this};
  }
  std::suspend_always await_transform(send_t&& s) {
    sends.clear();
    sends.push_back(std::move(s));
    state = State::SendOut;
    return {};
  }
  std::suspend_always await_transform(std::vector<send_t>&& v) {
    sends = std::move(v);
    state = State::SendOut;
    return {};
  }
  void return_void() { state = State::Complete; }
  Task get_return_object();
  void unhandled_exception() {
    error = std::current_exception();
    state = State::Complete;
  }
};
}  // namespace detail

struct Task {
  using promise_type = detail::promise_type;
  std::coroutine_handle<promise_type> h;
  Task() = default;
  explicit Task(std::coroutine_handle<promise_type> hh) : h(hh) {}
  Task(Task&& o) noexcept : h(std::exchange(o.h, {})) {}
  Task& operator=(Task&& o) noexcept {
    std::swap(h, o.h);
    return *this;
  }
  Task(const Task&) = delete;
  ~Task() {
    if (h) h.destroy();
  }
  bool completed() const { return !h || h.promise().state == detail::State::Complete; }
};

inline Task detail::promise_type::get_return_object() {
  return Task{std::coroutine_handle<promise_type>::from_promise(*this)};
}

}  // namespace ttg::device

namespace ttg {

// Drives one device task to completion. Owns the coroutine frame and the task's inputs.
template <typename TTT>
struct DeviceDriver {
  using Handle = std::coroutine_handle<device::detail::promise_type>;
  TTT* tt;
  typename TTT::key_store key{};  // the body holds `const Key&` across suspensions: keep it alive here
  std::function<void()> release;  // releases the task's inputs and its runtime count
  device::Task task;
  cudaStream_t stream = nullptr;      // stage-in copies (and the kernels, without a device queue)
  cudaStream_t rec_stream = nullptr;  // with a device queue: its recording stream, what the body sees
  int64_t prio = 0;
  std::vector<device::detail::BufRef> touched;  // every buffer selected by the task

  static void start(std::shared_ptr<DeviceDriver> self) { self->advance(self); }

  void set_current() {
    device::detail::tl_device() = device::Device(0);
    device::detail::tl_stream() = rec_stream ? rec_stream : stream;
    ttg::detail::tl_outputs() = &tt->out_ptrs_;
  }
  static void clear_current() {
    device::detail::tl_device() = device::Device();
    device::detail::tl_stream() = nullptr;
    ttg::detail::tl_outputs() = nullptr;
  }

  // Runs the state machine from the coroutine's current suspension point.
  void advance(std::shared_ptr<DeviceDriver> self) {
    auto& pr = task.h.promise();
    for (;;) {
      if (pr.error) {
        auto e = pr.error;
        finish();
        rt::Runtime::get().record_error(e);
        return;
      }
      switch (pr.state) {
        case device::detail::State::WaitTransfer: {
          std::shared_lock<std::shared_mutex> staging;  // with a device queue: copies, then recording
          if (rec_stream) staging = std::shared_lock<std::shared_mutex>(rt::Runtime::get().stage_mutex());
          set_current();
          for (auto& r : pr.select_refs) {
            const bool sync_in = r.st->sc != ttg::scope::Allocate;
            r.st->to_device(stream, sync_in);
            if (!r.is_const) r.st->mark_device_written();
            touched.push_back(r);
          }
          pr.select_refs.clear();
          task.h.resume();  // the body launches its kernels now
          clear_current();
          continue;
        }
        case device::detail::State::WaitKernel: {
          // with a device queue, what was recorded so far (this task's operations included) runs
          // now, and the copies back follow the run on its stream
          cudaStream_t ws = rec_stream ? rt::Runtime::get().flush() : stream;
          for (auto& r : pr.wait_refs) {
            // a buffer this task holds mutably may have been changed by any kernel since select
            for (auto& t : touched)
              if (t.st == r.st && !t.is_const) {
                r.st->mark_device_written();
                break;
              }
            r.st->to_host_async(ws);
          }
          pr.wait_refs.clear();
          rt::Runtime::get().when_stream_done(ws, prio, [self]() {
            self->set_current();
            self->task.h.resume();
            clear_current();
            self->advance(self);
          });
          return;
        }
        case device::detail::State::SendOut:
        case device::detail::State::Complete: {
          if (rec_stream) {  // device queue: the successors' operations are ordered by their operands
            ttg::detail::tl_outputs() = &tt->out_ptrs_;
            try {
              for (auto& s : pr.sends) s.fn();
            } catch (...) {
              rt::Runtime::get().record_error(std::current_exception());
            }
            ttg::detail::tl_outputs() = nullptr;
            pr.sends.clear();
            finish();
            return;
          }
          rt::Runtime::get().when_stream_done(stream, prio, [self]() {
            auto& p = self->task.h.promise();
            ttg::detail::tl_outputs() = &self->tt->out_ptrs_;
            try {
              for (auto& s : p.sends) s.fn();
            } catch (...) {
              rt::Runtime::get().record_error(std::current_exception());
            }
            ttg::detail::tl_outputs() = nullptr;
            p.sends.clear();
            self->finish();
          });
          return;
        }
        default:
          finish();
          return;
      }
    }
  }

  void finish() {
    task = device::Task{};  // destroys the coroutine frame (and its scratch) after completion
    if (release) {
      auto r = std::move(release);
      release = nullptr;
      r();
    }
  }
};

template <ExecutionSpace Space, typename Key, typename Func, typename OutTerms, typename... Values>
void TT<Space, Key, Func, OutTerms, Values...>::run_task(const key_store& k, std::shared_ptr<Pending> sp) {
  auto& R = rt::Runtime::get();
  if constexpr (Space == ExecutionSpace::Host) {
    // with a device queue, a host task that reads device data waits for the next batch to complete
    if (R.device_queue() && !device::detail::tl_after_flush() &&
        inputs_on_device(*sp, std::make_index_sequence<numins>{})) {
      R.defer_host(priority(k), [this, k, sp]() {
        device::detail::tl_after_flush() = true;
        run_task(k, sp);
        device::detail::tl_after_flush() = false;
      });
      return;
    }
    std::vector<detail::InputRef> refs;
    try {
      sync_inputs_to_host(*sp, std::make_index_sequence<numins>{});
      input_refs(*sp, refs, std::make_index_sequence<numins>{});
      detail::tl_inputs() = &refs;
      detail::tl_outputs() = &out_ptrs_;
      call_body(k, *sp);
      detail::tl_outputs() = nullptr;
      detail::tl_inputs() = nullptr;
    } catch (...) {
      detail::tl_outputs() = nullptr;
      detail::tl_inputs() = nullptr;
      R.record_error(std::current_exception());
    }
    refs.clear();
    release_inputs(*sp);
    R.done();
  } else {
    using Drv = DeviceDriver<TT>;
    auto drv = std::make_shared<Drv>();
    drv->tt = this;
    drv->prio = priority(k);
    int hint = -1;
    if (devicemap_) hint = -1;  // one GPU: the device map cannot move work elsewhere
    if (auto* dq = R.device_queue()) {  // stage-in on the copy stream; kernels recorded into the queue
      drv->stream = R.copy_stream();
      drv->rec_stream = dq->record_stream();
    } else {
      drv->stream = R.pick_stream(hint);
    }
    drv->release = [this, sp]() {
      release_inputs(*sp);
      rt::Runtime::get().done();
    };
    drv->key = k;
    try {
      detail::tl_outputs() = &out_ptrs_;
      drv->task = call_body(drv->key, *sp);  // runs until the first suspension (select / wait / send)
      detail::tl_outputs() = nullptr;
    } catch (...) {
      detail::tl_outputs() = nullptr;
      R.record_error(std::current_exception());
      drv->finish();
      return;
    }
    if (!drv->task.h) {
      drv->finish();
      return;
    }
    Drv::start(drv);
  }
}

}  // namespace ttg
