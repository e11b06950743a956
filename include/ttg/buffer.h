// ttg::Buffer, ttg::devicescratch and ttg::TTValue for the GB300 runtime.
//
// Buffer<T> is the host/device-mirrored array of the TTG API (ttg/ttg/buffer.h, the PaRSEC
// implementation in ttg/ttg/parsec/buffer.h:190-541): a host array (owned, or borrowed through a
// unique_ptr with a custom deleter as examples/matrixtile.h:82-88 does) plus at most one copy in
// the GPU's HBM, with a version on each side. `select` makes the device copy current (H2D only
// when the host copy is newer); a mutable selection makes the device copy the newest; a host task
// or `wait(buffer)` brings the host copy up to date. Device memory comes from the runtime's
// caching pool and is kept for the buffer's lifetime, so a tile moves to HBM once.
#pragma once
#include <cuda_runtime_api.h>

#include <cstring>
#include <memory>
#include <mutex>
#include <type_traits>
#include <utility>

#include "ttg/runtime.h"

namespace ttg {

namespace detail {
// Type-erased state of one buffer, shared by the runtime's coherence logic.
struct BufferState {
  void* host = nullptr;
  void* dev = nullptr;
  size_t bytes = 0;
  uint64_t host_version = 1;  // a fresh buffer is current on the host
  uint64_t dev_version = 0;
  ttg::scope sc = ttg::scope::SyncIn;
  std::mutex m;
  cudaEvent_t dev_ready = nullptr;  // completes when the device copy is valid

  ~BufferState() {
    if (dev) rt::Runtime::get().release_device(dev, bytes);  // deferred while a device queue may read it
    if (dev_ready) cudaEventDestroy(dev_ready);
  }

  // Makes the device copy current for a task on stream s. Called on the task's worker thread.
  void* to_device(cudaStream_t s, bool sync_in) {
    std::lock_guard<std::mutex> lk(m);
    auto& R = rt::Runtime::get();
    if (!dev) {
      dev = R.pool().alloc(bytes);
      dev_version = 0;
    }
    if (sync_in && host_version > dev_version) {
      rt::cuda_check(cudaMemcpyAsync(dev, host, bytes, cudaMemcpyHostToDevice, s), "H2D");
      dev_version = host_version;
      if (!dev_ready) rt::cuda_check(cudaEventCreateWithFlags(&dev_ready, cudaEventDisableTiming), "event");
      rt::cuda_check(cudaEventRecord(dev_ready, s), "event record");
    } else if (dev_ready) {
      // another task may have staged it on another stream moments ago
      rt::cuda_check(cudaStreamWaitEvent(s, dev_ready, 0), "stream wait");
    }
    if (!sync_in && host_version > dev_version) dev_version = host_version;  // allocate-only scope
    return dev;
  }
  void mark_device_written() {
    std::lock_guard<std::mutex> lk(m);
    dev_version = std::max(dev_version, host_version) + 1;
  }
  // Device -> host on stream s (asynchronous); host becomes current once s reaches this point.
  void to_host_async(cudaStream_t s) {
    std::lock_guard<std::mutex> lk(m);
    if (dev && dev_version > host_version && host) {
      rt::cuda_check(cudaMemcpyAsync(host, dev, bytes, cudaMemcpyDeviceToHost, s), "D2H");
      host_version = dev_version;
    }
  }
  bool device_newer() {
    std::lock_guard<std::mutex> lk(m);
    return dev && dev_version > host_version && host;
  }
  // Synchronous version for host tasks. With a device queue, the operations recorded so far (which
  // may write this buffer) run first, unless the calling host job already waited for a batch.
  void to_host_sync() {
    if (!device_newer()) return;
    auto& R = rt::Runtime::get();
    cudaStream_t s = R.copy_stream();
    if (R.device_queue() && !device::detail::tl_after_flush()) {
      s = R.flush();
      rt::cuda_check(cudaStreamSynchronize(s), "device queue sync");
    }
    to_host_async(s);
    rt::cuda_check(cudaStreamSynchronize(s), "D2H sync");
  }
  void mark_host_written() {
    std::lock_guard<std::mutex> lk(m);
    host_version = std::max(host_version, dev_version) + 1;
  }
};
}  // namespace detail

template <typename T, typename Allocator = std::allocator<std::remove_const_t<T>>>
class Buffer {
 public:
  using value_type = std::remove_const_t<T>;
  using element_type = T;
  using pointer_type = T*;
  using const_pointer_type = const value_type*;

  Buffer() = default;
  explicit Buffer(std::size_t n, ttg::scope sc = ttg::scope::SyncIn) { reset(n, sc); }
  template <typename Deleter>
  Buffer(std::unique_ptr<value_type[], Deleter> ptr, std::size_t n, ttg::scope sc = ttg::scope::SyncIn) {
    m_count = n;
    m_deleter = [d = ptr.get_deleter()](value_type* p) mutable { d(p); };
    m_host = ptr.release();
    make_state(sc);
  }
  Buffer(std::shared_ptr<value_type[]> ptr, std::size_t n, ttg::scope sc = ttg::scope::SyncIn) {
    m_count = n;
    m_shared_host = ptr;
    m_host = ptr.get();
    m_deleter = [](value_type*) {};
    make_state(sc);
  }
  Buffer(Buffer&& o) noexcept { swap(o); }
  Buffer& operator=(Buffer&& o) noexcept {
    Buffer tmp(std::move(o));
    swap(tmp);
    return *this;
  }
  Buffer(const Buffer&) = delete;
  Buffer& operator=(const Buffer&) = delete;
  ~Buffer() { release_host(); }

  void reset(std::size_t n, ttg::scope sc = ttg::scope::SyncIn) {
    release_host();
    m_count = n;
    m_host = n ? new value_type[n]() : nullptr;
    m_deleter = [](value_type* p) { delete[] p; };
    make_state(sc);
  }

  std::size_t size() const { return m_count; }
  value_type* host_ptr() { return m_host; }
  const value_type* host_ptr() const { return m_host; }
  /// Device pointer of the copy made current by the last select (nullptr before).
  value_type* current_device_ptr() { return m_state ? static_cast<value_type*>(m_state->dev) : nullptr; }
  const value_type* current_device_ptr() const {
    return m_state ? static_cast<const value_type*>(m_state->dev) : nullptr;
  }
  value_type* device_ptr_on(const device::Device& d) { return d.is_device() ? current_device_ptr() : m_host; }
  const value_type* device_ptr_on(const device::Device& d) const {
    return d.is_device() ? current_device_ptr() : m_host;
  }
  value_type* owner_device_ptr() { return get_owner_device().is_device() ? current_device_ptr() : m_host; }
  bool is_current_on(const device::Device& d) const {
    if (!m_state) return !d.is_device();
    std::lock_guard<std::mutex> lk(m_state->m);
    return d.is_device() ? (m_state->dev && m_state->dev_version >= m_state->host_version)
                         : m_state->host_version >= m_state->dev_version;
  }
  bool is_valid_on(const device::Device& d) const { return is_current_on(d); }
  device::Device get_owner_device() const {
    if (!m_state) return device::Device::host();
    std::lock_guard<std::mutex> lk(m_state->m);
    return m_state->dev_version > m_state->host_version ? device::Device(0) : device::Device::host();
  }
  /// Declares the host copy current (e.g. after the application wrote it).
  void set_current_device(const device::Device& d) {
    if (!m_state) return;
    if (d.is_device()) m_state->mark_device_written();
    else m_state->mark_host_written();
  }
  void prefer_device(const device::Device&) {}
  void allocate_on(const device::Device&) {}
  ttg::scope scope() const { return m_state ? m_state->sc : ttg::scope::SyncIn; }
  bool empty() const { return m_count == 0; }

  detail::BufferState* state() const { return m_state.get(); }

  template <typename Archive>
  void serialize(Archive&) {}  // buffers are discovered by buffer_apply, never serialised here

 private:
  void make_state(ttg::scope sc) {
    m_state = std::make_shared<detail::BufferState>();
    m_state->host = m_host;
    m_state->bytes = m_count * sizeof(value_type);
    m_state->sc = sc;
    if (sc == ttg::scope::Allocate) m_state->host_version = 0;
  }
  void release_host() {
    if (m_host && m_deleter) m_deleter(m_host);
    m_host = nullptr;
    m_shared_host.reset();
    m_state.reset();
    m_count = 0;
  }
  void swap(Buffer& o) noexcept {
    std::swap(m_host, o.m_host);
    std::swap(m_count, o.m_count);
    std::swap(m_deleter, o.m_deleter);
    std::swap(m_shared_host, o.m_shared_host);
    std::swap(m_state, o.m_state);
  }

  value_type* m_host = nullptr;
  std::size_t m_count = 0;
  std::function<void(value_type*)> m_deleter;
  std::shared_ptr<value_type[]> m_shared_host;
  std::shared_ptr<detail::BufferState> m_state;
};

/// Device scratch space of a task (ttg/ttg/devicescratch.h, parsec/devicescratch.h:28-115): a view
/// of `count` host elements that gets a device copy at `select` — allocated only (scope Allocate)
/// or copied in (scope SyncIn) — and is copied back by `wait(scratch)`.
template <typename T>
class devicescratch {
 public:
  using element_type = std::decay_t<T>;
  devicescratch(element_type* host, ttg::scope sc = ttg::scope::SyncIn, std::size_t count = 1)
      : m_host(host), m_count(count), m_state(std::make_shared<detail::BufferState>()) {
    m_state->host = host;
    m_state->bytes = count * sizeof(element_type);
    m_state->sc = sc;
    if (sc == ttg::scope::Allocate) m_state->host_version = 0;
  }
  devicescratch(devicescratch&&) = default;
  devicescratch(const devicescratch&) = delete;
  element_type* device_ptr() { return static_cast<element_type*>(m_state->dev); }
  const element_type* device_ptr() const { return static_cast<const element_type*>(m_state->dev); }
  element_type* host_ptr() { return m_host; }
  std::size_t size() const { return m_count; }
  ttg::scope scope() const { return m_state->sc; }
  detail::BufferState* state() const { return m_state.get(); }

 private:
  element_type* m_host;
  std::size_t m_count;
  std::shared_ptr<detail::BufferState> m_state;
};

template <typename T>
devicescratch<T> make_scratch(T* host, ttg::scope sc, std::size_t count = 1) {
  return devicescratch<T>(host, sc, count);
}

/// Base of values that carry buffers (ttg/ttg/ttvalue.h). Here it only marks the type.
template <typename Derived>
struct TTValue {};

namespace meta {
template <typename T>
struct is_buffer : std::false_type {};
template <typename T, typename A>
struct is_buffer<Buffer<T, A>> : std::true_type {};
template <typename T, typename A>
struct is_buffer<const Buffer<T, A>> : std::true_type {};
template <typename T>
inline constexpr bool is_buffer_v = is_buffer<std::remove_reference_t<T>>::value;
template <typename T>
struct is_devicescratch : std::false_type {};
template <typename T>
struct is_devicescratch<devicescratch<T>> : std::true_type {};
template <typename T>
struct is_devicescratch<const devicescratch<T>> : std::true_type {};
template <typename T>
inline constexpr bool is_devicescratch_v = is_devicescratch<std::remove_reference_t<T>>::value;
}  // namespace meta

namespace detail {
// Visits every ttg::Buffer inside a value through the value's serialize(ar) member, the way the
// reference enumerates buffers (ttg/ttg/buffer.h:58-147): the archive calls `fn` on buffers,
// recurses into members that have serialize(), and ignores everything else.
template <typename Fn>
struct BufferVisitor {
  Fn& fn;
  template <typename T>
  BufferVisitor& operator&(T& t) {
    visit(t);
    return *this;
  }
  template <typename T>
  BufferVisitor& operator<<(T& t) {
    visit(t);
    return *this;
  }
  template <typename T>
  void visit(T& t);
};

template <typename T, typename Ar, typename = void>
struct has_serialize1 : std::false_type {};
template <typename T, typename Ar>
struct has_serialize1<T, Ar, std::void_t<decltype(std::declval<T&>().serialize(std::declval<Ar&>()))>>
    : std::true_type {};
template <typename T, typename Ar, typename = void>
struct has_serialize2 : std::false_type {};
template <typename T, typename Ar>
struct has_serialize2<T, Ar, std::void_t<decltype(std::declval<T&>().serialize(std::declval<Ar&>(), 0u))>>
    : std::true_type {};

template <typename Fn>
template <typename T>
void BufferVisitor<Fn>::visit(T& t) {
  using U = std::remove_const_t<T>;
  if constexpr (meta::is_buffer_v<U>) {
    fn(const_cast<U&>(t));
  } else if constexpr (has_serialize1<U, BufferVisitor<Fn>>::value) {
    const_cast<U&>(t).serialize(*this);
  } else if constexpr (has_serialize2<U, BufferVisitor<Fn>>::value) {
    const_cast<U&>(t).serialize(*this, 0u);
  }
}

template <typename T, typename Fn>
void buffer_apply(T& value, Fn&& fn) {
  BufferVisitor<std::remove_reference_t<Fn>> v{fn};
  v.visit(value);
}

struct buffer_apply_dummy_fn {
  template <typename B>
  void operator()(B&) const {}
};
template <typename T>
inline constexpr bool has_buffer_apply_v =
    meta::is_buffer_v<T> || has_serialize1<T, BufferVisitor<buffer_apply_dummy_fn>>::value ||
    has_serialize2<T, BufferVisitor<buffer_apply_dummy_fn>>::value;

/// True when some buffer of `value` has a newer device copy than host copy.
template <typename T>
bool value_on_device(T& value) {
  bool any = false;
  if constexpr (has_buffer_apply_v<std::remove_const_t<T>>) {
    buffer_apply(value, [&any](auto& b) {
      if (auto* s = b.state()) any = any || s->device_newer();
    });
  }
  return any;
}

/// Brings every buffer of `value` up to date on the host (before a host task reads it).
template <typename T>
void sync_value_to_host(T& value) {
  if constexpr (has_buffer_apply_v<std::remove_const_t<T>>) {
    buffer_apply(value, [](auto& b) {
      if (auto* s = b.state()) s->to_host_sync();
    });
  }
}
}  // namespace detail

}  // namespace ttg
