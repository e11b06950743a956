// Device-task contract of the TTG API on the GB300 runtime: the scenarios of the reference's
// tests/unit/device_coro.cc:84-500 (devicebuf, devicebuf-inc, scratch, scratch-syncin, loop,
// device-host-tasks, empty-select), with the same increment kernel as tests/unit/cuda_kernel.cu.
// Prints "PASS <name>"; exits non-zero on the first failure.
#include <ttg.h>

#include <atomic>
#include <cstdio>

#define REQUIRE(c)                                                        \
  do {                                                                    \
    if (!(c)) {                                                           \
      std::fprintf(stderr, "FAIL %s:%d: %s\n", __FILE__, __LINE__, #c); \
      std::exit(1);                                                       \
    }                                                                     \
  } while (0)

__global__ void increment_kernel(double* buffer, std::size_t n, double* scratch) {
  const unsigned i = threadIdx.x;
  if (i < n) buffer[i] += 1.0;
  if (i == 0 && scratch) *scratch += 1.0;
}
static void increment_buffer(double* buffer, std::size_t n, double* scratch) {
  increment_kernel<<<1, (unsigned)(n < 32 ? 32 : n), 0, ttg::device::current_stream()>>>(buffer, n, scratch);
}

struct value_t {
  ttg::Buffer<double> db{1};
  int quark = 0;
  template <typename Archive>
  void serialize(Archive& ar) {
    ar& quark;
    ar& db;
  }
};

static void fence() { ttg::fence(ttg::default_execution_context()); }

int main(int argc, char** argv) {
  ttg::initialize(argc, argv, 4);
  {  // buffer discovery through serialize()
    value_t v;
    int n = 0;
    ttg::detail::buffer_apply(v, [&](auto&) { ++n; });
    REQUIRE(n == 1);
    std::puts("PASS buffer-inspection");
  }
  {  // devicebuf: select, an empty wait, forward a send — a 10-step chain
    ttg::Edge<int, value_t> edge;
    std::atomic<int> ran{0};
    auto fn = [&](const int& key, value_t&& val) -> ttg::device::Task {
      co_await ttg::device::select(val.db);
      REQUIRE(val.db.current_device_ptr() != nullptr);
      REQUIRE(ttg::device::current_device().is_device());
      co_await ttg::device::wait();
      ++ran;
      if (key < 10) co_await ttg::device::forward(ttg::device::send<0>(key + 1, std::move(val)));
    };
    auto tt = ttg::make_tt<ttg::ExecutionSpace::CUDA>(fn, ttg::edges(edge), ttg::edges(edge), "device_task", {"edge_in"},
                                                      {"edge_out"});
    ttg::make_graph_executable(tt);
    tt->invoke(0, value_t{});
    fence();
    REQUIRE(ran == 11);
    std::puts("PASS devicebuf");
  }
  {  // devicebuf-inc: a kernel increments the buffer each step; the host sees key+1 after wait
    ttg::Edge<int, value_t> edge;
    std::atomic<int> checks{0};
    auto fn = [&](const int& key, value_t&& val) -> ttg::device::Task {
      co_await ttg::device::select(val.db);
      increment_buffer(val.db.current_device_ptr(), val.db.size(), nullptr);
      co_await ttg::device::wait(val.db);
      REQUIRE(static_cast<int>(*val.db.host_ptr()) == key + 1);
      ++checks;
      if (key < 10) co_await ttg::device::forward(ttg::device::send<0>(key + 1, std::move(val)));
    };
    auto tt = ttg::make_tt<ttg::ExecutionSpace::CUDA>(fn, ttg::edges(edge), ttg::edges(edge), "device_task");
    ttg::make_graph_executable(tt);
    value_t v;
    *v.db.host_ptr() = 2.0;  // start from a non-zero value
    tt->invoke(2, std::move(v));
    fence();
    REQUIRE(checks == 9);
    std::puts("PASS devicebuf-inc");
  }
  {  // scratch (Allocate: nothing copied in) and scratch-syncin (copied in), both copied back by wait
    ttg::Edge<int, value_t> edge;
    std::atomic<int> ok{0};
    auto fn = [&](const int& key, value_t&& val) -> ttg::device::Task {
      double s_alloc = 0.0, s_sync = 5.0;
      auto a = ttg::make_scratch(&s_alloc, ttg::scope::Allocate);
      auto s = ttg::make_scratch(&s_sync, ttg::scope::SyncIn);
      co_await ttg::device::select(a, s, val.db);
      REQUIRE(a.device_ptr() != nullptr && s.device_ptr() != nullptr);
      cudaMemsetAsync(a.device_ptr(), 0, sizeof(double), ttg::device::current_stream());
      increment_buffer(val.db.current_device_ptr(), val.db.size(), a.device_ptr());
      increment_buffer(val.db.current_device_ptr(), val.db.size(), s.device_ptr());
      co_await ttg::device::wait(a, s);
      REQUIRE(static_cast<int>(s_alloc) == 1);
      REQUIRE(static_cast<int>(s_sync) == 6);
      ++ok;
      if (key < 5) co_await ttg::device::forward(ttg::device::send<0>(key + 1, std::move(val)));
    };
    auto tt = ttg::make_tt<ttg::ExecutionSpace::CUDA>(fn, ttg::edges(edge), ttg::edges(edge), "scratch");
    ttg::make_graph_executable(tt);
    tt->invoke(0, value_t{});
    fence();
    REQUIRE(ok == 6);
    std::puts("PASS scratch");
  }
  {  // loop: ten kernel/wait rounds inside one task
    ttg::Edge<int, value_t> edge;
    std::atomic<int> ok{0};
    auto fn = [&](const int& key, value_t&& val) -> ttg::device::Task {
      co_await ttg::device::select(val.db);
      for (int i = 0; i < 10; ++i) {
        increment_buffer(val.db.current_device_ptr(), val.db.size(), nullptr);
        co_await ttg::device::wait(val.db);
        REQUIRE(static_cast<int>(*val.db.host_ptr()) == i + 1);
      }
      ++ok;
    };
    auto tt = ttg::make_tt<ttg::ExecutionSpace::CUDA>(fn, ttg::edges(edge), ttg::edges(), "loop");
    ttg::make_graph_executable(tt);
    tt->invoke(0, value_t{});
    fence();
    REQUIRE(ok == 1);
    std::puts("PASS loop");
  }
  {  // device-host-tasks: the value ping-pongs between a device task and a host task
    ttg::Edge<int, value_t> d2h, h2d;
    std::atomic<int> host_checks{0};
    auto dev = ttg::make_tt<ttg::ExecutionSpace::CUDA>([&](const int& key, value_t&& val) -> ttg::device::Task {
      co_await ttg::device::select(val.db);
      increment_buffer(val.db.current_device_ptr(), val.db.size(), nullptr);
      co_await ttg::device::forward(ttg::device::send<0>(key, std::move(val)));
    }, ttg::edges(h2d), ttg::edges(d2h), "dev");
    auto host = ttg::make_tt([&](const int& key, value_t&& val, std::tuple<ttg::Out<int, value_t>>& out) {
      // the runtime brought the device's newest copy back before this host body runs
      REQUIRE(static_cast<int>(*val.db.host_ptr()) == 2 * key + 1);
      *val.db.host_ptr() += 1.0;
      val.db.set_current_device(ttg::device::Device::host());
      ++host_checks;
      if (key < 5) ttg::send<0>(key + 1, std::move(val), out);
    }, ttg::edges(d2h), ttg::edges(h2d), "host");
    ttg::make_graph_executable(dev.get());
    dev->invoke(0, value_t{});
    fence();
    REQUIRE(host_checks == 6);
    std::puts("PASS device-host-tasks");
  }
  {  // empty-select with a void key
    ttg::Edge<void, void> e;
    std::atomic<int> ok{0};
    auto tt = ttg::make_tt<ttg::ExecutionSpace::CUDA, void>([&]() -> ttg::device::Task {
      co_await ttg::device::select();
      ++ok;
    }, ttg::edges(), ttg::edges(), "empty");
    ttg::make_graph_executable(tt.get());
    tt->invoke();
    fence();
    REQUIRE(ok == 1);
    std::puts("PASS empty-select");
  }
  ttg::finalize();
  std::puts("ALL PASS");
  return 0;
}
