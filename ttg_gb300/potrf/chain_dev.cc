// Per-device-task overhead of the GB300 TTG runtime: a chain of device tasks, each waiting for its
// predecessor's output and sending to its successor (the measurement of the reference's
// examples/task-benchmarks/chain-ttg-dev.cc:191-192). Flows:
//   0  the chain is carried by keys only (no data; the task selects nothing)
//   1  one value with a one-int device buffer travels the chain (selected by every task)
// Usage: chain_dev [-f FLOWS] [-n TASKS] [-q]. Prints the time per task in microseconds. -q runs the
// device tasks through the device task queue (ttg/device/gbx_queue.h).
#include <ttg.h>
#include <ttg/device/gbx_queue.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <string>

struct Token : public ttg::TTValue<Token> {
  ttg::Buffer<int> b;
  Token() : b(1) {}
  Token(Token&&) = default;
  Token& operator=(Token&&) = default;
};

static int g_tasks = 20000;

static double run_keys() {
  ttg::Edge<int, void> I2N("I2N"), N2N("N2N");
  auto init = ttg::make_tt<void>([](std::tuple<ttg::Out<int, void>>& out) { ttg::sendk<0>(0, out); }, ttg::edges(),
                                 ttg::edges(I2N), "init", {}, {"start"});
  auto next = ttg::make_tt<ttg::ExecutionSpace::CUDA>(
      [](const int& key, std::tuple<ttg::Out<int, void>>& out) -> ttg::device::Task {
        co_await ttg::device::select();
        if (key < g_tasks) co_await ttg::device::forward(ttg::device::sendk<0>(key + 1, out));
      },
      ttg::edges(ttg::fuse(I2N, N2N)), ttg::edges(N2N), "next", {"in"}, {"out"});
  if (!ttg::make_graph_executable(init.get())) throw std::runtime_error("not connected");
  init->invoke();  // warm-up
  ttg::execute(ttg::default_execution_context());
  ttg::fence(ttg::default_execution_context());
  const auto t0 = std::chrono::high_resolution_clock::now();
  init->invoke();
  ttg::execute(ttg::default_execution_context());
  ttg::fence(ttg::default_execution_context());
  const auto t1 = std::chrono::high_resolution_clock::now();
  return std::chrono::duration<double, std::micro>(t1 - t0).count();
}

static double run_value() {
  ttg::Edge<int, Token> I2N("I2N"), N2N("N2N");
  auto init = ttg::make_tt<void>([](std::tuple<ttg::Out<int, Token>>& out) { ttg::send<0>(0, Token{}, out); },
                                 ttg::edges(), ttg::edges(I2N), "init", {}, {"start"});
  auto next = ttg::make_tt<ttg::ExecutionSpace::CUDA>(
      [](const int& key, Token&& v, std::tuple<ttg::Out<int, Token>>& out) -> ttg::device::Task {
        co_await ttg::device::select(v.b);
        if (key < g_tasks) co_await ttg::device::forward(ttg::device::send<0>(key + 1, std::move(v), out));
      },
      ttg::edges(ttg::fuse(I2N, N2N)), ttg::edges(N2N), "next", {"in"}, {"out"});
  if (!ttg::make_graph_executable(init.get())) throw std::runtime_error("not connected");
  init->invoke();  // warm-up
  ttg::execute(ttg::default_execution_context());
  ttg::fence(ttg::default_execution_context());
  const auto t0 = std::chrono::high_resolution_clock::now();
  init->invoke();
  ttg::execute(ttg::default_execution_context());
  ttg::fence(ttg::default_execution_context());
  const auto t1 = std::chrono::high_resolution_clock::now();
  return std::chrono::duration<double, std::micro>(t1 - t0).count();
}

int main(int argc, char** argv) {
  int flows = 0;
  bool queue = false;
  for (int i = 1; i < argc; ++i) {
    if (std::string(argv[i]) == "-q") queue = true;
    if (i + 1 >= argc) continue;
    if (std::string(argv[i]) == "-f") flows = std::atoi(argv[i + 1]);
    if (std::string(argv[i]) == "-n") g_tasks = std::atoi(argv[i + 1]);
  }
  ttg::initialize(argc, argv, -1);
  if (queue) ttg::device::use_gbx_queue();
  const double us = flows == 0 ? run_keys() : run_value();
  std::printf("# of tasks = %d\n", g_tasks + 1);
  std::printf("time elapsed (microseconds) = %g, avg %g\n", us, us / (g_tasks + 1));
  ttg::finalize();
  return 0;
}
