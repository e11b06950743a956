// Host-side semantics of the TTG runtime: keyed matching, broadcast sharing, deferred writers,
// void keys, fused edges, priorities, composites, error propagation. Prints "PASS <name>" lines;
// exits non-zero on the first failure.
#include <ttg.h>

#include <atomic>
#include <chrono>
#include <cstdio>
#include <string>
#include <thread>

#define REQUIRE(c)                                                        \
  do {                                                                    \
    if (!(c)) {                                                           \
      std::fprintf(stderr, "FAIL %s:%d: %s\n", __FILE__, __LINE__, #c); \
      std::exit(1);                                                       \
    }                                                                     \
  } while (0)

using Key2 = ttg::MultiIndex<2>;

struct Val {
  int x = 0;
  static inline std::atomic<int> copies{0};
  Val() = default;
  explicit Val(int v) : x(v) {}
  Val(const Val& o) : x(o.x) { ++copies; }
  Val(Val&&) = default;
  Val& operator=(Val&&) = default;
};

static void fence() { ttg::fence(ttg::default_execution_context()); }

int main(int argc, char** argv) {
  ttg::initialize(argc, argv, 4);
  {  // keyed chain with two inputs per task
    ttg::Edge<int, Val> a("a"), b("b");
    std::atomic<int> last{-1};
    auto tt = ttg::make_tt([&](const int& k, const Val& x, Val&& y, std::tuple<ttg::Out<int, Val>, ttg::Out<int, Val>>& out) {
      last = k;
      if (k < 20) {
        ttg::send<0>(k + 1, Val(x.x + 1), out);
        ttg::send<1>(k + 1, Val(y.x + 2), out);
      } else {
        REQUIRE(x.x == 20 && y.x == 40);
      }
    }, ttg::edges(a, b), ttg::edges(a, b), "two_input_chain");
    REQUIRE(ttg::make_graph_executable(tt.get()));
    tt->invoke(0, Val(0), Val(0));
    fence();
    REQUIRE(last == 20);
    std::puts("PASS keyed-chain");
  }
  {  // broadcast: one value to const readers and one deferred mutable writer; no copy is made
    ttg::Edge<int, Val> src("src"), to_r("to_r"), to_w("to_w");
    std::atomic<int> readers_done{0}, writer_saw{-1};
    Val::copies = 0;
    auto prod = ttg::make_tt([&](const int& k, Val&& v, std::tuple<ttg::Out<int, Val>, ttg::Out<int, Val>>& out) {
      std::vector<int> rk{1, 2, 3, 4};
      ttg::broadcast<0, 1>(std::make_tuple(rk, 99), std::move(v), out);
    }, ttg::edges(src), ttg::edges(to_r, to_w), "producer");
    auto rd = ttg::make_tt([&](const int& k, const Val& v) {
      std::this_thread::sleep_for(std::chrono::milliseconds(20));
      REQUIRE(v.x == 7);
      ++readers_done;
    }, ttg::edges(to_r), ttg::edges(), "reader");
    auto wr = ttg::make_tt([&](const int& k, Val&& v) {
      writer_saw = readers_done.load();
      v.x = -1;
    }, ttg::edges(to_w), ttg::edges(), "writer");
    wr->set_defer_writer(true);
    REQUIRE(!ttg::make_graph_executable(prod.get()));  // `src` has no producer: reported, still runnable
    prod->invoke(0, Val(7));
    fence();
    REQUIRE(readers_done == 4);
    REQUIRE(writer_saw == 4);  // the writer waited for every reader
    REQUIRE(Val::copies == 0);
    std::puts("PASS broadcast-deferred-writer");
  }
  {  // without deferral the writer gets its own copy at once
    ttg::Edge<int, Val> src("src"), to_r("to_r"), to_w("to_w");
    std::atomic<int> bad{0};
    Val::copies = 0;
    auto prod = ttg::make_tt([&](const int& k, Val&& v, std::tuple<ttg::Out<int, Val>, ttg::Out<int, Val>>& out) {
      ttg::broadcast<0, 1>(std::make_tuple(std::vector<int>{1, 2}, 5), std::move(v), out);
    }, ttg::edges(src), ttg::edges(to_r, to_w), "producer");
    auto rd = ttg::make_tt([&](const int&, const Val& v) {
      std::this_thread::sleep_for(std::chrono::milliseconds(20));
      if (v.x != 3) ++bad;
    }, ttg::edges(to_r), ttg::edges(), "reader");
    auto wr = ttg::make_tt([&](const int&, Val&& v) { v.x = 100; }, ttg::edges(to_w), ttg::edges(), "writer");
    ttg::make_graph_executable(prod.get());
    prod->invoke(0, Val(3));
    fence();
    REQUIRE(bad == 0);
    REQUIRE(Val::copies == 1);
    std::puts("PASS broadcast-copy-on-write");
  }
  {  // void key task + control-only edges + fused inputs
    ttg::Edge<Key2, void> start("start");
    ttg::Edge<Key2, Val> e1("e1"), e2("e2");
    std::atomic<int> seen{0};
    auto init = ttg::make_tt<void>([&](std::tuple<ttg::Out<Key2, void>>& out) {
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j <= i; ++j) ttg::sendk<0>(Key2{i, j}, out);
    }, ttg::edges(), ttg::edges(start), "init");
    auto gen = ttg::make_tt([&](const Key2& k, std::tuple<ttg::Out<Key2, Val>, ttg::Out<Key2, Val>>& out) {
      if (k[0] == k[1]) ttg::send<0>(k, Val(k[0]), out);
      else ttg::send<1>(k, Val(k[0] * 10 + k[1]), out);
    }, ttg::edges(start), ttg::edges(e1, e2), "gen");
    auto sink = ttg::make_tt([&](const Key2& k, Val&& v) { ++seen; }, ttg::edges(ttg::fuse(e1, e2)), ttg::edges(), "sink");
    REQUIRE(ttg::make_graph_executable(init.get()));
    const std::string dot = ttg::Dot()(init.get());
    REQUIRE(dot.find("digraph") != std::string::npos && dot.find("sink") != std::string::npos);
    init->invoke();
    fence();
    REQUIRE(seen == 6);
    std::puts("PASS void-key-fuse-dot");
  }
  {  // an exception in a body reaches fence()
    ttg::Edge<int, Val> e("e");
    auto tt = ttg::make_tt([](const int& k, Val&& v) {
      if (k == 3) throw std::runtime_error("boom");
    }, ttg::edges(e), ttg::edges(), "thrower");
    ttg::make_graph_executable(tt.get());
    for (int k = 0; k < 5; ++k) tt->invoke(k, Val(k));
    bool caught = false;
    try {
      fence();
    } catch (const std::runtime_error& ex) {
      caught = std::string(ex.what()) == "boom";
    }
    REQUIRE(caught);
    std::puts("PASS error-propagation");
  }
  {  // a duplicate input for one key is an error, not a silent overwrite
    ttg::Edge<int, Val> e("e");
    auto tt = ttg::make_tt([](const int&, const Val&, const Val&) {}, ttg::edges(e, ttg::Edge<int, Val>("other")),
                           ttg::edges(), "dup");
    ttg::make_graph_executable(tt.get());
    bool caught = false;
    int k = 1;
    tt->in<0>()->deliver(&k, std::make_shared<ttg::detail::Holder<Val>>(Val(1)), true);
    try {
      tt->in<0>()->deliver(&k, std::make_shared<ttg::detail::Holder<Val>>(Val(1)), true);
    } catch (const std::runtime_error&) {
      caught = true;
    }
    REQUIRE(caught);
    std::puts("PASS duplicate-input-detected");
  }
  ttg::finalize();
  {  // priorities: with one worker, queued tasks run highest priority first
    ttg::initialize(argc, argv, 1);
    ttg::Edge<int, Val> e("e");
    std::vector<int> order;
    std::mutex m;
    auto tt = ttg::make_tt([&](const int& k, Val&&) {
      std::lock_guard<std::mutex> lk(m);
      order.push_back(k);
    }, ttg::edges(e), ttg::edges(), "prio");
    tt->set_priomap([](const int& k) { return k; });
    ttg::make_graph_executable(tt.get());
    for (int k : {3, 1, 4, 0, 2}) tt->invoke(k, Val(k));
    fence();
    REQUIRE((order == std::vector<int>{4, 3, 2, 1, 0}));
    std::puts("PASS priorities");
    ttg::finalize();
  }
  {  // ttg::abort(): throws by default (the error surfaces from fence); the opt-in reference-faithful
     // mode ends the process, checked by the test driver in a child process (argument "abort")
    REQUIRE(!ttg::abort_terminates());
    bool thrown = false;
    try {
      ttg::abort();
    } catch (const std::runtime_error&) {
      thrown = true;
    }
    REQUIRE(thrown);
    std::puts("PASS abort-throws");
    if (argc > 1 && std::string(argv[1]) == "abort") {
      ttg::set_abort_terminates(true);
      std::fflush(stdout);
      ttg::abort();  // does not return
    }
  }
  std::puts("ALL PASS");
  return 0;
}
