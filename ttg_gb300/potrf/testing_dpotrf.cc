// Driver of the GB300 potrf flowgraph, with the command line of the reference's
// examples/potrf/testing_dpotrf.cc:41-87: -N order, -t tile size, -c worker threads, -n timed
// iterations, -x skip the check. Extra: -o FILE writes the factor tiles (tile-major lower
// storage) after the checked run; -s NRHS then solves A X = B through the solve flowgraph
// (potrs.h) for NRHS right-hand sides B(i, r) = ((7919 i + 104729 r) mod 1000) / 500 - 1, checks
// the normwise backward error and, with -p FILE, writes X (NRHS rows of N, row r = column r of X).
// -q runs the device tasks through the device task queue (ttg/device/gbx_queue.h): their tile
// kernels are recorded and each batch runs as one persistent launch.
//
// Each iteration generates the PLASMA test matrix (seed 3872, bump N) with one device task per
// tile, factorises it through the flowgraph and writes the factor back to the host matrix, all
// inside the timed region as the reference does. The check uses the reference's criterion
// ||L L^T - A||_inf / (||A||_inf N eps) < 60 (testing_dpotrf.cc:277-335).
#include <ttg.h>
#include <ttg/device/gbx_queue.h>

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <string>
#include <vector>

#include "potrf.h"
#include "potrs.h"

using namespace gbx_potrf;

static const char* opt(char** b, char** e, const std::string& o) {
  auto it = std::find(b, e, o);
  return (it != e && ++it != e) ? *it : nullptr;
}
static bool has(char** b, char** e, const std::string& o) { return std::find(b, e, o) != e; }

// device task per tile: the PLASMA generator into the matrix's tile slot
static auto make_plgsy_ttg(TiledMatrix<double>& A, int bump, unsigned long long seed, ttg::Edge<Key2, void>& start,
                           ttg::Edge<Key2, MatrixTile<double>>& out) {
  auto body = [&A, bump, seed](const Key2& key, std::tuple<ttg::Out<Key2, MatrixTile<double>>>& o) -> ttg::device::Task {
    const int I = key[0], J = key[1];
    MatrixTile<double> tile = A(I, J, ttg::scope::Allocate);  // generated on the device: nothing to copy in
    co_await ttg::device::select(tile.buffer());
    potrf::check_status(gbx_dplgsy_tile((double)bump, (int)tile.rows(), (int)tile.cols(), tile.buffer().current_device_ptr(),
                                        (int)tile.lda(), (int)A.rows_in_matrix(), I * (int)A.rows_in_tile(),
                                        J * (int)A.cols_in_tile(), seed, ttg::device::current_stream()),
                        "gbx_dplgsy_tile");
    co_await ttg::device::send<0>(key, std::move(tile), o);
  };
  return ttg::make_tt<ttg::ExecutionSpace::CUDA>(body, ttg::edges(start), ttg::edges(out), "PLGSY", {"startup"},
                                                 {"output"});
}

// host task per factor tile: bring it back into the host matrix (result.h of the reference)
static auto make_result_ttg(TiledMatrix<double>& A, ttg::Edge<Key2, MatrixTile<double>>& in) {
  auto body = [&A](const Key2& key, MatrixTile<double>&& tile, std::tuple<>&) {
    double* dst = A.tile_ptr(key[0], key[1]);
    if (dst != tile.data())  // a copy travelled: write every column of the tile back
      for (std::size_t j = 0; j < tile.cols(); ++j) std::copy_n(tile.data() + j * tile.lda(), tile.rows(), dst + j * tile.lda());
  };
  return ttg::make_tt(body, ttg::edges(in), ttg::edges(), "Result", {"result"}, {});
}

static double check_dpotrf(const TiledMatrix<double>& L, const TiledMatrix<double>& A0, int N) {
  auto at = [](const TiledMatrix<double>& M, long i, long j) {
    const int NB = (int)M.rows_in_tile();
    return M.tile_ptr((int)(i / NB), (int)(j / NB))[(i % NB) + (j % NB) * (long)NB];
  };
  std::vector<double> Ld((size_t)N * N, 0.0);
  for (long j = 0; j < N; ++j)
    for (long i = j; i < N; ++i) Ld[i + j * N] = at(L, i, j);
  double rnorm = 0, anorm = 0;
  std::vector<double> rowr(N, 0.0), rowa(N, 0.0);
  for (long j = 0; j < N; ++j)
    for (long i = 0; i < N; ++i) {
      const long lo = std::min(i, j);
      double s = 0;
      for (long k = 0; k <= lo; ++k) s += Ld[i + k * N] * Ld[j + k * N];
      const double a = i >= j ? at(A0, i, j) : at(A0, j, i);
      rowr[i] += std::fabs(s - a);
      rowa[i] += std::fabs(a);
    }
  for (int i = 0; i < N; ++i) {
    rnorm = std::max(rnorm, rowr[i]);
    anorm = std::max(anorm, rowa[i]);
  }
  return rnorm / (anorm * N * std::numeric_limits<double>::epsilon());
}

static void run_once(TiledMatrix<double>& A, int N, bool defer) {
  ttg::Edge<Key2, void> startup("startup");
  ttg::Edge<Key2, MatrixTile<double>> topotrf("To POTRF"), result("To result");
  auto init_tt = ttg::make_tt<void>([&](std::tuple<ttg::Out<Key2, void>>& out) {
    for (int i = 0; i < (int)A.rows(); i++)
      for (int j = 0; j <= i; j++) ttg::sendk<0>(Key2{i, j}, out);
  }, ttg::edges(), ttg::edges(startup), "Startup Trigger", {}, {"startup"});
  auto plgsy = make_plgsy_ttg(A, N, 3872, startup, topotrf);
  auto potrf_ttg = potrf::make_potrf_ttg(A, topotrf, result, defer);
  auto result_tt = make_result_ttg(A, result);
  if (!ttg::make_graph_executable(init_tt.get())) throw std::runtime_error("graph not connected");
  init_tt->invoke();
  ttg::execute(ttg::default_execution_context());
  ttg::fence(ttg::default_execution_context());
}

// the solve flowgraph on the factor in L; returns the normwise backward error against A0
static double run_solve(TiledMatrix<double>& L, const TiledMatrix<double>& A0, int N, int NB, int nrhs,
                        std::vector<double>& X) {
  std::vector<double> rhs(potrs::TiledRhs<double>::num_elements(N, NB, nrhs), 0.0);
  potrs::TiledRhs<double> B(rhs.data(), N, NB, nrhs);
  auto b_at = [](long i, int r) { return (double)((7919L * i + 104729L * r) % 1000) / 500.0 - 1.0; };
  for (long i = 0; i < N; ++i)
    for (int r = 0; r < nrhs; ++r) B.tile_ptr((int)(i / NB))[r + (i % NB) * nrhs] = b_at(i, r);
  ttg::Edge<Key2, potrs::Tile> lin("L tiles");
  ttg::Edge<Key1, potrs::Tile> bin("B tiles"), xout("X tiles");
  auto feed = ttg::make_tt<void>([&](std::tuple<ttg::Out<Key2, potrs::Tile>, ttg::Out<Key1, potrs::Tile>>& out) {
    for (int m = 0; m < (int)L.rows(); ++m)
      for (int k = 0; k <= m; ++k) ttg::send<0>(Key2{m, k}, L(m, k), out);
    for (int k = 0; k < B.tiles(); ++k) ttg::send<1>(Key1{k}, B(k), out);
  }, ttg::edges(), ttg::edges(lin, bin), "Solve inputs", {}, {"L", "B"});
  auto ops = potrs::make_potrs_ttg(L, nrhs, lin, bin, xout);
  auto result = ttg::make_tt([&B](const Key1& key, const potrs::Tile& x, std::tuple<>&) {
    double* dst = B.tile_ptr(key[0]);
    if (dst != x.data()) std::copy_n(x.data(), x.rows() * x.cols(), dst);
  }, ttg::edges(xout), ttg::edges(), "Solution", {"X"}, {});
  if (!ttg::make_graph_executable(feed.get())) throw std::runtime_error("solve graph not connected");
  feed->invoke();
  ttg::execute(ttg::default_execution_context());
  ttg::fence(ttg::default_execution_context());
  // X (row-major by right-hand side) and the backward error max_r ||b - A x||_inf / (||A||_inf ||x||_inf + ||b||_inf)
  X.assign((size_t)nrhs * N, 0.0);
  for (long i = 0; i < N; ++i)
    for (int r = 0; r < nrhs; ++r) X[(size_t)r * N + i] = B.tile_ptr((int)(i / NB))[r + (i % NB) * nrhs];
  auto a_at = [&](long i, long j) {
    if (i < j) std::swap(i, j);
    return A0.tile_ptr((int)(i / NB), (int)(j / NB))[(i % NB) + (j % NB) * (long)NB];
  };
  double anorm = 0.0, worst = 0.0;
  for (long i = 0; i < N; ++i) {
    double s = 0.0;
    for (long j = 0; j < N; ++j) s += std::fabs(a_at(i, j));
    anorm = std::max(anorm, s);
  }
  for (int r = 0; r < nrhs; ++r) {
    const double* x = X.data() + (size_t)r * N;
    double rmax = 0.0, xmax = 0.0, bmax = 0.0;
    for (long i = 0; i < N; ++i) {
      double s = b_at(i, r);
      for (long j = 0; j < N; ++j) s -= a_at(i, j) * x[j];
      rmax = std::max(rmax, std::fabs(s));
      xmax = std::max(xmax, std::fabs(x[i]));
      bmax = std::max(bmax, std::fabs(b_at(i, r)));
    }
    worst = std::max(worst, rmax / (anorm * xmax + bmax));
  }
  return worst;
}

int main(int argc, char** argv) {
  int NB = 32, N = 5 * NB, nthreads = -1, niter = 3;
  if (auto o = opt(argv + 1, argv + argc, "-N")) N = std::atoi(o);
  if (auto o = opt(argv + 1, argv + argc, "-t")) NB = std::atoi(o);
  if (auto o = opt(argv + 1, argv + argc, "-c")) nthreads = std::atoi(o);
  if (auto o = opt(argv + 1, argv + argc, "-n")) niter = std::atoi(o);
  const char* outfile = opt(argv + 1, argv + argc, "-o");
  const char* xfile = opt(argv + 1, argv + argc, "-p");
  int nrhs = 0;
  if (auto o = opt(argv + 1, argv + argc, "-s")) nrhs = std::atoi(o);
  const bool check = !has(argv + 1, argv + argc, "-x");
  const bool defer = !has(argv + 1, argv + argc, "-w");
  ttg::initialize(argc, argv, nthreads);
  if (has(argv + 1, argv + argc, "-q")) ttg::device::use_gbx_queue();
  std::printf("Creating 2D block cyclic matrix with NB %d N %d M %d P 1 Q 1\n", NB, N, N);
  std::vector<double> store(TiledMatrix<double>::num_elements(N, NB), 0.0);
  TiledMatrix<double> A(store.data(), N, NB);
  int ret = 0;
  try {
    for (int it = 0; it < (check ? 1 : niter); ++it) {
      auto beg = std::chrono::high_resolution_clock::now();
      run_once(A, N, defer);
      auto end = std::chrono::high_resolution_clock::now();
      const double us = std::chrono::duration_cast<std::chrono::microseconds>(end - beg).count();
      std::printf("TTG Execution Time (milliseconds) : %g : Flops %g %g GF/s\n", us / 1e3, potrf::FLOPS_DPOTRF(N),
                  potrf::FLOPS_DPOTRF(N) / 1e9 / (us / 1e6));
    }
    if (check) {
      std::vector<double> store0(store.size(), 0.0);
      TiledMatrix<double> A0(store0.data(), N, NB);
      // regenerate A0 on the device through the C ABI
      double* d = nullptr;
      cudaMalloc((void**)&d, store0.size() * sizeof(double));
      potrf::check_status(gbx_dplgsy_tiled(N, NB, (double)N, 3872, d, nullptr), "gbx_dplgsy_tiled");
      cudaMemcpy(store0.data(), d, store0.size() * sizeof(double), cudaMemcpyDeviceToHost);
      cudaFree(d);
      const double r = check_dpotrf(A, A0, N);
      std::printf("============\nChecking the Cholesky factorization\n-- ||LL'-A||_oo/(||A||_oo.N.eps) = %g\n", r);
      if (std::isnan(r) || std::isinf(r) || r > 60.0) {
        std::printf("-- Factorization is suspicious !\n");
        ret = 1;
      } else {
        std::printf("-- Factorization is CORRECT !\n");
      }
      if (outfile) {
        FILE* f = std::fopen(outfile, "wb");
        std::fwrite(store.data(), sizeof(double), store.size(), f);
        std::fclose(f);
      }
      if (nrhs > 0) {
        std::vector<double> X;
        auto beg = std::chrono::high_resolution_clock::now();
        const double be = run_solve(A, A0, N, NB, nrhs, X);
        auto end = std::chrono::high_resolution_clock::now();
        std::printf("TTG solve (%d right-hand sides) incl. check: %g ms\n", nrhs,
                    std::chrono::duration_cast<std::chrono::microseconds>(end - beg).count() / 1e3);
        std::printf("-- max_r ||b - A x||_oo / (||A||_oo ||x||_oo + ||b||_oo) = %g\n", be);
        if (!(be <= 1e-14)) {
          std::printf("-- Solve is suspicious !\n");
          ret = 1;
        } else {
          std::printf("-- Solve is CORRECT !\n");
        }
        if (xfile) {
          FILE* f = std::fopen(xfile, "wb");
          std::fwrite(X.data(), sizeof(double), X.size(), f);
          std::fclose(f);
        }
      }
    }
  } catch (const std::exception& e) {
    std::fprintf(stderr, "error: %s\n", e.what());
    ret = 2;
  }
  ttg::finalize();
  return ret;
}
