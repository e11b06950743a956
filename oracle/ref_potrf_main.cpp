// Runs the reference's own potrf flowgraph (examples/potrf/potrf.h, host branch), generator
// (plgsy.h) and result writer (result.h), unmodified, on the GB300 TTG runtime with the oracle's
// tile kernels, and writes the factor tiles — TEST INFRASTRUCTURE ONLY. Built by oracle/build.py
// into oracle/_ref/; the tests compare its output with the oracle's restated flowgraph.
// Usage: ref_potrf N NB out.bin
#include <ttg.h>

#include <cstdio>

#include "plgsy.h"
#include "pmw.h"
#include "potrf.h"
#include "result.h"

int main(int argc, char** argv) {
  if (argc != 4) return 2;
  const int N = std::atoi(argv[1]), NB = std::atoi(argv[2]);
  ttg::initialize(1, argv, 4);
  auto world = ttg::default_execution_context();
  parsec_matrix_sym_block_cyclic_t dcA;
  parsec_matrix_sym_block_cyclic_init(&dcA, parsec_matrix_type_t::PARSEC_MATRIX_DOUBLE, 0, NB, NB, N, N, 0, 0, N, N,
                                      1, 1, PARSEC_MATRIX_LOWER);
  dcA.mat = parsec_data_allocate((size_t)dcA.super.nb_local_tiles * (size_t)dcA.super.bsiz * sizeof(double));
  {
    ttg::Edge<Key2, void> startup("startup");
    ttg::Edge<Key2, MatrixTile<double>> topotrf("To POTRF");
    ttg::Edge<Key2, MatrixTile<double>> result("To result");
    MatrixT<double> A{&dcA};
    auto init_tt = ttg::make_tt<void>([&](std::tuple<ttg::Out<Key2, void>>& out) {
      for (int i = 0; i < (int)A.rows(); i++)
        for (int j = 0; j <= i && j < (int)A.cols(); j++) ttg::sendk<0>(Key2{i, j}, out);
    }, ttg::edges(), ttg::edges(startup), "Startup Trigger", {}, {"startup"});
    auto plgsy_ttg = make_plgsy_ttg(A, N, 3872, startup, topotrf, true);
    auto potrf_ttg = potrf::make_potrf_ttg(A, topotrf, result, true, true);
    auto result_ttg = make_result_ttg(A, result, true);
    bool connected = ttg::make_graph_executable(init_tt.get());
    if (!connected) return 3;
    init_tt->invoke();
    ttg::execute(world);
    ttg::fence(world);
  }
  FILE* f = std::fopen(argv[3], "wb");
  std::fwrite(dcA.mat, sizeof(double), (size_t)dcA.super.nb_local_tiles * dcA.super.bsiz, f);
  std::fclose(f);
  parsec_data_free(dcA.mat);
  parsec_tiled_matrix_destroy((parsec_tiled_matrix_t*)&dcA);
  ttg::finalize();
  return 0;
}
