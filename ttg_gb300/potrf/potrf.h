// The tiled Cholesky flowgraph on the GB300 TTG runtime, device branch.
//
// Same task graph as examples/potrf/potrf.h of the reference — five TTs (POTRF, TRSM, SYRK, GEMM
// and the input dispatcher), twelve edges, the successor rules of potrf.h:112-116, 259-268,
// 449-457, 578-586 and the DPLASMA priorities of potrf.h:742-752 — with each device body calling
// this project's sm_103a tile kernels (include/gbx_potrf.h) on ttg::device::current_stream()
// where the reference calls cuSOLVER/cuBLAS. A failing pivot raises potrf::NotPositiveDefinite
// from ttg::fence instead of aborting the process (the reference calls ttg::abort()); with
// ttg::set_abort_terminates(true) (or TTG_ABORT_TERMINATES=1) it ends the process as the reference does.
#pragma once
#include <ttg.h>

#include <cstdio>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "gbx_potrf.h"
#include "matrix.h"

namespace potrf {

using gbx_potrf::Key1;
using gbx_potrf::Key2;
using gbx_potrf::Key3;
using gbx_potrf::MatrixTile;

/* FLOP count of a dense Cholesky (the DPLASMA macros used by the reference, potrf.h:30-33) */
inline double FMULS_POTRF(double n) { return n * (((1. / 6.) * n + 0.5) * n + (1. / 3.)); }
inline double FADDS_POTRF(double n) { return n * (((1. / 6.) * n) * n - (1. / 6.)); }
inline double FLOPS_DPOTRF(double n) { return FMULS_POTRF(n) + FADDS_POTRF(n); }

struct NotPositiveDefinite : std::runtime_error {
  int tile, info;
  NotPositiveDefinite(int K, int i)
      : std::runtime_error("POTRF(" + std::to_string(K) + ") failed: info " + std::to_string(i)), tile(K), info(i) {}
};

inline void check_status(int st, const char* what) {
  if (st != GBX_OK) throw std::runtime_error(std::string(what) + " failed with status " + std::to_string(st));
}

template <typename MatrixT>
auto make_potrf(MatrixT& A, ttg::Edge<Key1, MatrixTile<double>>& from_dispatch, ttg::Edge<Key1, MatrixTile<double>>& from_syrk,
                ttg::Edge<Key2, MatrixTile<double>>& to_trsm, ttg::Edge<Key2, MatrixTile<double>>& to_result) {
  auto body = [&A](const Key1& key, MatrixTile<double>&& tile,
                   std::tuple<ttg::Out<Key2, MatrixTile<double>>, ttg::Out<Key2, MatrixTile<double>>>& out)
      -> ttg::device::Task {
    const int K = key[0];
    std::vector<Key2> trsm_keys;  // every tile below the diagonal in column K
    for (int m = K + 1; m < (int)A.rows(); ++m) trsm_keys.emplace_back(m, K);
    size_t lwork = 0;
    check_status(gbx_dpotrf_tile_bufferSize((int)tile.cols(), (int)tile.lda(), &lwork), "gbx_dpotrf_tile_bufferSize");
    std::vector<char> host_ws(lwork);
    int host_info = -32;
    auto ws = ttg::make_scratch(host_ws.data(), ttg::scope::Allocate, lwork);
    auto info = ttg::make_scratch(&host_info, ttg::scope::Allocate);
    co_await ttg::device::select(tile.buffer(), ws, info);
    check_status(gbx_dpotrf_tile((int)tile.cols(), tile.buffer().current_device_ptr(), (int)tile.lda(), ws.device_ptr(),
                                 lwork, info.device_ptr(), ttg::device::current_stream()),
                 "gbx_dpotrf_tile");
    co_await ttg::device::wait(info);
    if (host_info != 0) {
      if (ttg::abort_terminates()) {  // reference-faithful mode: end the process (potrf.h:184-186)
        std::fprintf(stderr, "POTRF(%d) failed: info %d\n", K, host_info);
        ttg::abort();
      }
      throw NotPositiveDefinite(K, host_info);
    }
    co_await ttg::device::forward(
        ttg::device::broadcast<0, 1>(std::make_tuple(Key2(K, K), std::move(trsm_keys)), std::move(tile), out));
  };
  return ttg::make_tt<ttg::ExecutionSpace::CUDA>(body, ttg::edges(ttg::fuse(from_syrk, from_dispatch)),
                                                 ttg::edges(to_result, to_trsm), "POTRF", {"tile_kk/dispatcher"},
                                                 {"output_result", "output_trsm"});
}

template <typename MatrixT>
auto make_trsm(MatrixT& A, ttg::Edge<Key2, MatrixTile<double>>& from_dispatch, ttg::Edge<Key2, MatrixTile<double>>& from_potrf,
               ttg::Edge<Key2, MatrixTile<double>>& from_gemm, ttg::Edge<Key2, MatrixTile<double>>& to_syrk,
               ttg::Edge<Key3, MatrixTile<double>>& to_gemm_row, ttg::Edge<Key3, MatrixTile<double>>& to_gemm_col,
               ttg::Edge<Key2, MatrixTile<double>>& to_result) {
  auto body = [&A](const Key2& key, const MatrixTile<double>& tile_kk, MatrixTile<double>&& tile_mk,
                   std::tuple<ttg::Out<Key2, MatrixTile<double>>, ttg::Out<Key2, MatrixTile<double>>,
                              ttg::Out<Key3, MatrixTile<double>>, ttg::Out<Key3, MatrixTile<double>>>& out)
      -> ttg::device::Task {
    const int M = key[0], K = key[1];
    std::vector<Key3> row_keys, col_keys;  // GEMMs that read this tile as A(M,K) / as A(N,K)
    for (int n = K + 1; n < M; ++n) row_keys.emplace_back(M, n, K);
    for (int m = M + 1; m < (int)A.rows(); ++m) col_keys.emplace_back(m, M, K);
    co_await ttg::device::select(tile_kk.buffer(), tile_mk.buffer());
    check_status(gbx_dtrsm_rlt_tile((int)tile_mk.rows(), (int)tile_mk.cols(), tile_kk.buffer().current_device_ptr(),
                                    (int)tile_kk.lda(), tile_mk.buffer().current_device_ptr(), (int)tile_mk.lda(),
                                    ttg::device::current_stream()),
                 "gbx_dtrsm_rlt_tile");
    co_await ttg::device::forward(ttg::device::broadcast<0, 1, 2, 3>(
        std::make_tuple(key, Key2(K, M), std::move(row_keys), std::move(col_keys)), std::move(tile_mk), out));
  };
  return ttg::make_tt<ttg::ExecutionSpace::CUDA>(body, ttg::edges(from_potrf, ttg::fuse(from_gemm, from_dispatch)),
                                                 ttg::edges(to_result, to_syrk, to_gemm_row, to_gemm_col), "TRSM",
                                                 {"tile_kk", "tile_mk/dispatcher"},
                                                 {"output_result", "tile_mk", "output_row", "output_col"});
}

template <typename MatrixT>
auto make_syrk(MatrixT& A, ttg::Edge<Key2, MatrixTile<double>>& from_dispatch, ttg::Edge<Key2, MatrixTile<double>>& from_trsm,
               ttg::Edge<Key2, MatrixTile<double>>& from_syrk, ttg::Edge<Key1, MatrixTile<double>>& to_potrf,
               ttg::Edge<Key2, MatrixTile<double>>& to_syrk) {
  auto body = [](const Key2& key, const MatrixTile<double>& tile_mk, MatrixTile<double>&& tile_kk,
                 std::tuple<ttg::Out<Key1, MatrixTile<double>>, ttg::Out<Key2, MatrixTile<double>>>& out)
      -> ttg::device::Task {
    const int K = key[0], M = key[1];  // step K updates the diagonal tile M
    co_await ttg::device::select(tile_kk.buffer(), tile_mk.buffer());
    check_status(gbx_dsyrk_ln_tile((int)tile_mk.rows(), (int)tile_mk.cols(), tile_mk.buffer().current_device_ptr(),
                                   (int)tile_mk.lda(), tile_kk.buffer().current_device_ptr(), (int)tile_kk.lda(),
                                   ttg::device::current_stream()),
                 "gbx_dsyrk_ln_tile");
    if (M == K + 1) co_await ttg::device::send<0>(Key1(K + 1), std::move(tile_kk), out);
    else co_await ttg::device::send<1>(Key2(K + 1, M), std::move(tile_kk), out);
  };
  (void)A;
  return ttg::make_tt<ttg::ExecutionSpace::CUDA>(body, ttg::edges(from_trsm, ttg::fuse(from_syrk, from_dispatch)),
                                                 ttg::edges(to_potrf, to_syrk), "SYRK", {"tile_mk", "tile_kk/dispatcher"},
                                                 {"output_potrf", "output_syrk"});
}

template <typename MatrixT>
auto make_gemm(MatrixT& A, ttg::Edge<Key3, MatrixTile<double>>& from_dispatch, ttg::Edge<Key3, MatrixTile<double>>& from_trsm_row,
               ttg::Edge<Key3, MatrixTile<double>>& from_trsm_col, ttg::Edge<Key3, MatrixTile<double>>& from_gemm,
               ttg::Edge<Key2, MatrixTile<double>>& to_trsm, ttg::Edge<Key3, MatrixTile<double>>& to_gemm) {
  auto body = [](const Key3& key, const MatrixTile<double>& tile_mk, const MatrixTile<double>& tile_nk,
                 MatrixTile<double>&& tile_mn,
                 std::tuple<ttg::Out<Key2, MatrixTile<double>>, ttg::Out<Key3, MatrixTile<double>>>& out)
      -> ttg::device::Task {
    const int M = key[0], N = key[1], K = key[2];
    co_await ttg::device::select(tile_mk.buffer(), tile_nk.buffer(), tile_mn.buffer());
    check_status(gbx_dgemm_nt_tile((int)tile_mk.rows(), (int)tile_nk.rows(), (int)tile_nk.cols(),
                                   tile_mk.buffer().current_device_ptr(), (int)tile_mk.lda(),
                                   tile_nk.buffer().current_device_ptr(), (int)tile_nk.lda(),
                                   tile_mn.buffer().current_device_ptr(), (int)tile_mn.lda(), ttg::device::current_stream()),
                 "gbx_dgemm_nt_tile");
    if (N == K + 1) co_await ttg::device::send<0>(Key2(M, N), std::move(tile_mn), out);
    else co_await ttg::device::send<1>(Key3(M, N, K + 1), std::move(tile_mn), out);
  };
  (void)A;
  return ttg::make_tt<ttg::ExecutionSpace::CUDA>(body, ttg::edges(from_trsm_row, from_trsm_col, ttg::fuse(from_dispatch, from_gemm)),
                                                 ttg::edges(to_trsm, to_gemm), "GEMM",
                                                 {"input_mk", "input_kn", "input_mn/dispatcher"}, {"output_trsm", "output_gemm"});
}

// routes each input tile to its first consumer (potrf.h:633-668)
inline auto make_dispatcher(ttg::Edge<Key2, MatrixTile<double>>& input, ttg::Edge<Key1, MatrixTile<double>>& to_potrf,
                            ttg::Edge<Key2, MatrixTile<double>>& to_trsm, ttg::Edge<Key2, MatrixTile<double>>& to_syrk,
                            ttg::Edge<Key3, MatrixTile<double>>& to_gemm) {
  auto body = [](const Key2& key, const MatrixTile<double>& tile,
                 std::tuple<ttg::Out<Key1, MatrixTile<double>>, ttg::Out<Key2, MatrixTile<double>>,
                            ttg::Out<Key2, MatrixTile<double>>, ttg::Out<Key3, MatrixTile<double>>>& out) {
    const int i = key[0], j = key[1];
    if (i == 0 && j == 0) ttg::send<0>(Key1{0}, tile, out);
    else if (i == j) ttg::send<2>(Key2{0, i}, tile, out);
    else if (j == 0) ttg::send<1>(key, tile, out);
    else ttg::send<3>(Key3{i, j, 0}, tile, out);
  };
  return ttg::make_tt(body, ttg::edges(input), ttg::edges(to_potrf, to_trsm, to_syrk, to_gemm), "POTRF Dispatch",
                      {"Input"}, {"POTRF", "TRSM", "SYRK", "GEMM"});
}

/// Builds the flowgraph; tiles enter through `input` (Key2 = tile index) and the factor tiles leave
/// through `output`.
template <typename MatrixT>
auto make_potrf_ttg(MatrixT& A, ttg::Edge<Key2, MatrixTile<double>>& input, ttg::Edge<Key2, MatrixTile<double>>& output,
                    bool defer_write, bool enable_device_map = true) {
  ttg::Edge<Key1, MatrixTile<double>> syrk_potrf("syrk_potrf"), disp_potrf("disp_potrf");
  ttg::Edge<Key2, MatrixTile<double>> potrf_trsm("potrf_trsm"), trsm_syrk("trsm_syrk"), gemm_trsm("gemm_trsm"),
      syrk_syrk("syrk_syrk"), disp_trsm("disp_trsm"), disp_syrk("disp_syrk");
  ttg::Edge<Key3, MatrixTile<double>> gemm_gemm("gemm_gemm"), trsm_gemm_row("trsm_gemm_row"),
      trsm_gemm_col("trsm_gemm_col"), disp_gemm("disp_gemm");

  auto tt_dispatch = make_dispatcher(input, disp_potrf, disp_trsm, disp_syrk, disp_gemm);
  auto tt_potrf = make_potrf(A, disp_potrf, syrk_potrf, potrf_trsm, output);
  auto tt_trsm = make_trsm(A, disp_trsm, potrf_trsm, gemm_trsm, trsm_syrk, trsm_gemm_row, trsm_gemm_col, output);
  auto tt_syrk = make_syrk(A, disp_syrk, trsm_syrk, syrk_syrk, syrk_potrf, syrk_syrk);
  auto tt_gemm = make_gemm(A, disp_gemm, trsm_gemm_row, trsm_gemm_col, gemm_gemm, gemm_trsm, gemm_gemm);
  tt_dispatch->set_defer_writer(defer_write);
  tt_potrf->set_defer_writer(defer_write);
  tt_trsm->set_defer_writer(defer_write);
  tt_syrk->set_defer_writer(defer_write);
  tt_gemm->set_defer_writer(defer_write);
  if (enable_device_map) {  // rows of tiles stay on one device (potrf.h:687-692); one GPU here
    tt_potrf->set_devicemap([](const Key1&) { return 0; });
    tt_trsm->set_devicemap([](const Key2&) { return 0; });
    tt_syrk->set_devicemap([](const Key2&) { return 0; });
    tt_gemm->set_devicemap([](const Key3&) { return 0; });
  }
  // DPLASMA priorities: work feeding the next panel first
  const long nt = (long)A.cols();
  tt_potrf->set_priomap([nt](const Key1& k) { return (nt - k[0]) * (nt - k[0]) * (nt - k[0]); });
  tt_trsm->set_priomap([nt](const Key2& k) {
    return (nt - k[0]) * (nt - k[0]) * (nt - k[0]) + 3 * ((2 * nt) - k[1] - k[0] - 1) * (k[0] - k[1]);
  });
  tt_syrk->set_priomap([nt](const Key2& k) { return (nt - k[0]) * (nt - k[0]) * (nt - k[0]) + 3 * (k[0] - k[1]); });
  tt_gemm->set_priomap([nt](const Key3& k) {
    return (nt - k[0]) * (nt - k[0]) * (nt - k[0]) + 3 * ((2 * nt) - k[0] - k[1] - 3) * (k[0] - k[1]) +
           6 * (k[0] - k[2]);
  });

  auto ins = std::make_tuple(tt_dispatch->template in<0>());
  auto outs = std::make_tuple(tt_potrf->template out<0>());
  std::vector<std::unique_ptr<ttg::TTBase>> ops;
  ops.push_back(std::move(tt_dispatch));
  ops.push_back(std::move(tt_potrf));
  ops.push_back(std::move(tt_syrk));
  ops.push_back(std::move(tt_trsm));
  ops.push_back(std::move(tt_gemm));
  return ttg::make_ttg(std::move(ops), ins, outs, "POTRF TTG");
}

}  // namespace potrf
