// The tiled solve (L L^T) X = B as a TTG flowgraph on the GB300 runtime, device branch.
//
// The reference's potrf example stops at the factor; this flowgraph adds the solve through the same
// API (make_tt device tasks, keyed terminals, ttg::device::select/send/broadcast/forward). The
// right-hand sides are held as NT tiles of nrhs x NB (column-major, lda = nrhs; column i of tile k
// is row k*NB + i of B), so both sweeps are right-side tile operations:
//   forward  L Y = B:    FWD_TRSM(k):   Y_k := B_k L_kk^{-T}            (gbx_dtrsm_rlt_tile)
//                        FWD_GEMM(m,k): B_m -= Y_k L_mk^T, m > k         (gbx_dgemm_nt_tile)
//   backward L^T X = Y:  BWD_TRSM(k):   X_k := Y_k L_kk^{-1}            (gbx_dtrsm_rln_tile)
//                        BWD_GEMM(m,k): Y_m -= X_k L_km, m < k           (gbx_dgemm_nn_tile)
// A right-hand-side tile flows through its chain of updates as the mutable (rvalue) input; the
// factor tiles and the solved tiles enter the updates as read-only (const) inputs. The forward
// updates of tile m go k = 0, 1, ..., m-1, then FWD_TRSM(m); the backward updates of tile m go
// k = NT-1, ..., m+1, then BWD_TRSM(m).
#pragma once
#include <ttg.h>

#include <vector>

#include "gbx_potrf.h"
#include "matrix.h"
#include "potrf.h"

namespace potrs {

using gbx_potrf::Key1;
using gbx_potrf::Key2;
using gbx_potrf::MatrixTile;
using Tile = MatrixTile<double>;

/// Right-hand sides of the tiled solve: NT tiles of nrhs x NB doubles, tile k at k * nrhs * NB.
template <typename T>
class TiledRhs {
  T* base_;
  int N_, NB_, NT_, nrhs_;

 public:
  TiledRhs(T* base, int N, int NB, int nrhs) : base_(base), N_(N), NB_(NB), NT_((N + NB - 1) / NB), nrhs_(nrhs) {}
  static std::size_t num_elements(int N, int NB, int nrhs) { return (std::size_t)((N + NB - 1) / NB) * NB * nrhs; }
  T* tile_ptr(int k) const { return base_ + (long)k * NB_ * nrhs_; }
  int tile_dim(int k) const { return k == NT_ - 1 ? N_ - (NT_ - 1) * NB_ : NB_; }
  MatrixTile<T> operator()(int k) const { return MatrixTile<T>(nrhs_, tile_dim(k), tile_ptr(k), nrhs_); }
  int tiles() const { return NT_; }
  int nrhs() const { return nrhs_; }
};

// routes the factor tiles and the right-hand-side tiles to their first consumers
template <typename MatrixT>
auto make_dispatch(MatrixT& L, ttg::Edge<Key2, Tile>& lin, ttg::Edge<Key1, Tile>& bin, ttg::Edge<Key1, Tile>& l_fwd_trsm,
                   ttg::Edge<Key1, Tile>& l_bwd_trsm, ttg::Edge<Key2, Tile>& l_fwd_gemm, ttg::Edge<Key2, Tile>& l_bwd_gemm,
                   ttg::Edge<Key1, Tile>& b_fwd_trsm, ttg::Edge<Key2, Tile>& b_fwd_gemm) {
  auto ltiles = [](const Key2& key, const Tile& tile,
                   std::tuple<ttg::Out<Key1, Tile>, ttg::Out<Key1, Tile>, ttg::Out<Key2, Tile>, ttg::Out<Key2, Tile>>& out) {
    const int m = key[0], k = key[1];
    if (m == k) ttg::broadcast<0, 1>(std::make_tuple(Key1(k), Key1(k)), tile, out);
    else ttg::broadcast<2, 3>(std::make_tuple(Key2(m, k), Key2(k, m)), tile, out);  // L_mk: FWD_GEMM(m,k), BWD_GEMM(k,m)
  };
  auto btiles = [](const Key1& key, const Tile& tile, std::tuple<ttg::Out<Key1, Tile>, ttg::Out<Key2, Tile>>& out) {
    const int k = key[0];
    if (k == 0) ttg::send<0>(Key1(0), tile, out);
    else ttg::send<1>(Key2(k, 0), tile, out);
  };
  (void)L;
  auto tl = ttg::make_tt(ltiles, ttg::edges(lin), ttg::edges(l_fwd_trsm, l_bwd_trsm, l_fwd_gemm, l_bwd_gemm),
                         "POTRS L Dispatch", {"L"}, {"FWD_TRSM", "BWD_TRSM", "FWD_GEMM", "BWD_GEMM"});
  auto tb = ttg::make_tt(btiles, ttg::edges(bin), ttg::edges(b_fwd_trsm, b_fwd_gemm), "POTRS B Dispatch", {"B"},
                         {"FWD_TRSM", "FWD_GEMM"});
  return std::make_pair(std::move(tl), std::move(tb));
}

/// The solve flowgraph. L (the factor, NT x NT tiles) and the right-hand sides enter through `lin`
/// (Key2 tile index, m >= k) and `bin` (Key1 tile index); the solution tiles leave through `out`.
template <typename MatrixT>
auto make_potrs_ttg(MatrixT& L, int nrhs, ttg::Edge<Key2, Tile>& lin, ttg::Edge<Key1, Tile>& bin,
                    ttg::Edge<Key1, Tile>& out) {
  const int NT = (int)L.rows();
  ttg::Edge<Key1, Tile> l_fwd_trsm("l_fwd_trsm"), l_bwd_trsm("l_bwd_trsm"), b_fwd_trsm("b_fwd_trsm"),
      y_fwd_trsm("y_fwd_trsm"), y_bwd_trsm("y_bwd_trsm"), y_solve("y_solve");
  ttg::Edge<Key2, Tile> l_fwd_gemm("l_fwd_gemm"), l_bwd_gemm("l_bwd_gemm"), b_fwd_gemm("b_fwd_gemm"),
      y_fwd_gemm("y_fwd_gemm"), chain_fwd("chain_fwd"), x_bwd_gemm("x_bwd_gemm"), chain_bwd("chain_bwd"),
      y_bwd_first("y_bwd_first");
  auto disp = make_dispatch(L, lin, bin, l_fwd_trsm, l_bwd_trsm, l_fwd_gemm, l_bwd_gemm, b_fwd_trsm, b_fwd_gemm);

  // FWD_TRSM(k): Y_k := B_k L_kk^{-T}; Y_k to the updates of the tiles below it and into the
  // backward chain of tile k
  auto fwd_trsm = ttg::make_tt<ttg::ExecutionSpace::CUDA>(
      [NT, nrhs](const Key1& key, const Tile& lkk, Tile&& b,
                 std::tuple<ttg::Out<Key2, Tile>, ttg::Out<Key2, Tile>, ttg::Out<Key1, Tile>>& o) -> ttg::device::Task {
        const int k = key[0];
        std::vector<Key2> below;
        for (int m = k + 1; m < NT; ++m) below.emplace_back(m, k);
        co_await ttg::device::select(lkk.buffer(), b.buffer());
        potrf::check_status(gbx_dtrsm_rlt_tile(nrhs, (int)b.cols(), lkk.buffer().current_device_ptr(), (int)lkk.lda(),
                                               b.buffer().current_device_ptr(), (int)b.lda(),
                                               ttg::device::current_stream()),
                            "gbx_dtrsm_rlt_tile");
        if (k == NT - 1)  // the last tile starts the backward sweep at once
          co_await ttg::device::forward(ttg::device::send<2>(Key1(k), std::move(b), o));
        else
          co_await ttg::device::forward(ttg::device::broadcast<0, 1>(
              std::make_tuple(std::move(below), Key2(k, NT - 1)), std::move(b), o));
      },
      ttg::edges(l_fwd_trsm, ttg::fuse(b_fwd_trsm, y_fwd_trsm)), ttg::edges(y_fwd_gemm, y_bwd_first, y_bwd_trsm),
      "FWD_TRSM", {"L_kk", "B_k"}, {"Y_k below", "Y_k backward chain", "Y_k backward solve"});

  // FWD_GEMM(m,k): B_m -= Y_k L_mk^T
  auto fwd_gemm = ttg::make_tt<ttg::ExecutionSpace::CUDA>(
      [nrhs](const Key2& key, const Tile& lmk, const Tile& yk, Tile&& bm,
             std::tuple<ttg::Out<Key2, Tile>, ttg::Out<Key1, Tile>>& o) -> ttg::device::Task {
        const int m = key[0], k = key[1];
        co_await ttg::device::select(lmk.buffer(), yk.buffer(), bm.buffer());
        potrf::check_status(gbx_dgemm_nt_tile(nrhs, (int)bm.cols(), (int)yk.cols(), yk.buffer().current_device_ptr(),
                                              (int)yk.lda(), lmk.buffer().current_device_ptr(), (int)lmk.lda(),
                                              bm.buffer().current_device_ptr(), (int)bm.lda(),
                                              ttg::device::current_stream()),
                            "gbx_dgemm_nt_tile");
        if (k + 1 < m) co_await ttg::device::send<0>(Key2(m, k + 1), std::move(bm), o);
        else co_await ttg::device::send<1>(Key1(m), std::move(bm), o);
      },
      ttg::edges(l_fwd_gemm, y_fwd_gemm, ttg::fuse(b_fwd_gemm, chain_fwd)), ttg::edges(chain_fwd, y_fwd_trsm),
      "FWD_GEMM", {"L_mk", "Y_k", "B_m"}, {"B_m next update", "B_m solve"});

  // BWD_TRSM(k): X_k := Y_k L_kk^{-1}; X_k to the updates of the tiles above it and out
  auto bwd_trsm = ttg::make_tt<ttg::ExecutionSpace::CUDA>(
      [nrhs](const Key1& key, const Tile& lkk, Tile&& y,
             std::tuple<ttg::Out<Key2, Tile>, ttg::Out<Key1, Tile>>& o) -> ttg::device::Task {
        const int k = key[0];
        std::vector<Key2> above;
        for (int m = 0; m < k; ++m) above.emplace_back(m, k);
        co_await ttg::device::select(lkk.buffer(), y.buffer());
        potrf::check_status(gbx_dtrsm_rln_tile(nrhs, (int)y.cols(), lkk.buffer().current_device_ptr(), (int)lkk.lda(),
                                               y.buffer().current_device_ptr(), (int)y.lda(),
                                               ttg::device::current_stream()),
                            "gbx_dtrsm_rln_tile");
        co_await ttg::device::forward(
            ttg::device::broadcast<0, 1>(std::make_tuple(std::move(above), Key1(k)), std::move(y), o));
      },
      ttg::edges(l_bwd_trsm, ttg::fuse(y_bwd_trsm, y_solve)), ttg::edges(x_bwd_gemm, out), "BWD_TRSM",
      {"L_kk", "Y_k"}, {"X_k above", "X_k out"});

  // BWD_GEMM(m,k), m < k: Y_m -= X_k L_km
  auto bwd_gemm = ttg::make_tt<ttg::ExecutionSpace::CUDA>(
      [nrhs](const Key2& key, const Tile& lkm, const Tile& xk, Tile&& ym,
             std::tuple<ttg::Out<Key2, Tile>, ttg::Out<Key1, Tile>>& o) -> ttg::device::Task {
        const int m = key[0], k = key[1];
        co_await ttg::device::select(lkm.buffer(), xk.buffer(), ym.buffer());
        potrf::check_status(gbx_dgemm_nn_tile(nrhs, (int)ym.cols(), (int)xk.cols(), xk.buffer().current_device_ptr(),
                                              (int)xk.lda(), lkm.buffer().current_device_ptr(), (int)lkm.lda(),
                                              ym.buffer().current_device_ptr(), (int)ym.lda(),
                                              ttg::device::current_stream()),
                            "gbx_dgemm_nn_tile");
        if (k - 1 > m) co_await ttg::device::send<0>(Key2(m, k - 1), std::move(ym), o);
        else co_await ttg::device::send<1>(Key1(m), std::move(ym), o);
      },
      ttg::edges(l_bwd_gemm, x_bwd_gemm, ttg::fuse(y_bwd_first, chain_bwd)), ttg::edges(chain_bwd, y_solve),
      "BWD_GEMM", {"L_km", "X_k", "Y_m"}, {"Y_m next update", "Y_m solve"});

  // a right-hand-side tile that is also read by other tasks (Y_k, X_k) is updated only after them
  fwd_trsm->set_defer_writer(true);
  fwd_gemm->set_defer_writer(true);
  bwd_trsm->set_defer_writer(true);
  bwd_gemm->set_defer_writer(true);
  std::vector<std::unique_ptr<ttg::TTBase>> ops;
  ops.emplace_back(std::move(disp.first));
  ops.emplace_back(std::move(disp.second));
  ops.emplace_back(std::move(fwd_trsm));
  ops.emplace_back(std::move(fwd_gemm));
  ops.emplace_back(std::move(bwd_trsm));
  ops.emplace_back(std::move(bwd_gemm));
  return ops;
}

}  // namespace potrs
