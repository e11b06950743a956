// Tile value and tile-major lower matrix for the GB300 potrf flowgraph.
//
// MatrixTile<T> plays the role of the reference's examples/matrixtile.h:42-194: a ttg::Buffer
// (HBM-mirrored) plus rows/cols/lda; it can borrow the matrix's own tile memory (no copy) and its
// copy constructor is a deep copy. TiledMatrix<T> is the storage the reference gets from PaRSEC's
// sym_block_cyclic distribution (examples/potrf/pmw.h:36-140), for one process: lower tiles of
// NB x NB doubles, lda = NB, in slot order n*NT - n*(n-1)/2 + (m-n) — the layout of
// include/gbx_potrf.h, so the same memory can go to gbx_dpotrf_tiled.
#pragma once
#include <ttg.h>

#include <algorithm>
#include <cstddef>
#include <memory>

namespace gbx_potrf {

using Key1 = ttg::MultiIndex<1>;
using Key2 = ttg::MultiIndex<2>;
using Key3 = ttg::MultiIndex<3>;

template <typename T>
class MatrixTile : public ttg::TTValue<MatrixTile<T>> {
  struct borrowed {
    void operator()(T*) const {}
  };
  ttg::Buffer<T> buf_;
  std::size_t rows_ = 0, cols_ = 0, lda_ = 0;

 public:
  MatrixTile() = default;
  MatrixTile(std::size_t rows, std::size_t cols, std::size_t lda) : buf_(lda * cols), rows_(rows), cols_(cols), lda_(lda) {}
  /// a view of memory the tile does not own (the matrix's tile slot)
  MatrixTile(std::size_t rows, std::size_t cols, T* data, std::size_t lda, ttg::scope sc = ttg::scope::SyncIn)
      : buf_(std::unique_ptr<T[], borrowed>(data, borrowed{}), lda * cols, sc), rows_(rows), cols_(cols), lda_(lda) {}
  MatrixTile(MatrixTile&&) = default;
  MatrixTile& operator=(MatrixTile&&) = default;
  MatrixTile(const MatrixTile& o) : buf_(o.lda_ * o.cols_), rows_(o.rows_), cols_(o.cols_), lda_(o.lda_) {
    std::copy_n(o.data(), lda_ * cols_, data());
  }
  T* data() { return buf_.host_ptr(); }
  const T* data() const { return buf_.host_ptr(); }
  std::size_t size() const { return cols_ * lda_; }
  std::size_t rows() const { return rows_; }
  std::size_t cols() const { return cols_; }
  std::size_t lda() const { return lda_; }
  ttg::Buffer<T>& buffer() { return buf_; }
  const ttg::Buffer<T>& buffer() const { return buf_; }
  template <typename Archive>
  void serialize(Archive& ar) {
    ar& rows_& cols_& lda_;
    ar& buf_;
  }
};

template <typename T>
class TiledMatrix {
  T* base_;
  int N_, NB_, NT_;

 public:
  using element_type = T;
  TiledMatrix(T* base, int N, int NB) : base_(base), N_(N), NB_(NB), NT_((N + NB - 1) / NB) {}
  static std::size_t num_elements(int N, int NB) {
    const std::size_t nt = (N + NB - 1) / NB;
    return nt * (nt + 1) / 2 * (std::size_t)NB * NB;
  }
  T* tile_ptr(int m, int n) const {
    const long slot = (long)n * NT_ - (long)n * (n - 1) / 2 + (m - n);
    return base_ + slot * (long)NB_ * NB_;
  }
  int tile_dim(int t) const { return t == NT_ - 1 ? N_ - (NT_ - 1) * NB_ : NB_; }
  MatrixTile<T> operator()(int m, int n, ttg::scope sc = ttg::scope::SyncIn) const {
    return MatrixTile<T>(tile_dim(m), tile_dim(n), tile_ptr(m, n), NB_, sc);
  }
  std::size_t rows() const { return NT_; }
  std::size_t cols() const { return NT_; }
  std::size_t rows_in_tile() const { return NB_; }
  std::size_t cols_in_tile() const { return NB_; }
  std::size_t rows_in_matrix() const { return N_; }
  std::size_t cols_in_matrix() const { return N_; }
  int P() const { return 1; }
  int Q() const { return 1; }
  int rank_of(int, int) const { return 0; }
  bool is_local(int, int) const { return true; }
  bool in_matrix(int m, int n) const { return n <= m; }
  T* data() const { return base_; }
};

}  // namespace gbx_potrf
