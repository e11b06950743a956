// Minimal stand-in for the PaRSEC data-distribution types that the reference's potrf example
// touches (examples/potrf/pmw.h, testing_dpotrf.cc) — TEST INFRASTRUCTURE ONLY.
// One process, one rank: a lower sym_block_cyclic matrix is a set of NB x NB tiles stored in the
// oracle's slot order (slot(m,n) = n*NT - n*(n-1)/2 + (m-n)), lda = mb.
#pragma once
#include <cstdarg>
#include <cstddef>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <unistd.h>

struct parsec_data_copy_t {
  void* ptr;
};
struct parsec_data_t {
  parsec_data_copy_t copy;
};
struct parsec_data_collection_t {
  parsec_data_t* (*data_of)(parsec_data_collection_t* d, ...);
  uint32_t (*rank_of)(parsec_data_collection_t* d, ...);
  const char* key;
};
typedef enum parsec_matrix_type_e { PARSEC_MATRIX_FLOAT, PARSEC_MATRIX_DOUBLE } parsec_matrix_type_t;
enum { PARSEC_MATRIX_LOWER = 0, PARSEC_MATRIX_UPPER = 1 };

struct parsec_tiled_matrix_t {
  parsec_data_collection_t super;
  parsec_matrix_type_t mtype;
  int mb, nb, bsiz, lm, ln, i, j, m, n, mt, nt, nb_local_tiles;
};
struct parsec_grid_t {
  int rows, cols;
};
struct parsec_matrix_sym_block_cyclic_t {
  parsec_tiled_matrix_t super;
  parsec_grid_t grid;
  int uplo;
  void* mat;
  parsec_data_t* tiles;  // one descriptor per lower tile, slot order
};

inline parsec_data_copy_t* parsec_data_get_copy(parsec_data_t* d, int) { return &d->copy; }
inline void* parsec_data_copy_get_ptr(parsec_data_copy_t* c) { return c->ptr; }
inline size_t parsec_datadist_getsizeoftype(parsec_matrix_type_t t) {
  return t == PARSEC_MATRIX_FLOAT ? sizeof(float) : sizeof(double);
}

inline parsec_data_t* shim_sym_data_of(parsec_data_collection_t* d, ...) {
  va_list ap;
  va_start(ap, d);
  const int m = va_arg(ap, int), n = va_arg(ap, int);
  va_end(ap);
  auto* A = reinterpret_cast<parsec_matrix_sym_block_cyclic_t*>(d);
  const int NT = A->super.mt;
  const long slot = (long)n * NT - (long)n * (n - 1) / 2 + (m - n);
  parsec_data_t* t = &A->tiles[slot];
  t->copy.ptr = static_cast<char*>(A->mat) + slot * (long)A->super.bsiz * (long)parsec_datadist_getsizeoftype(A->super.mtype);
  return t;
}
inline uint32_t shim_rank_of(parsec_data_collection_t*, ...) { return 0; }

inline void parsec_matrix_sym_block_cyclic_init(parsec_matrix_sym_block_cyclic_t* A, parsec_matrix_type_t mtype,
                                                int /*myrank*/, int mb, int nb, int lm, int ln, int i, int j, int m,
                                                int n, int P, int Q, int uplo) {
  std::memset(A, 0, sizeof(*A));
  A->super.super.data_of = shim_sym_data_of;
  A->super.super.rank_of = shim_rank_of;
  A->super.mtype = mtype;
  A->super.mb = mb;
  A->super.nb = nb;
  A->super.bsiz = mb * nb;
  A->super.lm = lm;
  A->super.ln = ln;
  A->super.i = i;
  A->super.j = j;
  A->super.m = m;
  A->super.n = n;
  A->super.mt = (m + mb - 1) / mb;
  A->super.nt = (n + nb - 1) / nb;
  A->super.nb_local_tiles = A->super.mt * (A->super.mt + 1) / 2;
  A->grid.rows = P;
  A->grid.cols = Q;
  A->uplo = uplo;
  A->tiles = new parsec_data_t[A->super.nb_local_tiles];
}
inline void* parsec_data_allocate(size_t bytes) { return std::calloc(1, bytes); }
inline void parsec_data_free(void* p) { std::free(p); }
inline void parsec_data_collection_set_key(parsec_data_collection_t* d, char* key) { d->key = key; }
inline void parsec_tiled_matrix_destroy(parsec_tiled_matrix_t* A) {
  delete[] reinterpret_cast<parsec_matrix_sym_block_cyclic_t*>(A)->tiles;
}
inline void parsec_devices_release_memory() {}
#define BLKLDD(desc, m) ((desc)->mb)
