/*
 * CPU oracle for the tiled Cholesky (potrf) path — TEST INFRASTRUCTURE ONLY.
 *
 * This library restates, on the host, what the reference computes on the potrf path:
 *   - the PLASMA symmetric test-matrix generator (examples/potrf/core_plgsy.h:64-150,
 *     examples/potrf/random.h:19-41), bit for bit;
 *   - the seeded "(M+M^T)/2 + n*I, M ~ U[-0.5,0.5]" generator used by the benchmark
 *     configurations (a counter-based generator, identical on CPU and GPU);
 *   - the tile kernels of the host branch of the flowgraph (LAPACK potrf lower,
 *     examples/potrf/potrf.h:201; trsm Right/Lower/Trans/NonUnit, potrf.h:345-346;
 *     syrk Lower/NoTrans alpha=-1 beta=1, potrf.h:480-481; gemm NoTrans/Trans alpha=-1
 *     beta=1, potrf.h:609-611) as plain loops, or OpenBLAS when loaded;
 *   - the flowgraph itself (dispatcher potrf.h:633-668, successor rules potrf.h:112-116,
 *     259-268, 449-457, 578-586, DPLASMA priorities potrf.h:742-752) on a keyed host task
 *     runtime with a thread pool and a priority ready queue;
 *   - the reference's correctness check (examples/potrf/testing_dpotrf.cc:277-335).
 *
 * Only the tests, the smoke check and the CPU-baseline leg of the benchmark use it. The
 * product path (the CUDA library) never links or calls it.
 *
 * Tile storage (shared with the CUDA library): the lower triangle of an N x N matrix split
 * into NT = ceil(N/NB) tile rows/columns; each tile (m,n), m >= n, occupies an NB*NB slot
 * of doubles, column-major with lda = NB, slots packed column of tiles by column of tiles:
 *   slot(m,n) = n*NT - n*(n-1)/2 + (m-n).
 * The last tile row/column is ragged when NB does not divide N (rows = N - (NT-1)*NB).
 */
#pragma once
#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- layout ---- */
int64_t orc_tile_slot(int m, int n, int NT);
/* tiles <-> full column-major (only the lower triangle is read/written; upper set to 0 on export) */
void orc_tiles_from_colmajor(int N, int NB, const double* A, int64_t lda, double* tiles);
void orc_tiles_to_colmajor(int N, int NB, const double* tiles, double* A, int64_t lda);

/* ---- generators ---- */
/* PLASMA CORE_dplgsy on one tile (core_plgsy.h:64-150), double precision */
void orc_plgsy_tile(double bump, int m, int n, double* A, int lda, int gM, int m0, int n0,
                    unsigned long long seed);
/* the whole lower-tiled matrix with CORE_plgsy per tile, as examples/potrf/plgsy.h:8-34 does */
void orc_plgsy_tiles(int N, int NB, double bump, unsigned long long seed, double* tiles);
/* uniform element M_ij in [-0.5,0.5) of the counter-based generator (seed, i, j) */
double orc_uniform_elem(uint64_t seed, int64_t i, int64_t j);
/* A = (M+M^T)/2 + N*I into lower tiles (or full col-major if tiles==NULL and A!=NULL) */
void orc_gen_uniform_sym_tiles(int N, int NB, uint64_t seed, double shift, double* tiles);
void orc_gen_uniform_sym_colmajor(int N, uint64_t seed, double shift, double* A, int64_t lda);

/* ---- tile kernels (plain loops, -ffp-contract=off) ---- */
int  orc_potrf_tile(int n, double* A, int lda);                 /* returns info */
void orc_trsm_rlt_tile(int m, int n, const double* L, int ldl, double* B, int ldb);
void orc_syrk_ln_tile(int n, int k, const double* A, int lda, double* C, int ldc);
void orc_gemm_nt_tile(int m, int n, int k, const double* A, int lda, const double* B, int ldb,
                      double* C, int ldc);
void orc_trsm_rln_tile(int m, int n, const double* L, int ldl, double* B, int ldb);
void orc_gemm_nn_tile(int m, int n, int k, const double* A, int lda, const double* B, int ldb,
                      double* C, int ldc);

/* ---- OpenBLAS tile kernels (optional, for timing the CPU baseline) ---- */
/* loads the given shared library; returns 0 on success */
int  orc_blas_load(const char* path);
int  orc_blas_loaded(void);

/* ---- the flowgraph ---- */
/* factorises the lower-tiled matrix in place; nthreads workers; use_blas: 0 plain loops,
 * 1 OpenBLAS (single-threaded per task). Returns 0, or K+1 of the first failing POTRF(K)
 * tile with its LAPACK info in *tile_info. Writes the executed task order to trace
 * (type<<60 | m<<40 | n<<20 | k) when trace != NULL (capacity trace_cap). */
int  orc_potrf_tiled(int N, int NB, double* tiles, int nthreads, int use_blas, int* tile_info,
                     int64_t* trace, int64_t trace_cap, int64_t* ntrace);
/* the DPLASMA priorities of potrf.h:742-752 (type 0 POTRF(K), 1 TRSM(M,K), 2 SYRK(K,M), 3 GEMM(M,N,K)) */
int64_t orc_priority(int type, int nt, int a, int b, int c);

/* ---- solve and checks ---- */
/* x := (L L^T)^{-1} x for nrhs columns, L lower tiled */
void orc_potrs_tiled(int N, int NB, const double* tiles, int nrhs, double* X, int64_t ldx);
/* examples/potrf/testing_dpotrf.cc:277-335: ||LL^T - A0||_inf / (||A0||_inf N eps); A, A0 col-major N x N */
double orc_check_dpotrf(int N, const double* L, const double* A0);
/* ||A0 - L L^T||_F / (N ||A0||_F), A0 full symmetric col-major, L lower col-major */
double orc_frob_residual(int N, const double* L, const double* A0);

/* ---- inverse from the factor (the reference's POTRI chain, examples/potrf/potri.h, trtri_L.h,
 * lauum.h): the PLASMA tile algorithms TRTRI (lower, non-unit) then LAUUM, plain loops, in place
 * on the lower tiles of the factor; returns 0 ---- */
int orc_potri_tiled(int N, int NB, double* tiles);

/* ---- batched solves (the per-matrix LAPACK loop a CPU user runs for many small systems) ---- */
/* matrix k: n[k] x n[k] column-major at A + offA[k] (lower triangle read, factor written in place),
 * right-hand sides n[k] x nrhs at B + offB[k] (overwritten by the solution). Matrices are taken
 * largest first by nthreads workers (0 = all cores); use_blas: OpenBLAS dpotrf + dtrsm, else the
 * plain-loop tile kernels. info[k] = 0 or the LAPACK info of the failed factorisation. */
void orc_dposv_batched(int batch, const int* n, const int64_t* offA, const int64_t* offB, double* A,
                       double* B, int nrhs, int nthreads, int use_blas, int* info);
/* matrix k of the batched generator: (M+M^T)/2 + n*I, M from seed + k * 0x9e3779b97f4a7c15 */
void orc_gen_uniform_sym_batched(int batch, const int* n, const int64_t* offA, uint64_t seed, double* A);

#ifdef __cplusplus
}
#endif
