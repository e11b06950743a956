/*
 * gbx_potrf.h — C ABI of the GB300 (sm_103a) tiled-Cholesky library.
 *
 * Plain pointers, sizes and a cudaStream_t passed as void*; no C++ or torch types. Every
 * function returns an int status:
 *    0                 success
 *   >0                 (factorisations) LAPACK-style info: 1-based global index of the first
 *                      non-positive pivot; the factor is left partially computed
 *   GBX_ERR_ARG        invalid argument (nothing launched)
 *   GBX_ERR_CUDA       a CUDA runtime call failed
 *   GBX_ERR_TIMEOUT    a device-side dependency wait ran out of time (the kernel returned
 *                      without hanging; the context stays usable)
 *   GBX_ERR_WORKSPACE  the caller's workspace is too small
 *
 * Matrix layouts.
 *   Tile-major lower storage (the layout of the reference's sym_block_cyclic matrix,
 *   examples/potrf/pmw.h:52-59 and testing_dpotrf.cc:99-102): NT = ceil(N/NB) tile rows and
 *   columns; tile (m,n), m >= n, is an NB x NB column-major slot with lda = NB at slot index
 *   n*NT - n*(n-1)/2 + (m-n). The last tile row/column holds N-(NT-1)*NB valid rows/columns.
 *   Tile-level calls take ordinary column-major tiles with their leading dimension.
 *
 * Streams. Every call is asynchronous on `stream` (NULL = legacy default stream) unless its
 * comment says otherwise. Statuses written by kernels live in device memory and are read
 * back by the *_status calls, which synchronise the stream.
 *
 * Thread safety. Calls on different streams with disjoint workspaces may run concurrently.
 * Mutable global state, each part guarded by a mutex or set only by its own setter: per-device
 * caches of launch attributes and of the FP64 solve's scratch, the wait time limit
 * (gbx_set_wait_timeout_ns), the trace buffer (gbx_set_trace_buffer), the copy stream and
 * events of gbx_dposv_tiled_host (one caller at a time), the static scratch of
 * gbx_dpotrf_tiled_noalloc with its per-device address, and the executor settings
 * (gbx_set_dag_block_edge, gbx_set_fp64_update, gbx_set_dag_lead: read at each launch; set them
 * before the calls they are meant for, not concurrently with other calls).
 */
#ifndef GBX_POTRF_H
#define GBX_POTRF_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GBX_OK 0
#define GBX_ERR_ARG (-1)
#define GBX_ERR_CUDA (-2)
#define GBX_ERR_TIMEOUT (-3)
#define GBX_ERR_WORKSPACE (-4)
#define GBX_ERR_NOCONV (-5)
#define GBX_ERR_NOALLOC_LIMIT (-6)

/* Library version and the device architecture it was built for (e.g. 1030). */
int gbx_version(void);
int gbx_built_arch(void);

/* Default time limit of one device-side dependency wait, in nanoseconds (default 20 s). A wait
 * that runs out sets GBX_ERR_TIMEOUT and makes every CTA of the launch return. */
void gbx_set_wait_timeout_ns(uint64_t ns);
uint64_t gbx_get_wait_timeout_ns(void);

/* Per-task timeline of the persistent executors (gbx_dpotrf_tiled, gbx_potrf_mixed and their
 * variants), the counterpart of the reference's PaRSEC task tracing (bin/pbt_to_ctf.py). While a
 * device buffer is set, every task of a later launch appends a record: buf[0] counts records,
 * record i is buf[2+4i .. 5+4i] = {start ns, end ns (globaltimer), key = type<<60 | a<<40 | b<<20 | c
 * (type 0 POTRF(a), 1 TRSM(a,b), 2 SYRK(a,b), 3 GEMM(a,b,c)), sub-task << 32 | CTA}. Records beyond
 * `capacity` are dropped (the count keeps growing). Pass NULL to stop tracing. The caller zeroes
 * buf[0] before a launch. ttg_gb300.trace_to_chrome() writes Chrome trace JSON. */
void gbx_set_trace_buffer(unsigned long long* buf, int capacity);

/* ============================================================================================
 * Tile kernels: drop-in replacements for the four vendor-library calls of the device bodies
 * of the potrf flowgraph. FP64, column-major tiles.
 * ========================================================================================== */

/* Replaces cusolverDnDpotrf_bufferSize (examples/potrf/potrf.h:39-42): bytes of device
 * workspace gbx_dpotrf_tile needs for an n x n tile. */
int gbx_dpotrf_tile_bufferSize(int n, int lda, size_t* bytes);

/* Replaces cusolverDnDpotrf(handle, CUBLAS_FILL_MODE_LOWER, n, A, lda, work, lwork, devInfo)
 * (examples/potrf/potrf.h:62-66): A = L L^T in place, lower triangle only (the strict upper
 * triangle is not touched). devInfo (device int) receives 0 or the 1-based index of the first
 * non-positive pivot, exactly as cuSOLVER reports it. */
int gbx_dpotrf_tile(int n, double* A, int lda, void* work, size_t work_bytes, int* devInfo, void* stream);

/* Replaces cublasDtrsm(handle, CUBLAS_SIDE_RIGHT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_T,
 * CUBLAS_DIAG_NON_UNIT, m, n, &one, L, ldl, B, ldb) (examples/potrf/potrf.h:292-297):
 * B := B * L^{-T}, B m x n, L n x n lower. */
int gbx_dtrsm_rlt_tile(int m, int n, const double* L, int ldl, double* B, int ldb, void* stream);

/* Replaces cublasDsyrk(handle, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_N, n, k, &minus_one, A, lda,
 * &one, C, ldc) (examples/potrf/potrf.h:422-427): C := C - A A^T on the lower triangle. */
int gbx_dsyrk_ln_tile(int n, int k, const double* A, int lda, double* C, int ldc, void* stream);

/* Replaces cublasDgemm(handle, CUBLAS_OP_N, CUBLAS_OP_T, m, n, k, &minus_one, A, lda, B, ldb,
 * &one, C, ldc) (examples/potrf/potrf.h:547-553): C := C - A B^T. */
int gbx_dgemm_nt_tile(int m, int n, int k, const double* A, int lda, const double* B, int ldb,
                      double* C, int ldc, void* stream);

/* Tile kernels of the backward sweep of the tiled solve flowgraph (ttg_gb300/potrf/potrs.h). The
 * reference has no solve; these are the non-transposed forms of its TRSM and GEMM calls
 * (examples/potrf/potrf.h:292-297 and 547-553), for right-hand-side tiles stored as nrhs x NB:
 *   gbx_dtrsm_rln_tile: B := B * L^{-1}, B m x n, L n x n lower non-unit (n <= 3200);
 *   gbx_dgemm_nn_tile:  C := C - A * B, A m x k, B k x n. */
int gbx_dtrsm_rln_tile(int m, int n, const double* L, int ldl, double* B, int ldb, void* stream);
int gbx_dgemm_nn_tile(int m, int n, int k, const double* A, int lda, const double* B, int ldb, double* C, int ldc,
                      void* stream);

/* ============================================================================================
 * Whole-flowgraph device executor. One persistent launch runs every POTRF/TRSM/SYRK/GEMM task
 * of the potrf flowgraph (examples/potrf/potrf.h:670-764) over a tile-major lower matrix: CTAs
 * take tasks from a device-side ready queue (the flowgraph's keys in a lookahead order) and
 * wait, with a time limit, on per-block completion counters that encode the flowgraph's
 * successor rules (potrf.h:112-116, 259-268, 449-457, 578-586). Tiles larger than 128 are
 * processed as 128 x 128 blocks inside the tile.
 * Supported NB: any NB <= 128, or a multiple of 32 above that.
 * ========================================================================================== */

/* Bytes of device workspace gbx_dpotrf_tiled needs. */
int gbx_dpotrf_tiled_bufferSize(int N, int NB, size_t* bytes);

/* Block edge of the executor (the reference's tile tasks run as tasks on blocks inside the tiles):
 * 0 (default) = automatic, 64-blocks for N <= 4096 with FP64 FMA updates and for N <= 2048 with the
 * tensor-core updates (gbx_set_fp64_update; a small matrix is bound by its chain of block steps),
 * 128 above; 32, 64 or 128 forces that edge where it divides the tile (else the
 * automatic edge). Applies to later gbx_dpotrf_tiled / gbx_dpotrs_tiled / bufferSize calls, which
 * must agree: size the workspace after setting it. Returns 0 or GBX_ERR_ARG. */
int gbx_set_dag_block_edge(int b);

/* FP64 update mode of the tiled executor (gbx_dpotrf_tiled, gbx_dposv_tiled_host and their
 * bufferSize calls; replaces the cublasDsyrk / cublasDgemm tile calls at examples/potrf/potrf.h:422-427
 * and 547-553 inside it):
 *   0 (default)  FP64 FMA block GEMMs;
 *   1            the same products on the bf16 tensor cores, exactly: each finished block of L is
 *                split into seven 8-bit digit planes with a power-of-two scale per row, the 28 plane
 *                products of the seven leading digit groups accumulate exactly in FP32, and each
 *                element is composed from the exact integer sum with one rounding to FP64 and
 *                subtracted from C with one FP64 add (product error ~2^-55 of the rows' largest
 *                entries, the FP64 dot product's is ~k 2^-53). POTRF and TRSM tasks stay FP64.
 *                Needs 128-blocks (the tile edge a multiple of 128 and N above the small-matrix
 *                threshold, or gbx_set_dag_block_edge(128)); other block edges run mode 0. The
 *                workspace grows by 7 x 32 KB + 512 B per lower 128-block (7.6 GB at N = 32768).
 * Size the workspace after setting it. Returns 0 or GBX_ERR_ARG. */
int gbx_set_fp64_update(int mode);
int gbx_get_fp64_update(void);

/* Factorises the tile-major lower matrix in place (asynchronous). The status is kept in the
 * workspace; read it with gbx_dpotrf_tiled_status. */
int gbx_dpotrf_tiled(int N, int NB, double* tiles, void* work, size_t work_bytes, void* stream);

/* Allocation-free variant of gbx_dpotrf_tiled, for callers that cannot call cudaMalloc (device
 * memory owned by another allocator or budgeted up front; latency-critical paths that cannot take
 * cudaMalloc's device synchronisation). No counterpart in the reference. Its scratch is a
 * library-owned static device array of 525,376 bytes that every GPU loading the library keeps until
 * the process exits; it limits the problem to 512 blocks per edge (N <= 65536 with 128-blocks:
 * NB <= 128 gives blocks of NB, larger NB blocks of 128, 64 or 32) and larger problems return
 * GBX_ERR_NOALLOC_LIMIT. The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress) and keeps it for later calls: make that first call before any stream
 * capture. cudaDeviceReset invalidates the kept address (the module is loaded again at a new
 * address), so do not call this entry point in a process after a cudaDeviceReset of that device.
 * All calls share the array, so calls that overlap on the GPU (other streams, other threads) race;
 * serialise them. The factorisation
 * status (0, first bad pivot, GBX_ERR_TIMEOUT) is written to the device int devInfo. Asynchronous. */
int gbx_dpotrf_tiled_noalloc(int N, int NB, double* tiles, int* devInfo, void* stream);

/* Synchronises `stream` and returns the status of the last gbx_dpotrf_tiled on `work`:
 * 0, >0 (first bad pivot, 1-based global index) or GBX_ERR_TIMEOUT. */
int gbx_dpotrf_tiled_status(const void* work, void* stream);

/* Solves (L L^T) X = B in place for nrhs right-hand sides (B column-major, N x nrhs, ldb),
 * using the tile-major factor written by gbx_dpotrf_tiled (asynchronous). */
int gbx_dpotrs_tiled(int N, int NB, const double* tiles, int nrhs, double* B, int ldb, void* stream);

/* Fills a tile-major lower matrix on the device (asynchronous).
 * gbx_dplgsy_tiled: the PLASMA generator of the reference (examples/potrf/core_plgsy.h:64-150
 *   with the LCG of examples/potrf/random.h), bump added to the diagonal, bit-identical to it.
 * gbx_dgen_uniform_sym_tiled: A = (M + M^T)/2 + shift*I with M_ij uniform in [-0.5, 0.5) from a
 *   counter-based generator keyed by (seed, i, j). */
int gbx_dplgsy_tiled(int N, int NB, double bump, unsigned long long seed, double* tiles, void* stream);
int gbx_dgen_uniform_sym_tiled(int N, int NB, unsigned long long seed, double shift, double* tiles,
                               void* stream);

/* A = Q diag(lam) Q^T on the device, Q = I - U V^T the compact-WY form of a product of r <= 8
 * Householder reflectors (U, V column-major N x r, G = V^T diag(lam) V column-major r x r; all
 * device pointers). The generator of the ill-conditioned (kappa = max lam / min lam) workloads. */
int gbx_dgen_lowrank_sym_tiled(int N, int NB, const double* lam, const double* U, const double* V, const double* G,
                               int r, double* tiles, void* stream);

/* Replaces CORE_dplgsy (examples/potrf/core_plgsy.h:64-150) for one tile: fills the m x n
 * column-major tile A (lda) holding rows m0.. and columns n0.. of the gM x gM PLASMA test matrix,
 * bit-identical to the reference generator (diagonal tiles mirrored and bumped). */
int gbx_dplgsy_tile(double bump, int m, int n, double* A, int lda, int gM, int m0, int n0, unsigned long long seed,
                    void* stream);

/* ============================================================================================
 * Tensor-core building block (tcgen05, sm_103a)
 * ========================================================================================== */

/* D := A * B^T in fp32 on the 5th-generation tensor cores: A is M x K and B is N x K, both bf16
 * and K-major (row-major, leading dimensions lda/ldb multiples of 8, 16-byte aligned), D is
 * column-major M x N (ldd). No reference counterpart: this is the low-precision contraction the
 * mixed-precision factorisation is built on, exposed for testing and reuse. `status` (device int,
 * may be NULL) receives GBX_ERR_TIMEOUT if a pipeline wait ran out of time. */
int gbx_gemm_bf16_nt_f32(int M, int N, int K, const void* A, int lda, const void* B, int ldb, float* D, int ldd,
                         int* status, void* stream);

/* ============================================================================================
 * Mixed precision: low-precision tensor-core factorisation + FP64 refinement. No counterpart in
 * the reference (which has no solve and no mixed precision); built on the same flowgraph.
 * ========================================================================================== */

/* Precision of the off-diagonal tensor-core operands (E4M3: fp8, tcgen05 kind::f8f6f4). */
#define GBX_PREC_BF16 0
#define GBX_PREC_FP16 1
#define GBX_PREC_E4M3 2

/* Bytes of workspace gbx_potrf_mixed needs (NB 256 or 512). */
int gbx_potrf_mixed_bufferSize(int N, int NB, size_t* bytes);

/* Low-precision Cholesky of the FP64 tile-major lower matrix A into the FP32 tile-major factor W
 * (same layout): diagonal POTRF and TRSM in FP32, SYRK/GEMM updates on the tensor cores with
 * bf16/fp16/fp8-e4m3 operands scaled per row by powers of two and FP32 accumulation. The diagonal of A is
 * multiplied by (1 + shift) first (0 for none).
 * fp64_diag_cond: a diagonal tile whose condition estimate, max_i a_ii / min_i a_ii of the tile after
 * its updates (a lower bound of its condition number), exceeds this threshold (or which has a
 * non-positive diagonal entry) is factorised in FP64 instead (the reference's diagonal POTRF is
 * FP64, examples/potrf/potrf.h:62-66); 0 sends every diagonal tile to FP64, a huge value (1e300)
 * none. The FP64 route uses one NB x NB FP64 scratch tile per diagonal tile in the workspace.
 * Asynchronous; the status (0, first bad pivot, or GBX_ERR_TIMEOUT), the largest diagonal-tile
 * condition estimate (from the factor's diagonal) and the number of diagonal tiles factorised in
 * FP64 come from gbx_potrf_mixed_info, which synchronises the stream. */
int gbx_potrf_mixed(int N, int NB, const double* A, float* W, int prec, double shift, double fp64_diag_cond,
                    void* work, size_t work_bytes, void* stream);
int gbx_potrf_mixed_info(const void* work, int N, int NB, float* cond_est, int* fp64_tiles, void* stream);

/* Inverses of the FP32 diagonal factor tiles: Inv holds NT tiles of NB*NB floats, tile K =
 * L_KK^{-T} column-major. */
int gbx_spotri_diag(int N, int NB, const float* W, float* Inv, void* stream);

/* Z := (W W^T)^{-1} R for nrhs <= 16 column-major FP64 right-hand sides (FP32 arithmetic inside);
 * tmp holds 2*N*nrhs floats. */
int gbx_sprecond(int N, int NB, const float* W, const float* Inv, int nrhs, const double* R, double* Z, float* tmp,
                 void* stream);

/* Y := alpha A X + beta Y in FP64 with A symmetric, stored as FP64 tile-major lower tiles;
 * X and Y column-major N x nrhs (nrhs <= 16). */
int gbx_dsymm_tiled(int N, int NB, const double* A, int nrhs, double alpha, const double* X, double beta, double* Y,
                    void* stream);

typedef struct gbx_refine_info {
  int iterations;        /* preconditioned CG iterations */
  int factor_retries;    /* low-precision factorisations repeated with a larger diagonal shift */
  double shift;          /* diagonal shift of the factorisation that succeeded */
  double backward_error; /* max over right-hand sides of ||b - A x||_inf / (||A||_inf ||x||_inf + ||b||_inf) */
  double anorm;          /* ||A||_inf */
  float cond_estimate;   /* largest diagonal-tile condition estimate seen by the factorisation */
  int fp64_diag_tiles;   /* diagonal tiles the factorisation sent to the FP64 route */
} gbx_refine_info;

/* Batched mixed-precision factorisation: the flowgraphs of many SPD matrices of uneven orders
 * n[k] (host array) in ONE persistent launch whose device queue holds every matrix's tile tasks,
 * largest matrix first. A and W: the matrices' tile-major lower storage (tile NB) concatenated in
 * batch order (matrix k's tile slots follow matrix k-1's). sel (host, optional): factorise only the
 * matrices with sel[k] != 0. A breakdown stops only its own matrix; gbx_potrf_mixed_batched_info
 * returns per-matrix info (0 or the first bad pivot) and condition estimates, and synchronises.
 * No counterpart in the reference. */
int gbx_potrf_mixed_batched_bufferSize(int batch, const int* n, int NB, size_t* bytes);
int gbx_potrf_mixed_batched(int batch, const int* n, int NB, const double* A, float* W, int prec, double shift,
                            double fp64_diag_cond, const unsigned char* sel, void* work, size_t work_bytes,
                            void* stream);
int gbx_potrf_mixed_batched_info(const void* work, int batch, const int* n, int NB, int* info, float* cond_est,
                                 int* fp64_tiles, void* stream);

/* Bytes of workspace gbx_dposv_mixed needs (NB 256 or 512, nrhs <= 16). */
int gbx_dposv_mixed_bufferSize(int N, int NB, int nrhs, size_t* bytes);

/* Solves A X = B (A FP64 tile-major lower, B and X column-major N x nrhs, nrhs <= 16) to the FP64
 * backward error `tol`: low-precision factorisation into W (fp64_diag_cond as for
 * gbx_potrf_mixed), then CG in FP64 preconditioned by W. Synchronises the stream. Returns 0, a
 * positive pivot index if every shifted factorisation broke down, GBX_ERR_NOCONV if `maxiter`
 * iterations did not reach `tol`, or another error. */
int gbx_dposv_mixed(int N, int NB, const double* A, int nrhs, const double* B, double* X, int prec,
                    double fp64_diag_cond, double tol, int maxiter, float* W, void* work, size_t work_bytes,
                    gbx_refine_info* info, void* stream);

/* Batched gbx_dposv_mixed: matrices as for gbx_potrf_mixed_batched, right-hand sides and solutions
 * of matrix k column-major n[k] x nrhs, concatenated in batch order. One factorisation launch for
 * the batch (matrices that break down are factorised again with a growing diagonal shift, up to 8
 * attempts), then preconditioned CG in FP64 in which every step runs over the matrices that have
 * not yet met `tol`. The PCG coefficients, the convergence tests and the selection of the matrices
 * still iterating are computed on the device; the retries and the iterations are CUDA-graph WHILE
 * nodes, so the whole solve is one graph with no host synchronisation. No counterpart in the
 * reference.
 *   _plan:   builds the task tables of a batch shape (batch, n, NB, nrhs, prec) and uploads them
 *            into `work`; synchronises `stream`. Not capturable. Once per shape and workspace.
 *            sched: the factorisation queue's order within each panel step, 0 the trailing
 *            updates before the panel's TRSMs (CTAs update while the diagonal POTRF runs), 1 the
 *            TRSMs first (the next panel's chain starts earlier); gbx_dposv_mixed_batched uses 0
 *            and ttg_gb300.autotune.tune_mixed_batched picks one per batch.
 *   _exec:   the solve itself, asynchronous on `stream`: no host synchronisation, no allocation, no
 *            host-to-device copy. When `stream` is capturing, the solve's nodes (with its two
 *            conditional nodes) are added to the caller's graph, which can then be replayed; else
 *            the library builds, launches and releases a graph of its own. Needs a plan of the
 *            same shape in `work` (a mismatch makes the run do nothing and _result return
 *            GBX_ERR_ARG) made earlier in this process on this device.
 *   _result: synchronises `stream` and returns 0 when every matrix met `tol`, GBX_ERR_NOCONV
 *            otherwise, a pivot index for a one-matrix batch whose every factorisation broke
 *            down, or GBX_ERR_TIMEOUT / GBX_ERR_ARG; info (optional) receives one record per
 *            matrix.
 * gbx_dposv_mixed_batched = _plan + _exec + _result. */
int gbx_dposv_mixed_batched_bufferSize(int batch, const int* n, int NB, int nrhs, size_t* bytes);
int gbx_dposv_mixed_batched_plan(int batch, const int* n, int NB, int nrhs, int prec, int sched, void* work,
                                 size_t work_bytes, void* stream);
int gbx_dposv_mixed_batched_exec(int batch, const int* n, int NB, const double* A, int nrhs, const double* B,
                                 double* X, int prec, double fp64_diag_cond, double tol, int maxiter, float* W,
                                 void* work, size_t work_bytes, void* stream);
int gbx_dposv_mixed_batched_result(int batch, const int* n, int NB, int nrhs, double tol, const void* work,
                                   gbx_refine_info* info, void* stream);
int gbx_dposv_mixed_batched(int batch, const int* n, int NB, const double* A, int nrhs, const double* B, double* X,
                            int prec, double fp64_diag_cond, double tol, int maxiter, float* W, void* work,
                            size_t work_bytes, gbx_refine_info* info, void* stream);

/* hi[i] + lo[i] = a[i] for n FP64 values: hi = fl32(a), lo = fl32(a - hi), rounded to nearest even
 * (the double-float split of the refinement's residual products, computed on the bit pattern;
 * bitwise equal to the FP64 conversions). Asynchronous on `stream`. No counterpart in the reference. */
int gbx_split_f64(const double* a, float* hi, float* lo, long long n, void* stream);

/* Inverse of the SPD matrix from its factor, in place (replaces the reference's host-only POTRI
 * chain, examples/potrf/potri.h:18-29: TRTRI of the lower factor, trtri_L.h, then LAUUM,
 * lauum.h): on entry the lower tiles hold L from gbx_dpotrf_tiled, on exit the lower triangle of
 * A^{-1} (strict upper parts of diagonal tiles and padding past N: unspecified). FP64, NB a
 * multiple of 128; asynchronous on `stream`. */
int gbx_dpotri_tiled_bufferSize(int N, int NB, size_t* bytes);
int gbx_dpotri_tiled(int N, int NB, double* tiles, void* work, size_t work_bytes, void* stream);

/* Factorisation and solve from host buffers (pinned for full copy speed): A_host and L_host hold
 * the tile-major lower storage (tiled_numel doubles), B_host / X_host are column-major N x nrhs;
 * tiles and X are device buffers of the same sizes. A and B are copied in, the executor runs, then
 * L is copied back on a second stream while X = (L L^T)^{-1} B is solved and copied back on
 * `stream`. Returns once the factorisation has finished on the device; the solve and the copies
 * are still queued (`stream` waits for the copy of L). gbx_dpotrf_tiled_status(work) gives the
 * factorisation status. If the factorisation stopped early (a non-positive pivot or a timed-out
 * wait), the solve is skipped, L_host receives the partial factor before the call returns, and
 * the call returns the status itself (>0 first bad pivot, or GBX_ERR_TIMEOUT). The workspace is
 * gbx_dpotrf_tiled's. No
 * counterpart in the reference, whose tiles reach the device through PaRSEC's stage-in
 * (parsec/ttg.h:1434-1672) and come back on wait() (parsec/devicefunc.h:232-256). */
int gbx_dposv_tiled_host_bufferSize(int N, int NB, size_t* bytes);
int gbx_dposv_tiled_host(int N, int NB, const double* A_host, double* L_host, int nrhs, const double* B_host,
                         double* X_host, double* tiles, double* X, void* work, size_t work_bytes, void* stream);

/* ============================================================================================
 * Batched solves of many independent SPD matrices of uneven sizes in one persistent launch
 * (capturable in a CUDA graph: no host synchronisation, no allocation). No counterpart in the
 * reference.
 * ========================================================================================== */

/* Fills matrix k of a batch (device arrays n, offA) with (M + M^T)/2 + n_k I, M_ij uniform in
 * [-0.5, 0.5) from the counter-based generator of gbx_dgen_uniform_sym_tiled with seed
 * seed + k * 0x9e3779b97f4a7c15 (full column-major storage). */
int gbx_dgen_uniform_sym_batched(int batch, const int* n, const long long* offA, unsigned long long seed, double* A,
                                 void* stream);

/* Host helper: the longest-processing-time order (largest matrix first) of a batch. */
int gbx_batched_order(int batch, const int* n_host, int* order_host);

/* For every matrix i (device arrays n, offA, offB, order): A_i = column-major n_i x n_i at
 * A + offA[i] (lower triangle read), right-hand sides column-major n_i x nrhs at B + offB[i],
 * overwritten with the solution. mode 0: FP64 factor + solve (A_i overwritten by L_i); mode 1: FP32
 * factor into L32 (offA layout) + `refine` steps of FP64 iterative refinement (A_i untouched).
 * info[i] = 0 or the first bad pivot. n_i <= 1024. `work` >= 256 bytes (the queue head). */
int gbx_dposv_batched(int batch, const int* n, const long long* offA, const long long* offB, const int* order,
                      double* A, double* B, int nrhs, int mode, int refine, float* L32, int* info, void* work,
                      size_t work_bytes, void* stream);

/* gbx_dposv_batched with an explicit number of CTAs (0 = every resident CTA slot): the knob of the
 * batched autotuner (ttg_gb300/autotune.py). */
int gbx_dposv_batched_ex(int batch, const int* n, const long long* offA, const long long* offB, const int* order,
                         double* A, double* B, int nrhs, int mode, int refine, float* L32, int* info, int ctas,
                         void* work, size_t work_bytes, void* stream);

/* ============================================================================================
 * Device task queue: the persistent device-side ready queue behind the TTG API's device tasks
 * (include/ttg/device/gbx_queue.h). Replaces the reference's per-task hand-off of device tasks to
 * PaRSEC's GPU manager (parsec/ttg.h:1521-1672, 2678-2727).
 * ========================================================================================== */

/* Creates / destroys a queue (at most 64 live queues). */
int gbx_taskq_create(void** q);
int gbx_taskq_destroy(void* q);

/* The queue's recording stream handle. Passed as the `stream` of gbx_dpotrf_tile,
 * gbx_dtrsm_rlt_tile, gbx_dsyrk_ln_tile, gbx_dgemm_nt_tile, gbx_dtrsm_rln_tile or
 * gbx_dgemm_nn_tile, it makes the call append its tile operation to the queue instead of launching
 * a kernel (nothing runs, nothing is read). The handle is not a CUDA stream: give it to no other
 * call. An operation waits for the last writer of every tile it reads or writes and for the
 * readers of every tile it writes (tiles are identified by their base device pointers). The
 * operands must stay allocated until the run that executes the operation has completed. */
void* gbx_taskq_stream(void* q);

/* Operations recorded and not yet run. */
long long gbx_taskq_pending(void* q);

/* Runs every operation recorded since the previous run, in one persistent launch on `stream`
 * (asynchronous; operations of earlier runs are complete once their run is). A POTRF operation
 * writes 0 or its first bad pivot to its devInfo. */
int gbx_taskq_run(void* q, void* stream);

/* Synchronises `stream` and returns the status of the last run: 0 or GBX_ERR_TIMEOUT. */
int gbx_taskq_status(void* q, void* stream);

/* Test hook for the failure path: launches the executor on a 2 x 2 block problem whose first
 * task is skipped, so the dependency wait of the second task can never be satisfied and must
 * run out after `timeout_ns`. Returns the status the kernel reported (GBX_ERR_TIMEOUT when the
 * time limit works). `work` must hold gbx_dpotrf_tiled_bufferSize(2*NB, NB) bytes, `tiles`
 * 3 tiles of NB*NB doubles. Synchronises the stream. */
int gbx_dag_timeout_selftest(int NB, double* tiles, void* work, size_t work_bytes, uint64_t timeout_ns,
                             void* stream);

/* The task orders the persistent executors follow (host-side introspection, no GPU needed): task t
 * of gbx_dpotrf_tiled's order over NTb x NTb blocks, and of the mixed factorisation's order over
 * NT x NT tiles, written to key[4] = {type, a, b, c}: type 0 POTRF of block (a,a); 1 TRSM of
 * block (a,b) by the factor of (b,b); 2 SYRK of block (b,b) with column a; 3 GEMM of block (a,b)
 * with column c. Each returns the number of tasks in the order (t and key are ignored when
 * t < 0), or GBX_ERR_ARG. The orders are the executors' task lists, in which every task's
 * predecessors come earlier, so CTAs that take tasks in order cannot deadlock. */
long long gbx_dag_task(int NTb, long long t, int* key);
/* The same order with `lead` tasks of each step's trailing updates queued ahead of that step's
 * TRSMs (the emulated executor's order; lead 0 is gbx_dag_task's). */
long long gbx_dag_task_lead(int NTb, long long lead, long long t, int* key);
/* Tasks of each step's trailing updates the executor queues ahead of the step's TRSMs: -1 (default)
 * automatic (16 per CTA with tensor-core updates, none with FP64 FMA updates), else that count.
 * Returns 0 or GBX_ERR_ARG. */
int gbx_set_dag_lead(long long tasks);
long long gbx_mixed_task(int NT, long long t, int* key);

#ifdef __cplusplus
}
#endif

#endif /* GBX_POTRF_H */
