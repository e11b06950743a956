// CPU oracle for the tiled Cholesky (potrf) path — TEST INFRASTRUCTURE ONLY.
// See oracle.h for what each part restates and where in the reference it comes from.
// Built with -ffp-contract=off so that x86-64 and aarch64 produce the same bits.
#include "oracle.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <dlfcn.h>
#include <limits>
#include <mutex>
#include <queue>
#include <thread>
#include <unordered_map>
#include <vector>

// ------------------------------------------------------------------------------------------------
// layout
// ------------------------------------------------------------------------------------------------
extern "C" int64_t orc_tile_slot(int m, int n, int NT) {
  return (int64_t)n * NT - (int64_t)n * (n - 1) / 2 + (m - n);
}

static inline int tile_dim(int t, int NT, int N, int NB) { return (t == NT - 1) ? N - (NT - 1) * NB : NB; }

extern "C" void orc_tiles_from_colmajor(int N, int NB, const double* A, int64_t lda, double* tiles) {
  const int NT = (N + NB - 1) / NB;
  for (int n = 0; n < NT; ++n)
    for (int m = n; m < NT; ++m) {
      double* t = tiles + orc_tile_slot(m, n, NT) * (int64_t)NB * NB;
      const int mb = tile_dim(m, NT, N, NB), nb = tile_dim(n, NT, N, NB);
      std::memset(t, 0, sizeof(double) * (size_t)NB * NB);
      for (int j = 0; j < nb; ++j)
        for (int i = 0; i < mb; ++i) t[i + (int64_t)j * NB] = A[(int64_t)(m * NB + i) + (int64_t)(n * NB + j) * lda];
    }
}

extern "C" void orc_tiles_to_colmajor(int N, int NB, const double* tiles, double* A, int64_t lda) {
  const int NT = (N + NB - 1) / NB;
  for (int j = 0; j < N; ++j)
    for (int i = 0; i < N; ++i) A[i + (int64_t)j * lda] = 0.0;
  for (int n = 0; n < NT; ++n)
    for (int m = n; m < NT; ++m) {
      const double* t = tiles + orc_tile_slot(m, n, NT) * (int64_t)NB * NB;
      const int mb = tile_dim(m, NT, N, NB), nb = tile_dim(n, NT, N, NB);
      for (int j = 0; j < nb; ++j)
        for (int i = 0; i < mb; ++i) {
          const int gi = m * NB + i, gj = n * NB + j;
          if (gi >= gj) A[gi + (int64_t)gj * lda] = t[i + (int64_t)j * NB];
        }
    }
}

// ------------------------------------------------------------------------------------------------
// generators
// ------------------------------------------------------------------------------------------------
// PLASMA LCG (examples/potrf/random.h:19-41): x_{k+1} = A x_k + C mod 2^64, with a log-time jump.
static const unsigned long long kLcgA = 6364136223846793005ULL;
static const unsigned long long kLcgC = 1ULL;
static const float kLcgToFloat = 5.4210108624275222e-20f;  // 2^-64 as a float literal

static unsigned long long lcg_jump(unsigned long long n, unsigned long long seed) {
  unsigned long long a = kLcgA, c = kLcgC, x = seed;
  while (n) {
    if (n & 1ULL) x = a * x + c;
    c *= (a + 1);
    a *= a;
    n >>= 1;
  }
  return x;
}

// One entry: the reference evaluates `0.5f - ran * RndF_Mul` in float (ran converted to float),
// then stores the float into a double (core_plgsy.h:86,115).
static inline double lcg_entry(unsigned long long ran) {
  const float r = (float)ran;
  const float p = r * kLcgToFloat;
  const float v = 0.5f - p;
  return (double)v;
}

extern "C" void orc_plgsy_tile(double bump, int m, int n, double* A, int lda, int gM, int m0, int n0,
                               unsigned long long seed) {
  // Tiles on or below the diagonal draw column j's entries from the stream position of global
  // element (m0, n0+j) onwards; diagonal tiles draw from the diagonal down and mirror the lower
  // part up, then add `bump` to the diagonal; tiles above the diagonal are drawn row by row from
  // the transposed position (core_plgsy.h:78-148).
  if (m0 == n0) {
    unsigned long long pos = (unsigned long long)m0 + (unsigned long long)n0 * (unsigned long long)gM;
    for (int j = 0; j < n; ++j) {
      unsigned long long ran = lcg_jump(pos, seed);
      for (int i = j; i < m; ++i) {
        A[i + (int64_t)j * lda] = lcg_entry(ran);
        ran = kLcgA * ran + kLcgC;
      }
      pos += (unsigned long long)gM + 1;
    }
    for (int j = 0; j < n; ++j) {
      A[j + (int64_t)j * lda] += bump;
      for (int i = 0; i < j; ++i) A[i + (int64_t)j * lda] = A[j + (int64_t)i * lda];
    }
  } else if (m0 > n0) {
    unsigned long long pos = (unsigned long long)m0 + (unsigned long long)n0 * (unsigned long long)gM;
    for (int j = 0; j < n; ++j) {
      unsigned long long ran = lcg_jump(pos, seed);
      for (int i = 0; i < m; ++i) {
        A[i + (int64_t)j * lda] = lcg_entry(ran);
        ran = kLcgA * ran + kLcgC;
      }
      pos += (unsigned long long)gM;
    }
  } else {
    unsigned long long pos = (unsigned long long)n0 + (unsigned long long)m0 * (unsigned long long)gM;
    for (int i = 0; i < m; ++i) {
      unsigned long long ran = lcg_jump(pos, seed);
      for (int j = 0; j < n; ++j) {
        A[i + (int64_t)j * lda] = lcg_entry(ran);
        ran = kLcgA * ran + kLcgC;
      }
      pos += (unsigned long long)gM;
    }
  }
}

extern "C" void orc_plgsy_tiles(int N, int NB, double bump, unsigned long long seed, double* tiles) {
  const int NT = (N + NB - 1) / NB;
  for (int n = 0; n < NT; ++n)
    for (int m = n; m < NT; ++m) {
      double* t = tiles + orc_tile_slot(m, n, NT) * (int64_t)NB * NB;
      std::memset(t, 0, sizeof(double) * (size_t)NB * NB);
      orc_plgsy_tile(bump, tile_dim(m, NT, N, NB), tile_dim(n, NT, N, NB), t, NB, N, m * NB, n * NB, seed);
    }
}

// Counter-based generator: element (i,j) of stream `seed` is a function of (seed, i, j) only, so
// any tile can be produced independently on the host or on the device with identical bits.
static inline uint64_t mix64(uint64_t z) {
  z += 0x9e3779b97f4a7c15ULL;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
  return z ^ (z >> 31);
}

extern "C" double orc_uniform_elem(uint64_t seed, int64_t i, int64_t j) {
  const uint64_t r = mix64(mix64(seed) ^ (((uint64_t)i << 32) | (uint64_t)(uint32_t)j));
  return (double)(r >> 11) * (1.0 / 9007199254740992.0) - 0.5;  // exact: k*2^-53 - 1/2
}

static inline double sym_elem(uint64_t seed, double shift, int64_t i, int64_t j) {
  if (i == j) return orc_uniform_elem(seed, i, i) + shift;
  return 0.5 * (orc_uniform_elem(seed, i, j) + orc_uniform_elem(seed, j, i));  // exact
}

extern "C" void orc_gen_uniform_sym_tiles(int N, int NB, uint64_t seed, double shift, double* tiles) {
  const int NT = (N + NB - 1) / NB;
  for (int n = 0; n < NT; ++n)
    for (int m = n; m < NT; ++m) {
      double* t = tiles + orc_tile_slot(m, n, NT) * (int64_t)NB * NB;
      const int mb = tile_dim(m, NT, N, NB), nb = tile_dim(n, NT, N, NB);
      for (int j = 0; j < NB; ++j)
        for (int i = 0; i < NB; ++i)
          t[i + (int64_t)j * NB] = (i < mb && j < nb) ? sym_elem(seed, shift, (int64_t)m * NB + i, (int64_t)n * NB + j) : 0.0;
    }
}

extern "C" void orc_gen_uniform_sym_colmajor(int N, uint64_t seed, double shift, double* A, int64_t lda) {
  for (int64_t j = 0; j < N; ++j)
    for (int64_t i = 0; i < N; ++i) A[i + j * lda] = sym_elem(seed, shift, i, j);
}

// ------------------------------------------------------------------------------------------------
// tile kernels (plain loops)
// ------------------------------------------------------------------------------------------------
// Unblocked left-looking Cholesky, lower (the LAPACK dpotf2 algorithm). Returns info = j+1 for the
// first non-positive pivot, as LAPACK does.
extern "C" int orc_potrf_tile(int n, double* A, int lda) {
  for (int j = 0; j < n; ++j) {
    double ajj = A[j + (int64_t)j * lda];
    for (int k = 0; k < j; ++k) ajj -= A[j + (int64_t)k * lda] * A[j + (int64_t)k * lda];
    if (!(ajj > 0.0)) {
      A[j + (int64_t)j * lda] = ajj;
      return j + 1;
    }
    ajj = std::sqrt(ajj);
    A[j + (int64_t)j * lda] = ajj;
    for (int i = j + 1; i < n; ++i) {
      double s = A[i + (int64_t)j * lda];
      for (int k = 0; k < j; ++k) s -= A[i + (int64_t)k * lda] * A[j + (int64_t)k * lda];
      A[i + (int64_t)j * lda] = s / ajj;
    }
  }
  return 0;
}

// B := B * L^{-T} (Right, Lower, Trans, NonUnit) — column by column, left to right.
extern "C" void orc_trsm_rlt_tile(int m, int n, const double* L, int ldl, double* B, int ldb) {
  for (int j = 0; j < n; ++j) {
    double* bj = B + (int64_t)j * ldb;
    for (int k = 0; k < j; ++k) {
      const double l = L[j + (int64_t)k * ldl];
      const double* bk = B + (int64_t)k * ldb;
      for (int i = 0; i < m; ++i) bj[i] -= bk[i] * l;
    }
    const double d = L[j + (int64_t)j * ldl];
    for (int i = 0; i < m; ++i) bj[i] = bj[i] / d;
  }
}

// C := C - A A^T on the lower triangle (n x n), A is n x k.
extern "C" void orc_syrk_ln_tile(int n, int k, const double* A, int lda, double* C, int ldc) {
  for (int j = 0; j < n; ++j)
    for (int l = 0; l < k; ++l) {
      const double b = A[j + (int64_t)l * lda];
      const double* al = A + (int64_t)l * lda;
      double* cj = C + (int64_t)j * ldc;
      for (int i = j; i < n; ++i) cj[i] -= al[i] * b;
    }
}

// C := C - A B^T, A m x k, B n x k.
extern "C" void orc_gemm_nt_tile(int m, int n, int k, const double* A, int lda, const double* B, int ldb,
                                 double* C, int ldc) {
  for (int j = 0; j < n; ++j)
    for (int l = 0; l < k; ++l) {
      const double b = B[j + (int64_t)l * ldb];
      const double* al = A + (int64_t)l * lda;
      double* cj = C + (int64_t)j * ldc;
      for (int i = 0; i < m; ++i) cj[i] -= al[i] * b;
    }
}

// The backward sweep's tile operations of the tiled solve on nrhs x NB right-hand-side tiles (the
// reference has no solve; these are the non-transposed forms of its TRSM and GEMM).
// B := B * L^{-1} (Right, Lower, NoTrans, NonUnit) — column by column, right to left.
extern "C" void orc_trsm_rln_tile(int m, int n, const double* L, int ldl, double* B, int ldb) {
  for (int j = n - 1; j >= 0; --j) {
    double* bj = B + (int64_t)j * ldb;
    for (int k = j + 1; k < n; ++k) {
      const double l = L[k + (int64_t)j * ldl];
      const double* bk = B + (int64_t)k * ldb;
      for (int i = 0; i < m; ++i) bj[i] -= bk[i] * l;
    }
    const double d = L[j + (int64_t)j * ldl];
    for (int i = 0; i < m; ++i) bj[i] = bj[i] / d;
  }
}

// C := C - A B, A m x k, B k x n.
extern "C" void orc_gemm_nn_tile(int m, int n, int k, const double* A, int lda, const double* B, int ldb,
                                 double* C, int ldc) {
  for (int j = 0; j < n; ++j)
    for (int l = 0; l < k; ++l) {
      const double b = B[l + (int64_t)j * ldb];
      const double* al = A + (int64_t)l * lda;
      double* cj = C + (int64_t)j * ldc;
      for (int i = 0; i < m; ++i) cj[i] -= al[i] * b;
    }
}

// ------------------------------------------------------------------------------------------------
// OpenBLAS tile kernels (Fortran ABI, hidden string lengths appended)
// ------------------------------------------------------------------------------------------------
namespace {
typedef void (*potrf_fn)(const char*, const int*, double*, const int*, int*, size_t);
typedef void (*trsm_fn)(const char*, const char*, const char*, const char*, const int*, const int*,
                        const double*, const double*, const int*, double*, const int*, size_t, size_t,
                        size_t, size_t);
typedef void (*syrk_fn)(const char*, const char*, const int*, const int*, const double*, const double*,
                        const int*, const double*, double*, const int*, size_t, size_t);
typedef void (*gemm_fn)(const char*, const char*, const int*, const int*, const int*, const double*,
                        const double*, const int*, const double*, const int*, const double*, double*,
                        const int*, size_t, size_t);
typedef void (*nthreads_fn)(int);
struct Blas {
  potrf_fn potrf = nullptr;
  trsm_fn trsm = nullptr;
  syrk_fn syrk = nullptr;
  gemm_fn gemm = nullptr;
  nthreads_fn set_threads = nullptr;
} g_blas;

void* find_sym(void* h, const char* base) {
  char name[128];
  const char* pats[] = {"scipy_%s_", "%s_", "scipy_%s", "%s"};
  for (const char* p : pats) {
    std::snprintf(name, sizeof name, p, base);
    if (void* s = dlsym(h, name)) return s;
  }
  return nullptr;
}
}  // namespace

extern "C" int orc_blas_load(const char* path) {
  void* h = dlopen(path, RTLD_NOW | RTLD_LOCAL);
  if (!h) return -1;
  g_blas.potrf = (potrf_fn)find_sym(h, "dpotrf");
  g_blas.trsm = (trsm_fn)find_sym(h, "dtrsm");
  g_blas.syrk = (syrk_fn)find_sym(h, "dsyrk");
  g_blas.gemm = (gemm_fn)find_sym(h, "dgemm");
  g_blas.set_threads = (nthreads_fn)dlsym(h, "scipy_openblas_set_num_threads");
  if (!g_blas.set_threads) g_blas.set_threads = (nthreads_fn)dlsym(h, "openblas_set_num_threads");
  if (!g_blas.potrf || !g_blas.trsm || !g_blas.syrk || !g_blas.gemm) {
    g_blas = Blas{};
    return -2;
  }
  if (g_blas.set_threads) g_blas.set_threads(1);
  return 0;
}

extern "C" int orc_blas_loaded(void) { return g_blas.gemm != nullptr; }

// ------------------------------------------------------------------------------------------------
// the flowgraph on a keyed host task runtime
// ------------------------------------------------------------------------------------------------
namespace {
enum TaskType { POTRF = 0, TRSM = 1, SYRK = 2, GEMM = 3 };

struct Task {
  int type, a, b, c;  // POTRF(K): a=K; TRSM(M,K): a=M b=K; SYRK(K,M): a=K b=M; GEMM(M,N,K): a=M b=N c=K
  int64_t prio;
  bool operator<(const Task& o) const { return prio < o.prio; }  // max-heap on priority
};

inline uint64_t pack(int type, int a, int b, int c) {
  return ((uint64_t)type << 60) | ((uint64_t)(uint32_t)a << 40) | ((uint64_t)(uint32_t)b << 20) | (uint64_t)(uint32_t)c;
}

// number of inputs of each task type (make_tt input lists of potrf.h:189, 323, 459, 588)
inline int num_inputs(int type) { return type == POTRF ? 1 : (type == GEMM ? 3 : 2); }

struct Graph {
  int N, NB, NT;
  double* tiles;
  int use_blas;
  std::mutex mtx;
  std::condition_variable cv;
  std::priority_queue<Task> ready;
  std::unordered_map<uint64_t, int> pending;  // inputs received so far per task key
  int64_t remaining = 0;                      // tasks not yet finished
  int failed = 0, fail_info = 0;
  int64_t* trace = nullptr;
  int64_t trace_cap = 0, ntrace = 0;

  double* tile(int m, int n) { return tiles + orc_tile_slot(m, n, NT) * (int64_t)NB * NB; }
  int dim(int t) const { return tile_dim(t, NT, N, NB); }

  // deliver one input to task (type,a,b,c); caller holds mtx
  void deliver(int type, int a, int b, int c) {
    const uint64_t k = pack(type, a, b, c);
    int& cnt = pending[k];
    if (++cnt == num_inputs(type)) {
      pending.erase(k);
      ready.push(Task{type, a, b, c, orc_priority(type, NT, a, b, c)});
      cv.notify_one();
    }
  }

  // dispatcher (potrf.h:633-668): route tile (i,j) to its first consumer
  void dispatch(int i, int j) {
    if (i == 0 && j == 0) deliver(POTRF, 0, 0, 0);
    else if (i == j) deliver(SYRK, 0, i, 0);
    else if (j == 0) deliver(TRSM, i, 0, 0);
    else deliver(GEMM, i, j, 0);
  }

  int run_body(const Task& t) {
    const int ld = NB;
    switch (t.type) {
      case POTRF: {
        const int K = t.a, nb = dim(K);
        int info = 0;
        if (use_blas) g_blas.potrf("L", &nb, tile(K, K), &ld, &info, 1);
        else info = orc_potrf_tile(nb, tile(K, K), ld);
        return info;
      }
      case TRSM: {
        const int M = t.a, K = t.b, mb = dim(M), nb = dim(K);
        const double one = 1.0;
        if (use_blas) g_blas.trsm("R", "L", "T", "N", &mb, &nb, &one, tile(K, K), &ld, tile(M, K), &ld, 1, 1, 1, 1);
        else orc_trsm_rlt_tile(mb, nb, tile(K, K), ld, tile(M, K), ld);
        return 0;
      }
      case SYRK: {
        const int K = t.a, M = t.b, mb = dim(M), nb = dim(K);
        const double alpha = -1.0, beta = 1.0;
        if (use_blas) g_blas.syrk("L", "N", &mb, &nb, &alpha, tile(M, K), &ld, &beta, tile(M, M), &ld, 1, 1);
        else orc_syrk_ln_tile(mb, nb, tile(M, K), ld, tile(M, M), ld);
        return 0;
      }
      default: {
        const int M = t.a, Nn = t.b, K = t.c, mb = dim(M), nb = dim(Nn), kb = dim(K);
        const double alpha = -1.0, beta = 1.0;
        if (use_blas)
          g_blas.gemm("N", "T", &mb, &nb, &kb, &alpha, tile(M, K), &ld, tile(Nn, K), &ld, &beta, tile(M, Nn), &ld, 1, 1);
        else orc_gemm_nt_tile(mb, nb, kb, tile(M, K), ld, tile(Nn, K), ld, tile(M, Nn), ld);
        return 0;
      }
    }
  }

  // successor rules: potrf.h:112-116 (POTRF), 259-268 (TRSM), 449-457 (SYRK), 578-586 (GEMM)
  void release(const Task& t) {
    switch (t.type) {
      case POTRF:
        for (int m = t.a + 1; m < NT; ++m) deliver(TRSM, m, t.a, 0);
        break;
      case TRSM: {
        const int M = t.a, K = t.b;
        deliver(SYRK, K, M, 0);
        for (int n = K + 1; n < M; ++n) deliver(GEMM, M, n, K);   // row: GEMM's tile_mk
        for (int m = M + 1; m < NT; ++m) deliver(GEMM, m, M, K);  // column: GEMM's tile_nk
        break;
      }
      case SYRK: {
        const int K = t.a, M = t.b;
        if (M == K + 1) deliver(POTRF, K + 1, 0, 0);
        else deliver(SYRK, K + 1, M, 0);
        break;
      }
      default: {
        const int M = t.a, Nn = t.b, K = t.c;
        if (Nn == K + 1) deliver(TRSM, M, Nn, 0);
        else deliver(GEMM, M, Nn, K + 1);
        break;
      }
    }
  }

  void worker() {
    std::unique_lock<std::mutex> lk(mtx);
    for (;;) {
      cv.wait(lk, [&] { return !ready.empty() || remaining == 0 || failed; });
      if (remaining == 0 || failed) return;
      Task t = ready.top();
      ready.pop();
      if (trace && ntrace < trace_cap) trace[ntrace] = (int64_t)pack(t.type, t.a, t.b, t.c);
      ++ntrace;
      lk.unlock();
      const int info = run_body(t);
      lk.lock();
      if (info != 0) {  // the reference aborts here (potrf.h:179-187); the oracle reports instead
        failed = t.a + 1;
        fail_info = info;
        cv.notify_all();
        return;
      }
      release(t);
      if (--remaining == 0) cv.notify_all();
    }
  }
};
}  // namespace

extern "C" int64_t orc_priority(int type, int nt, int a, int b, int c) {
  const int64_t n = nt;
  switch (type) {
    case POTRF: return (n - a) * (n - a) * (n - a);
    case TRSM: return (n - a) * (n - a) * (n - a) + 3 * ((2 * n) - b - a - 1) * (int64_t)(a - b);
    case SYRK: return (n - a) * (n - a) * (n - a) + 3 * (int64_t)(a - b);
    default: return (n - a) * (n - a) * (n - a) + 3 * ((2 * n) - a - b - 3) * (int64_t)(a - b) + 6 * (int64_t)(a - c);
  }
}

extern "C" int orc_potrf_tiled(int N, int NB, double* tiles, int nthreads, int use_blas, int* tile_info,
                               int64_t* trace, int64_t trace_cap, int64_t* ntrace) {
  if (N <= 0 || NB <= 0) return -1;
  if (use_blas && !orc_blas_loaded()) return -2;
  Graph g;
  g.N = N;
  g.NB = NB;
  g.NT = (N + NB - 1) / NB;
  g.tiles = tiles;
  g.use_blas = use_blas;
  g.trace = trace;
  g.trace_cap = trace_cap;
  const int64_t nt = g.NT;
  g.remaining = nt + nt * (nt - 1) / 2 * 2 + nt * (nt - 1) * (nt - 2) / 6;  // POTRF + TRSM + SYRK + GEMM
  {
    std::lock_guard<std::mutex> lk(g.mtx);
    for (int i = 0; i < g.NT; ++i)
      for (int j = 0; j <= i; ++j) g.dispatch(i, j);
  }
  if (nthreads <= 0) nthreads = (int)std::max(1u, std::thread::hardware_concurrency());
  std::vector<std::thread> pool;
  for (int t = 0; t < nthreads; ++t) pool.emplace_back([&g] { g.worker(); });
  for (auto& th : pool) th.join();
  if (ntrace) *ntrace = g.ntrace;
  if (tile_info) *tile_info = g.fail_info;
  return g.failed;
}

// ------------------------------------------------------------------------------------------------
// solve and checks
// ------------------------------------------------------------------------------------------------
extern "C" void orc_potrs_tiled(int N, int NB, const double* tiles, int nrhs, double* X, int64_t ldx) {
  const int NT = (N + NB - 1) / NB;
  auto L = [&](int64_t i, int64_t j) -> double {
    const int m = (int)(i / NB), n = (int)(j / NB);
    return tiles[orc_tile_slot(m, n, NT) * (int64_t)NB * NB + (i % NB) + (j % NB) * (int64_t)NB];
  };
  for (int r = 0; r < nrhs; ++r) {
    double* x = X + (int64_t)r * ldx;
    for (int64_t j = 0; j < N; ++j) {  // L y = b (column-oriented forward substitution)
      x[j] /= L(j, j);
      const double xj = x[j];
      for (int64_t i = j + 1; i < N; ++i) x[i] -= L(i, j) * xj;
    }
    for (int64_t i = N - 1; i >= 0; --i) {  // L^T x = y
      double s = x[i];
      for (int64_t k = i + 1; k < N; ++k) s -= L(k, i) * x[k];
      x[i] = s / L(i, i);
    }
  }
}

static void lower_llt(int N, const double* L, std::vector<double>& R) {
  // R = L L^T (full), blocked over k for cache reuse
  R.assign((size_t)N * N, 0.0);
  for (int64_t k = 0; k < N; ++k)
    for (int64_t j = k; j < N; ++j) {
      const double b = L[j + k * N];
      if (b == 0.0) continue;
      double* rj = R.data() + j * N;
      const double* lk = L + k * N;
      for (int64_t i = j; i < N; ++i) rj[i] += lk[i] * b;
    }
  for (int64_t j = 0; j < N; ++j)
    for (int64_t i = 0; i < j; ++i) R[i + j * N] = R[j + i * N];
}

extern "C" double orc_check_dpotrf(int N, const double* L, const double* A0) {
  std::vector<double> R;
  lower_llt(N, L, R);
  double rnorm = 0.0, anorm = 0.0;
  for (int64_t i = 0; i < N; ++i) {
    double rs = 0.0, as = 0.0;
    for (int64_t j = 0; j < N; ++j) {
      rs += std::fabs(R[i + j * N] - A0[i + j * N]);
      as += std::fabs(A0[i + j * N]);
    }
    rnorm = std::max(rnorm, rs);
    anorm = std::max(anorm, as);
  }
  return rnorm / (anorm * N * std::numeric_limits<double>::epsilon());
}

extern "C" double orc_frob_residual(int N, const double* L, const double* A0) {
  std::vector<double> R;
  lower_llt(N, L, R);
  double r2 = 0.0, a2 = 0.0;
  for (int64_t k = 0; k < (int64_t)N * N; ++k) {
    const double d = R[k] - A0[k];
    r2 += d * d;
    a2 += A0[k] * A0[k];
  }
  return std::sqrt(r2) / (N * std::sqrt(a2));
}

// ------------------------------------------------------------------------------------------------
// batched solves: one LAPACK-style dpotrf + dpotrs per matrix, matrices spread over a thread pool
// (the CPU counterpart of many independent small systems; the reference has no batched path)
// ------------------------------------------------------------------------------------------------
extern "C" void orc_dposv_batched(int batch, const int* n, const int64_t* offA, const int64_t* offB, double* A,
                                  double* B, int nrhs, int nthreads, int use_blas, int* info) {
  if (batch <= 0) return;
  if (use_blas && !orc_blas_loaded()) use_blas = 0;
  std::vector<int> order(batch);
  for (int k = 0; k < batch; ++k) order[k] = k;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return n[a] > n[b]; });
  std::atomic<int> next{0};
  auto work = [&]() {
    for (;;) {
      const int t = next.fetch_add(1);
      if (t >= batch) return;
      const int k = order[t], nk = n[k];
      double* a = A + offA[k];
      double* b = B + offB[k];
      int inf = 0;
      if (use_blas) {
        g_blas.potrf("L", &nk, a, &nk, &inf, 1);
        if (inf == 0) {
          const double one = 1.0;
          g_blas.trsm("L", "L", "N", "N", &nk, &nrhs, &one, a, &nk, b, &nk, 1, 1, 1, 1);
          g_blas.trsm("L", "L", "T", "N", &nk, &nrhs, &one, a, &nk, b, &nk, 1, 1, 1, 1);
        }
      } else {
        inf = orc_potrf_tile(nk, a, nk);
        if (inf == 0)
          for (int r = 0; r < nrhs; ++r) {
            double* x = b + (int64_t)r * nk;
            for (int64_t j = 0; j < nk; ++j) {
              x[j] /= a[j + j * nk];
              for (int64_t i = j + 1; i < nk; ++i) x[i] -= a[i + j * nk] * x[j];
            }
            for (int64_t i = nk - 1; i >= 0; --i) {
              double s = x[i];
              for (int64_t q = i + 1; q < nk; ++q) s -= a[q + i * nk] * x[q];
              x[i] = s / a[i + i * nk];
            }
          }
      }
      info[k] = inf;
    }
  };
  if (nthreads <= 0) nthreads = (int)std::max(1u, std::thread::hardware_concurrency());
  std::vector<std::thread> pool;
  for (int t = 0; t < nthreads; ++t) pool.emplace_back(work);
  for (auto& th : pool) th.join();
}

extern "C" void orc_gen_uniform_sym_batched(int batch, const int* n, const int64_t* offA, uint64_t seed, double* A) {
  for (int k = 0; k < batch; ++k)
    orc_gen_uniform_sym_colmajor(n[k], seed + (uint64_t)k * 0x9e3779b97f4a7c15ULL, (double)n[k], A + offA[k], n[k]);
}

// ------------------------------------------------------------------------------------------------
// inverse from the factor: TRTRI (examples/potrf/trtri_L.h: TRSMR, GEMM, TRSML, TRTRI tasks) then
// LAUUM (examples/potrf/lauum.h: SYRK/GEMM, TRMM, LAUUM tasks), restated step by step on tiles
// ------------------------------------------------------------------------------------------------
namespace {
struct TileMat {
  int N, NB, NT;
  double* t;
  double* at(int m, int n) { return t + orc_tile_slot(m, n, NT) * (int64_t)NB * NB; }
  int dim(int k) const { return tile_dim(k, NT, N, NB); }
};
// inverse of a lower triangular n x n block (column-major, ld), written as a dense lower matrix
void tri_inverse_lower(int n, const double* L, int ld, std::vector<double>& X) {
  X.assign((size_t)n * n, 0.0);
  for (int j = 0; j < n; ++j) {  // column j of L^{-1}: forward substitution of e_j
    X[j + (size_t)j * n] = 1.0 / L[j + (int64_t)j * ld];
    for (int i = j + 1; i < n; ++i) {
      double s = 0.0;
      for (int p = j; p < i; ++p) s += L[i + (int64_t)p * ld] * X[p + (size_t)j * n];
      X[i + (size_t)j * n] = -s / L[i + (int64_t)i * ld];
    }
  }
}
// C (m x n, ld NB) := beta C + alpha op(A) op(B) with op(X) = X or X^T, contraction length kd;
// lowA / lowB: only the stored lower triangle of the operand counts
void tile_gemm(int m, int n, int kd, bool ta, bool tb, bool lowA, bool lowB, const double* A, int lda, const double* B,
               int ldb, double* C, int ldc, double alpha, double beta) {
  std::vector<double> out((size_t)m * n, 0.0);
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < m; ++i) {
      double s = 0.0;
      for (int p = 0; p < kd; ++p) {
        const int ar = ta ? p : i, ac = ta ? i : p, br = tb ? j : p, bc = tb ? p : j;
        if ((lowA && ar < ac) || (lowB && br < bc)) continue;
        s += A[ar + (int64_t)ac * lda] * B[br + (int64_t)bc * ldb];
      }
      out[i + (size_t)j * m] = s;
    }
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < m; ++i) {
      double& c = C[i + (int64_t)j * ldc];
      c = (beta == 0.0 ? 0.0 : beta * c) + alpha * out[i + (size_t)j * m];
    }
}
}  // namespace

extern "C" int orc_potri_tiled(int N, int NB, double* tiles) {
  TileMat A{N, NB, (N + NB - 1) / NB, tiles};
  const int NT = A.NT;
  std::vector<double> Linv, tmp;
  for (int k = 0; k < NT; ++k) {  // TRTRI
    const int kk = A.dim(k);
    tri_inverse_lower(kk, A.at(k, k), NB, Linv);
    for (int m = k + 1; m < NT; ++m) {  // A_mk := -A_mk L_kk^{-1}
      const int mm = A.dim(m);
      tmp.assign(A.at(m, k), A.at(m, k) + (size_t)NB * NB);
      tile_gemm(mm, kk, kk, false, false, false, false, tmp.data(), NB, Linv.data(), kk, A.at(m, k), NB, -1.0, 0.0);
    }
    for (int m = k + 1; m < NT; ++m)  // A_mn += A_mk A_kn
      for (int n = 0; n < k; ++n)
        tile_gemm(A.dim(m), NB, kk, false, false, false, false, A.at(m, k), NB, A.at(k, n), NB, A.at(m, n), NB, 1.0, 1.0);
    for (int n = 0; n < k; ++n) {  // A_kn := L_kk^{-1} A_kn
      tmp.assign(A.at(k, n), A.at(k, n) + (size_t)NB * NB);
      tile_gemm(kk, NB, kk, false, false, false, false, Linv.data(), kk, tmp.data(), NB, A.at(k, n), NB, 1.0, 0.0);
    }
    for (int j = 0; j < kk; ++j)
      for (int i = j; i < kk; ++i) A.at(k, k)[i + (int64_t)j * NB] = Linv[i + (size_t)j * kk];
  }
  for (int k = 0; k < NT; ++k) {  // LAUUM
    const int kk = A.dim(k);
    for (int m = 0; m < k; ++m)  // A_mn += A_km^T A_kn
      for (int n = 0; n <= m; ++n)
        tile_gemm(NB, NB, kk, true, false, false, false, A.at(k, m), NB, A.at(k, n), NB, A.at(m, n), NB, 1.0, 1.0);
    for (int n = 0; n < k; ++n) {  // A_kn := A_kk^T A_kn (A_kk lower)
      tmp.assign(A.at(k, n), A.at(k, n) + (size_t)NB * NB);
      tile_gemm(kk, NB, kk, true, false, true, false, A.at(k, k), NB, tmp.data(), NB, A.at(k, n), NB, 1.0, 0.0);
    }
    tmp.assign(A.at(k, k), A.at(k, k) + (size_t)NB * NB);  // A_kk := A_kk^T A_kk (lower)
    std::vector<double> d((size_t)NB * NB, 0.0);
    tile_gemm(kk, kk, kk, true, false, true, true, tmp.data(), NB, tmp.data(), NB, d.data(), NB, 1.0, 0.0);
    for (int j = 0; j < kk; ++j)
      for (int i = j; i < kk; ++i) A.at(k, k)[i + (int64_t)j * NB] = d[i + (size_t)j * NB];
  }
  return 0;
}
