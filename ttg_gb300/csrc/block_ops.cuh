// Block operations of the tiled Cholesky, templated on the element type (double for the FP64
// path, float for the working precision of the mixed path). One CTA of 256 threads per call.
#pragma once
#include <type_traits>
#include <cuda_runtime.h>

namespace gbx {

constexpr int kThreads = 256;  // threads per CTA of every FP64 block kernel
constexpr int kBlk = 128;      // largest block edge handled by one CTA
constexpr int kKC = 16;        // k-chunk of the GEMM staging
constexpr int kPW = 32;        // panel width of the TRSM

// CTA barrier of the block operations: every thread of the CTA, or (kNamed) the first 256 threads
// only, with named barrier 1, so that a larger CTA can run an operation on 256 of its threads
template <bool kNamed>
__device__ __forceinline__ void ops_sync() {
  if (kNamed) asm volatile("bar.sync 1, 256;" ::: "memory");
  else __syncthreads();
}

// four consecutive elements from shared memory in 16-byte loads (p 16-byte aligned)
__device__ __forceinline__ void lds4(const float* p, float (&v)[4]) {
  const float4 f = *(const float4*)p;
  v[0] = f.x;
  v[1] = f.y;
  v[2] = f.z;
  v[3] = f.w;
}
__device__ __forceinline__ void lds4(const double* p, double (&v)[4]) {
  const double2 a = *(const double2*)p, b = *(const double2*)(p + 2);
  v[0] = a.x;
  v[1] = a.y;
  v[2] = b.x;
  v[3] = b.y;
}

// pivot of the Cholesky column: l = sqrt(d) and 1/l. FP32: hardware reciprocal square root with
// one Newton step (r <- r (3 - d r^2) / 2), a few ulp, short latency on the factor's serial chain;
// FP64: rsqrt (within an ulp or two) and one multiply.
__device__ __forceinline__ void chol_pivot(float d, float& l, float& inv) {
  float r = rsqrtf(d);
  r = r * fmaf(-0.5f * d * r, r, 1.5f);
  inv = r;
  l = d * r;
}
__device__ __forceinline__ void chol_pivot(double d, double& l, double& inv) {
  inv = rsqrt(d);  // about half the FP64 work of sqrt and a division (each FP64 op is slow on GB300)
  l = d * inv;
}

// ------------------------------------------------------------------------------------------------
// block GEMM:  C(m x n) := C - A(m x k) * B(n x k)^T   (lower: only i >= j of C is written)
// 256 threads, each owning an 8 x 8 micro-tile (rows 4tx..4tx+3 and 64+4tx..64+4tx+3, the same
// pattern of columns from ty), read from shared memory with 16-byte vector loads; k staged through
// double-buffered chunks of 16 with a register prefetch of the next chunk.
// kSmall (m, n <= 64): each thread owns only the first 4 x 4 quarter of that pattern, so a 64 x 64
// block keeps every thread's FMAs useful (the 8 x 8 form would spend three quarters on zeros).
// smem: 2 * 2 * 16 * 128 elements (64 KB in FP64)
// ------------------------------------------------------------------------------------------------
template <typename T, bool kSmall = false>
__device__ __forceinline__ void op_gemm_nt(const T* __restrict__ A, int lda, const T* __restrict__ B, int ldb, T* C,
                                           int ldc, int m, int n, int k, bool lower, T* sm) {
  constexpr int R = kSmall ? 4 : 8;  // micro-tile edge
  T* As = sm;                       // [2][kKC][kBlk]
  T* Bs = sm + 2 * kKC * kBlk;      // [2][kKC][kBlk]
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int lrow = tid & 127, lk0 = tid >> 7;
  T acc[R][R];
#pragma unroll
  for (int i = 0; i < R; ++i)
#pragma unroll
    for (int j = 0; j < R; ++j) acc[i][j] = T(0);

  const int nchunks = (k + kKC - 1) / kKC;
  T ra[8], rb[8];
  auto gload = [&](int k0) {
#pragma unroll
    for (int s = 0; s < 8; ++s) {
      const int kk = k0 + lk0 + 2 * s;
      ra[s] = (lrow < m && kk < k) ? __ldcg(A + lrow + (long long)kk * lda) : T(0);
      rb[s] = (lrow < n && kk < k) ? __ldcg(B + lrow + (long long)kk * ldb) : T(0);
    }
  };
  auto sstore = [&](int buf) {
#pragma unroll
    for (int s = 0; s < 8; ++s) {
      As[(buf * kKC + lk0 + 2 * s) * kBlk + lrow] = ra[s];
      Bs[(buf * kKC + lk0 + 2 * s) * kBlk + lrow] = rb[s];
    }
  };
  if (nchunks > 0) {
    gload(0);
    sstore(0);
    __syncthreads();
    for (int c = 0; c < nchunks; ++c) {
      const int buf = c & 1;
      if (c + 1 < nchunks) gload((c + 1) * kKC);
      const T* as = As + buf * kKC * kBlk;
      const T* bs = Bs + buf * kKC * kBlk;
#pragma unroll
      for (int kk = 0; kk < kKC; ++kk) {
        T a0[4], a1[4], b0[4], b1[4];
        lds4(as + kk * kBlk + 4 * tx, a0);
        lds4(bs + kk * kBlk + 4 * ty, b0);
        if (!kSmall) {
          lds4(as + kk * kBlk + 64 + 4 * tx, a1);
          lds4(bs + kk * kBlk + 64 + 4 * ty, b1);
        }
#pragma unroll
        for (int i = 0; i < R; ++i)
#pragma unroll
          for (int j = 0; j < R; ++j) {
            const T ai = i < 4 ? a0[i & 3] : a1[i & 3], bj = j < 4 ? b0[j & 3] : b1[j & 3];
            acc[i][j] = fma(ai, bj, acc[i][j]);
          }
      }
      if (c + 1 < nchunks) sstore(buf ^ 1);
      __syncthreads();
    }
  }
#pragma unroll
  for (int j = 0; j < R; ++j) {
    const int col = (j < 4 ? 0 : 60) + 4 * ty + j;
#pragma unroll
    for (int i = 0; i < R; ++i) {
      const int row = (i < 4 ? 0 : 60) + 4 * tx + i;
      if (row < m && col < n && (!lower || row >= col)) {
        T* p = C + row + (long long)col * ldc;
        __stcg(p, __ldcg(p) - acc[i][j]);
      }
    }
  }
  __syncthreads();
}

// FP32 reciprocal without a branch: the hardware approximation refined by one Newton-Raphson step,
// r <- r + r (1 - d r) (within an ulp or so of 1/d). The IEEE division carries a slow-path branch
// that splits an unrolled solve into many scheduling regions and keeps its loads from being hoisted.
__device__ __forceinline__ float rcp_nr(float d) {
  const float r = __fdividef(1.f, d);
  return fmaf(r, fmaf(-d, r, 1.f), r);
}

// ------------------------------------------------------------------------------------------------
// block POTRF (lower, n <= 128) in shared memory, blocked by 32 columns:
//   1. warp 0 factors the 32 x 32 diagonal block (warp-synchronous, no CTA barrier per column)
//   2. every thread solves one row below the block against it (row-wise substitution)
//   3. all threads apply the block's rank-32 update to the trailing lower triangle
// Returns 0 or the 1-based local index of the first non-positive pivot (LAPACK info); the strict
// upper triangle of A is not touched. smem: 128 * 128 elements + 1 int.
// ------------------------------------------------------------------------------------------------
// One row of a 32-column panel held in registers: x := x * L_blk^{-T} (row-wise forward
// substitution against the panel's lower triangle Lp, column-major with leading dimension ldp).
// rinv (optional): the 32 reciprocals of the panel's diagonal at rinv[rinv_at(c)], computed once
// for all rows (an FP64 division per row and column is ~500 clocks of a warp on GB300).
__device__ __forceinline__ int rinv_at(int c, int ldp) { return (c & 15) + ldp * (16 + (c >> 4)); }
template <typename T>
__device__ __forceinline__ void row_solve32(T (&x)[32], const T* Lp, int ldp, int pw, const T* rinv = nullptr) {
#pragma unroll
  for (int c = 0; c < 32; ++c) {
    if (c < pw) {
      T s0 = x[c], s1 = T(0);
#pragma unroll
      for (int c2 = 0; c2 + 1 < c; c2 += 2) {
        s0 = fma(-x[c2], Lp[c + ldp * c2], s0);
        s1 = fma(-x[c2 + 1], Lp[c + ldp * (c2 + 1)], s1);
      }
      if (c & 1) s0 = fma(-x[c - 1], Lp[c + ldp * (c - 1)], s0);
      // the reciprocal does not depend on x: off the chain
      x[c] = (s0 + s1) * (rinv ? rinv[rinv_at(c, ldp)] : (T(1) / Lp[c + ldp * c]));
    }
  }
}
// the reciprocals of a 32 x 32 lower panel Lp (column-major, ldp) into its strict upper triangle at
// rinv_at(c): rows 0-15 of columns 16 and 17, never read as part of the lower triangle. One warp.
template <typename T>
__device__ __forceinline__ void panel_reciprocals(T* Lp, int ldp, int pw, int lane) {
  const T v = lane < pw ? T(1) / Lp[lane + ldp * lane] : T(0);
  __syncwarp();
  Lp[rinv_at(lane, ldp)] = v;
}

// The same solve column by column for a full FP32 panel: once x(c) is final it is subtracted from
// the later entries, so column c of Lp is read with 16-byte loads that do not depend on x, and the
// chain per column is one multiply and one FMA. Lp is 16-byte aligned and ldp a multiple of 4. The
// warp sync every 8 columns bounds how far ahead the compiler hoists the loads (register pressure
// inside the persistent mixed kernel). It is a full-warp sync: every caller runs this on all 32
// lanes of its warps (a partial warp would never meet the sync).
__device__ __forceinline__ void col_solve32(float (&x)[32], const float* Lp, int ldp) {
#pragma unroll
  for (int c = 0; c < 32; ++c) {
    float l[32];
#pragma unroll
    for (int q = c / 4; q < 8; ++q) lds4(Lp + c * ldp + 4 * q, *reinterpret_cast<float(*)[4]>(&l[4 * q]));
    x[c] *= rcp_nr(l[c]);
#pragma unroll
    for (int r = c + 1; r < 32; ++r) x[r] = fmaf(-l[r], x[c], x[r]);
    if ((c + 1) % 8 == 0 && c < 31) __syncwarp();  // keeps the loads hoisted at most 8 columns ahead
  }
}

template <typename T, bool kNamed = false>
__device__ int op_potrf(T* A, int lda, int n, T* sm) {
  T* S = sm;                              // col-major, ld 128
  int* flag = (int*)(sm + kBlk * kBlk);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) *flag = 0;
  for (int idx = tid; idx < kBlk * n; idx += kThreads) {
    const int i = idx & (kBlk - 1), j = idx >> 7;
    if (i < n && i >= j) S[i + kBlk * j] = __ldcg(A + i + (long long)j * lda);
  }
  ops_sync<kNamed>();
  int info = 0;
  for (int p0 = 0; p0 < n; p0 += 32) {
    const int pw = min(32, n - p0);
    if (sizeof(T) == 8 && warp < 4) {
      // FP64: the 32 x 32 diagonal block on four warps, warp w holding columns 8w..8w+7 of every
      // row (lane = row). Per column j the owner warp takes the pivot and publishes column j of L;
      // after one barrier every warp applies it to its columns, the next pivot's column first, so
      // only the pivot and one FMA per column stay on the serial chain (each warp-wide FP64
      // instruction occupies a GB300 SM sub-partition for 64 clocks)
      T* colbuf = S + p0 + kBlk * (p0 + 20);  // [2][32] at rows 0-15 of columns 20-23: upper, unused
      auto cb = [&](int b, int r) -> T& { return colbuf[(r & 15) + kBlk * (2 * b + (r >> 4))]; };
      T xw[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int c = 8 * warp + q;
        xw[q] = (lane < pw && c <= lane) ? S[(p0 + lane) + kBlk * (p0 + c)] : T(0);
      }
      for (int j = 0; j < pw; ++j) {
        if (warp == (j >> 3)) {
          T xj = T(0);
#pragma unroll
          for (int q = 0; q < 8; ++q) xj = q == (j & 7) ? xw[q] : xj;
          const T d = __shfl_sync(0xffffffffu, xj, j);
          if (!(d > T(0))) {
            if (lane == 0) *flag = p0 + j + 1;
          } else {
            T ljj, inv;
            chol_pivot(d, ljj, inv);
            if (lane == 0) S[p0 + rinv_at(j, kBlk) + kBlk * p0] = inv;  // for the rows below the block
            const T lij = lane == j ? ljj : (lane > j ? xj * inv : T(0));
#pragma unroll
            for (int q = 0; q < 8; ++q) xw[q] = q == (j & 7) ? lij : xw[q];
            cb(j & 1, lane) = lij;
          }
        }
        asm volatile("bar.sync 2, 128;" ::: "memory");
        if (*(volatile int*)flag) break;
        const T lj = cb(j & 1, lane);
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const int cc = 8 * warp + q;
          if (cc > j && cc < pw) {
            const T upd = fma(-lj, cb(j & 1, cc), xw[q]);
            xw[q] = lane >= cc ? upd : xw[q];
          }
        }
      }
      if (*(volatile int*)flag == 0 && lane < pw)
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const int c = 8 * warp + q;
          if (c <= lane && c < pw) S[(p0 + lane) + kBlk * (p0 + c)] = xw[q];
        }
    } else if (sizeof(T) == 4 && warp == 0) {
      // 32 x 32 diagonal block: lane = row, the row in registers, columns exchanged by shuffles
      T x[32];
#pragma unroll
      for (int c = 0; c < 32; ++c) x[c] = (lane < pw && c <= lane) ? S[(p0 + lane) + kBlk * (p0 + c)] : T(0);
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        if (j < pw) {
          const T d = __shfl_sync(0xffffffffu, x[j], j);
          if (!(d > T(0))) {  // same value in every lane: the whole warp leaves together
            if (lane == 0) *flag = p0 + j + 1;
            break;
          }
          T ljj, inv;
          chol_pivot(d, ljj, inv);
          if (lane == 0) S[p0 + rinv_at(j, kBlk) + kBlk * p0] = inv;  // for the rows below the block
          // column j of L in every lane (0 above the diagonal); selects, not branches, so the
          // warp never diverges inside the column loop
          const T lij = lane == j ? ljj : (lane > j ? x[j] * inv : T(0));
          x[j] = lij;
#pragma unroll
          for (int cc = j + 1; cc < 32; ++cc) {
            const T lcj = __shfl_sync(0xffffffffu, lij, cc);
            const T upd = fma(-lij, lcj, x[cc]);
            x[cc] = lane >= cc ? upd : x[cc];
          }
        }
      }
      __syncwarp();
      if (*flag == 0 && lane < pw)
#pragma unroll
        for (int c = 0; c < 32; ++c)
          if (c <= lane) S[(p0 + lane) + kBlk * (p0 + c)] = x[c];
    }
    ops_sync<kNamed>();
    info = *flag;
    if (info) break;
    // rows below the block: X := X L_d^{-T}
    const int rb = p0 + pw, ng = (n - rb + 31) >> 5;  // rows rb..n-1 in groups of 32 (<= 3)
    if (sizeof(T) == 8 && ng > 0 && n <= 64) {
      // FP64 blocks of at most 64: the columns dealt to the eight warps (column c to warp c % 8),
      // all rows in each (lane = row of a group), right-looking: per column j its owner scales x_j
      // by the reciprocal and stores it, one barrier, then every warp subtracts it from its later
      // columns (a warp's smallest column above j first: the next owner's). One row per thread
      // leaves the 32 rows on one sub-partition's FP64 pipe (GB300, N=2048 with 64-blocks: 7.23
      // -> 7.10 ms). On 128-blocks the 32 barriers per panel cost more than the balance gains
      // (N=8192 32.6 -> 34.4 ms), so they keep the per-row solve.
      const T* Ld = S + p0 + kBlk * p0;
      T xv[3][4];  // [row group][column j = warp + 8 q]
#pragma unroll
      for (int g = 0; g < 3; ++g)
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int r = rb + 32 * g + lane, c = warp + 8 * q;
          xv[g][q] = (g < ng && r < n && c < pw) ? S[r + kBlk * (p0 + c)] : T(0);
        }
      for (int j = 0; j < pw; ++j) {
        if (warp == (j & 7)) {
          const T rj = Ld[rinv_at(j, kBlk)];
          auto own = [&](auto qc) {
            constexpr int q = decltype(qc)::value;
#pragma unroll
            for (int g = 0; g < 3; ++g)
              if (g < ng) {
                const int r = rb + 32 * g + lane;
                xv[g][q] *= rj;
                if (r < n) S[r + kBlk * (p0 + j)] = xv[g][q];
              }
          };
          switch (j >> 3) {
            case 0: own(std::integral_constant<int, 0>{}); break;
            case 1: own(std::integral_constant<int, 1>{}); break;
            case 2: own(std::integral_constant<int, 2>{}); break;
            default: own(std::integral_constant<int, 3>{}); break;
          }
        }
        ops_sync<kNamed>();
        if (j + 1 < pw) {
          T xj[3];
#pragma unroll
          for (int g = 0; g < 3; ++g) {
            const int r = rb + 32 * g + lane;
            xj[g] = (g < ng && r < n) ? S[r + kBlk * (p0 + j)] : T(0);
          }
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const int c = warp + 8 * q;
            if (c > j && c < pw) {
              const T l = Ld[c + kBlk * j];
#pragma unroll
              for (int g = 0; g < 3; ++g)
                if (g < ng) xv[g][q] = fma(-l, xj[g], xv[g][q]);
            }
          }
        }
      }
    } else {
      // each thread solves one row in registers
      for (int r = rb + tid; r < n; r += kThreads) {
        T x[32];
#pragma unroll
        for (int c = 0; c < 32; ++c) x[c] = c < pw ? S[r + kBlk * (p0 + c)] : T(0);
        row_solve32<T>(x, S + p0 + kBlk * p0, kBlk, pw, S + p0 + kBlk * p0);
#pragma unroll
        for (int c = 0; c < 32; ++c)
          if (c < pw) S[r + kBlk * (p0 + c)] = x[c];
      }
    }
    ops_sync<kNamed>();
    // trailing update S(i, c) -= sum_k S(i, k) S(c, k), p0+pw <= c <= i < n
    const int t0 = p0 + pw, t = n - t0;
    if (sizeof(T) == 8 && t > 0) {
      // FP64: one element per thread. A warp-wide FP64 instruction holds its sub-partition's FP64
      // pipe ~80 clocks however many lanes are active, so what counts is the warp instructions on
      // the busiest sub-partition: 4 x 4 blocks (300 / 136 / 36 of them for t = 96 / 64 / 32) leave
      // a second round on one or two warps; single elements spread evenly (per sub-partition
      // 1536 -> ~1184, 1024 -> ~544, 512 -> ~160 instructions). Same k order: the same sums.
      const int ne = t * (t + 1) / 2;
      for (int e = tid; e < ne; e += kThreads) {
        int i = (int)((sqrtf(8.0f * (float)e + 1.0f) - 1.0f) * 0.5f);  // row: i (i + 1) / 2 <= e
        i -= (i * (i + 1) / 2 > e) ? 1 : 0;
        i += ((i + 1) * (i + 2) / 2 <= e) ? 1 : 0;
        const int c = e - i * (i + 1) / 2;
        const T* Si = S + (t0 + i) + kBlk * p0;
        const T* Sc = S + (t0 + c) + kBlk * p0;
        T acc = T(0);
#pragma unroll 8
        for (int k = 0; k < pw; ++k) acc = fma(Si[kBlk * k], Sc[kBlk * k], acc);
        S[(t0 + i) + kBlk * (t0 + c)] -= acc;
      }
    } else if (t > 0) {  // FP32: 4 x 4 register blocks
      const int nb4 = (t + 3) / 4;
      const int nblk = nb4 * (nb4 + 1) / 2;
      for (int q = tid; q < nblk; q += kThreads) {
        int bj = 0, rem = q;  // lower 4 x 4 block (bi >= bj)
        while (rem >= nb4 - bj) {
          rem -= nb4 - bj;
          ++bj;
        }
        const int bi = bj + rem;
        const int i0 = t0 + 4 * bi, c0 = t0 + 4 * bj;
        T acc[4][4];
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
          for (int b = 0; b < 4; ++b) acc[a][b] = T(0);
        for (int k = p0; k < p0 + pw; ++k) {
          T vi[4], vc[4];
#pragma unroll
          for (int a = 0; a < 4; ++a) vi[a] = (i0 + a < n) ? S[(i0 + a) + kBlk * k] : T(0);
#pragma unroll
          for (int b = 0; b < 4; ++b) vc[b] = (c0 + b < n) ? S[(c0 + b) + kBlk * k] : T(0);
#pragma unroll
          for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int b = 0; b < 4; ++b) acc[a][b] = fma(vi[a], vc[b], acc[a][b]);
        }
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
          for (int b = 0; b < 4; ++b) {
            const int i = i0 + a, c = c0 + b;
            if (i < n && c < n && i >= c) S[i + kBlk * c] -= acc[a][b];
          }
      }
    }
    ops_sync<kNamed>();
  }
  for (int idx = tid; idx < kBlk * n; idx += kThreads) {
    const int i = idx & (kBlk - 1), j = idx >> 7;
    if (i < n && i >= j) __stcg(A + i + (long long)j * lda, S[i + kBlk * j]);
  }
  ops_sync<kNamed>();
  return info;
}

// ------------------------------------------------------------------------------------------------
// block TRSM (Right, Lower, Trans, NonUnit): B(m x n) := B * L^{-T}, m <= 128, any n.
// Column panels of 32: left-looking update of the panel from the already-solved columns (a
// 128 x 32 x p0 GEMM, 4 x 4 micro-tiles), then each thread solves its own row across the panel.
// smem: panel 32*128 + X chunk 16*128 + L chunk 16*32 + diagonal 32*32 doubles = 60 KB
// ------------------------------------------------------------------------------------------------
// k-chunk of the TRSM update: 64 for float (enough FMAs per chunk to cover the L2 latency of the
// next chunk's prefetch), 16 for double (the FP64 pipe already hides it)
template <typename T>
struct TrsmChunk {
  static constexpr int value = sizeof(T) == 4 ? 64 : kKC;
};
template <typename T>
constexpr size_t op_trsm_smem_elems() {
  return (size_t)kPW * kBlk + (size_t)TrsmChunk<T>::value * kBlk + (size_t)TrsmChunk<T>::value * kPW + kPW * kPW;
}

// kColSolve (FP32 only): the panel solve in the column-wise form with the branch-free reciprocal,
// for kernels with registers to spare; the default keeps the row-wise form and IEEE division.
template <typename T, bool kColSolve = false, bool kNamed = false>
__device__ void op_trsm(const T* __restrict__ L, int ldl, T* B, int ldb, int m, int n, T* sm) {
  constexpr int KC = TrsmChunk<T>::value;
  T* P = sm;                    // [kPW][128]  panel, P[c*128 + r]
  T* Xc = P + kPW * kBlk;       // [KC][128]
  T* Lc = Xc + KC * kBlk;       // [KC][kPW]
  T* Ld = Lc + KC * kPW;        // [kPW][kPW]  Ld[c2*32 + c] = L(p0+c, p0+c2)
  const int tid = threadIdx.x, tx = tid & 31, ty = tid >> 5;
  for (int p0 = 0; p0 < n; p0 += kPW) {
    const int pw = min(kPW, n - p0);
    for (int idx = tid; idx < kPW * kBlk; idx += kThreads) {
      const int r = idx & (kBlk - 1), c = idx >> 7;
      P[idx] = (r < m && c < pw) ? __ldcg(B + r + (long long)(p0 + c) * ldb) : T(0);
    }
    for (int idx = tid; idx < kPW * kPW; idx += kThreads) {
      const int c = idx & 31, c2 = idx >> 5;
      Ld[idx] = (c < pw && c2 <= c) ? __ldcg(L + (p0 + c) + (long long)(p0 + c2) * ldl) : T(0);
    }
    ops_sync<kNamed>();
    if (p0 > 0) {
      // P -= X(:, 0:p0) L(p0:p0+pw, 0:p0)^T, k in chunks of KC; the next chunk is prefetched into
      // registers while the current one is multiplied (hides the L2 latency)
      T acc[4][4];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = T(0);
      T rx[KC * kBlk / kThreads], rl[(KC * kPW + kThreads - 1) / kThreads];
      auto gload = [&](int k0) {
#pragma unroll
        for (int u = 0; u < KC * kBlk / kThreads; ++u) {
          const int idx = tid + u * kThreads;
          const int r = idx & (kBlk - 1), kk = idx >> 7;
          rx[u] = (r < m && k0 + kk < p0) ? __ldcg(B + r + (long long)(k0 + kk) * ldb) : T(0);
        }
#pragma unroll
        for (int u = 0; u < (KC * kPW + kThreads - 1) / kThreads; ++u) {
          const int idx = tid + u * kThreads;
          const int c = idx & 31, kk = idx >> 5;
          rl[u] = (idx < KC * kPW && c < pw && k0 + kk < p0) ? __ldcg(L + (p0 + c) + (long long)(k0 + kk) * ldl) : T(0);
        }
      };
      auto sstore = [&]() {
#pragma unroll
        for (int u = 0; u < KC * kBlk / kThreads; ++u) Xc[tid + u * kThreads] = rx[u];
#pragma unroll
        for (int u = 0; u < (KC * kPW + kThreads - 1) / kThreads; ++u)
          if (tid + u * kThreads < KC * kPW) Lc[tid + u * kThreads] = rl[u];
      };
      // m <= 32 (a row sub-task): lane = row, warp = four columns, so that no FP64 instruction
      // works on absent rows (a warp-wide FP64 instruction costs the same with any active lanes)
      const bool narrow = m <= 32;
      gload(0);
      for (int k0 = 0; k0 < p0; k0 += KC) {
        sstore();
        ops_sync<kNamed>();
        if (k0 + KC < p0) gload(k0 + KC);
        if (narrow) {
#pragma unroll
          for (int kk = 0; kk < KC; ++kk) {  // row tx x columns 4ty..4ty+3
            const T a = Xc[kk * kBlk + tx];
            T b[4];
            lds4(Lc + kk * kPW + 4 * ty, b);
#pragma unroll
            for (int j = 0; j < 4; ++j) acc[0][j] = fma(a, b[j], acc[0][j]);
          }
        } else {
#pragma unroll
          for (int kk = 0; kk < KC; ++kk) {  // rows 4tx..4tx+3 x columns 4ty..4ty+3, vector loads
            T a[4], b[4];
            lds4(Xc + kk * kBlk + 4 * tx, a);
            lds4(Lc + kk * kPW + 4 * ty, b);
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
              for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
          }
        }
        ops_sync<kNamed>();
      }
      if (narrow) {
#pragma unroll
        for (int j = 0; j < 4; ++j) P[(4 * ty + j) * kBlk + tx] -= acc[0][j];
      } else {
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int j = 0; j < 4; ++j) P[(4 * ty + j) * kBlk + 4 * tx + i] -= acc[i][j];
      }
      ops_sync<kNamed>();
    }
    if (!kColSolve) {  // the panel's reciprocals once, into Ld's unused upper triangle
      if (tid < 32) panel_reciprocals<T>(Ld, kPW, pw, tid);
      ops_sync<kNamed>();
    }
    // each thread solves its row of the panel in registers; the column-wise solve synchronises its
    // warp, so it runs on whole warps (rows past m are zero in P and are never stored back)
    const int solvers = kColSolve ? ((m + 31) & ~31) : m;
    if (tid < solvers && tid < kBlk) {
      const int r = tid;
      T x[kPW];
#pragma unroll
      for (int c = 0; c < kPW; ++c) x[c] = P[c * kBlk + r];
      if constexpr (kColSolve) {
        if (pw == kPW) col_solve32(x, Ld, kPW);
        else row_solve32<T>(x, Ld, kPW, pw);
      } else {
        row_solve32<T>(x, Ld, kPW, pw, Ld);  // Ld holds L(p0+c, p0+c2) at c + 32*c2
      }
#pragma unroll
      for (int c = 0; c < kPW; ++c) P[c * kBlk + r] = x[c];
    }
    ops_sync<kNamed>();
    for (int idx = tid; idx < kPW * kBlk; idx += kThreads) {
      const int r = idx & (kBlk - 1), c = idx >> 7;
      if (r < m && c < pw) __stcg(B + r + (long long)(p0 + c) * ldb, P[idx]);
    }
    ops_sync<kNamed>();
  }
}


// Triangular solves of one right-hand side held in shared memory xs[0..n) against the lower
// factor L (column-major, ld), by 32-column panels: warp 0 solves the panel's triangle with its
// rows in registers, the solved value broadcast by a shuffle and the diagonal's reciprocals taken
// once per panel (an FP64 division is ~500 clocks of a warp on GB300), then the whole CTA applies
// the panel to the other rows (two CTA barriers per panel instead of two per column).
template <typename T>
__device__ void fwd_solve(const T* L, int n, int ld, T* xs) {  // L y = x
  __shared__ T tri[32 * 33];  // the panel's 32 x 32 triangle, staged once per panel
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int p0 = 0; p0 < n; p0 += 32) {
    const int pw = min(32, n - p0);
    for (int idx = tid; idx < 32 * 32; idx += blockDim.x) {
      const int r = idx & 31, c = idx >> 5;
      tri[r + 33 * c] = (r < pw && c < pw && r >= c) ? L[(p0 + r) + (long long)(p0 + c) * ld] : T(0);
    }
    __syncthreads();
    if (warp == 0) {  // lane = row of the panel, x in a register; the reciprocals once per panel
      T x = lane < pw ? xs[p0 + lane] : T(0);
      const T ri = lane < pw ? T(1) / tri[lane * 34] : T(0);
      for (int c = 0; c < pw; ++c) {
        const T xc = __shfl_sync(0xffffffffu, x * ri, c);
        if (lane == c) x = xc;
        else if (lane > c) x = fma(-tri[lane + 33 * c], xc, x);
      }
      if (lane < pw) xs[p0 + lane] = x;
    }
    __syncthreads();
    for (int i = p0 + pw + tid; i < n; i += blockDim.x) {
      T s = T(0);
#pragma unroll 8
      for (int c = 0; c < pw; ++c) s += L[i + (long long)(p0 + c) * ld] * xs[p0 + c];
      xs[i] -= s;
    }
    __syncthreads();
  }
}

template <typename T>
__device__ void bwd_solve(const T* L, int n, int ld, T* xs) {  // L^T x = y
  __shared__ T tri[32 * 33];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int last = ((n - 1) / 32) * 32;
  for (int p0 = last; p0 >= 0; p0 -= 32) {
    const int pw = min(32, n - p0);
    // contributions of the already solved rows below the panel: xs[r] -= sum_i L(i, r) x_i
    for (int r = warp; r < pw; r += blockDim.x / 32) {
      T s = T(0);
      for (int i = p0 + pw + lane; i < n; i += 32) s += L[i + (long long)(p0 + r) * ld] * xs[i];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if (lane == 0) xs[p0 + r] -= s;
    }
    for (int idx = tid; idx < 32 * 32; idx += blockDim.x) {
      const int r = idx & 31, c = idx >> 5;
      tri[r + 33 * c] = (r < pw && c < pw && r >= c) ? L[(p0 + r) + (long long)(p0 + c) * ld] : T(0);
    }
    __syncthreads();
    if (warp == 0) {  // as in fwd_solve, from the last row up
      T x = lane < pw ? xs[p0 + lane] : T(0);
      const T ri = lane < pw ? T(1) / tri[lane * 34] : T(0);
      for (int c = pw - 1; c >= 0; --c) {
        const T xc = __shfl_sync(0xffffffffu, x * ri, c);
        if (lane == c) x = xc;
        else if (lane < c) x = fma(-tri[c + 33 * lane], xc, x);
      }
      if (lane < pw) xs[p0 + lane] = x;
    }
    __syncthreads();
  }
}

// x := (L L^T)^{-1} x
template <typename T>
__device__ void solve_vec(const T* L, int n, int ld, T* xs) {
  fwd_solve<T>(L, n, ld, xs);
  bwd_solve<T>(L, n, ld, xs);
}

}  // namespace gbx
