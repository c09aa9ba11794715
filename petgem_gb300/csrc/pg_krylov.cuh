// Shared pieces of the Krylov solvers (GMRES, COCG in FP64 / complex64 /
// double-float, several systems): complex helpers, the complex128 and
// complex64 CSR products used for true residuals, per-RHS norms, the entity
// block check, the launch switch over the RHS count, and the solver plan.
//
// Vectors with k right-hand sides are stored row-major, RHS fastest:
// v[row * k + rhs].  k must be 1, 2, 4, 8, 16 or 32.  All reductions are
// two-stage with a fixed order, so results are bitwise reproducible.
#pragma once
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <stdio.h>

#include <mutex>
#include <vector>

#include "pg_common.cuh"
#include "pg_df.cuh"
#include "pg_blockjac.cuh"

namespace pgk {

// problem shape of one solve (shared by the solver translation units)
struct Plan {
  int64_t n, nnz;
  int k, m;
  int prec;           // 0 fp64 Arnoldi, 1 fp32 Arnoldi
  int nb;             // reduction blocks
  size_t csize;       // sizeof Arnoldi complex
  BjInfo bj;          // COCG entity block-Jacobi (bj.p == 0: diagonal Jacobi)
  int64_t gn = 0;     // gradient correction (COCG, GMRES): columns of G (0: off)
};

}  // namespace pgk

namespace {

using pgk::Plan;

constexpr int kThreads = 256;
constexpr int kMaxM = 64;    // restart length limit
constexpr int kMaxK = 32;    // RHS per block limit

// ---------------------------------------------------------------- complex helpers
__device__ __forceinline__ float2 cmul(float2 a, float2 b) { return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cfma(float2 a, float2 b, float2 c) {  // c + a*b
  return make_float2(fmaf(a.x, b.x, fmaf(-a.y, b.y, c.x)), fmaf(a.x, b.y, fmaf(a.y, b.x, c.y)));
}
__device__ __forceinline__ double2 cfma(double2 a, double2 b, double2 c) {
  return make_double2(fma(a.x, b.x, fma(-a.y, b.y, c.x)), fma(a.x, b.y, fma(a.y, b.x, c.y)));
}
__device__ __forceinline__ float2 cconjfma(float2 a, float2 b, float2 c) {  // c + conj(a)*b
  return make_float2(fmaf(a.x, b.x, fmaf(a.y, b.y, c.x)), fmaf(a.x, b.y, fmaf(-a.y, b.x, c.y)));
}
__device__ __forceinline__ double2 cconjfma(double2 a, double2 b, double2 c) {
  return make_double2(fma(a.x, b.x, fma(a.y, b.y, c.x)), fma(a.x, b.y, fma(-a.y, b.x, c.y)));
}
template <typename C> struct Real;
template <> struct Real<float2> { typedef float T; };
template <> struct Real<double2> { typedef double T; };
template <typename C> __device__ __forceinline__ C czero();
template <> __device__ __forceinline__ float2 czero<float2>() { return make_float2(0.f, 0.f); }
template <> __device__ __forceinline__ double2 czero<double2>() { return make_double2(0.0, 0.0); }
template <typename C> __device__ __forceinline__ C cfrom(double2 v);
template <> __device__ __forceinline__ float2 cfrom<float2>(double2 v) { return make_float2((float)v.x, (float)v.y); }
template <> __device__ __forceinline__ double2 cfrom<double2>(double2 v) { return v; }
__device__ __forceinline__ double2 to_d(float2 v) { return make_double2(v.x, v.y); }
__device__ __forceinline__ double2 to_d(double2 v) { return v; }

// acc = sum_j g_j v[c_j * K + rhs] over [j0, j1) of a row of the auxiliary
// map (or of its transpose), in FP64 and in entry order; four entries'
// index and value loads are issued before their four gathers, so a thread
// keeps four independent gathers in flight instead of one dependent chain.
template <int K, typename V>
__device__ __forceinline__ double2 grad_row_sum64(const int32_t* __restrict__ gc, const double* __restrict__ gv,
                                                  const V* __restrict__ v, int64_t j0, int64_t j1, int rhs) {
  double2 acc = make_double2(0.0, 0.0);
  int64_t j = j0;
  for (; j + 4 <= j1; j += 4) {
    int32_t c[4];
    double g[4];
    double2 w[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      c[i] = gc[j + i];
      g[i] = gv[j + i];
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) w[i] = to_d(v[(int64_t)c[i] * K + rhs]);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      acc.x = fma(g[i], w[i].x, acc.x);
      acc.y = fma(g[i], w[i].y, acc.y);
    }
  }
  for (; j < j1; ++j) {
    const double2 w = to_d(v[(int64_t)gc[j] * K + rhs]);
    acc.x = fma(gv[j], w.x, acc.x);
    acc.y = fma(gv[j], w.y, acc.y);
  }
  return acc;
}

__device__ __forceinline__ double2 dadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 dsub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 dscale(double s, double2 a) { return make_double2(s * a.x, s * a.y); }
__device__ __forceinline__ double dabs2(double2 a) { return a.x * a.x + a.y * a.y; }
__device__ __forceinline__ double2 dconj(double2 a) { return make_double2(a.x, -a.y); }
__device__ __forceinline__ double2 ddiv(double2 a, double2 b) {
  const double d = b.x * b.x + b.y * b.y;
  return make_double2((a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d);
}

template <typename T> __device__ __forceinline__ T shfl_xor(T v, int m) { return __shfl_xor_sync(0xffffffffu, v, m); }
__device__ __forceinline__ float2 shfl_xor(float2 v, int m) {
  return make_float2(__shfl_xor_sync(0xffffffffu, v.x, m), __shfl_xor_sync(0xffffffffu, v.y, m));
}
__device__ __forceinline__ double2 shfl_xor(double2 v, int m) {
  return make_double2(__shfl_xor_sync(0xffffffffu, v.x, m), __shfl_xor_sync(0xffffffffu, v.y, m));
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }

struct Ctl {
  int any_active;  // some RHS still iterating in this cycle
  int nonfinite;
};

// ---------------------------------------------------------------- SpMV / SpMM
// y = A x for k = 1, G lanes per row.  Optionally y = b - A x (resid).
template <typename C, int G>
__global__ void __launch_bounds__(kThreads) k_spmv1(const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                                                    const C* __restrict__ val, int64_t n, const C* __restrict__ x,
                                                    C* __restrict__ y, const C* __restrict__ bsub, const Ctl* ctl) {
  if (ctl && !ctl->any_active) return;
  // The row loop is warp-uniform (all 32 lanes run the same trip count) so
  // the full-mask shuffles below are always executed by the whole warp.
  const int lane = threadIdx.x % G;
  const int64_t groups = ((int64_t)gridDim.x * blockDim.x) / G;
  const int64_t gid = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / G;
  const int64_t warp_base = gid - (threadIdx.x & 31) / G;
  for (int64_t rw = warp_base; rw < n; rw += groups) {
    const int64_t r = rw + (gid - warp_base);
    const bool valid = r < n;
    C acc = czero<C>();
    if (valid) {
      const int64_t e = rowptr[r + 1];
      for (int64_t q = rowptr[r] + lane; q < e; q += G) acc = cfma(val[q], x[col[q]], acc);
    }
#pragma unroll
    for (int off = G / 2; off > 0; off >>= 1) acc = cadd(acc, shfl_xor(acc, off));
    if (valid && lane == 0) {
      if (bsub) {
        C bb = bsub[r];
        acc.x = bb.x - acc.x;
        acc.y = bb.y - acc.y;
      }
      y[r] = acc;
    }
  }
}

// k > 1: thread (row, rhs); rows of a block stride by kThreads / K
template <typename C, int K>
__global__ void __launch_bounds__(kThreads) k_spmm(const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                                                   const C* __restrict__ val, int64_t n, const C* __restrict__ x,
                                                   C* __restrict__ y, const C* __restrict__ bsub, const Ctl* ctl) {
  if (ctl && !ctl->any_active) return;
  const int rhs = threadIdx.x % K;
  const int64_t rows_per_pass = ((int64_t)gridDim.x * blockDim.x) / K;
  for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / K; r < n; r += rows_per_pass) {
    C acc = czero<C>();
    const int64_t e = rowptr[r + 1];
    for (int64_t q = rowptr[r]; q < e; ++q) acc = cfma(val[q], x[(int64_t)col[q] * K + rhs], acc);
    if (bsub) {
      C bb = bsub[r * K + rhs];
      acc.x = bb.x - acc.x;
      acc.y = bb.y - acc.y;
    }
    y[r * K + rhs] = acc;
  }
}

// ---------------------------------------------------------------- reductions
// Block-reduce per-thread values that all belong to rhs = tid % K; writes
// out[rhs] for this block (double2).  Fixed order => deterministic.
template <int K>
__device__ void block_reduce_rhs(double2 v, double2* smem, double2* out) {
  // warp stage: lanes with equal (lane % K) combine
#pragma unroll
  for (int off = 16; off >= K; off >>= 1) v = dadd(v, shfl_xor(v, off));
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane < K) smem[warp * K + lane] = v;
  __syncthreads();
  if (threadIdx.x < K) {
    double2 s = make_double2(0.0, 0.0);
    for (int w = 0; w < kThreads / 32; ++w) s = dadd(s, smem[w * K + threadIdx.x]);
    out[threadIdx.x] = s;
  }
  __syncthreads();
}

// per-RHS norms: block partials, then one warp per RHS
template <int K>
__global__ void __launch_bounds__(kThreads) k_norm2(const double2* __restrict__ r, int64_t n, double2* partial) {
  __shared__ double2 smem[(kThreads / 32) * kMaxK];
  const int64_t total = n * K;
  const int64_t chunk = ((total + gridDim.x - 1) / gridDim.x + K - 1) / K * K;
  const int64_t lo = (int64_t)blockIdx.x * chunk, hi = min(total, lo + chunk);
  double s = 0.0;
  for (int64_t e = lo + threadIdx.x; e < hi; e += kThreads) s += dabs2(r[e]);
  block_reduce_rhs<K>(make_double2(s, 0.0), smem, partial + (int64_t)blockIdx.x * K);
}

template <int K>
__global__ void k_norm_final(const double2* partial, int nblocks, double* out) {
  const int lane = threadIdx.x & 31, rhs = threadIdx.x >> 5;  // one warp per rhs
  if (rhs >= K) return;
  double s = 0.0;
  for (int b = lane; b < nblocks; b += 32) s += partial[(int64_t)b * K + rhs].x;
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
  if (lane == 0) out[rhs] = sqrt(s);
}

// rows of one entity must share their column list (entity-pair pattern);
// checked through row lengths and first / last columns before block scaling
__global__ void k_bj_check(const int64_t* rowptr, const int32_t* col, BjInfo B, int* status) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < B.n; r += (int64_t)gridDim.x * blockDim.x) {
    int64_t f, so;
    int na, loc;
    B.block(r, f, na, loc, so);
    const int64_t l0 = rowptr[f + 1] - rowptr[f], l = rowptr[r + 1] - rowptr[r];
    if (l != l0 || l < 1 || col[rowptr[r]] != col[rowptr[f]] || col[rowptr[r + 1] - 1] != col[rowptr[f + 1] - 1])
      *status = PG_ERR_ARG;
  }
}

__global__ void k_fill_one(double2* S, int64_t n) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x)
    S[r] = make_double2(1.0, 0.0);
}

int pick_blocks(int64_t n, int k) {
  int64_t nb = (n * k + 1023) / 1024;
  if (nb > 152 * 8) nb = 152 * 8;
  if (nb < 1) nb = 1;
  return (int)nb;
}

// Lanes per row: complex128 is FP64-pipe bound, so few lanes keep the
// shuffle reduction (FP64 adds) small; complex64 is bandwidth bound and uses
// more lanes for wider coalesced row segments.
template <typename C> struct LanesPerRow { static int pick(int64_t npr) { return npr > 48 ? 32 : (npr > 20 ? 16 : 8); } };
template <> struct LanesPerRow<double2> { static int pick(int64_t npr) { return npr > 64 ? 8 : 4; } };

template <typename C>
void launch_spmv(const Plan& P, const int64_t* rowptr, const int32_t* col, const C* val, const C* x, C* y,
                 const C* bsub, const Ctl* ctl, int64_t nnz_per_row, cudaStream_t s) {
  const unsigned grid = 152 * 16;
  switch (P.k) {
    case 1:
      switch (LanesPerRow<C>::pick(nnz_per_row)) {
        case 32: k_spmv1<C, 32><<<grid, kThreads, 0, s>>>(rowptr, col, val, P.n, x, y, bsub, ctl); break;
        case 16: k_spmv1<C, 16><<<grid, kThreads, 0, s>>>(rowptr, col, val, P.n, x, y, bsub, ctl); break;
        case 8: k_spmv1<C, 8><<<grid, kThreads, 0, s>>>(rowptr, col, val, P.n, x, y, bsub, ctl); break;
        default: k_spmv1<C, 4><<<grid, kThreads, 0, s>>>(rowptr, col, val, P.n, x, y, bsub, ctl); break;
      }
      break;
    case 2: k_spmm<C, 2><<<grid, kThreads, 0, s>>>(rowptr, col, val, P.n, x, y, bsub, ctl); break;
    case 4: k_spmm<C, 4><<<grid, kThreads, 0, s>>>(rowptr, col, val, P.n, x, y, bsub, ctl); break;
    case 8: k_spmm<C, 8><<<grid, kThreads, 0, s>>>(rowptr, col, val, P.n, x, y, bsub, ctl); break;
    case 16: k_spmm<C, 16><<<grid, kThreads, 0, s>>>(rowptr, col, val, P.n, x, y, bsub, ctl); break;
    case 32: k_spmm<C, 32><<<grid, kThreads, 0, s>>>(rowptr, col, val, P.n, x, y, bsub, ctl); break;
  }
}

#define PG_KSWITCH(KVAR, CALL)              \
  switch (KVAR) {                           \
    case 1: { constexpr int K = 1; CALL; } break;   \
    case 2: { constexpr int K = 2; CALL; } break;   \
    case 4: { constexpr int K = 4; CALL; } break;   \
    case 8: { constexpr int K = 8; CALL; } break;   \
    case 16: { constexpr int K = 16; CALL; } break; \
    case 32: { constexpr int K = 32; CALL; } break; \
  }

bool valid_k(int k) { return k == 1 || k == 2 || k == 4 || k == 8 || k == 16 || k == 32; }

// Gradient correction shared by COCG and GMRES: G (real, DOF rows x H1
// columns, from pg_gradient_map) and its transpose (rows ascending).
// invD[phi] = 1 / (G^T A G)_{phi phi} (0 for an empty or vanishing column;
// raw != 0 stores the diagonal itself).  (A G_phi)_r = sum_k A_rk G_{k phi};
// G_{k phi} is looked up by binary search in the transpose row of phi.  One
// warp per column (launch 32 threads per column): the warp walks the
// column's rows r in order, lane l takes the stored entries l, l + 32, ... of
// row r of A (coalesced loads), each lane keeps its own partial sum, and the
// lanes' sums are combined in a fixed tree, so the result does not depend on
// scheduling.
__global__ void k_grad_diag(const int64_t* rowptr, const int32_t* col, const double2* A, const int64_t* gtp,
                            const int32_t* gtr, const double* gtv, int64_t gn, double2* invD, int raw = 0) {
  const int lane = threadIdx.x & 31;
  const int64_t w0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t c = w0; c < gn; c += nw) {
    const int64_t lo = gtp[c], hi = gtp[c + 1];
    double2 d = make_double2(0.0, 0.0);
    for (int64_t j = lo; j < hi; ++j) {
      const int64_t r = gtr[j];
      const double gj = gtv[j];
      for (int64_t k = rowptr[r] + lane; k < rowptr[r + 1]; k += 32) {
        const int32_t s = col[k];
        int64_t a = lo, b = hi;
        while (a < b) {
          const int64_t m = (a + b) >> 1;
          if (gtr[m] < s) a = m + 1;
          else b = m;
        }
        if (a < hi && gtr[a] == s) {
          const double w = gj * gtv[a];
          d.x = fma(A[k].x, w, d.x);
          d.y = fma(A[k].y, w, d.y);
        }
      }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      d.x += __shfl_down_sync(0xffffffffu, d.x, off);
      d.y += __shfl_down_sync(0xffffffffu, d.y, off);
    }
    if (lane != 0) continue;
    if (raw) invD[c] = d;
    else invD[c] = (d.x == 0.0 && d.y == 0.0) ? make_double2(0.0, 0.0) : ddiv(make_double2(1.0, 0.0), d);
  }
}



}  // namespace
