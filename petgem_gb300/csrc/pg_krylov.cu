// Restarted GMRES for petgem's complex system A x = b (petgem/solver.py:584-594,
// PETSc KSP with -ksp_type gmres -pc_type jacobi), for one or several
// right-hand sides at once.
//
// Structure (same code for both precisions, templated on the Arnoldi scalar):
//   loop over restarts:
//     r = b - A x                    complex128 CSR SpMV/SpMM with the original A
//     stop when ||r|| <= rtol ||b|| for every RHS (true residual, FP64)
//     one Arnoldi cycle of m steps on  Ahat = A D^-1  (right Jacobi), in the
//     Arnoldi precision: complex128 ("fp64") or complex64 ("mixed")
//     x += D^-1 V y                  FP64 update
// In the mixed form every restart is an FP64 iterative-refinement step around
// a complex64 GMRES(m) cycle; in the plain form both parts are complex128.
//
// Orthogonalisation is classical Gram-Schmidt (PETSc's default), optionally
// repeated once (CGS2).  Basis vectors are stored unnormalised with a scale
// alpha_i = 1/||v~_i|| that is folded into the small Hessenberg scalars, so
// no kernel rewrites a vector only to normalise it.  All reductions are
// two-stage with a fixed order: results are bitwise reproducible.  Within a
// cycle the host does not synchronise: a one-block kernel applies the Givens
// rotations, tracks the residual estimate and switches the remaining launches
// of the cycle off once every RHS is below its target.
//
// Vectors with k right-hand sides are stored row-major, RHS fastest:
// v[row * k + rhs].  k must be 1, 2, 4, 8, 16 or 32.
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <stdio.h>

#include <mutex>
#include <vector>

#include "pg_common.cuh"
#include "pg_df.cuh"
#include "pg_blockjac.cuh"

namespace {

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

// ---------------------------------------------------------------- per-RHS cycle state
struct RhsState {
  double2 H[kMaxM * (kMaxM + 1)];  // column j: H[j*(m+1) + i]
  double2 g[kMaxM + 1];
  double2 sn[kMaxM];
  double cs[kMaxM];
  double alpha[kMaxM + 1];         // 1 / ||v~_i||
  double2 y[kMaxM];
  double target;                   // absolute residual target for this RHS
  double res_est;                  // current Arnoldi residual estimate
  double rnorm;                    // ||r|| at cycle start
  int active;                      // still iterating in this cycle
  int kdone;                       // Arnoldi steps completed in this cycle
  int breakdown;
  int pad;
};

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

// partial[b][i][rhs] = sum over this block's rows of conj(v~_i) . w~   for i <= j
// Basis vectors are processed 8 at a time (accumulators stay in registers).
template <typename C, int K>
__global__ void __launch_bounds__(kThreads) k_dots(const C* __restrict__ V, int64_t stride, const C* __restrict__ w,
                                                   int64_t n, int j, double2* partial, const Ctl* ctl) {
  if (!ctl->any_active) return;
  constexpr int GB = 8;
  __shared__ double2 smem[(kThreads / 32) * kMaxK];
  const int64_t total = n * K;
  const int64_t chunk = ((total + gridDim.x - 1) / gridDim.x + K - 1) / K * K;
  const int64_t lo = (int64_t)blockIdx.x * chunk, hi = min(total, lo + chunk);
  double2* out = partial + (int64_t)blockIdx.x * (kMaxM + 1) * K;
  for (int i0 = 0; i0 <= j; i0 += GB) {
    C acc[GB];
#pragma unroll
    for (int t = 0; t < GB; ++t) acc[t] = czero<C>();
    for (int64_t e = lo + threadIdx.x; e < hi; e += kThreads) {
      const C we = w[e];
#pragma unroll
      for (int t = 0; t < GB; ++t)
        if (i0 + t <= j) acc[t] = cconjfma(V[(int64_t)(i0 + t) * stride + e], we, acc[t]);
    }
#pragma unroll
    for (int t = 0; t < GB; ++t)
      if (i0 + t <= j) block_reduce_rhs<K>(to_d(acc[t]), smem, out + (i0 + t) * K);
  }
}

// sums of |w|^2 per rhs for this block
template <typename C, int K>
__device__ void norm_partial(double2 v, double2* smem, double2* out) {
  block_reduce_rhs<K>(v, smem, out);
}

// h_ij = alpha_i * alpha_j * sum_b partial ; coef[i][rhs] = h_ij * alpha_i (as C)
// `accumulate` adds into the existing column (second CGS pass, alpha_j := 1).
template <typename C, int K>
__global__ void k_dots_final(const double2* partial, int nblocks, int j, int m, RhsState* st, C* coef, int second,
                             const Ctl* ctl) {
  if (!ctl->any_active) return;
  // one warp per (i, rhs) item; lanes sum the block partials in a fixed pattern
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  for (int t = warp; t < (j + 1) * K; t += nwarps) {  // t = i * K + rhs
    const int i = t / K, rhs = t % K;
    double2 s = make_double2(0.0, 0.0);
    for (int b = lane; b < nblocks; b += 32) s = dadd(s, partial[((int64_t)b * (kMaxM + 1) + i) * K + rhs]);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) s = dadd(s, shfl_xor(s, off));
    if (lane == 0) {
      RhsState& S = st[rhs];
      const double aj = second ? 1.0 : S.alpha[j];
      const double2 h = dscale(S.alpha[i] * aj, s);
      if (S.active) {
        if (second) S.H[j * (m + 1) + i] = dadd(S.H[j * (m + 1) + i], h);
        else S.H[j * (m + 1) + i] = h;
      }
      coef[i * K + rhs] = cfrom<C>(dscale(S.alpha[i], h));
    }
  }
}

// w~ <- a_j w~ - sum_i coef_i v~_i ; partial norms of the result
template <typename C, int K>
__global__ void __launch_bounds__(kThreads) k_update(const C* __restrict__ V, int64_t stride, C* __restrict__ w,
                                                     int64_t n, int j, const C* __restrict__ coef,
                                                     const RhsState* st, int second, double2* partial,
                                                     const Ctl* ctl) {
  if (!ctl->any_active) return;
  __shared__ double2 smem[(kThreads / 32) * kMaxK];
  __shared__ C cf[kMaxM * kMaxK];
  __shared__ typename Real<C>::T aj[kMaxK];
  for (int t = threadIdx.x; t < (j + 1) * K; t += kThreads) cf[t] = coef[t];
  if (threadIdx.x < K) aj[threadIdx.x] = second ? 1 : (typename Real<C>::T)st[threadIdx.x].alpha[j];
  __syncthreads();
  const int rhs = threadIdx.x % K;
  const int64_t total = n * K;
  const int64_t chunk = ((total + gridDim.x - 1) / gridDim.x + K - 1) / K * K;
  const int64_t lo = (int64_t)blockIdx.x * chunk, hi = min(total, lo + chunk);
  double nrm = 0.0;
  typename Real<C>::T nrm_f = 0;
  for (int64_t e = lo + threadIdx.x; e < hi; e += kThreads) {
    C v = w[e];
    v.x *= aj[rhs];
    v.y *= aj[rhs];
#pragma unroll 4
    for (int i = 0; i <= j; ++i) {
      const C c = cf[i * K + rhs];
      const C b = V[(int64_t)i * stride + e];
      v.x -= c.x * b.x - c.y * b.y;
      v.y -= c.x * b.y + c.y * b.x;
    }
    w[e] = v;
    nrm_f += v.x * v.x + v.y * v.y;
  }
  nrm = (double)nrm_f;
  block_reduce_rhs<K>(make_double2(nrm, 0.0), smem, partial + (int64_t)blockIdx.x * K);
}

// Finish step j: h_{j+1,j} = ||w||, Givens, residual estimate, activity.
template <int K>
__global__ void k_givens(const double2* partial, int nblocks, int j, int m, RhsState* st, Ctl* ctl, int last) {
  if (!ctl->any_active) return;
  __shared__ int any;
  if (threadIdx.x == 0) any = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, rhs = threadIdx.x >> 5;  // one warp per rhs
  if (rhs < K) {
    RhsState& S = st[rhs];
    double ss = 0.0;
    for (int b = lane; b < nblocks; b += 32) ss += partial[(int64_t)b * K + rhs].x;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) ss += __shfl_xor_sync(0xffffffffu, ss, off);
    if (lane == 0 && S.active) {
      const double hn = sqrt(ss);
      double2* Hc = S.H + j * (m + 1);
      Hc[j + 1] = make_double2(hn, 0.0);
      if (!isfinite(hn)) ctl->nonfinite = 1;
      S.alpha[j + 1] = hn > 0.0 ? 1.0 / hn : 0.0;
      // apply previous rotations to column j
      for (int i = 0; i < j; ++i) {
        const double2 a = Hc[i], b = Hc[i + 1];
        const double c = S.cs[i];
        const double2 s = S.sn[i];
        Hc[i] = dadd(dscale(c, a), cmul(s, b));
        Hc[i + 1] = dsub(dscale(c, b), cmul(dconj(s), a));
      }
      // new rotation zeroing H[j+1][j]
      const double2 a = Hc[j], b = Hc[j + 1];
      const double na = sqrt(dabs2(a)), nb = sqrt(dabs2(b));
      double c;
      double2 s;
      if (nb == 0.0) {
        c = 1.0;
        s = make_double2(0.0, 0.0);
      } else if (na == 0.0) {
        c = 0.0;
        s = make_double2(1.0, 0.0);
      } else {
        const double r = sqrt(na * na + nb * nb);
        c = na / r;
        const double2 ph = dscale(1.0 / na, a);  // a/|a|
        s = dscale(1.0 / r, cmul(ph, dconj(b)));
      }
      S.cs[j] = c;
      S.sn[j] = s;
      Hc[j] = dadd(dscale(c, a), cmul(s, b));
      Hc[j + 1] = make_double2(0.0, 0.0);
      const double2 gj = S.g[j];
      S.g[j] = dscale(c, gj);
      S.g[j + 1] = dscale(-1.0, cmul(dconj(s), gj));
      S.res_est = sqrt(dabs2(S.g[j + 1]));
      S.kdone = j + 1;
      const bool lucky = !(hn > 1e-300 * (S.rnorm > 0 ? S.rnorm : 1.0));
      if (lucky) S.breakdown = 1;
      if (S.res_est <= S.target || lucky || last || !isfinite(S.res_est)) S.active = 0;
    }
    __syncwarp();
    if (lane == 0 && S.active) atomicOr(&any, 1);
  }
  __syncthreads();
  if (threadIdx.x == 0) ctl->any_active = any;
}

// y = H^-1 g (upper triangular, kdone x kdone); coef_i = y_i alpha_i
template <int K>
__global__ void k_backsolve(RhsState* st, int m, double2* ycoef) {
  const int rhs = threadIdx.x;
  if (rhs >= K) return;
  RhsState& S = st[rhs];
  const int k = S.kdone;
  for (int i = k - 1; i >= 0; --i) {
    double2 s = S.g[i];
    for (int l = i + 1; l < k; ++l) s = dsub(s, cmul(S.H[l * (m + 1) + i], S.y[l]));
    const double2 d = S.H[i * (m + 1) + i];
    S.y[i] = (d.x == 0.0 && d.y == 0.0) ? make_double2(0.0, 0.0) : ddiv(s, d);
  }
  for (int i = 0; i < kMaxM; ++i) ycoef[i * K + rhs] = i < k ? dscale(S.alpha[i], S.y[i]) : make_double2(0.0, 0.0);
}

// x += D^-1 sum_i ycoef_i v~_i   (FP64 accumulation)
template <typename C, int K>
__global__ void __launch_bounds__(kThreads) k_update_x(const C* __restrict__ V, int64_t stride, int kmax, int64_t n,
                                                       const double2* __restrict__ ycoef, const double2* __restrict__ dinv,
                                                       double2* __restrict__ x) {
  __shared__ double2 yc[kMaxM * kMaxK];
  for (int t = threadIdx.x; t < kmax * K; t += kThreads) yc[t] = ycoef[t];
  __syncthreads();
  const int64_t total = n * K;
  for (int64_t e = (int64_t)blockIdx.x * kThreads + threadIdx.x; e < total; e += (int64_t)gridDim.x * kThreads) {
    const int rhs = (int)(e % K);
    double2 s = make_double2(0.0, 0.0);
    for (int i = 0; i < kmax; ++i) {
      const double2 c = yc[i * K + rhs];
      if (c.x != 0.0 || c.y != 0.0) s = cfma(c, to_d(V[(int64_t)i * stride + e]), s);
    }
    x[e] = dadd(x[e], cmul(dinv[e / K], s));
  }
}

// v~_0 = r / ||r|| (cast to C); per-RHS norms partials first
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

template <typename C, int K>
__global__ void __launch_bounds__(kThreads) k_start(const double2* __restrict__ r, int64_t n, const double* rnorm,
                                                    C* __restrict__ v0) {
  __shared__ double inv[kMaxK];
  if (threadIdx.x < K) inv[threadIdx.x] = rnorm[threadIdx.x] > 0 ? 1.0 / rnorm[threadIdx.x] : 0.0;
  __syncthreads();
  const int64_t total = n * K;
  for (int64_t e = (int64_t)blockIdx.x * kThreads + threadIdx.x; e < total; e += (int64_t)gridDim.x * kThreads)
    v0[e] = cfrom<C>(dscale(inv[e % K], r[e]));
}

template <int K>
__global__ void k_cycle_init(RhsState* st, const double* rnorm, const double* target, const int* want, Ctl* ctl) {
  __shared__ int any;
  if (threadIdx.x == 0) any = 0;
  __syncthreads();
  const int rhs = threadIdx.x;
  if (rhs < K) {
    RhsState& S = st[rhs];
    S.rnorm = rnorm[rhs];
    S.target = target[rhs];
    S.alpha[0] = 1.0;
    S.g[0] = make_double2(rnorm[rhs], 0.0);
    S.res_est = rnorm[rhs];
    S.kdone = 0;
    S.breakdown = 0;
    S.active = want[rhs] && rnorm[rhs] > 0.0;
    if (S.active) atomicOr(&any, 1);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    ctl->any_active = any;
    ctl->nonfinite = 0;
  }
}

// Ahat = A D^-1 in the Arnoldi precision; dinv = 1 / diag(A)
__global__ void k_diag_inv(const int64_t* rowptr, const int32_t* col, const double2* val, int64_t n, double2* dinv,
                           int* status) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    double2 d = make_double2(0.0, 0.0);
    for (int64_t q = rowptr[r]; q < rowptr[r + 1]; ++q)
      if (col[q] == r) d = val[q];
    if (d.x == 0.0 && d.y == 0.0) {
      *status = PG_ERR_BREAKDOWN;
      dinv[r] = make_double2(1.0, 0.0);
    } else {
      dinv[r] = ddiv(make_double2(1.0, 0.0), d);
    }
  }
}

template <typename C>
__global__ void k_scale_cols(const int32_t* col, const double2* val, int64_t nnz, const double2* dinv, C* out) {
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < nnz; q += (int64_t)gridDim.x * blockDim.x)
    out[q] = cfrom<C>(cmul(val[q], dinv[col[q]]));
}

// ---------------------------------------------------------------- host driver
struct Plan {
  int64_t n, nnz;
  int k, m;
  int prec;           // 0 fp64 Arnoldi, 1 fp32 Arnoldi
  int nb;             // reduction blocks
  size_t csize;       // sizeof Arnoldi complex
  BjInfo bj;          // COCG entity block-Jacobi (bj.p == 0: diagonal Jacobi)
};

size_t ws_layout(const Plan& P, size_t* off /* 16 */) {
  size_t o = 0;
  auto put = [&](int idx, size_t bytes) { off[idx] = o; o += pg_align256(bytes); };
  put(0, P.nnz * P.csize);                                   // Ahat
  put(1, sizeof(double2) * P.n);                             // dinv
  put(2, P.csize * (size_t)(P.m + 1) * P.n * P.k);           // V
  put(3, sizeof(double2) * P.n * P.k);                       // r
  put(4, sizeof(double2) * (size_t)P.nb * (kMaxM + 1) * P.k);  // dot partials
  put(5, sizeof(double2) * (size_t)P.nb * P.k);              // norm partials
  put(6, sizeof(RhsState) * P.k);                            // state
  put(7, sizeof(Ctl));                                       // ctl
  put(8, P.csize * kMaxM * P.k);                             // coef
  put(9, sizeof(double2) * kMaxM * P.k);                     // ycoef
  put(10, sizeof(double) * P.k);                             // rnorm
  put(11, sizeof(double) * P.k);                             // target
  put(12, sizeof(int) * P.k);                                // want
  put(13, sizeof(int));                                      // status
  put(14, P.bj.p ? sizeof(double2) * P.bj.s_size() : 0);    // block-Jacobi factors S
  put(15, P.bj.p ? sizeof(double2) * P.bj.s_size() : 0);    // block inverses M^-1
  return o;
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

// GMRES block-Jacobi: Minv_a = A_aa^-1 = S_a^T S_a per entity block
// (row-major na x na, complex symmetric), from the COCG factors S_a
__global__ void k_bj_minv(const double2* S, BjInfo B, double2* Minv) {
  for (int64_t r0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r0 < B.n; r0 += (int64_t)gridDim.x * blockDim.x) {
    int64_t first, soff;
    int na, loc;
    B.block(r0, first, na, loc, soff);
    if (loc != 0) continue;
    const double2* Sa = S + soff;
    double2* Ma = Minv + soff;
    for (int l = 0; l < na; ++l)
      for (int j = 0; j < na; ++j) {
        double2 acc = make_double2(0.0, 0.0);
        for (int t = l > j ? l : j; t < na; ++t) {
          const double2 u = bj_mul(Sa[t * na + l], Sa[t * na + j]);
          acc.x += u.x;
          acc.y += u.y;
        }
        Ma[l * na + j] = acc;
      }
  }
}

// out = A M^-1 row by row: the entry at column fb + j of entity b is
// sum_l A[r, fb + l] Minv_b[l, j] (entity b's columns are contiguous in the row)
template <typename CM>
__global__ void k_bj_right_scale(const int64_t* rowptr, const int32_t* col, const double2* val, BjInfo B,
                                 const double2* Minv, CM* out) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < B.n; r += (int64_t)gridDim.x * blockDim.x) {
    for (int64_t k = rowptr[r]; k < rowptr[r + 1]; ++k) {
      int64_t fb, sb;
      int nb, j;
      B.block(col[k] - B.c0, fb, nb, j, sb);
      const double2* Mb = Minv + sb;
      double2 acc = make_double2(0.0, 0.0);
      for (int l = 0; l < nb; ++l) {
        const double2 t = bj_mul(val[k - j + l], Mb[l * nb + j]);
        acc.x += t.x;
        acc.y += t.y;
      }
      out[k] = cfrom<CM>(acc);
    }
  }
}

// x[:, c] += Minv t[:, c] (full entity blocks), K columns
template <int K>
__global__ void k_bj_minv_apply_add(const double2* Minv, BjInfo B, const double2* t, double2* x) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < B.n * K; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = e / K;
    const int c = (int)(e % K);
    int64_t fa, sa;
    int na, i;
    B.block(r, fa, na, i, sa);
    double2 acc = x[e];
    for (int l = 0; l < na; ++l) {
      const double2 u = bj_mul(Minv[sa + i * na + l], t[(fa + l) * K + c]);
      acc.x += u.x;
      acc.y += u.y;
    }
    x[e] = acc;
  }
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

template <typename C>
int run_gmres(const Plan& P, const int64_t* rowptr, const int32_t* col, const double2* A, const double2* b, double2* x,
              const pg_gmres_opts* o, pg_gmres_result* res, double* relres_out, char* ws, cudaStream_t s) {
  size_t off[16];
  ws_layout(P, off);
  C* Ahat = reinterpret_cast<C*>(ws + off[0]);
  double2* dinv = reinterpret_cast<double2*>(ws + off[1]);
  C* V = reinterpret_cast<C*>(ws + off[2]);
  double2* r = reinterpret_cast<double2*>(ws + off[3]);
  double2* dpart = reinterpret_cast<double2*>(ws + off[4]);
  double2* npart = reinterpret_cast<double2*>(ws + off[5]);
  RhsState* st = reinterpret_cast<RhsState*>(ws + off[6]);
  Ctl* ctl = reinterpret_cast<Ctl*>(ws + off[7]);
  C* coef = reinterpret_cast<C*>(ws + off[8]);
  double2* ycoef = reinterpret_cast<double2*>(ws + off[9]);
  double* rnorm = reinterpret_cast<double*>(ws + off[10]);
  double* target = reinterpret_cast<double*>(ws + off[11]);
  int* want = reinterpret_cast<int*>(ws + off[12]);
  int* dstatus = reinterpret_cast<int*>(ws + off[13]);
  const int k = P.k, m = P.m, nb = P.nb;
  const int64_t stride = P.n * k;
  const int64_t npr = P.nnz / (P.n > 0 ? P.n : 1);

  const bool bj = P.bj.p > 0;
  double2* Sblk = reinterpret_cast<double2*>(ws + off[14]);
  double2* Minv = reinterpret_cast<double2*>(ws + off[15]);
  PG_CUDA_TRY(cudaMemsetAsync(dstatus, 0, sizeof(int), s));
  if (bj) {
    // right preconditioning with the entity blocks' inverses: Ahat = A M^-1
    k_bj_check<<<pg_blocks(P.n, 256), 256, 0, s>>>(rowptr, col, P.bj, dstatus);
    int hchk = 0;
    PG_CUDA_TRY(cudaMemcpyAsync(&hchk, dstatus, sizeof(int), cudaMemcpyDeviceToHost, s));
    PG_CUDA_TRY(cudaStreamSynchronize(s));
    if (hchk) {
      pg_set_error("pg_gmres: block-Jacobi needs the entity-block pattern (rows of one entity share their columns)");
      return PG_ERR_ARG;
    }
    // |D| of the factorisation is not needed here: dinv serves as its scratch
    k_bj_factor<<<pg_blocks(P.n, 128), 128, 0, s>>>(rowptr, col, A, P.bj, Sblk, reinterpret_cast<double*>(dinv),
                                                     dstatus);
    k_bj_minv<<<pg_blocks(P.n, 128), 128, 0, s>>>(Sblk, P.bj, Minv);
    k_bj_right_scale<C><<<pg_blocks(P.n, 128), 128, 0, s>>>(rowptr, col, A, P.bj, Minv, Ahat);
    k_fill_one<<<pg_blocks(P.n, 256), 256, 0, s>>>(dinv, P.n);   // the basis combination is added unscaled
  } else {
    k_diag_inv<<<pg_blocks(P.n, 256), 256, 0, s>>>(rowptr, col, A, P.n, dinv, dstatus);
    k_scale_cols<C><<<pg_blocks(P.nnz, 256), 256, 0, s>>>(col, A, P.nnz, dinv, Ahat);
  }
  PG_LAUNCH_CHECK();

  // ||b|| per RHS
  std::vector<double> bnorm(k), rn(k), tgt(k);
  std::vector<int> wnt(k);
  PG_KSWITCH(k, (k_norm2<K><<<nb, kThreads, 0, s>>>(b, P.n, npart), k_norm_final<K><<<1, 32 * K, 0, s>>>(npart, nb, rnorm)));
  PG_LAUNCH_CHECK();
  PG_CUDA_TRY(cudaMemcpyAsync(bnorm.data(), rnorm, sizeof(double) * k, cudaMemcpyDeviceToHost, s));
  int hstatus = 0;
  PG_CUDA_TRY(cudaMemcpyAsync(&hstatus, dstatus, sizeof(int), cudaMemcpyDeviceToHost, s));
  PG_CUDA_TRY(cudaStreamSynchronize(s));
  if (hstatus) {
    pg_set_error("pg_gmres: zero diagonal entry or block pivot (Jacobi preconditioner undefined)");
    return PG_ERR_BREAKDOWN;
  }
  for (int i = 0; i < k; ++i) {
    if (!isfinite(bnorm[i])) {
      pg_set_error("pg_gmres: non-finite right-hand side");
      return PG_ERR_NONFINITE;
    }
  }
  int64_t its = 0, restarts = 0;
  int status = PG_OK;
  // PG_KSP_MONITOR=1 prints the true residual at every restart (like PETSc -ksp_monitor_true_residual)
  const char* mon_env = getenv("PG_KSP_MONITOR");
  const bool monitor = mon_env && mon_env[0] && mon_env[0] != '0';
  if (monitor)
    for (int i = 0; i < k; ++i) fprintf(stderr, "pg_gmres: rhs %d ||b|| = %.6e\n", i, bnorm[i]);
  const int64_t max_it = o->max_it > 0 ? o->max_it : 10000;
  for (;;) {
    // r = b - A x (FP64), ||r||
    launch_spmv<double2>(P, rowptr, col, A, x, r, b, nullptr, npr, s);
    PG_KSWITCH(k, (k_norm2<K><<<nb, kThreads, 0, s>>>(r, P.n, npart), k_norm_final<K><<<1, 32 * K, 0, s>>>(npart, nb, rnorm)));
    PG_LAUNCH_CHECK();
    PG_CUDA_TRY(cudaMemcpyAsync(rn.data(), rnorm, sizeof(double) * k, cudaMemcpyDeviceToHost, s));
    PG_CUDA_TRY(cudaStreamSynchronize(s));
    bool all = true;
    if (monitor)
      for (int i = 0; i < k; ++i)
        fprintf(stderr, "pg_gmres: restart %lld its %lld rhs %d true ||r||/||b|| = %.6e\n", (long long)restarts,
                (long long)its, i, bnorm[i] > 0 ? rn[i] / bnorm[i] : 0.0);
    for (int i = 0; i < k; ++i) {
      if (!isfinite(rn[i])) {
        pg_set_error("pg_gmres: non-finite residual");
        status = PG_ERR_NONFINITE;
      }
      const double tb = o->rtol * bnorm[i];
      const bool ok = rn[i] <= tb || bnorm[i] == 0.0;
      wnt[i] = ok ? 0 : 1;
      // inner target: aim slightly below the outer target (estimate vs true residual)
      tgt[i] = tb * 0.5;
      if (!ok) all = false;
    }
    if (status) break;
    if (all) break;
    if (its >= max_it) {
      status = PG_ERR_NOT_CONVERGED;
      break;
    }
    PG_CUDA_TRY(cudaMemcpyAsync(target, tgt.data(), sizeof(double) * k, cudaMemcpyHostToDevice, s));
    PG_CUDA_TRY(cudaMemcpyAsync(want, wnt.data(), sizeof(int) * k, cudaMemcpyHostToDevice, s));
    PG_KSWITCH(k, (k_start<C, K><<<pg_blocks(P.n * K, kThreads), kThreads, 0, s>>>(r, P.n, rnorm, V),
                   k_cycle_init<K><<<1, 32, 0, s>>>(st, rnorm, target, want, ctl)));
    int steps = (int)((max_it - its) < m ? (max_it - its) : m);
    for (int j = 0; j < steps; ++j) {
      C* vj = V + (int64_t)j * stride;
      C* w = V + (int64_t)(j + 1) * stride;
      launch_spmv<C>(P, rowptr, col, Ahat, vj, w, nullptr, ctl, npr, s);
      const int passes = o->reorth ? 2 : 1;
      for (int pass = 0; pass < passes; ++pass) {
        PG_KSWITCH(k, (k_dots<C, K><<<nb, kThreads, 0, s>>>(V, stride, w, P.n, j, dpart, ctl),
                       k_dots_final<C, K><<<1, 1024, 0, s>>>(dpart, nb, j, m, st, coef, pass, ctl),
                       k_update<C, K><<<nb, kThreads, 0, s>>>(V, stride, w, P.n, j, coef, st, pass, npart, ctl)));
      }
      PG_KSWITCH(k, (k_givens<K><<<1, 32 * K, 0, s>>>(npart, nb, j, m, st, ctl, j == steps - 1)));
    }
    PG_LAUNCH_CHECK();
    if (bj) {
      // x += M^-1 (V y): the combination into r (free until the next true residual), then the blocks
      PG_CUDA_TRY(cudaMemsetAsync(r, 0, sizeof(double2) * P.n * k, s));
      PG_KSWITCH(k, (k_backsolve<K><<<1, 32, 0, s>>>(st, m, ycoef),
                     k_update_x<C, K><<<pg_blocks(P.n * K, kThreads), kThreads, 0, s>>>(V, stride, steps, P.n,
                                                                                        ycoef, dinv, r),
                     k_bj_minv_apply_add<K><<<pg_blocks(P.n * K, 256), 256, 0, s>>>(Minv, P.bj, r, x)));
    } else {
      PG_KSWITCH(k, (k_backsolve<K><<<1, 32, 0, s>>>(st, m, ycoef),
                     k_update_x<C, K><<<pg_blocks(P.n * K, kThreads), kThreads, 0, s>>>(V, stride, steps, P.n,
                                                                                        ycoef, dinv, x)));
    }
    // iterations actually used this cycle (max over RHS)
    std::vector<int> hs(k);
    for (int i = 0; i < k; ++i)
      PG_CUDA_TRY(cudaMemcpyAsync(&hs[i], &st[i].kdone, sizeof(int), cudaMemcpyDeviceToHost, s));
    Ctl hctl;
    PG_CUDA_TRY(cudaMemcpyAsync(&hctl, ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, s));
    PG_CUDA_TRY(cudaStreamSynchronize(s));
    int used = 0;
    for (int i = 0; i < k; ++i) used = hs[i] > used ? hs[i] : used;
    its += used > 0 ? used : 1;
    ++restarts;
    if (hctl.nonfinite) {
      pg_set_error("pg_gmres: non-finite Arnoldi norm");
      status = PG_ERR_NONFINITE;
      break;
    }
  }
  double worst = 0.0;
  for (int i = 0; i < k; ++i) {
    const double rr = bnorm[i] > 0 ? rn[i] / bnorm[i] : 0.0;
    if (relres_out) relres_out[i] = rr;
    worst = rr > worst ? rr : worst;
  }
  if (res) {
    res->iterations = its;
    res->restarts = restarts;
    res->relres = worst;
    res->status = status;
  }
  if (status == PG_ERR_NOT_CONVERGED) pg_set_error("pg_gmres: max_it reached before rtol");
  return status;
}


// ============================================================================
// COCG: conjugate orthogonal CG for complex-symmetric A (A^T = A, not
// Hermitian), the short-recurrence Krylov method for the complex symmetric
// systems of frequency-domain edge-element EM.  Jacobi enters as a symmetric
// scaling  At = S A S,  S = D^-1/2  (complex principal square root), which
// keeps At complex symmetric; the iteration solves At y = S r and x += S y.
// The recurrence works in the Arnoldi-equivalent "compute" precision (complex
// 128 or 64).  At every host check (every `check_every` iterations) the FP64
// true residual  r = b - A x  replaces the recurrence residual (reliable
// update: the search direction p is kept), and convergence is decided on it.
// Per iteration: SpMV fused with mu = p^T q; alpha; y += alpha p, r -= alpha q
// fused with rho = r^T r and the true-residual weight sum |r_i|^2 |D_i|; beta;
// p = r + beta p.  Reductions are fixed-order (deterministic).
// ============================================================================

struct CgState {
  double2 rho;     // r^T r (bilinear)
  double2 alpha, beta;
  double target;   // absolute true-residual target
  double res;      // recurrence estimate of the true residual
  double res0;     // true residual at the start of this cycle
  int active;      // iterating (not converged)
  int its;
  int breakdown;
  int beta_iter;   // launch index whose beta is current (p is updated once per beta)
};

struct CgCtl {
  int any_active;      // some RHS still iterating in this cycle
  int nonfinite;
  unsigned counter;    // last-block-done counter (reset by the last block)
  int pending;         // double-float path: a p update is due (set by the update, cleared by the product)
};

template <typename C>
__device__ __forceinline__ double2 bilin(C a, C b) {  // a*b (no conjugate) in double
  const double2 x = to_d(a), y = to_d(b);
  return make_double2(x.x * y.x - x.y * y.y, x.x * y.y + x.y * y.x);
}

// Every block publishes its partial; the block that arrives last (atomic
// ticket) reduces all partials in block order - a fixed order, so the result
// does not depend on which block is last.  Nothing waits: no spin.
__device__ __forceinline__ bool arrive_last(unsigned* counter) {
  __shared__ bool last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(counter, 1u) == gridDim.x - 1;
  __syncthreads();
  return last;
}

// block-wide fixed-order sum of partial[b * K + rhs] over b, per rhs (K <= 32)
template <int K>
__device__ double2 sum_partials(const double2* partial, int nblocks, int rhs, double2* smem) {
  // thread t handles rhs = t % K, blocks b = t / K, t / K + 256 / K, ...
  const int my_rhs = threadIdx.x % K;
  double2 acc = make_double2(0.0, 0.0);
  for (int b = threadIdx.x / K; b < nblocks; b += kThreads / K) acc = dadd(acc, __ldcg(partial + (int64_t)b * K + my_rhs));
  block_reduce_rhs<K>(acc, smem, smem + (kThreads / 32) * K);
  const double2 out = smem[(kThreads / 32) * K + rhs];
  __syncthreads();
  return out;
}

// q = At p (k = 1, G lanes per row) in the matrix precision CM, gathering
// the CM-typed copy pm of p; partial mu = p^T q with p in FP64; last block:
// alpha = rho / mu.
template <typename CM, int G>
__global__ void __launch_bounds__(kThreads) k_cg_spmv1(const int64_t* __restrict__ rowptr,
                                                       const int32_t* __restrict__ col, const CM* __restrict__ val,
                                                       int64_t n, const CM* __restrict__ pm,
                                                       const double2* __restrict__ p64, CM* __restrict__ q,
                                                       double2* partial, CgState* st, CgCtl* ctl) {
  if (!ctl->any_active) return;
  __shared__ double2 smem[2 * (kThreads / 32) * kMaxK];
  const int lane = threadIdx.x % G;
  const int64_t groups = ((int64_t)gridDim.x * blockDim.x) / G;
  const int64_t gid = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / G;
  const int64_t warp_base = gid - (threadIdx.x & 31) / G;
  double2 mu = make_double2(0.0, 0.0);
  for (int64_t rw = warp_base; rw < n; rw += groups) {
    const int64_t r = rw + (gid - warp_base);
    const bool valid = r < n;
    CM acc = czero<CM>();
    if (valid) {
      const int64_t e = rowptr[r + 1];
      for (int64_t k = rowptr[r] + lane; k < e; k += G) acc = cfma(val[k], pm[col[k]], acc);
    }
#pragma unroll
    for (int off = G / 2; off > 0; off >>= 1) acc = cadd(acc, shfl_xor(acc, off));
    if (valid && lane == 0) {
      q[r] = acc;
      mu = dadd(mu, cmul(p64[r], to_d(acc)));
    }
  }
  block_reduce_rhs<1>(mu, smem, partial + blockIdx.x);
  if (arrive_last(&ctl->counter)) {
    const double2 m = sum_partials<1>(partial, gridDim.x, 0, smem);
    if (threadIdx.x == 0) {
      CgState& S = st[0];
      if (S.active) {
        if (m.x == 0.0 && m.y == 0.0) {
          S.breakdown = 1;
          S.active = 0;
          S.alpha = make_double2(0.0, 0.0);
        } else {
          S.alpha = ddiv(S.rho, m);
        }
      } else {
        S.alpha = make_double2(0.0, 0.0);
      }
      ctl->counter = 0;
    }
  }
}

// q = At p for k > 1 RHS (thread per (row, rhs)), partial mu; last block: alpha
template <typename CM, int K>
__global__ void __launch_bounds__(kThreads) k_cg_spmm(const int64_t* __restrict__ rowptr,
                                                      const int32_t* __restrict__ col, const CM* __restrict__ val,
                                                      int64_t n, const CM* __restrict__ pm,
                                                      const double2* __restrict__ p64, CM* __restrict__ q,
                                                      double2* partial, CgState* st, CgCtl* ctl) {
  if (!ctl->any_active) return;
  __shared__ double2 smem[2 * (kThreads / 32) * kMaxK];
  const int rhs = threadIdx.x % K;
  const int64_t rows_per_pass = ((int64_t)gridDim.x * blockDim.x) / K;
  double2 mu = make_double2(0.0, 0.0);
  for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / K; r < n; r += rows_per_pass) {
    CM acc = czero<CM>();
    const int64_t e = rowptr[r + 1];
    for (int64_t k = rowptr[r]; k < e; ++k) acc = cfma(val[k], pm[(int64_t)col[k] * K + rhs], acc);
    q[r * K + rhs] = acc;
    mu = dadd(mu, cmul(p64[r * K + rhs], to_d(acc)));
  }
  block_reduce_rhs<K>(mu, smem, partial + (int64_t)blockIdx.x * K);
  if (arrive_last(&ctl->counter)) {
    const double2 m = sum_partials<K>(partial, gridDim.x, threadIdx.x < K ? threadIdx.x : 0, smem);
    if (threadIdx.x < K) {
      CgState& S = st[threadIdx.x];
      if (S.active) {
        if (m.x == 0.0 && m.y == 0.0) {
          S.breakdown = 1;
          S.active = 0;
          S.alpha = make_double2(0.0, 0.0);
        } else {
          S.alpha = ddiv(S.rho, m);
        }
      } else {
        S.alpha = make_double2(0.0, 0.0);
      }
    }
    if (threadIdx.x == 0) ctl->counter = 0;
  }
}

// y += alpha p ; r -= alpha q (FP64) ; partials rho = r^T r, w = sum |r|^2 |D|.
// Last block: beta, residual estimate, activity; the cycle stops for every
// RHS when one needs a reliable update (estimate dropped below delta * res0
// or grew above 1e3 * res0), or when all have converged.
template <typename CM, int K>
__global__ void __launch_bounds__(kThreads) k_cg_update(double2* __restrict__ y, double2* __restrict__ r,
                                                        const double2* __restrict__ pv, const CM* __restrict__ q,
                                                        const double* __restrict__ wd, int64_t n, CgState* st,
                                                        double2* prho, double2* pw, CgCtl* ctl, int iter,
                                                        double delta) {
  if (!ctl->any_active) return;
  __shared__ double2 smem[2 * (kThreads / 32) * kMaxK];
  __shared__ double2 al[kMaxK];
  if (threadIdx.x < K) al[threadIdx.x] = st[threadIdx.x].alpha;
  __syncthreads();
  const int rhs = threadIdx.x % K;
  const double2 a = al[rhs];
  const int64_t total = n * K;
  const int64_t chunk = ((total + gridDim.x - 1) / gridDim.x + K - 1) / K * K;
  const int64_t lo = (int64_t)blockIdx.x * chunk, hi = min(total, lo + chunk);
  double rr = 0, ri = 0, ww = 0;
  for (int64_t e = lo + threadIdx.x; e < hi; e += kThreads) {
    const double2 pe = pv[e], qe = to_d(q[e]);
    double2 ye = y[e], re = r[e];
    ye = cfma(a, pe, ye);
    re.x -= a.x * qe.x - a.y * qe.y;
    re.y -= a.x * qe.y + a.y * qe.x;
    y[e] = ye;
    r[e] = re;
    rr += re.x * re.x - re.y * re.y;
    ri += 2 * re.x * re.y;
    ww += (re.x * re.x + re.y * re.y) * wd[e / K];
  }
  block_reduce_rhs<K>(make_double2(rr, ri), smem, prho + (int64_t)blockIdx.x * K);
  block_reduce_rhs<K>(make_double2(ww, 0.0), smem, pw + (int64_t)blockIdx.x * K);
  if (arrive_last(&ctl->counter)) {
    const int my = threadIdx.x < K ? threadIdx.x : 0;
    const double2 rho = sum_partials<K>(prho, gridDim.x, my, smem);
    const double2 w = sum_partials<K>(pw, gridDim.x, my, smem);
    __shared__ int any, stop;
    if (threadIdx.x == 0) { any = 0; stop = 0; }
    __syncthreads();
    if (threadIdx.x < K) {
      CgState& S = st[threadIdx.x];
      if (S.active) {
        S.beta_iter = iter;
        S.its += 1;
        S.res = sqrt(w.x);
        if (!isfinite(S.res)) ctl->nonfinite = 1;
        if (S.rho.x == 0.0 && S.rho.y == 0.0) {
          S.breakdown = 1;
          S.active = 0;
          S.beta = make_double2(0.0, 0.0);
        } else {
          S.beta = ddiv(rho, S.rho);
        }
        S.rho = rho;
        if (S.res <= S.target || !isfinite(S.res)) S.active = 0;
        else if (S.res <= delta * S.res0 || S.res > 1e3 * S.res0) atomicOr(&stop, 1);
      } else {
        S.beta = make_double2(0.0, 0.0);
      }
      if (S.active) atomicOr(&any, 1);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      ctl->any_active = any && !stop;
      ctl->counter = 0;
    }
  }
}

// p = r + beta p (FP64) and its matrix-precision copy pm, for every RHS whose
// beta was computed in this launch (iteration `iter`).
template <typename CM, int K>
__global__ void __launch_bounds__(kThreads) k_cg_pupdate(double2* __restrict__ pv, CM* __restrict__ pm,
                                                         const double2* __restrict__ r, int64_t n, const CgState* st,
                                                         int iter, int write_pm) {
  __shared__ double2 bt[kMaxK];
  __shared__ int use[kMaxK];
  if (threadIdx.x < K) {
    bt[threadIdx.x] = st[threadIdx.x].beta;
    use[threadIdx.x] = st[threadIdx.x].beta_iter == iter;
  }
  __syncthreads();
  int anyuse = 0;
  for (int i = 0; i < K; ++i) anyuse |= use[i];
  if (!anyuse) return;
  const int64_t total = n * K;
  for (int64_t e = (int64_t)blockIdx.x * kThreads + threadIdx.x; e < total; e += (int64_t)gridDim.x * kThreads)
    if (use[e % K]) {
      const double2 v = cfma(bt[e % K], pv[e], r[e]);
      pv[e] = v;
      if (write_pm) pm[e] = cfrom<CM>(v);
    }
}

// S = D^-1/2 (principal root), wd = |D|, At = S A S in precision CM
__global__ void k_cg_scaling(const int64_t* rowptr, const int32_t* col, const double2* val, int64_t n, double2* S,
                             double* wd, int* status) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    double2 d = make_double2(0.0, 0.0);
    for (int64_t k = rowptr[r]; k < rowptr[r + 1]; ++k)
      if (col[k] == r) d = val[k];
    const double ad = sqrt(dabs2(d));
    if (ad == 0.0) {
      *status = PG_ERR_BREAKDOWN;
      S[r] = make_double2(1.0, 0.0);
      wd[r] = 1.0;
      continue;
    }
    const double sr = sqrt(0.5 * (ad + d.x));
    double si = sqrt(fmax(0.0, 0.5 * (ad - d.x)));
    if (d.y < 0) si = -si;
    S[r] = ddiv(make_double2(1.0, 0.0), make_double2(sr, si));
    wd[r] = ad;
  }
}

template <typename CM>
__global__ void k_cg_scale_matrix(const int64_t* rowptr, const int32_t* col, const double2* val, int64_t n,
                                  const double2* S, CM* out) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    const double2 sr = S[r];
    for (int64_t k = rowptr[r]; k < rowptr[r + 1]; ++k) out[k] = cfrom<CM>(cmul(sr, cmul(val[k], S[col[k]])));
  }
}

// r = S r64, y = 0 ; first cycle also p = r (and pm) ; partial rho
template <typename CM, int K>
__global__ void k_cg_start(const double2* __restrict__ r64, const double2* __restrict__ S, int64_t n, double2* r,
                           double2* y, double2* pv, CM* pm, int set_p, int write_pm, double2* prho) {
  __shared__ double2 smem[(kThreads / 32) * kMaxK];
  const int64_t total = n * K;
  const int64_t chunk = ((total + gridDim.x - 1) / gridDim.x + K - 1) / K * K;
  const int64_t lo = (int64_t)blockIdx.x * chunk, hi = min(total, lo + chunk);
  double2 rho = make_double2(0.0, 0.0);
  for (int64_t e = lo + threadIdx.x; e < hi; e += kThreads) {
    const double2 v = cmul(S[e / K], r64[e]);
    r[e] = v;
    y[e] = make_double2(0.0, 0.0);
    if (set_p) {
      pv[e] = v;
      if (write_pm) pm[e] = cfrom<CM>(v);
    }
    rho = dadd(rho, cmul(v, v));
  }
  block_reduce_rhs<K>(rho, smem, prho + (int64_t)blockIdx.x * K);
}

template <int K>
__global__ void k_cg_cycle_init(const double2* prho, int nblocks, CgState* st, const double* rnorm,
                                const double* target, const int* want, CgCtl* ctl, int first) {
  __shared__ int any;
  if (threadIdx.x == 0) any = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, rhs = threadIdx.x >> 5;
  if (rhs < K) {
    double2 rho = make_double2(0.0, 0.0);
    for (int b = lane; b < nblocks; b += 32) rho = dadd(rho, prho[(int64_t)b * K + rhs]);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) rho = dadd(rho, shfl_xor(rho, off));
    if (lane == 0) {
      CgState& S = st[rhs];
      if (first) {
        S.its = 0;
        S.breakdown = 0;
        S.beta_iter = 0;
      }
      S.rho = rho;
      S.target = target[rhs];
      S.res = rnorm[rhs];
      S.res0 = rnorm[rhs];
      S.active = want[rhs] && rnorm[rhs] > 0.0;
      S.alpha = S.beta = make_double2(0.0, 0.0);
      if (S.active) atomicOr(&any, 1);
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    ctl->any_active = any;
    ctl->nonfinite = 0;
    ctl->counter = 0;
  }
}

// x += S y
template <int K>
__global__ void k_cg_xupdate(const double2* __restrict__ y, const double2* __restrict__ S, int64_t n, double2* x) {
  const int64_t total = n * K;
  for (int64_t e = (int64_t)blockIdx.x * kThreads + threadIdx.x; e < total; e += (int64_t)gridDim.x * kThreads)
    x[e] = dadd(x[e], cmul(S[e / K], y[e]));
}

struct ToCM64 {
  __device__ double2 operator()(double2 v) const { return v; }
};
struct ToCM32 {
  __device__ float2 operator()(double2 v) const { return make_float2((float)v.x, (float)v.y); }
};
struct IdD2 {
  __device__ double2 operator()(double2 v) const { return v; }
};

// block-Jacobi setup shared by the COCG drivers: S (diagonal) := 1, the
// entity factors into Sblk, |D| into wd, At = S A S^T in the solver's precision
template <typename CM, typename Conv>
int bj_setup(const Plan& P, const int64_t* rowptr, const int32_t* col, const double2* A, double2* S, double* wd,
             double2* Sblk, CM* At, Conv conv, int* dstatus, cudaStream_t s) {
  k_fill_one<<<pg_blocks(P.n, 256), 256, 0, s>>>(S, P.n);
  k_bj_check<<<pg_blocks(P.n, 256), 256, 0, s>>>(rowptr, col, P.bj, dstatus);
  int h = 0;
  PG_CUDA_TRY(cudaMemcpyAsync(&h, dstatus, sizeof(int), cudaMemcpyDeviceToHost, s));
  PG_CUDA_TRY(cudaStreamSynchronize(s));
  if (h) {
    pg_set_error("pg_cocg: block-Jacobi needs the entity-block pattern (rows of one entity share their columns)");
    return PG_ERR_ARG;
  }
  k_bj_factor<<<pg_blocks(P.n, 128), 128, 0, s>>>(rowptr, col, A, P.bj, Sblk, wd, dstatus);
  k_bj_scale_matrix<<<pg_blocks(P.n, 128), 128, 0, s>>>(rowptr, col, A, P.bj, Sblk, At, conv);
  PG_LAUNCH_CHECK();
  return PG_OK;
}

size_t cg_layout(const Plan& P, size_t* off /* 20 */) {
  size_t o = 0;
  auto put = [&](int idx, size_t bytes) { off[idx] = o; o += pg_align256(bytes); };
  put(0, P.nnz * P.csize);                      // At (matrix precision)
  put(1, sizeof(double2) * P.n);                // S
  put(2, sizeof(double) * P.n);                 // |D|
  put(3, P.csize * P.n * P.k);                  // p in matrix precision (gathered by the SpMV)
  put(4, sizeof(double2) * P.n * P.k);          // p
  put(5, P.csize * P.n * P.k);                  // q (matrix precision)
  put(6, sizeof(double2) * P.n * P.k);          // r
  put(7, sizeof(double2) * P.n * P.k);          // y
  put(8, sizeof(double2) * P.n * P.k);          // r64
  put(9, sizeof(double2) * (size_t)P.nb * P.k * 3);  // partials (mu/rho, w)
  put(10, sizeof(CgState) * P.k);
  put(11, sizeof(CgCtl));
  put(12, sizeof(double) * P.k * 3);            // rnorm, target, (spare)
  put(13, sizeof(int) * (P.k + 1));             // want, status
  put(18, P.bj.p ? sizeof(double2) * P.bj.s_size() : 0);     // block-Jacobi factors
  put(19, P.bj.p ? sizeof(double2) * P.n * P.k : 0);         // S r64
  return o;
}

template <typename CM>
void launch_cg_spmv(const Plan& P, const int64_t* rowptr, const int32_t* col, const CM* val, const CM* pm,
                    const double2* p64, CM* q, double2* partial, CgState* st, CgCtl* ctl, int64_t npr, int grid,
                    cudaStream_t s) {
  switch (P.k) {
    case 1:
      switch (LanesPerRow<CM>::pick(npr)) {
        case 32: k_cg_spmv1<CM, 32><<<grid, kThreads, 0, s>>>(rowptr, col, val, P.n, pm, p64, q, partial, st, ctl); break;
        case 16: k_cg_spmv1<CM, 16><<<grid, kThreads, 0, s>>>(rowptr, col, val, P.n, pm, p64, q, partial, st, ctl); break;
        case 8: k_cg_spmv1<CM, 8><<<grid, kThreads, 0, s>>>(rowptr, col, val, P.n, pm, p64, q, partial, st, ctl); break;
        default: k_cg_spmv1<CM, 4><<<grid, kThreads, 0, s>>>(rowptr, col, val, P.n, pm, p64, q, partial, st, ctl); break;
      }
      break;
    case 2: k_cg_spmm<CM, 2><<<grid, kThreads, 0, s>>>(rowptr, col, val, P.n, pm, p64, q, partial, st, ctl); break;
    case 4: k_cg_spmm<CM, 4><<<grid, kThreads, 0, s>>>(rowptr, col, val, P.n, pm, p64, q, partial, st, ctl); break;
    case 8: k_cg_spmm<CM, 8><<<grid, kThreads, 0, s>>>(rowptr, col, val, P.n, pm, p64, q, partial, st, ctl); break;
    case 16: k_cg_spmm<CM, 16><<<grid, kThreads, 0, s>>>(rowptr, col, val, P.n, pm, p64, q, partial, st, ctl); break;
    case 32: k_cg_spmm<CM, 32><<<grid, kThreads, 0, s>>>(rowptr, col, val, P.n, pm, p64, q, partial, st, ctl); break;
  }
}

template <typename CM>
int run_cocg(const Plan& P, const int64_t* rowptr, const int32_t* col, const double2* A, const double2* b, double2* x,
             const pg_cocg_opts* o, pg_gmres_result* res, double* relres_out, char* ws, cudaStream_t s) {
  size_t off[20];
  cg_layout(P, off);
  const bool bj = P.bj.p > 0;
  double2* Sblk = reinterpret_cast<double2*>(ws + off[18]);
  double2* r64b = reinterpret_cast<double2*>(ws + off[19]);
  CM* At = reinterpret_cast<CM*>(ws + off[0]);
  double2* S = reinterpret_cast<double2*>(ws + off[1]);
  double* wd = reinterpret_cast<double*>(ws + off[2]);
  const bool same = sizeof(CM) == sizeof(double2);   // fp64: p doubles as its own matrix-precision copy
  double2* pv = reinterpret_cast<double2*>(ws + off[4]);
  CM* pm = same ? reinterpret_cast<CM*>(pv) : reinterpret_cast<CM*>(ws + off[3]);
  CM* q = reinterpret_cast<CM*>(ws + off[5]);
  double2* r = reinterpret_cast<double2*>(ws + off[6]);
  double2* y = reinterpret_cast<double2*>(ws + off[7]);
  double2* r64 = reinterpret_cast<double2*>(ws + off[8]);
  double2* part = reinterpret_cast<double2*>(ws + off[9]);
  double2* part2 = part + (size_t)P.nb * P.k;
  CgState* st = reinterpret_cast<CgState*>(ws + off[10]);
  CgCtl* ctl = reinterpret_cast<CgCtl*>(ws + off[11]);
  double* rnorm = reinterpret_cast<double*>(ws + off[12]);
  double* target = rnorm + P.k;
  int* want = reinterpret_cast<int*>(ws + off[13]);
  int* dstatus = want + P.k;
  const int write_pm = same ? 0 : 1;
  const int k = P.k, nb = P.nb;
  // vector-update grid: at least ~4 elements per thread, so the per-block
  // reduction does not dominate on small systems (its last block sums
  // gridDim.x partials)
  const int nbu = (int)std::min<int64_t>(nb, std::max<int64_t>(152 * 2, (P.n * P.k + 4 * kThreads - 1) / (4 * kThreads)));
  const int64_t npr = P.nnz / (P.n > 0 ? P.n : 1);
  const int spmv_grid = 152 * 16;
  if (spmv_grid > nb) return PG_ERR_ARG;  // partial buffers are sized by nb

  PG_CUDA_TRY(cudaMemsetAsync(dstatus, 0, sizeof(int), s));
  if (bj) {
    int st0;
    if (sizeof(CM) == sizeof(double2))
      st0 = bj_setup(P, rowptr, col, A, S, wd, Sblk, reinterpret_cast<double2*>(At), ToCM64(), dstatus, s);
    else
      st0 = bj_setup(P, rowptr, col, A, S, wd, Sblk, reinterpret_cast<float2*>(At), ToCM32(), dstatus, s);
    if (st0) return st0;
  } else {
    k_cg_scaling<<<pg_blocks(P.n, 256), 256, 0, s>>>(rowptr, col, A, P.n, S, wd, dstatus);
    k_cg_scale_matrix<CM><<<pg_blocks(P.n, 256), 256, 0, s>>>(rowptr, col, A, P.n, S, At);
  }
  PG_LAUNCH_CHECK();
  std::vector<double> bnorm(k), rn(k), tgt(k);
  std::vector<int> wnt(k);
  PG_KSWITCH(k, (k_norm2<K><<<nb, kThreads, 0, s>>>(b, P.n, part), k_norm_final<K><<<1, 32 * K, 0, s>>>(part, nb, rnorm)));
  PG_LAUNCH_CHECK();
  PG_CUDA_TRY(cudaMemcpyAsync(bnorm.data(), rnorm, sizeof(double) * k, cudaMemcpyDeviceToHost, s));
  int hstatus = 0;
  PG_CUDA_TRY(cudaMemcpyAsync(&hstatus, dstatus, sizeof(int), cudaMemcpyDeviceToHost, s));
  PG_CUDA_TRY(cudaStreamSynchronize(s));
  if (hstatus) {
    pg_set_error("pg_cocg: zero diagonal entry (Jacobi scaling undefined)");
    return PG_ERR_BREAKDOWN;
  }
  const char* mon_env = getenv("PG_KSP_MONITOR");
  const bool monitor = mon_env && mon_env[0] && mon_env[0] != '0';
  int64_t its = 0, checks = 0;
  int status = PG_OK;
  const int64_t max_it = o->max_it > 0 ? o->max_it : 100000;
  int chunk = o->check_every > 0 ? o->check_every : 50;
  bool first = true;
  int64_t launch_iter = 1;
  for (;;) {
    launch_spmv<double2>(P, rowptr, col, A, x, r64, b, nullptr, npr, s);
    PG_KSWITCH(k, (k_norm2<K><<<nb, kThreads, 0, s>>>(r64, P.n, part),
                   k_norm_final<K><<<1, 32 * K, 0, s>>>(part, nb, rnorm)));
    PG_LAUNCH_CHECK();
    PG_CUDA_TRY(cudaMemcpyAsync(rn.data(), rnorm, sizeof(double) * k, cudaMemcpyDeviceToHost, s));
    CgCtl hctl;
    PG_CUDA_TRY(cudaMemcpyAsync(&hctl, ctl, sizeof(CgCtl), cudaMemcpyDeviceToHost, s));
    PG_CUDA_TRY(cudaStreamSynchronize(s));
    if (!first && hctl.nonfinite) {
      pg_set_error("pg_cocg: non-finite residual");
      status = PG_ERR_NONFINITE;
      break;
    }
    bool all = true;
    for (int i = 0; i < k; ++i) {
      if (monitor)
        fprintf(stderr, "pg_cocg: check %lld its %lld rhs %d true ||r||/||b|| = %.6e\n", (long long)checks,
                (long long)its, i, bnorm[i] > 0 ? rn[i] / bnorm[i] : 0.0);
      if (!isfinite(rn[i])) {
        pg_set_error("pg_cocg: non-finite residual");
        status = PG_ERR_NONFINITE;
      }
      const double tb = o->rtol * bnorm[i];
      const bool ok = rn[i] <= tb || bnorm[i] == 0.0;
      wnt[i] = ok ? 0 : 1;
      tgt[i] = 0.5 * tb;
      if (!ok) all = false;
    }
    if (status || all) break;
    if (its >= max_it) {
      status = PG_ERR_NOT_CONVERGED;
      break;
    }
    PG_CUDA_TRY(cudaMemcpyAsync(target, tgt.data(), sizeof(double) * k, cudaMemcpyHostToDevice, s));
    PG_CUDA_TRY(cudaMemcpyAsync(want, wnt.data(), sizeof(int) * k, cudaMemcpyHostToDevice, s));
    if (bj) PG_KSWITCH(k, (k_bj_apply<K><<<pg_blocks(P.n * K, 256), 256, 0, s>>>(Sblk, P.bj, r64, r64b)));
    PG_KSWITCH(k, (k_cg_start<CM, K><<<nb, kThreads, 0, s>>>(bj ? r64b : r64, S, P.n, r, y, pv, pm, first ? 1 : 0,
                                                             write_pm, part),
                   k_cg_cycle_init<K><<<1, 32 * K, 0, s>>>(part, nb, st, rnorm, target, want, ctl, first ? 1 : 0)));
    first = false;
    const int steps = (int)((max_it - its) < chunk ? (max_it - its) : chunk);
    const double delta = P.prec ? 0.1 : 0.0;
    for (int it = 0; it < steps; ++it) {
      const int iter = (int)(launch_iter + it);
      launch_cg_spmv<CM>(P, rowptr, col, At, pm, pv, q, part, st, ctl, npr, spmv_grid, s);
      PG_KSWITCH(k, (k_cg_update<CM, K><<<nbu, kThreads, 0, s>>>(y, r, pv, q, wd, P.n, st, part, part2, ctl, iter, delta),
                     k_cg_pupdate<CM, K><<<pg_blocks(P.n * K, kThreads), kThreads, 0, s>>>(pv, pm, r, P.n, st, iter,
                                                                                          write_pm)));
    }
    PG_LAUNCH_CHECK();
    launch_iter += steps;
    if (bj) {
      PG_KSWITCH(k, (k_bj_apply_t_add<K><<<pg_blocks(P.n * K, 256), 256, 0, s>>>(Sblk, P.bj, y, x, IdD2())));
    } else {
      PG_KSWITCH(k, (k_cg_xupdate<K><<<pg_blocks(P.n * K, kThreads), kThreads, 0, s>>>(y, S, P.n, x)));
    }
    std::vector<int> hits(k);
    std::vector<int> hbrk(k);
    for (int i = 0; i < k; ++i) {
      PG_CUDA_TRY(cudaMemcpyAsync(&hits[i], &st[i].its, sizeof(int), cudaMemcpyDeviceToHost, s));
      PG_CUDA_TRY(cudaMemcpyAsync(&hbrk[i], &st[i].breakdown, sizeof(int), cudaMemcpyDeviceToHost, s));
    }
    PG_CUDA_TRY(cudaStreamSynchronize(s));
    int used = 0;
    for (int i = 0; i < k; ++i) used = hits[i] > used ? hits[i] : used;
    const int64_t cycle_its = used - its;
    its = used;
    ++checks;
    bool brk = false;
    for (int i = 0; i < k; ++i) brk = brk || hbrk[i];
    if (brk) {
      pg_set_error("pg_cocg: breakdown (p^T A p = 0 or r^T r = 0)");
      status = PG_ERR_BREAKDOWN;
      // still report the residual of the last iterate below
      launch_spmv<double2>(P, rowptr, col, A, x, r64, b, nullptr, npr, s);
      PG_KSWITCH(k, (k_norm2<K><<<nb, kThreads, 0, s>>>(r64, P.n, part),
                     k_norm_final<K><<<1, 32 * K, 0, s>>>(part, nb, rnorm)));
      PG_CUDA_TRY(cudaMemcpyAsync(rn.data(), rnorm, sizeof(double) * k, cudaMemcpyDeviceToHost, s));
      PG_CUDA_TRY(cudaStreamSynchronize(s));
      break;
    }
    if (P.prec) {
      // cycles end on-device at the reliable-update trigger; size the next
      // launch batch from this cycle's length to limit no-op launches
      int64_t c2 = cycle_its + cycle_its / 4 + 8;
      chunk = (int)(c2 < 16 ? 16 : (c2 > 2000 ? 2000 : c2));
    } else if (chunk < 400) {
      chunk *= 2;
    }
  }
  double worst = 0.0;
  for (int i = 0; i < k; ++i) {
    const double rr = bnorm[i] > 0 ? rn[i] / bnorm[i] : 0.0;
    if (relres_out) relres_out[i] = rr;
    worst = rr > worst ? rr : worst;
  }
  if (res) {
    res->iterations = its;
    res->restarts = checks;
    res->relres = worst;
    res->status = status;
  }
  if (status == PG_ERR_NOT_CONVERGED) pg_set_error("pg_cocg: max_it reached before rtol");
  return status;
}


// ============================================================================
// df64: FP64-accurate COCG on the FP32 pipes.  Values are double-float pairs
// (hi + lo, ~48-bit mantissa); a complex number is a float4
// (re.hi, re.lo, im.hi, im.lo), 16 bytes like complex128.  Products are made
// error-free with FMA, sums are compensated (two-sum), so every operation
// costs ~11 FP32 instructions instead of one FP64 instruction - and GB300's
// FP32 pipe is ~57x faster than its FP64 pipe, which makes the SpMV HBM-bound
// instead of FP64-bound.  FP64 is kept for the scaling, the true residual, the
// reliable updates and x.
// ============================================================================

__device__ __forceinline__ float4 df_norm(float4 v) {
  const float s = __fadd_rn(v.x, v.y);
  const float e1 = __fsub_rn(v.y, __fsub_rn(s, v.x));
  const float t = __fadd_rn(v.z, v.w);
  const float e2 = __fsub_rn(v.w, __fsub_rn(t, v.z));
  return make_float4(s, e1, t, e2);
}

// c += a * b (complex double-float)
__device__ __forceinline__ void cdf_mac(float4& c, float4 a, float4 b) {
  df_mac(c.x, c.y, a.x, a.y, b.x, b.y);
  df_mac(c.x, c.y, -a.z, -a.w, b.z, b.w);
  df_mac(c.z, c.w, a.x, a.y, b.z, b.w);
  df_mac(c.z, c.w, a.z, a.w, b.x, b.y);
}

__device__ __forceinline__ float4 cdf_from(double2 v) {
  const float rh = __double2float_rn(v.x), ih = __double2float_rn(v.y);
  return make_float4(rh, __double2float_rn(v.x - (double)rh), ih, __double2float_rn(v.y - (double)ih));
}
__device__ __forceinline__ double2 cdf_to(float4 v) {
  return make_double2((double)v.x + (double)v.y, (double)v.z + (double)v.w);
}
__device__ __forceinline__ float4 shfl_xor4(float4 v, int m) {
  return make_float4(__shfl_xor_sync(0xffffffffu, v.x, m), __shfl_xor_sync(0xffffffffu, v.y, m),
                     __shfl_xor_sync(0xffffffffu, v.z, m), __shfl_xor_sync(0xffffffffu, v.w, m));
}
__device__ __forceinline__ void cdf_add(float4& a, float4 b) {
  df_add(a.x, a.y, b.x, b.y);
  df_add(a.z, a.w, b.z, b.w);
}

// Block reductions of double-float values: the warp and block stages add in
// double-float on the FP32 pipes and only the block total is converted to
// double (GB300's FP64 pipe runs ~2 operations per clock per SM, so a
// per-thread conversion plus a double-precision shuffle tree cost more than
// the vector update they reduce).  Lanes with equal lane % K combine.
template <int K>
__device__ void block_reduce_df(float4 v, float4* smf, double2* out) {
#pragma unroll
  for (int off = 16; off >= K; off >>= 1) cdf_add(v, shfl_xor4(v, off));
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane < K) smf[warp * K + lane] = v;
  __syncthreads();
  if (threadIdx.x < K) {
    float4 t = smf[threadIdx.x];
    for (int w = 1; w < kThreads / 32; ++w) cdf_add(t, smf[w * K + threadIdx.x]);
    out[threadIdx.x] = cdf_to(t);
  }
  __syncthreads();
}

template <int K>
__device__ void block_reduce_f(float v, float* smf, double2* out) {
#pragma unroll
  for (int off = 16; off >= K; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane < K) smf[warp * K + lane] = v;
  __syncthreads();
  if (threadIdx.x < K) {
    float t = smf[threadIdx.x];
    for (int w = 1; w < kThreads / 32; ++w) t += smf[w * K + threadIdx.x];
    out[threadIdx.x] = make_double2((double)t, 0.0);
  }
  __syncthreads();
}

// alpha / beta finalisation shared by the df kernels (last block only)
template <int K>
__device__ void cg_alpha_final(const double2* partial, int nblocks, CgState* st, CgCtl* ctl, double2* smem) {
  const double2 m = sum_partials<K>(partial, nblocks, threadIdx.x < K ? threadIdx.x : 0, smem);
  if (threadIdx.x < K) {
    CgState& S = st[threadIdx.x];
    if (S.active) {
      if (m.x == 0.0 && m.y == 0.0) {
        S.breakdown = 1;
        S.active = 0;
        S.alpha = make_double2(0.0, 0.0);
      } else {
        S.alpha = ddiv(S.rho, m);
      }
    } else {
      S.alpha = make_double2(0.0, 0.0);
    }
  }
  if (threadIdx.x == 0) ctl->counter = 0;
}

template <int K>
__device__ void cg_beta_final(const double2* prho, const double2* pw, int nblocks, CgState* st, CgCtl* ctl, int iter,
                              double delta, double2* smem) {
  const int my = threadIdx.x < K ? threadIdx.x : 0;
  const double2 rho = sum_partials<K>(prho, nblocks, my, smem);
  const double2 w = sum_partials<K>(pw, nblocks, my, smem);
  __shared__ int any, stop;
  if (threadIdx.x == 0) { any = 0; stop = 0; }
  __syncthreads();
  if (threadIdx.x < K) {
    CgState& S = st[threadIdx.x];
    if (S.active) {
      S.beta_iter = 1;   // fresh beta: the next p update applies it once
      S.its += 1;
      S.res = sqrt(w.x);
      if (!isfinite(S.res)) ctl->nonfinite = 1;
      if (S.rho.x == 0.0 && S.rho.y == 0.0) {
        S.breakdown = 1;
        S.active = 0;
        S.beta = make_double2(0.0, 0.0);
      } else {
        S.beta = ddiv(rho, S.rho);
      }
      S.rho = rho;
      if (S.res <= S.target || !isfinite(S.res)) S.active = 0;
      else if (S.res <= delta * S.res0 || S.res > 1e3 * S.res0) atomicOr(&stop, 1);
    } else {
      S.beta = make_double2(0.0, 0.0);
      S.beta_iter = 0;
    }
    if (S.active) atomicOr(&any, 1);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    ctl->any_active = any && !stop;
    ctl->pending = 1;
    ctl->counter = 0;
  }
}

// q = At p (double-float), partial mu = p^T q; last block: alpha
template <int G, int U = 1>
__global__ void __launch_bounds__(kThreads) k_df_spmv1(const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                                                       const float4* __restrict__ val, int64_t n,
                                                       const float4* __restrict__ pv, float4* __restrict__ q,
                                                       double2* partial, CgState* st, CgCtl* ctl) {
  if (blockIdx.x == 0 && threadIdx.x == 0) ctl->pending = 0;   // the previous p update has run
  if (!ctl->any_active) return;
  __shared__ double2 smem[2 * (kThreads / 32) * kMaxK];
  const int lane = threadIdx.x % G;
  const int64_t groups = ((int64_t)gridDim.x * blockDim.x) / G;
  const int64_t gid = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / G;
  const int64_t warp_base = gid - (threadIdx.x & 31) / G;
  float4 mu = make_float4(0.f, 0.f, 0.f, 0.f);
  for (int64_t rw = warp_base; rw < n; rw += groups) {
    const int64_t r = rw + (gid - warp_base);
    const bool valid = r < n;
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    if (valid) {
      const int64_t e = rowptr[r + 1];
      int64_t k = rowptr[r] + lane;
      if (U == 2) {
        // two independent accumulators: two gathers in flight per lane
        float4 acc1 = make_float4(0.f, 0.f, 0.f, 0.f);
        for (; k + G < e; k += 2 * G) {
          const int32_t c0 = col[k], c1 = col[k + G];
          const float4 v0 = val[k], v1 = val[k + G];
          cdf_mac(acc, v0, pv[c0]);
          cdf_mac(acc1, v1, pv[c1]);
        }
        if (k < e) cdf_mac(acc, val[k], pv[col[k]]);
        cdf_add(acc, acc1);
      } else {
        for (; k < e; k += G) cdf_mac(acc, val[k], pv[col[k]]);
      }
    }
#pragma unroll
    for (int off = G / 2; off > 0; off >>= 1) cdf_add(acc, shfl_xor4(acc, off));
    if (valid && lane == 0) {
      acc = df_norm(acc);
      q[r] = acc;
      cdf_mac(mu, pv[r], acc);
    }
  }
  __shared__ float4 smf[(kThreads / 32) * kMaxK];
  block_reduce_df<1>(mu, smf, partial + blockIdx.x);
  if (arrive_last(&ctl->counter)) cg_alpha_final<1>(partial, gridDim.x, st, ctl, smem);
}

template <int K, int U = 1>
__global__ void __launch_bounds__(kThreads) k_df_spmm(const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                                                      const float4* __restrict__ val, int64_t n,
                                                      const float4* __restrict__ pv, float4* __restrict__ q,
                                                      double2* partial, CgState* st, CgCtl* ctl) {
  if (blockIdx.x == 0 && threadIdx.x == 0) ctl->pending = 0;   // the previous p update has run
  if (!ctl->any_active) return;
  __shared__ double2 smem[2 * (kThreads / 32) * kMaxK];
  const int rhs = threadIdx.x % K;
  const int64_t rows_per_pass = ((int64_t)gridDim.x * blockDim.x) / K;
  float4 mu = make_float4(0.f, 0.f, 0.f, 0.f);
  for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / K; r < n; r += rows_per_pass) {
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    const int64_t e = rowptr[r + 1];
    int64_t k = rowptr[r];
    if (U == 2) {
      float4 acc1 = make_float4(0.f, 0.f, 0.f, 0.f);
      for (; k + 1 < e; k += 2) {
        const int32_t c0 = col[k], c1 = col[k + 1];
        const float4 v0 = val[k], v1 = val[k + 1];
        cdf_mac(acc, v0, pv[(int64_t)c0 * K + rhs]);
        cdf_mac(acc1, v1, pv[(int64_t)c1 * K + rhs]);
      }
      if (k < e) cdf_mac(acc, val[k], pv[(int64_t)col[k] * K + rhs]);
      cdf_add(acc, acc1);
    } else {
      for (; k < e; ++k) cdf_mac(acc, val[k], pv[(int64_t)col[k] * K + rhs]);
    }
    acc = df_norm(acc);
    q[r * K + rhs] = acc;
    cdf_mac(mu, pv[r * K + rhs], acc);
  }
  __shared__ float4 smf[(kThreads / 32) * kMaxK];
  block_reduce_df<K>(mu, smf, partial + (int64_t)blockIdx.x * K);
  if (arrive_last(&ctl->counter)) cg_alpha_final<K>(partial, gridDim.x, st, ctl, smem);
}

// y += alpha p ; r -= alpha q ; partials rho = r^T r (df), w = sum |r|^2 |D| (FP32 estimate)
template <int K, bool PC = false>
__global__ void __launch_bounds__(kThreads) k_df_update(float4* __restrict__ y, float4* __restrict__ r,
                                                        const float4* __restrict__ pv, const float4* __restrict__ q,
                                                        const float* __restrict__ wd, int64_t n, CgState* st,
                                                        double2* prho, double2* pw, CgCtl* ctl, int iter,
                                                        double delta) {
  if (!ctl->any_active) return;
  __shared__ double2 smem[2 * (kThreads / 32) * kMaxK];
  __shared__ float4 al[kMaxK];
  if (threadIdx.x < K) {
    const double2 a = st[threadIdx.x].alpha;
    al[threadIdx.x] = cdf_from(a);
  }
  __syncthreads();
  const int rhs = threadIdx.x % K;
  const float4 a = al[rhs];
  const float4 na = make_float4(-a.x, -a.y, -a.z, -a.w);
  const int64_t total = n * K;
  const int64_t chunk = ((total + gridDim.x - 1) / gridDim.x + K - 1) / K * K;
  const int64_t lo = (int64_t)blockIdx.x * chunk, hi = min(total, lo + chunk);
  float4 rho = make_float4(0.f, 0.f, 0.f, 0.f);
  float ww = 0.f;
  for (int64_t e = lo + threadIdx.x; e < hi; e += kThreads) {
    float4 ye = y[e], re = r[e];
    cdf_mac(ye, a, pv[e]);
    cdf_mac(re, na, q[e]);
    ye = df_norm(ye);
    re = df_norm(re);
    y[e] = ye;
    r[e] = re;
    cdf_mac(rho, re, re);
    ww += (re.x * re.x + re.z * re.z) * wd[PC ? e : e / K];
  }
  __shared__ float4 smf[(kThreads / 32) * kMaxK];
  block_reduce_df<K>(rho, smf, prho + (int64_t)blockIdx.x * K);
  block_reduce_f<K>(ww, reinterpret_cast<float*>(smf), pw + (int64_t)blockIdx.x * K);
  if (arrive_last(&ctl->counter)) cg_beta_final<K>(prho, pw, gridDim.x, st, ctl, iter, delta, smem);
}

template <int K, bool PC = false>
__global__ void __launch_bounds__(kThreads) k_df_pupdate(float4* __restrict__ pv, const float4* __restrict__ r, int64_t n,
                                                         const CgState* st, const CgCtl* ctl,
                                                         float4* __restrict__ ps = nullptr,
                                                         const float4* __restrict__ Sdf = nullptr) {
  __shared__ float4 bt[kMaxK];
  __shared__ int use[kMaxK];
  if (!ctl->pending) return;
  if (threadIdx.x < K) {
    bt[threadIdx.x] = cdf_from(st[threadIdx.x].beta);
    use[threadIdx.x] = st[threadIdx.x].beta_iter == 1;
  }
  __syncthreads();
  int anyuse = 0;
  for (int i = 0; i < K; ++i) anyuse |= use[i];
  if (!anyuse) return;
  const int64_t total = n * K;
  for (int64_t e = (int64_t)blockIdx.x * kThreads + threadIdx.x; e < total; e += (int64_t)gridDim.x * kThreads)
    if (use[e % K]) {
      float4 v = r[e];
      cdf_mac(v, bt[e % K], pv[e]);
      v = df_norm(v);
      pv[e] = v;
      if (PC) {
        float4 w = make_float4(0.f, 0.f, 0.f, 0.f);
        cdf_mac(w, Sdf[e], v);
        ps[e] = df_norm(w);
      }
    }
}

__global__ void k_df_scale_matrix(const int64_t* rowptr, const int32_t* col, const double2* val, int64_t n,
                                  const double2* S, float4* out, float* wdf, const double* wd) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    const double2 sr = S[r];
    for (int64_t k = rowptr[r]; k < rowptr[r + 1]; ++k) out[k] = cdf_from(cmul(sr, cmul(val[k], S[col[k]])));
    wdf[r] = (float)wd[r];
  }
}

template <int K, bool PC = false>
__global__ void k_df_start(const double2* __restrict__ r64, const double2* __restrict__ S, int64_t n, float4* r,
                           float4* y, float4* pv, int set_p, double2* prho, float4* ps = nullptr) {
  __shared__ double2 smem[(kThreads / 32) * kMaxK];
  const int64_t total = n * K;
  const int64_t chunk = ((total + gridDim.x - 1) / gridDim.x + K - 1) / K * K;
  const int64_t lo = (int64_t)blockIdx.x * chunk, hi = min(total, lo + chunk);
  double2 rho = make_double2(0.0, 0.0);
  for (int64_t e = lo + threadIdx.x; e < hi; e += kThreads) {
    const double2 sc = S[PC ? e : e / K];
    const double2 v = cmul(sc, r64[e]);
    const float4 vf = cdf_from(v);
    r[e] = vf;
    y[e] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (set_p) pv[e] = vf;
    if (PC && set_p) ps[e] = cdf_from(cmul(sc, v));
    rho = dadd(rho, cmul(v, v));
  }
  block_reduce_rhs<K>(rho, smem, prho + (int64_t)blockIdx.x * K);
}

// v[:, c] *= f[c] (FP64 vectors)
template <int K>
__global__ void k_scale_cols_d2(double2* v, int64_t n, const double* f) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n * K; e += (int64_t)gridDim.x * blockDim.x)
    v[e] = dscale(f[e % K], v[e]);
}

// v[:, c] *= f[c] (double-float vectors; f split into hi + lo)
template <int K>
__global__ void k_scale_cols_df(float4* v, int64_t n, const double* f) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n * K; e += (int64_t)gridDim.x * blockDim.x) {
    const double fc = f[e % K];
    const float fh = __double2float_rn(fc);
    const float fl = __double2float_rn(fc - (double)fh);
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    cdf_mac(acc, v[e], make_float4(fh, fl, 0.f, 0.f));
    v[e] = df_norm(acc);
  }
}

template <int K, bool PC = false>
__global__ void k_df_xupdate(const float4* __restrict__ y, const double2* __restrict__ S, int64_t n, double2* x) {
  const int64_t total = n * K;
  for (int64_t e = (int64_t)blockIdx.x * kThreads + threadIdx.x; e < total; e += (int64_t)gridDim.x * kThreads)
    x[e] = dadd(x[e], cmul(S[PC ? e : e / K], cdf_to(y[e])));
}

// ---- several frequencies in one solve --------------------------------------
// Column j solves (Re A0 + i s_j Im A0) x_j = b_j: A0 assembled at omega_0
// (K - i omega_0 mu M, PEC rows unit), s_j = omega_j / omega_0.  The matrix is
// read once per iteration for all columns; each column has its own Jacobi
// scaling S_j = diag(A_j)^(-1/2), applied to the direction (ps = S_j o p, kept
// by the p update) and to the product's rows.

// S[r * K + j], |D|[r * K + j] for every column
template <int K>
__global__ void k_mf_scaling(const int64_t* rowptr, const int32_t* col, const double2* val, int64_t n,
                             const double* scale, double2* S, double* wd, float* wdf, int* status) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    double2 d = make_double2(0.0, 0.0);
    for (int64_t k = rowptr[r]; k < rowptr[r + 1]; ++k)
      if (col[k] == r) d = val[k];
    for (int j = 0; j < K; ++j) {
      const double2 dj = make_double2(d.x, scale[j] * d.y);
      const double m = hypot(dj.x, dj.y);
      if (!(m > 0.0)) {
        *status = 1;
        S[r * K + j] = make_double2(1.0, 0.0);
        wd[r * K + j] = 1.0;
        wdf[r * K + j] = 1.0f;
        continue;
      }
      // principal square root of 1/d
      const double2 inv = make_double2(dj.x / (m * m), -dj.y / (m * m));
      const double mi = 1.0 / m;
      const double re = sqrt(0.5 * (mi + inv.x));
      const double im = inv.y >= 0.0 ? sqrt(fmax(0.5 * (mi - inv.x), 0.0)) : -sqrt(fmax(0.5 * (mi - inv.x), 0.0));
      S[r * K + j] = make_double2(re, im);
      wd[r * K + j] = m;
      wdf[r * K + j] = (float)m;
    }
  }
}

__global__ void k_mf_df_matrix(const double2* val, int64_t nnz, float4* out) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nnz; k += (int64_t)gridDim.x * blockDim.x)
    out[k] = cdf_from(val[k]);
}

__global__ void k_mf_sdf(const double2* S, int64_t total, float4* out) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x)
    out[e] = cdf_from(S[e]);
}

// q = S o (A_j ps), A_j = Re A0 + i s_j Im A0, partial mu = p^T q; last block: alpha
template <int K>
__global__ void __launch_bounds__(kThreads) k_mf_spmm(const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                                                      const float4* __restrict__ val, int64_t n,
                                                      const float* __restrict__ scale_hl,
                                                      const float4* __restrict__ Sdf, const float4* __restrict__ pv,
                                                      const float4* __restrict__ ps, float4* __restrict__ q,
                                                      double2* partial, CgState* st, CgCtl* ctl) {
  if (blockIdx.x == 0 && threadIdx.x == 0) ctl->pending = 0;   // the previous p update has run
  if (!ctl->any_active) return;
  __shared__ double2 smem[2 * (kThreads / 32) * kMaxK];
  const int rhs = threadIdx.x % K;
  const float sh = scale_hl[2 * rhs], sl = scale_hl[2 * rhs + 1];
  const int64_t rows_per_pass = ((int64_t)gridDim.x * blockDim.x) / K;
  float4 mu = make_float4(0.f, 0.f, 0.f, 0.f);
  for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / K; r < n; r += rows_per_pass) {
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    const int64_t e = rowptr[r + 1];
    for (int64_t k = rowptr[r]; k < e; ++k) {
      const float4 a = val[k];
      // imaginary part times s_j (double-float product)
      const dfv im = df_mul(dfv{a.z, a.w}, dfv{sh, sl});
      cdf_mac(acc, make_float4(a.x, a.y, im.h, im.l), ps[(int64_t)col[k] * K + rhs]);
    }
    float4 out = make_float4(0.f, 0.f, 0.f, 0.f);
    cdf_mac(out, Sdf[r * K + rhs], df_norm(acc));
    out = df_norm(out);
    q[r * K + rhs] = out;
    cdf_mac(mu, pv[r * K + rhs], out);
  }
  __shared__ float4 smf[(kThreads / 32) * kMaxK];
  block_reduce_df<K>(mu, smf, partial + (int64_t)blockIdx.x * K);
  if (arrive_last(&ctl->counter)) cg_alpha_final<K>(partial, gridDim.x, st, ctl, smem);
}

// r64 = b - A_j x (FP64), one thread per (row, column)
template <int K>
__global__ void k_mf_resid(const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                           const double2* __restrict__ val, int64_t n, const double* __restrict__ scale,
                           const double2* __restrict__ x, const double2* __restrict__ b, double2* __restrict__ r64) {
  const int64_t total = n * K;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = e / K;
    const int j = (int)(e % K);
    const double sj = scale[j];
    double ar = 0.0, ai = 0.0;
    for (int64_t k = rowptr[r]; k < rowptr[r + 1]; ++k) {
      const double2 a = val[k];
      const double2 xv = x[(int64_t)col[k] * K + j];
      const double im = sj * a.y;
      ar = fma(a.x, xv.x, fma(-im, xv.y, ar));
      ai = fma(a.x, xv.y, fma(im, xv.x, ai));
    }
    r64[e] = make_double2(b[e].x - ar, b[e].y - ai);
  }
}

size_t df_layout(const Plan& P, size_t* off /* 20 */, bool mf = false) {
  size_t o = 0;
  auto put = [&](int idx, size_t bytes) { off[idx] = o; o += pg_align256(bytes); };
  const size_t ns = mf ? (size_t)P.n * P.k : (size_t)P.n;   // scaling entries: per column with several frequencies
  put(0, P.nnz * sizeof(float4));               // At (double-float)
  put(1, sizeof(double2) * ns);                 // S
  put(2, sizeof(double) * ns);                  // |D|
  put(3, sizeof(float) * ns);                   // |D| f32
  put(4, sizeof(float4) * P.n * P.k);           // p
  put(5, sizeof(float4) * P.n * P.k);           // q
  put(6, sizeof(float4) * P.n * P.k);           // r
  put(7, sizeof(float4) * P.n * P.k);           // y
  put(8, sizeof(double2) * P.n * P.k);          // r64
  put(9, sizeof(double2) * (size_t)P.nb * P.k * 3);
  put(10, sizeof(CgState) * P.k);
  put(11, sizeof(CgCtl));
  put(12, sizeof(double) * P.k * 6);              // rnorm, target, column scales, inverses, ratios
  put(13, sizeof(int) * (P.k + 1));
  put(14, mf ? sizeof(float4) * P.n * P.k : 0);   // ps = S o p
  put(15, mf ? sizeof(float4) * ns : 0);          // S (double-float)
  put(16, sizeof(double) * P.k);                  // column frequency scales
  put(17, sizeof(float) * 2 * P.k);               // the same as (hi, lo)
  put(18, P.bj.p ? sizeof(double2) * P.bj.s_size() : 0);     // block-Jacobi factors
  put(19, P.bj.p ? sizeof(double2) * P.n * P.k : 0);         // S r64
  return o;
}

// ---- entity-group products --------------------------------------------------
// DOFs are numbered entity by entity with p, p(p-1) and p(p-1)(p-2)/2 DOFs per
// edge, face and volume: all multiples of p, and every entity starts at a
// multiple of p.  So rows [R i, R i + R) with R = p belong to one entity and
// share their column list (entity-pair pattern; checked column by column
// before use).  The group product loads each column index and p value once
// and uses them for R rows: fewer loads per stored entry and R independent
// accumulations per lane.

// 0 if rows of every aligned group of R have the first row's column list
__global__ void k_group_check(const int64_t* rowptr, const int32_t* col, int64_t n, int R, int* status) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    const int64_t f = r - r % R;
    if (f == r) continue;
    const int64_t o = rowptr[r], of = rowptr[f], len = rowptr[r + 1] - o;
    if (len != rowptr[f + 1] - of) {
      *status = 1;
      continue;
    }
    for (int64_t k = 0; k < len; ++k)
      if (col[o + k] != col[of + k]) {
        *status = 1;
        break;
      }
  }
}

// one RHS: G lanes per group of R rows, U column steps per loop pass
template <int R, int G, int U = 1>
__global__ void __launch_bounds__(kThreads) k_df_spmv_grp(const int64_t* __restrict__ rowptr,
                                                          const int32_t* __restrict__ col,
                                                          const float4* __restrict__ val, int64_t n,
                                                          const float4* __restrict__ pv, float4* __restrict__ q,
                                                          double2* partial, CgState* st, CgCtl* ctl) {
  if (blockIdx.x == 0 && threadIdx.x == 0) ctl->pending = 0;   // the previous p update has run
  if (!ctl->any_active) return;
  __shared__ double2 smem[2 * (kThreads / 32) * kMaxK];
  const int lane = threadIdx.x % G;
  const int64_t ngroups = n / R;
  const int64_t groups = ((int64_t)gridDim.x * blockDim.x) / G;
  const int64_t gid = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / G;
  const int64_t warp_base = gid - (threadIdx.x & 31) / G;
  float4 mu = make_float4(0.f, 0.f, 0.f, 0.f);
  for (int64_t gw = warp_base; gw < ngroups; gw += groups) {
    const int64_t gi = gw + (gid - warp_base);
    const bool valid = gi < ngroups;
    float4 acc[R];
#pragma unroll
    for (int i = 0; i < R; ++i) acc[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (valid) {
      const int64_t r0 = gi * R;
      int64_t off[R];
#pragma unroll
      for (int i = 0; i < R; ++i) off[i] = rowptr[r0 + i];
      const int64_t len = rowptr[r0 + 1] - off[0];
      int64_t k = lane;
      if (U == 2) {
        // a second set of accumulators: two column steps in flight per lane
        float4 acc1[R];
#pragma unroll
        for (int i = 0; i < R; ++i) acc1[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        for (; k + G < len; k += 2 * G) {
          const int32_t c0 = col[off[0] + k], c1 = col[off[0] + k + G];
          float4 v0[R], v1[R];
#pragma unroll
          for (int i = 0; i < R; ++i) {
            v0[i] = val[off[i] + k];
            v1[i] = val[off[i] + k + G];
          }
          const float4 x0 = pv[c0], x1 = pv[c1];
#pragma unroll
          for (int i = 0; i < R; ++i) {
            cdf_mac(acc[i], v0[i], x0);
            cdf_mac(acc1[i], v1[i], x1);
          }
        }
#pragma unroll
        for (int i = 0; i < R; ++i) cdf_add(acc[i], acc1[i]);
      }
      for (; k < len; k += G) {
        const float4 x = pv[col[off[0] + k]];
#pragma unroll
        for (int i = 0; i < R; ++i) cdf_mac(acc[i], val[off[i] + k], x);
      }
    }
#pragma unroll
    for (int i = 0; i < R; ++i)
#pragma unroll
      for (int o = G / 2; o > 0; o >>= 1) cdf_add(acc[i], shfl_xor4(acc[i], o));
    if (valid && lane == 0) {
      const int64_t r0 = gi * R;
#pragma unroll
      for (int i = 0; i < R; ++i) {
        const float4 a = df_norm(acc[i]);
        q[r0 + i] = a;
        cdf_mac(mu, pv[r0 + i], a);
      }
    }
  }
  __shared__ float4 smf[(kThreads / 32) * kMaxK];
  block_reduce_df<1>(mu, smf, partial + blockIdx.x);
  if (arrive_last(&ctl->counter)) cg_alpha_final<1>(partial, gridDim.x, st, ctl, smem);
}

// one RHS, G lanes per group of R rows; each lane issues the column, value
// and p loads of B column steps back to back before using them, so a warp
// keeps B times more bytes in flight than one step at a time
template <int R, int G, int B>
__global__ void __launch_bounds__(kThreads) k_df_spmv_grpb(const int64_t* __restrict__ rowptr,
                                                           const int32_t* __restrict__ col,
                                                           const float4* __restrict__ val, int64_t n,
                                                           const float4* __restrict__ pv, float4* __restrict__ q,
                                                           double2* partial, CgState* st, CgCtl* ctl) {
  if (blockIdx.x == 0 && threadIdx.x == 0) ctl->pending = 0;   // the previous p update has run
  if (!ctl->any_active) return;
  __shared__ double2 smem[2 * (kThreads / 32) * kMaxK];
  const int lane = threadIdx.x % G;
  const int64_t ngroups = n / R;
  const int64_t groups = ((int64_t)gridDim.x * blockDim.x) / G;
  const int64_t gid = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / G;
  const int64_t warp_base = gid - (threadIdx.x & 31) / G;
  float4 mu = make_float4(0.f, 0.f, 0.f, 0.f);
  for (int64_t gw = warp_base; gw < ngroups; gw += groups) {
    const int64_t gi = gw + (gid - warp_base);
    const bool valid = gi < ngroups;
    float4 acc[R];
#pragma unroll
    for (int i = 0; i < R; ++i) acc[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (valid) {
      const int64_t r0 = gi * R;
      int64_t off[R];
#pragma unroll
      for (int i = 0; i < R; ++i) off[i] = rowptr[r0 + i];
      const int len = (int)(rowptr[r0 + 1] - off[0]);
      for (int k0 = lane; k0 < len; k0 += G * B) {
        int c[B];
        float4 v[B][R], x[B];
#pragma unroll
        for (int j = 0; j < B; ++j) {
          const int k = k0 + j * G;
          c[j] = k < len ? col[off[0] + k] : 0;
#pragma unroll
          for (int i = 0; i < R; ++i) v[j][i] = k < len ? val[off[i] + k] : make_float4(0.f, 0.f, 0.f, 0.f);
        }
#pragma unroll
        for (int j = 0; j < B; ++j) x[j] = k0 + j * G < len ? pv[c[j]] : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int j = 0; j < B; ++j)
          if (k0 + j * G < len) {
#pragma unroll
            for (int i = 0; i < R; ++i) cdf_mac(acc[i], v[j][i], x[j]);
          }
      }
    }
#pragma unroll
    for (int i = 0; i < R; ++i)
#pragma unroll
      for (int o = G / 2; o > 0; o >>= 1) cdf_add(acc[i], shfl_xor4(acc[i], o));
    if (valid && lane == 0) {
      const int64_t r0 = gi * R;
#pragma unroll
      for (int i = 0; i < R; ++i) {
        const float4 a = df_norm(acc[i]);
        q[r0 + i] = a;
        cdf_mac(mu, pv[r0 + i], a);
      }
    }
  }
  __shared__ float4 smf[(kThreads / 32) * kMaxK];
  block_reduce_df<1>(mu, smf, partial + blockIdx.x);
  if (arrive_last(&ctl->counter)) cg_alpha_final<1>(partial, gridDim.x, st, ctl, smem);
}

// K RHS: one thread per (group of R rows, rhs)
template <int K, int R>
__global__ void __launch_bounds__(kThreads) k_df_spmm_grp(const int64_t* __restrict__ rowptr,
                                                          const int32_t* __restrict__ col,
                                                          const float4* __restrict__ val, int64_t n,
                                                          const float4* __restrict__ pv, float4* __restrict__ q,
                                                          double2* partial, CgState* st, CgCtl* ctl) {
  if (blockIdx.x == 0 && threadIdx.x == 0) ctl->pending = 0;   // the previous p update has run
  if (!ctl->any_active) return;
  __shared__ double2 smem[2 * (kThreads / 32) * kMaxK];
  const int rhs = threadIdx.x % K;
  const int64_t items = (n / R) * K;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  float4 mu = make_float4(0.f, 0.f, 0.f, 0.f);
  for (int64_t it = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; it < items; it += stride) {
    const int64_t r0 = (it / K) * R;
    int64_t off[R];
#pragma unroll
    for (int i = 0; i < R; ++i) off[i] = rowptr[r0 + i];
    const int64_t len = rowptr[r0 + 1] - off[0];
    float4 acc[R];
#pragma unroll
    for (int i = 0; i < R; ++i) acc[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int64_t k = 0; k < len; ++k) {
      const float4 x = pv[(int64_t)col[off[0] + k] * K + rhs];
#pragma unroll
      for (int i = 0; i < R; ++i) cdf_mac(acc[i], val[off[i] + k], x);
    }
#pragma unroll
    for (int i = 0; i < R; ++i) {
      const float4 a = df_norm(acc[i]);
      q[(r0 + i) * K + rhs] = a;
      cdf_mac(mu, pv[(r0 + i) * K + rhs], a);
    }
  }
  __shared__ float4 smf[(kThreads / 32) * kMaxK];
  block_reduce_df<K>(mu, smf, partial + (int64_t)blockIdx.x * K);
  if (arrive_last(&ctl->counter)) cg_alpha_final<K>(partial, gridDim.x, st, ctl, smem);
}

// ---- SpMV variant autotuner ------------------------------------------------
// The double-float product's best lanes-per-row / unrolling depends on the
// matrix (rows, stored entries per row) and the RHS count.  At the first
// cycle of a solve each candidate runs 3 times on the actual operands (the
// product is the first kernel of an iteration and recomputes alpha, so extra
// runs change no solver state) and the fastest is kept per (n, nnz, k).
// PG_AUTOTUNE=0 keeps the default variant.
struct TuneEntry {
  int64_t n, nnz;
  int k, group, variant;
};
std::vector<TuneEntry> g_tune;
std::mutex g_tune_mu;

int tuned_variant(int64_t n, int64_t nnz, int k, int group) {
  std::lock_guard<std::mutex> lock(g_tune_mu);
  for (const TuneEntry& t : g_tune)
    if (t.n == n && t.nnz == nnz && t.k == k && t.group == group) return t.variant;
  return -1;
}

void store_variant(int64_t n, int64_t nnz, int k, int group, int v) {
  std::lock_guard<std::mutex> lock(g_tune_mu);
  g_tune.push_back(TuneEntry{n, nnz, k, group, v});
}

// PG_SPMV_VARIANT=v forces a product variant when it is valid for the solve
// (a group variant only when the rows were checked to group by R); -1 otherwise
int forced_variant(int k, int group) {
  const char* e = getenv("PG_SPMV_VARIANT");
  if (!(e && e[0])) return -1;
  const int v = atoi(e);
  if (k == 1) {
    if (v == 21 || v == 22 || v == 41 || v == 42 || v == 81 || v == 82) return v;
    const int gv = v - 100 * group;
    if (group && (gv == 2 || gv == 4 || gv == 8 || gv == 12 || gv == 14 || gv == 32 || gv == 34)) return v;
  } else {
    if (v == 1 || v == 2) return v;
    if (group && v == 100 * group) return v;
  }
  return -1;
}

bool autotune_enabled() {
  const char* e = getenv("PG_AUTOTUNE");
  return !(e && e[0] == '0');
}

// single RHS: variant = lanes per row G (1..8) * 10 + unroll U, or
// 100 R + 10 (U - 1) + G for the product over groups of R rows with G lanes
// per group and unroll U, 100 R + 30 + G for the group product with 4 column
// steps batched;
// several RHS: unroll 1 or 2, or 100 R for the group product
void launch_df_spmv1(int variant, int grid, cudaStream_t s, const int64_t* rowptr, const int32_t* col,
                     const float4* At, int64_t n, const float4* pv, float4* q, double2* part, CgState* st,
                     CgCtl* ctl) {
  switch (variant) {
    case 202: k_df_spmv_grp<2, 2><<<grid, kThreads, 0, s>>>(rowptr, col, At, n, pv, q, part, st, ctl); break;
    case 204: k_df_spmv_grp<2, 4><<<grid, kThreads, 0, s>>>(rowptr, col, At, n, pv, q, part, st, ctl); break;
    case 208: k_df_spmv_grp<2, 8><<<grid, kThreads, 0, s>>>(rowptr, col, At, n, pv, q, part, st, ctl); break;
    case 302: k_df_spmv_grp<3, 2><<<grid, kThreads, 0, s>>>(rowptr, col, At, n, pv, q, part, st, ctl); break;
    case 304: k_df_spmv_grp<3, 4><<<grid, kThreads, 0, s>>>(rowptr, col, At, n, pv, q, part, st, ctl); break;
    case 308: k_df_spmv_grp<3, 8><<<grid, kThreads, 0, s>>>(rowptr, col, At, n, pv, q, part, st, ctl); break;
    case 212: k_df_spmv_grp<2, 2, 2><<<grid, kThreads, 0, s>>>(rowptr, col, At, n, pv, q, part, st, ctl); break;
    case 232: k_df_spmv_grpb<2, 2, 4><<<grid, kThreads, 0, s>>>(rowptr, col, At, n, pv, q, part, st, ctl); break;
    case 234: k_df_spmv_grpb<2, 4, 4><<<grid, kThreads, 0, s>>>(rowptr, col, At, n, pv, q, part, st, ctl); break;
    case 332: k_df_spmv_grpb<3, 2, 4><<<grid, kThreads, 0, s>>>(rowptr, col, At, n, pv, q, part, st, ctl); break;
    case 334: k_df_spmv_grpb<3, 4, 4><<<grid, kThreads, 0, s>>>(rowptr, col, At, n, pv, q, part, st, ctl); break;
    case 214: k_df_spmv_grp<2, 4, 2><<<grid, kThreads, 0, s>>>(rowptr, col, At, n, pv, q, part, st, ctl); break;
    case 312: k_df_spmv_grp<3, 2, 2><<<grid, kThreads, 0, s>>>(rowptr, col, At, n, pv, q, part, st, ctl); break;
    case 314: k_df_spmv_grp<3, 4, 2><<<grid, kThreads, 0, s>>>(rowptr, col, At, n, pv, q, part, st, ctl); break;
    case 21: k_df_spmv1<2, 1><<<grid, kThreads, 0, s>>>(rowptr, col, At, n, pv, q, part, st, ctl); break;
    case 22: k_df_spmv1<2, 2><<<grid, kThreads, 0, s>>>(rowptr, col, At, n, pv, q, part, st, ctl); break;
    case 42: k_df_spmv1<4, 2><<<grid, kThreads, 0, s>>>(rowptr, col, At, n, pv, q, part, st, ctl); break;
    case 81: k_df_spmv1<8, 1><<<grid, kThreads, 0, s>>>(rowptr, col, At, n, pv, q, part, st, ctl); break;
    case 82: k_df_spmv1<8, 2><<<grid, kThreads, 0, s>>>(rowptr, col, At, n, pv, q, part, st, ctl); break;
    default: k_df_spmv1<4, 1><<<grid, kThreads, 0, s>>>(rowptr, col, At, n, pv, q, part, st, ctl); break;
  }
}

template <int K>
void launch_df_spmm(int variant, int grid, cudaStream_t s, const int64_t* rowptr, const int32_t* col,
                    const float4* At, int64_t n, const float4* pv, float4* q, double2* part, CgState* st, CgCtl* ctl) {
  if (variant == 200)
    k_df_spmm_grp<K, 2><<<grid, kThreads, 0, s>>>(rowptr, col, At, n, pv, q, part, st, ctl);
  else if (variant == 300)
    k_df_spmm_grp<K, 3><<<grid, kThreads, 0, s>>>(rowptr, col, At, n, pv, q, part, st, ctl);
  else if (variant == 2)
    k_df_spmm<K, 2><<<grid, kThreads, 0, s>>>(rowptr, col, At, n, pv, q, part, st, ctl);
  else
    k_df_spmm<K, 1><<<grid, kThreads, 0, s>>>(rowptr, col, At, n, pv, q, part, st, ctl);
}

// time each candidate (3 runs after 1 warm-up) and return the fastest
template <typename F>
int pick_fastest(const std::vector<int>& cands, F&& launch, cudaStream_t s) {
  cudaEvent_t a, b;
  if (cudaEventCreate(&a) != cudaSuccess) return cands[0];
  if (cudaEventCreate(&b) != cudaSuccess) {
    cudaEventDestroy(a);
    return cands[0];
  }
  int best = cands[0];
  float best_ms = 1e30f;
  for (int v : cands) {
    launch(v);
    cudaEventRecord(a, s);
    for (int i = 0; i < 3; ++i) launch(v);
    cudaEventRecord(b, s);
    if (cudaEventSynchronize(b) != cudaSuccess) break;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    if (ms < best_ms) {
      best_ms = ms;
      best = v;
    }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return best;
}

struct ToDF {
  __device__ float4 operator()(double2 v) const { return cdf_from(v); }
};

__global__ void k_wd_to_f32(const double* wd, int64_t n, float* wdf) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x)
    wdf[r] = (float)wd[r];
}
struct DfToD2 {
  __device__ double2 operator()(float4 v) const { return cdf_to(v); }
};

constexpr int kGraphIters = 16;   // iterations per captured CUDA graph

int run_cocg_df(const Plan& P, const int64_t* rowptr, const int32_t* col, const double2* A, const double2* b, double2* x,
                const pg_cocg_opts* o, pg_gmres_result* res, double* relres_out, char* ws, cudaStream_t s,
                const double* col_scale = nullptr) {
  const bool mf = col_scale != nullptr;
  size_t off[20];
  df_layout(P, off, mf);
  float4* ps = reinterpret_cast<float4*>(ws + off[14]);
  float4* Sdf = reinterpret_cast<float4*>(ws + off[15]);
  double* dscale = reinterpret_cast<double*>(ws + off[16]);
  float* dscale_hl = reinterpret_cast<float*>(ws + off[17]);
  const bool bj = !mf && P.bj.p > 0;
  double2* Sblk = reinterpret_cast<double2*>(ws + off[18]);
  double2* r64b = reinterpret_cast<double2*>(ws + off[19]);
  float4* At = reinterpret_cast<float4*>(ws + off[0]);
  double2* S = reinterpret_cast<double2*>(ws + off[1]);
  double* wd = reinterpret_cast<double*>(ws + off[2]);
  float* wdf = reinterpret_cast<float*>(ws + off[3]);
  float4* pv = reinterpret_cast<float4*>(ws + off[4]);
  float4* q = reinterpret_cast<float4*>(ws + off[5]);
  float4* r = reinterpret_cast<float4*>(ws + off[6]);
  float4* y = reinterpret_cast<float4*>(ws + off[7]);
  double2* r64 = reinterpret_cast<double2*>(ws + off[8]);
  double2* part = reinterpret_cast<double2*>(ws + off[9]);
  double2* part2 = part + (size_t)P.nb * P.k;
  CgState* st = reinterpret_cast<CgState*>(ws + off[10]);
  CgCtl* ctl = reinterpret_cast<CgCtl*>(ws + off[11]);
  double* rnorm = reinterpret_cast<double*>(ws + off[12]);
  double* target = rnorm + P.k;
  // per-column scales of the double-float recurrence: every cycle starts from
  // the true residual scaled to unit norm, so r^T r stays far inside the
  // FP32 exponent range whatever the units of b
  double* cscale = rnorm + 2 * P.k;
  double* cinv = rnorm + 3 * P.k;
  double* clam = rnorm + 4 * P.k;
  int* want = reinterpret_cast<int*>(ws + off[13]);
  int* dstatus = want + P.k;
  const int k = P.k, nb = P.nb;
  // vector-update grid: at least ~4 elements per thread, so the per-block
  // reduction does not dominate on small systems (its last block sums
  // gridDim.x partials)
  const int nbu = (int)std::min<int64_t>(nb, std::max<int64_t>(152 * 2, (P.n * P.k + 4 * kThreads - 1) / (4 * kThreads)));
  const int64_t npr = P.nnz / (P.n > 0 ? P.n : 1);
  const int spmv_grid = 152 * 16;
  if (spmv_grid > nb) return PG_ERR_ARG;

  PG_CUDA_TRY(cudaMemsetAsync(dstatus, 0, sizeof(int), s));
  PG_CUDA_TRY(cudaMemsetAsync(ctl, 0, sizeof(CgCtl), s));
  int group = 0;   // rows per entity group for the group product (0: not used)
  if (mf) {
    std::vector<float> hl(2 * (size_t)k);
    for (int i = 0; i < k; ++i) {
      hl[2 * i] = (float)col_scale[i];
      hl[2 * i + 1] = (float)(col_scale[i] - (double)hl[2 * i]);
    }
    PG_CUDA_TRY(cudaMemcpyAsync(dscale, col_scale, sizeof(double) * k, cudaMemcpyHostToDevice, s));
    PG_CUDA_TRY(cudaMemcpyAsync(dscale_hl, hl.data(), sizeof(float) * 2 * k, cudaMemcpyHostToDevice, s));
    PG_KSWITCH(k, (k_mf_scaling<K><<<pg_blocks(P.n, 256), 256, 0, s>>>(rowptr, col, A, P.n, dscale, S, wd, wdf,
                                                                          dstatus)));
    k_mf_sdf<<<pg_blocks(P.n * k, 256), 256, 0, s>>>(S, P.n * k, Sdf);
    k_mf_df_matrix<<<pg_blocks(P.nnz, 256), 256, 0, s>>>(A, P.nnz, At);
    // the host copy of the scales must outlive the asynchronous copy
    PG_CUDA_TRY(cudaStreamSynchronize(s));
  } else if (bj) {
    const int st0 = bj_setup(P, rowptr, col, A, S, wd, Sblk, At, ToDF(), dstatus, s);
    if (st0) return st0;
    k_wd_to_f32<<<pg_blocks(P.n, 256), 256, 0, s>>>(wd, P.n, wdf);
    if ((P.bj.p == 2 || P.bj.p == 3) && P.n % P.bj.p == 0) {
      // the group product needs every aligned group of p rows on one column list
      int* gflag = reinterpret_cast<int*>(part);
      int hg = 1;
      PG_CUDA_TRY(cudaMemsetAsync(gflag, 0, sizeof(int), s));
      k_group_check<<<pg_blocks(P.n, 256), 256, 0, s>>>(rowptr, col, P.n, P.bj.p, gflag);
      PG_LAUNCH_CHECK();
      PG_CUDA_TRY(cudaMemcpyAsync(&hg, gflag, sizeof(int), cudaMemcpyDeviceToHost, s));
      PG_CUDA_TRY(cudaStreamSynchronize(s));
      group = hg == 0 ? P.bj.p : 0;
    }
  } else {
    k_cg_scaling<<<pg_blocks(P.n, 256), 256, 0, s>>>(rowptr, col, A, P.n, S, wd, dstatus);
    k_df_scale_matrix<<<pg_blocks(P.n, 256), 256, 0, s>>>(rowptr, col, A, P.n, S, At, wdf, wd);
  }
  PG_LAUNCH_CHECK();
  std::vector<double> bnorm(k), rn(k), tgt(k), sc(k), sc_prev(k, 1.0), scal(4 * (size_t)k);
  std::vector<int> wnt(k);
  PG_KSWITCH(k, (k_norm2<K><<<nb, kThreads, 0, s>>>(b, P.n, part), k_norm_final<K><<<1, 32 * K, 0, s>>>(part, nb, rnorm)));
  PG_LAUNCH_CHECK();
  PG_CUDA_TRY(cudaMemcpyAsync(bnorm.data(), rnorm, sizeof(double) * k, cudaMemcpyDeviceToHost, s));
  int hstatus = 0;
  PG_CUDA_TRY(cudaMemcpyAsync(&hstatus, dstatus, sizeof(int), cudaMemcpyDeviceToHost, s));
  PG_CUDA_TRY(cudaStreamSynchronize(s));
  if (hstatus) {
    pg_set_error("pg_cocg: zero diagonal entry (Jacobi scaling undefined)");
    return PG_ERR_BREAKDOWN;
  }
  auto true_residual = [&]() {
    if (mf) {
      PG_KSWITCH(k, (k_mf_resid<K><<<pg_blocks(P.n * K, 256), 256, 0, s>>>(rowptr, col, A, P.n, dscale, x, b, r64)));
    } else {
      launch_spmv<double2>(P, rowptr, col, A, x, r64, b, nullptr, npr, s);
    }
  };
  const char* mon_env = getenv("PG_KSP_MONITOR");
  const bool monitor = mon_env && mon_env[0] && mon_env[0] != '0';
  int64_t its = 0, checks = 0;
  int status = PG_OK;
  const int64_t max_it = o->max_it > 0 ? o->max_it : 100000;
  int chunk = o->check_every > 0 ? o->check_every : 50;
  bool first = true;
  int variant = 41;
  const double delta = 1e-3;   // double-float recurrence: replace after 3 decades
  auto launch_single = [&](int v, cudaStream_t ss) {
    launch_df_spmv1(v, spmv_grid, ss, rowptr, col, At, P.n, pv, q, part, st, ctl);
  };
  // one iteration: product (alpha), vector update (beta), direction update;
  // no per-iteration launch arguments, so a run of them can be captured once
  // in a CUDA graph and replayed
  auto one_iteration = [&](cudaStream_t ss) {
    if (mf) {
      PG_KSWITCH(k, (k_mf_spmm<K><<<spmv_grid, kThreads, 0, ss>>>(rowptr, col, At, P.n, dscale_hl, Sdf, pv, ps, q,
                                                                  part, st, ctl),
                     k_df_update<K, true><<<nbu, kThreads, 0, ss>>>(y, r, pv, q, wdf, P.n, st, part, part2, ctl, 0,
                                                                    delta),
                     k_df_pupdate<K, true><<<pg_blocks(P.n * K, kThreads), kThreads, 0, ss>>>(pv, r, P.n, st, ctl,
                                                                                              ps, Sdf)));
      return;
    }
    if (k == 1)
      launch_single(variant, ss);
    else
      PG_KSWITCH(k, (launch_df_spmm<K>(variant, spmv_grid, ss, rowptr, col, At, P.n, pv, q, part, st, ctl)));
    PG_KSWITCH(k, (k_df_update<K><<<nbu, kThreads, 0, ss>>>(y, r, pv, q, wdf, P.n, st, part, part2, ctl, 0, delta),
                   k_df_pupdate<K><<<pg_blocks(P.n * K, kThreads), kThreads, 0, ss>>>(pv, r, P.n, st, ctl)));
  };
  const char* genv = getenv("PG_GRAPHS");
  const bool use_graphs = !(genv && genv[0] == '0');
  cudaStream_t cs = nullptr;
  cudaEvent_t ev_in = nullptr, ev_out = nullptr;
  cudaGraphExec_t gexec = nullptr;
  bool graph_failed = false;
  auto build_graph = [&]() {
    if (graph_failed) return;
    cudaGraph_t graph = nullptr;
    bool ok = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) == cudaSuccess &&
              cudaEventCreateWithFlags(&ev_in, cudaEventDisableTiming) == cudaSuccess &&
              cudaEventCreateWithFlags(&ev_out, cudaEventDisableTiming) == cudaSuccess;
    if (ok) ok = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
    if (ok) {
      for (int g = 0; g < kGraphIters; ++g) one_iteration(cs);
      ok = cudaStreamEndCapture(cs, &graph) == cudaSuccess && graph != nullptr;
    }
    if (ok) ok = cudaGraphInstantiate(&gexec, graph, 0) == cudaSuccess;
    if (graph) cudaGraphDestroy(graph);
    if (!ok) {
      cudaGetLastError();   // capture unavailable: keep launching directly
      gexec = nullptr;
      graph_failed = true;
    }
  };
  struct GraphCleanup {
    cudaStream_t& cs;
    cudaEvent_t& a;
    cudaEvent_t& b;
    cudaGraphExec_t& g;
    ~GraphCleanup() {
      if (g) cudaGraphExecDestroy(g);
      if (a) cudaEventDestroy(a);
      if (b) cudaEventDestroy(b);
      if (cs) cudaStreamDestroy(cs);
    }
  } graph_cleanup{cs, ev_in, ev_out, gexec};
  for (;;) {
    true_residual();
    PG_KSWITCH(k, (k_norm2<K><<<nb, kThreads, 0, s>>>(r64, P.n, part),
                   k_norm_final<K><<<1, 32 * K, 0, s>>>(part, nb, rnorm)));
    PG_LAUNCH_CHECK();
    PG_CUDA_TRY(cudaMemcpyAsync(rn.data(), rnorm, sizeof(double) * k, cudaMemcpyDeviceToHost, s));
    CgCtl hctl;
    PG_CUDA_TRY(cudaMemcpyAsync(&hctl, ctl, sizeof(CgCtl), cudaMemcpyDeviceToHost, s));
    PG_CUDA_TRY(cudaStreamSynchronize(s));
    if (!first && hctl.nonfinite) {
      pg_set_error("pg_cocg: non-finite residual");
      status = PG_ERR_NONFINITE;
      break;
    }
    bool all = true;
    for (int i = 0; i < k; ++i) {
      if (monitor)
        fprintf(stderr, "pg_cocg(df64): check %lld its %lld rhs %d true ||r||/||b|| = %.6e\n", (long long)checks,
                (long long)its, i, bnorm[i] > 0 ? rn[i] / bnorm[i] : 0.0);
      if (!isfinite(rn[i])) {
        pg_set_error("pg_cocg: non-finite residual");
        status = PG_ERR_NONFINITE;
      }
      const double tb = o->rtol * bnorm[i];
      const bool ok = rn[i] <= tb || bnorm[i] == 0.0;
      wnt[i] = ok ? 0 : 1;
      sc[i] = rn[i] > 0.0 && isfinite(rn[i]) ? rn[i] : 1.0;
      tgt[i] = 0.5 * tb / sc[i];
      if (!ok) all = false;
    }
    if (status || all) break;
    if (its >= max_it) {
      status = PG_ERR_NOT_CONVERGED;
      break;
    }
    // unit-norm cycle: the residual estimate starts at 1 (0 for an exact
    // column), p is carried over in the new scale
    for (int i = 0; i < k; ++i) {
      scal[i] = rn[i] > 0.0 ? 1.0 : 0.0;
      scal[k + i] = sc[i];
      scal[2 * k + i] = 1.0 / sc[i];
      scal[3 * k + i] = sc_prev[i] / sc[i];
      sc_prev[i] = sc[i];
    }
    PG_CUDA_TRY(cudaMemcpyAsync(target, tgt.data(), sizeof(double) * k, cudaMemcpyHostToDevice, s));
    PG_CUDA_TRY(cudaMemcpyAsync(want, wnt.data(), sizeof(int) * k, cudaMemcpyHostToDevice, s));
    PG_CUDA_TRY(cudaMemcpyAsync(rnorm, scal.data(), sizeof(double) * k, cudaMemcpyHostToDevice, s));
    PG_CUDA_TRY(cudaMemcpyAsync(cscale, scal.data() + k, sizeof(double) * 3 * k, cudaMemcpyHostToDevice, s));
    PG_KSWITCH(k, (k_scale_cols_d2<K><<<pg_blocks(P.n * K, 256), 256, 0, s>>>(r64, P.n, cinv)));
    if (!first) {
      PG_KSWITCH(k, (k_scale_cols_df<K><<<pg_blocks(P.n * K, 256), 256, 0, s>>>(pv, P.n, clam)));
      if (mf) PG_KSWITCH(k, (k_scale_cols_df<K><<<pg_blocks(P.n * K, 256), 256, 0, s>>>(ps, P.n, clam)));
    }
    if (mf) {
      PG_KSWITCH(k, (k_df_start<K, true><<<nb, kThreads, 0, s>>>(r64, S, P.n, r, y, pv, first ? 1 : 0, part, ps)));
    } else {
      if (bj) PG_KSWITCH(k, (k_bj_apply<K><<<pg_blocks(P.n * K, 256), 256, 0, s>>>(Sblk, P.bj, r64, r64b)));
      PG_KSWITCH(k, (k_df_start<K><<<nb, kThreads, 0, s>>>(bj ? r64b : r64, S, P.n, r, y, pv, first ? 1 : 0, part)));
    }
    PG_KSWITCH(k, (k_cg_cycle_init<K><<<1, 32 * K, 0, s>>>(part, nb, st, rnorm, target, want, ctl, first ? 1 : 0)));
    if (first && !mf) {
      variant = forced_variant(k, group);
      if (variant < 0) variant = tuned_variant(P.n, P.nnz, k, group);
      if (variant < 0) {
        if (autotune_enabled()) {
          if (k == 1) {
            std::vector<int> cands = {41, 42, 22, 82, 21};
            if (group)
              for (int gv : {2, 4, 8, 12, 14, 32, 34}) cands.push_back(100 * group + gv);
            variant = pick_fastest(cands, [&](int v) { launch_single(v, s); }, s);
          } else {
            std::vector<int> cands = {1, 2};
            if (group) cands.push_back(100 * group);
            variant = pick_fastest(cands, [&](int v) {
              PG_KSWITCH(k, (launch_df_spmm<K>(v, spmv_grid, s, rowptr, col, At, P.n, pv, q, part, st, ctl)));
            }, s);
          }
          PG_LAUNCH_CHECK();
        } else {
          variant = k == 1 ? 41 : 1;
        }
        store_variant(P.n, P.nnz, k, group, variant);
      }
      if (monitor) fprintf(stderr, "pg_cocg(df64): SpMV variant %d for n=%lld nnz=%lld k=%d\n", variant,
                           (long long)P.n, (long long)P.nnz, k);
    }
    first = false;
    const int steps = (int)((max_it - its) < chunk ? (max_it - its) : chunk);
    int done = 0;
    if (use_graphs && steps >= kGraphIters) {
      if (!gexec) build_graph();
      if (gexec) {
        // replay the captured iterations on the capture stream, joined to s
        cudaEventRecord(ev_in, s);
        cudaStreamWaitEvent(cs, ev_in, 0);
        for (; done + kGraphIters <= steps; done += kGraphIters) cudaGraphLaunch(gexec, cs);
        cudaEventRecord(ev_out, cs);
        cudaStreamWaitEvent(s, ev_out, 0);
      }
    }
    for (; done < steps; ++done) one_iteration(s);
    PG_LAUNCH_CHECK();
    PG_KSWITCH(k, (k_scale_cols_df<K><<<pg_blocks(P.n * K, 256), 256, 0, s>>>(y, P.n, cscale)));
    if (mf) {
      PG_KSWITCH(k, (k_df_xupdate<K, true><<<pg_blocks(P.n * K, kThreads), kThreads, 0, s>>>(y, S, P.n, x)));
    } else if (bj) {
      PG_KSWITCH(k, (k_bj_apply_t_add<K><<<pg_blocks(P.n * K, 256), 256, 0, s>>>(Sblk, P.bj, y, x, DfToD2())));
    } else {
      PG_KSWITCH(k, (k_df_xupdate<K><<<pg_blocks(P.n * K, kThreads), kThreads, 0, s>>>(y, S, P.n, x)));
    }
    std::vector<int> hits(k), hbrk(k);
    for (int i = 0; i < k; ++i) {
      PG_CUDA_TRY(cudaMemcpyAsync(&hits[i], &st[i].its, sizeof(int), cudaMemcpyDeviceToHost, s));
      PG_CUDA_TRY(cudaMemcpyAsync(&hbrk[i], &st[i].breakdown, sizeof(int), cudaMemcpyDeviceToHost, s));
    }
    PG_CUDA_TRY(cudaStreamSynchronize(s));
    int used = 0;
    for (int i = 0; i < k; ++i) used = hits[i] > used ? hits[i] : used;
    const int64_t cycle_its = used - its;
    its = used;
    ++checks;
    bool brk = false;
    for (int i = 0; i < k; ++i) brk = brk || hbrk[i];
    if (brk) {
      pg_set_error("pg_cocg: breakdown (p^T A p = 0 or r^T r = 0)");
      status = PG_ERR_BREAKDOWN;
      true_residual();
      PG_KSWITCH(k, (k_norm2<K><<<nb, kThreads, 0, s>>>(r64, P.n, part),
                     k_norm_final<K><<<1, 32 * K, 0, s>>>(part, nb, rnorm)));
      PG_CUDA_TRY(cudaMemcpyAsync(rn.data(), rnorm, sizeof(double) * k, cudaMemcpyDeviceToHost, s));
      PG_CUDA_TRY(cudaStreamSynchronize(s));
      break;
    }
    int64_t c2 = cycle_its + cycle_its / 4 + 8;
    chunk = (int)(c2 < 16 ? 16 : (c2 > 4000 ? 4000 : c2));
  }
  double worst = 0.0;
  for (int i = 0; i < k; ++i) {
    const double rr = bnorm[i] > 0 ? rn[i] / bnorm[i] : 0.0;
    if (relres_out) relres_out[i] = rr;
    worst = rr > worst ? rr : worst;
  }
  if (res) {
    res->iterations = its;
    res->restarts = checks;
    res->relres = worst;
    res->status = status;
  }
  if (status == PG_ERR_NOT_CONVERGED) pg_set_error("pg_cocg: max_it reached before rtol");
  return status;
}

// ---- several systems in one solve -------------------------------------------
// Independent complex-symmetric systems (meshes of different sizes, or one
// mesh at several frequencies) stored as one block-diagonal CSR matrix: system
// j owns rows [row[j], row[j+1]) and only references its own columns.  Each
// system keeps its own COCG scalars, convergence test and iteration count, so
// the result is the one each would reach alone, while every launch covers all
// of them: small systems no longer leave most of the GPU idle, and one graph
// replay advances every system.  Every launch splits its blocks over the
// systems in proportion to their rows (blk[j] .. blk[j+1] - 1 for system j),
// so a block's partial sums belong to one system and the per-system totals
// are fixed-order sums over that block range.
struct Seg {
  const int64_t* row;   // [S + 1] first row of each system (device)
  const int* blk;       // [S + 1] first block of each system (device)
  int S;
};

struct SegPos {
  int j, lb, nbj;       // system, block index inside it, blocks it owns
  int64_t r0, r1;       // its rows
};

__device__ __forceinline__ SegPos seg_pos(const Seg& g) {
  __shared__ int sj;
  if (threadIdx.x == 0) {
    int lo = 0, hi = g.S - 1;   // largest j with blk[j] <= blockIdx.x
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (g.blk[mid] <= (int)blockIdx.x) lo = mid;
      else hi = mid - 1;
    }
    sj = lo;
  }
  __syncthreads();
  SegPos p;
  p.j = sj;
  p.lb = (int)blockIdx.x - g.blk[sj];
  p.nbj = g.blk[sj + 1] - g.blk[sj];
  p.r0 = g.row[sj];
  p.r1 = g.row[sj + 1];
  return p;
}

// sum of partial[b * K + rhs] over the blocks of system t / K (one warp; fixed order)
template <int K>
__device__ double2 seg_pair_sum(const double2* partial, const Seg& g, int t) {
  const int lane = threadIdx.x & 31, j = t / K, rhs = t % K;
  double2 acc = make_double2(0.0, 0.0);
  for (int b = g.blk[j] + lane; b < g.blk[j + 1]; b += 32) acc = dadd(acc, __ldcg(partial + (int64_t)b * K + rhs));
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) acc = dadd(acc, shfl_xor(acc, off));
  return acc;
}

// 1 if some right-hand side of system j is iterating
template <int K>
__device__ int seg_live(const CgState* st, int j) {
  __shared__ int live;
  if (threadIdx.x == 0) live = 0;
  __syncthreads();
  if (threadIdx.x < K && st[j * K + threadIdx.x].active) atomicOr(&live, 1);
  __syncthreads();
  return live;
}

template <int K>
__device__ void seg_alpha_final(const double2* partial, const Seg& g, CgState* st, CgCtl* ctl) {
  for (int t = threadIdx.x >> 5; t < g.S * K; t += kThreads / 32) {
    const double2 m = seg_pair_sum<K>(partial, g, t);
    if ((threadIdx.x & 31) == 0) {
      CgState& S = st[t];
      if (S.active) {
        if (m.x == 0.0 && m.y == 0.0) {
          S.breakdown = 1;
          S.active = 0;
          S.alpha = make_double2(0.0, 0.0);
        } else {
          S.alpha = ddiv(S.rho, m);
        }
      } else {
        S.alpha = make_double2(0.0, 0.0);
      }
    }
  }
  if (threadIdx.x == 0) ctl->counter = 0;
}

template <int K>
__device__ void seg_beta_final(const double2* prho, const double2* pw, const Seg& g, CgState* st, CgCtl* ctl,
                               double delta) {
  __shared__ int any, stop;
  if (threadIdx.x == 0) {
    any = 0;
    stop = 0;
  }
  __syncthreads();
  for (int t = threadIdx.x >> 5; t < g.S * K; t += kThreads / 32) {
    const double2 rho = seg_pair_sum<K>(prho, g, t);
    const double2 w = seg_pair_sum<K>(pw, g, t);
    if ((threadIdx.x & 31) == 0) {
      CgState& S = st[t];
      if (S.active) {
        S.beta_iter = 1;
        S.its += 1;
        S.res = sqrt(w.x);
        if (!isfinite(S.res)) ctl->nonfinite = 1;
        if (S.rho.x == 0.0 && S.rho.y == 0.0) {
          S.breakdown = 1;
          S.active = 0;
          S.beta = make_double2(0.0, 0.0);
        } else {
          S.beta = ddiv(rho, S.rho);
        }
        S.rho = rho;
        if (S.res <= S.target || !isfinite(S.res)) S.active = 0;
        else if (S.res <= delta * S.res0 || S.res > 1e3 * S.res0) atomicOr(&stop, 1);
      } else {
        S.beta = make_double2(0.0, 0.0);
        S.beta_iter = 0;
      }
      if (S.active) atomicOr(&any, 1);
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    ctl->any_active = any && !stop;
    ctl->pending = 1;
    ctl->counter = 0;
  }
}

// q = At p for every system (G lanes per (row, rhs) item; G > 1 only for one
// RHS), partial mu = p^T q; last block: alpha of every system
template <int K, int G, int U>
__global__ void __launch_bounds__(kThreads) k_sg_spmm(const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                                                      const float4* __restrict__ val, Seg g,
                                                      const float4* __restrict__ pv, float4* __restrict__ q,
                                                      double2* partial, CgState* st, CgCtl* ctl) {
  static_assert(K == 1 || G == 1, "several lanes per item only for one right-hand side");
  if (blockIdx.x == 0 && threadIdx.x == 0) ctl->pending = 0;
  if (!ctl->any_active) return;
  const SegPos sp = seg_pos(g);
  float4 mu = make_float4(0.f, 0.f, 0.f, 0.f);
  if (seg_live<K>(st, sp.j)) {
    const int64_t items = (sp.r1 - sp.r0) * K;
    const int lane = threadIdx.x % G;
    const int64_t groups = ((int64_t)sp.nbj * kThreads) / G;
    const int64_t gid = ((int64_t)sp.lb * kThreads + threadIdx.x) / G;
    const int64_t warp_base = gid - (threadIdx.x & 31) / G;
    for (int64_t iw = warp_base; iw < items; iw += groups) {
      const int64_t it = iw + (gid - warp_base);
      const bool valid = it < items;
      const int64_t r = sp.r0 + it / K;
      const int rhs = (int)(it % K);
      float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
      if (valid) {
        const int64_t e = rowptr[r + 1];
        int64_t kk = rowptr[r] + lane;
        if (U == 2) {
          // two independent accumulators: two gathers in flight per lane
          float4 acc1 = make_float4(0.f, 0.f, 0.f, 0.f);
          for (; kk + G < e; kk += 2 * G) {
            const int32_t c0 = col[kk], c1 = col[kk + G];
            const float4 v0 = val[kk], v1 = val[kk + G];
            cdf_mac(acc, v0, pv[(int64_t)c0 * K + rhs]);
            cdf_mac(acc1, v1, pv[(int64_t)c1 * K + rhs]);
          }
          if (kk < e) cdf_mac(acc, val[kk], pv[(int64_t)col[kk] * K + rhs]);
          cdf_add(acc, acc1);
        } else {
          for (; kk < e; kk += G) cdf_mac(acc, val[kk], pv[(int64_t)col[kk] * K + rhs]);
        }
      }
#pragma unroll
      for (int off = G / 2; off > 0; off >>= 1) cdf_add(acc, shfl_xor4(acc, off));
      if (valid && lane == 0) {
        acc = df_norm(acc);
        q[r * K + rhs] = acc;
        cdf_mac(mu, pv[r * K + rhs], acc);
      }
    }
  }
  __shared__ float4 smf[(kThreads / 32) * kMaxK];
  block_reduce_df<K>(mu, smf, partial + (int64_t)blockIdx.x * K);
  if (arrive_last(&ctl->counter)) seg_alpha_final<K>(partial, g, st, ctl);
}

// y += alpha p ; r -= alpha q with each system's alpha; partial rho and w
template <int K>
__global__ void __launch_bounds__(kThreads) k_sg_update(float4* __restrict__ y, float4* __restrict__ r,
                                                        const float4* __restrict__ pv, const float4* __restrict__ q,
                                                        const float* __restrict__ wd, Seg g, CgState* st,
                                                        double2* prho, double2* pw, CgCtl* ctl, double delta) {
  if (!ctl->any_active) return;
  const SegPos sp = seg_pos(g);
  __shared__ float4 al[kMaxK];
  if (threadIdx.x < K) al[threadIdx.x] = cdf_from(st[sp.j * K + threadIdx.x].alpha);
  const int live = seg_live<K>(st, sp.j);   // synchronises al as well
  const float4 a = al[threadIdx.x % K];
  const float4 na = make_float4(-a.x, -a.y, -a.z, -a.w);
  const int64_t base = sp.r0 * K, total = (sp.r1 - sp.r0) * K;
  const int64_t chunk = ((total + sp.nbj - 1) / sp.nbj + K - 1) / K * K;
  const int64_t lo = base + (int64_t)sp.lb * chunk, hi = min(base + total, lo + chunk);
  float4 rho = make_float4(0.f, 0.f, 0.f, 0.f);
  float ww = 0.f;
  if (live)
    for (int64_t e = lo + threadIdx.x; e < hi; e += kThreads) {
      float4 ye = y[e], re = r[e];
      cdf_mac(ye, a, pv[e]);
      cdf_mac(re, na, q[e]);
      ye = df_norm(ye);
      re = df_norm(re);
      y[e] = ye;
      r[e] = re;
      cdf_mac(rho, re, re);
      ww += (re.x * re.x + re.z * re.z) * wd[e / K];
    }
  __shared__ float4 smf[(kThreads / 32) * kMaxK];
  block_reduce_df<K>(rho, smf, prho + (int64_t)blockIdx.x * K);
  block_reduce_f<K>(ww, reinterpret_cast<float*>(smf), pw + (int64_t)blockIdx.x * K);
  if (arrive_last(&ctl->counter)) seg_beta_final<K>(prho, pw, g, st, ctl, delta);
}

// p = r + beta p with each system's beta
template <int K>
__global__ void __launch_bounds__(kThreads) k_sg_pupdate(float4* __restrict__ pv, const float4* __restrict__ r, Seg g,
                                                         const CgState* st, const CgCtl* ctl) {
  if (!ctl->pending) return;
  const SegPos sp = seg_pos(g);
  __shared__ float4 bt[kMaxK];
  __shared__ int use[kMaxK];
  __shared__ int anyuse;
  if (threadIdx.x == 0) anyuse = 0;
  __syncthreads();
  if (threadIdx.x < K) {
    const CgState& S = st[sp.j * K + threadIdx.x];
    bt[threadIdx.x] = cdf_from(S.beta);
    use[threadIdx.x] = S.beta_iter == 1;
    if (S.beta_iter == 1) atomicOr(&anyuse, 1);
  }
  __syncthreads();
  if (!anyuse) return;
  const int64_t hi = sp.r1 * K;
  for (int64_t e = sp.r0 * K + (int64_t)sp.lb * kThreads + threadIdx.x; e < hi; e += (int64_t)sp.nbj * kThreads)
    if (use[e % K]) {
      float4 v = r[e];
      cdf_mac(v, bt[e % K], pv[e]);
      pv[e] = df_norm(v);
    }
}

// r = S r64 (double-float), y = 0, first cycle p = r; partial rho (FP64)
template <int K>
__global__ void k_sg_start(const double2* __restrict__ r64, const double2* __restrict__ S, Seg g, float4* r, float4* y,
                           float4* pv, int set_p, double2* prho) {
  __shared__ double2 smem[(kThreads / 32) * kMaxK];
  const SegPos sp = seg_pos(g);
  const int64_t base = sp.r0 * K, total = (sp.r1 - sp.r0) * K;
  const int64_t chunk = ((total + sp.nbj - 1) / sp.nbj + K - 1) / K * K;
  const int64_t lo = base + (int64_t)sp.lb * chunk, hi = min(base + total, lo + chunk);
  double2 rho = make_double2(0.0, 0.0);
  for (int64_t e = lo + threadIdx.x; e < hi; e += kThreads) {
    const double2 v = cmul(S[e / K], r64[e]);
    const float4 vf = cdf_from(v);
    r[e] = vf;
    y[e] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (set_p) pv[e] = vf;
    rho = dadd(rho, cmul(v, v));
  }
  block_reduce_rhs<K>(rho, smem, prho + (int64_t)blockIdx.x * K);
}

// per-block sums of |r|^2 per right-hand side
template <int K>
__global__ void __launch_bounds__(kThreads) k_sg_norm2(const double2* __restrict__ r, Seg g, double2* partial) {
  __shared__ double2 smem[(kThreads / 32) * kMaxK];
  const SegPos sp = seg_pos(g);
  const int64_t base = sp.r0 * K, total = (sp.r1 - sp.r0) * K;
  const int64_t chunk = ((total + sp.nbj - 1) / sp.nbj + K - 1) / K * K;
  const int64_t lo = base + (int64_t)sp.lb * chunk, hi = min(base + total, lo + chunk);
  double s = 0.0;
  for (int64_t e = lo + threadIdx.x; e < hi; e += kThreads) s += dabs2(r[e]);
  block_reduce_rhs<K>(make_double2(s, 0.0), smem, partial + (int64_t)blockIdx.x * K);
}

template <int K>
__global__ void k_sg_norm_final(const double2* partial, Seg g, double* out) {
  for (int t = threadIdx.x >> 5; t < g.S * K; t += blockDim.x / 32) {
    const double2 s = seg_pair_sum<K>(partial, g, t);
    if ((threadIdx.x & 31) == 0) out[t] = sqrt(s.x);
  }
}

template <int K>
__global__ void k_sg_cycle_init(const double2* prho, Seg g, CgState* st, const double* rnorm, const double* target,
                                const int* want, CgCtl* ctl, int first) {
  __shared__ int any;
  if (threadIdx.x == 0) any = 0;
  __syncthreads();
  for (int t = threadIdx.x >> 5; t < g.S * K; t += blockDim.x / 32) {
    const double2 rho = seg_pair_sum<K>(prho, g, t);
    if ((threadIdx.x & 31) == 0) {
      CgState& S = st[t];
      if (first) {
        S.its = 0;
        S.breakdown = 0;
        S.beta_iter = 0;
      }
      S.rho = rho;
      S.target = target[t];
      S.res = rnorm[t];
      S.res0 = rnorm[t];
      S.active = want[t] && rnorm[t] > 0.0;
      S.alpha = S.beta = make_double2(0.0, 0.0);
      if (S.active) atomicOr(&any, 1);
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    ctl->any_active = any;
    ctl->nonfinite = 0;
    ctl->counter = 0;
  }
}

__device__ __forceinline__ int seg_of_row(const Seg& g, int64_t r) {
  int lo = 0, hi = g.S - 1;   // largest j with row[j] <= r
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (g.row[mid] <= r) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// v[r, c] *= f[system(r) * K + c] (FP64 vectors)
template <int K>
__global__ void k_sg_scale_d2(double2* v, Seg g, int64_t n, const double* f) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n * K; e += (int64_t)gridDim.x * blockDim.x)
    v[e] = dscale(f[seg_of_row(g, e / K) * K + e % K], v[e]);
}

// the same for double-float vectors
template <int K>
__global__ void k_sg_scale_df(float4* v, Seg g, int64_t n, const double* f) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n * K; e += (int64_t)gridDim.x * blockDim.x) {
    const double fc = f[seg_of_row(g, e / K) * K + e % K];
    const float fh = __double2float_rn(fc);
    const float fl = __double2float_rn(fc - (double)fh);
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    cdf_mac(acc, v[e], make_float4(fh, fl, 0.f, 0.f));
    v[e] = df_norm(acc);
  }
}

// every stored column of system j lies in its own rows (block-diagonal)
__global__ void k_sg_check(const int64_t* rowptr, const int32_t* col, Seg g, int64_t n, int* status) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    const int j = seg_of_row(g, r);
    const int64_t c0 = g.row[j], c1 = g.row[j + 1];
    for (int64_t k = rowptr[r]; k < rowptr[r + 1]; ++k)
      if (col[k] < c0 || col[k] >= c1) *status = PG_ERR_ARG;
  }
}

// host block map: blocks of system j in proportion to its rows, at least 1
// and at most one per kThreads (row, rhs) items
std::vector<int> seg_blocks(const int64_t* rows, int S, int k) {
  const int64_t n = rows[S] - rows[0];
  const double target = 152.0 * 16.0;
  std::vector<int> blk(S + 1, 0);
  for (int j = 0; j < S; ++j) {
    const int64_t nj = rows[j + 1] - rows[j];
    int64_t b = n > 0 ? (int64_t)(target * (double)nj / (double)n) : 1;
    const int64_t cap = (nj * k + kThreads - 1) / kThreads;
    b = std::min<int64_t>(b, cap);
    blk[j + 1] = blk[j] + (int)std::max<int64_t>(b, 1);
  }
  return blk;
}

// the same total of blocks re-split over the systems still iterating: a
// converged system keeps one (idle) block, the others share the rest in
// proportion to their rows; blocks no system can use go to the largest
// active system, where they find no rows
void seg_rebalance(const int64_t* rows, int S, int k, const std::vector<char>& active, int total,
                   std::vector<int>& blk) {
  blk.assign(S + 1, 0);
  int64_t n_act = 0;
  int big = -1;
  for (int j = 0; j < S; ++j) {
    const int64_t nj = rows[j + 1] - rows[j];
    if (active[j]) {
      n_act += nj;
      if (big < 0 || nj > rows[big + 1] - rows[big]) big = j;
    }
  }
  // every system holds one block; the total - S others go to the active
  // systems (total >= S: the first map gives each system at least one)
  const int spare = total - S;
  std::vector<int> b(S, 1);
  int used = S;
  for (int j = 0; j < S; ++j) {
    if (!active[j]) continue;
    const int64_t nj = rows[j + 1] - rows[j];
    int64_t v = n_act > 0 ? (int64_t)((double)spare * (double)nj / (double)n_act) : 0;
    v = std::min<int64_t>(v, std::max<int64_t>((nj * k + kThreads - 1) / kThreads - 1, 0));
    b[j] += (int)v;
    used += (int)v;
  }
  if (used < total) b[big >= 0 ? big : S - 1] += total - used;
  for (int j = 0; j < S; ++j) blk[j + 1] = blk[j] + b[j];
}

struct SegPlan {
  int64_t n, nnz;
  int k, S, nb;
  int p;                    // block-Jacobi order (0: diagonal)
  std::vector<BjInfo> bj;   // per system, c0 = its first row
  std::vector<int64_t> soff;  // per system offset of its factors (S + 1 entries)
};

size_t sg_layout(const SegPlan& P, size_t* off /* 18 */) {
  size_t o = 0;
  auto put = [&](int idx, size_t bytes) { off[idx] = o; o += pg_align256(bytes); };
  const size_t pairs = (size_t)P.S * P.k;
  put(0, P.nnz * sizeof(float4));                // At
  put(1, sizeof(double2) * P.n);                 // S
  put(2, sizeof(double) * P.n);                  // |D|
  put(3, sizeof(float) * P.n);                   // |D| f32
  put(4, sizeof(float4) * P.n * P.k);            // p
  put(5, sizeof(float4) * P.n * P.k);            // q
  put(6, sizeof(float4) * P.n * P.k);            // r
  put(7, sizeof(float4) * P.n * P.k);            // y
  put(8, sizeof(double2) * P.n * P.k);           // r64
  put(9, sizeof(double2) * (size_t)P.nb * P.k * 3);
  put(10, sizeof(CgState) * pairs);
  put(11, sizeof(CgCtl));
  put(12, sizeof(double) * pairs * 6);           // rnorm, target, pair scales, inverses, ratios
  put(13, sizeof(int) * (pairs + 1));            // want, status
  put(14, sizeof(int64_t) * (P.S + 1));          // system rows
  put(15, sizeof(int) * (P.S + 1));              // system blocks
  put(16, P.p ? sizeof(double2) * P.soff[P.S] : 0);      // block-Jacobi factors
  put(17, P.p ? sizeof(double2) * P.n * P.k : 0);        // S r64
  return o;
}

int seg_plan(int64_t n, int64_t nnz, int k, const int64_t* rows, int S, const int64_t* ents, int bp, SegPlan& P) {
  if (S < 1 || rows == nullptr || rows[0] != 0 || rows[S] != n) return PG_ERR_ARG;
  for (int j = 0; j < S; ++j)
    if (rows[j + 1] < rows[j]) return PG_ERR_ARG;
  P.n = n;
  P.nnz = nnz;
  P.k = k;
  P.S = S;
  const std::vector<int> blk = seg_blocks(rows, S, k);
  P.nb = blk[S];
  P.p = bp >= 1 && bp <= 6 ? bp : 0;
  P.bj.clear();
  P.soff.assign(S + 1, 0);
  if (P.p) {
    if (ents == nullptr) return PG_ERR_ARG;
    for (int j = 0; j < S; ++j) {
      BjInfo B{ents[3 * j], ents[3 * j + 1], ents[3 * j + 2], P.p, rows[j + 1] - rows[j]};
      B.c0 = rows[j];
      if (B.nE < 0 || B.nF < 0 || B.nV < 0 ||
          B.nE * B.de() + B.nF * (int64_t)B.df() + B.nV * (int64_t)B.dv() != B.n)
        return PG_ERR_ARG;
      P.bj.push_back(B);
      P.soff[j + 1] = P.soff[j] + B.s_size();
    }
  }
  return PG_OK;
}

int run_cocg_seg(const SegPlan& P, const int64_t* hrows, const int64_t* rowptr, const int32_t* col, const double2* A,
                 const double2* b, double2* x, const pg_cocg_opts* o, pg_gmres_result* res, double* relres_out,
                 int64_t* its_out, char* ws, cudaStream_t s) {
  size_t off[18];
  sg_layout(P, off);
  float4* At = reinterpret_cast<float4*>(ws + off[0]);
  double2* Sd = reinterpret_cast<double2*>(ws + off[1]);
  double* wd = reinterpret_cast<double*>(ws + off[2]);
  float* wdf = reinterpret_cast<float*>(ws + off[3]);
  float4* pv = reinterpret_cast<float4*>(ws + off[4]);
  float4* q = reinterpret_cast<float4*>(ws + off[5]);
  float4* r = reinterpret_cast<float4*>(ws + off[6]);
  float4* y = reinterpret_cast<float4*>(ws + off[7]);
  double2* r64 = reinterpret_cast<double2*>(ws + off[8]);
  double2* part = reinterpret_cast<double2*>(ws + off[9]);
  double2* part2 = part + (size_t)P.nb * P.k;
  CgState* st = reinterpret_cast<CgState*>(ws + off[10]);
  CgCtl* ctl = reinterpret_cast<CgCtl*>(ws + off[11]);
  const int pairs = P.S * P.k;
  double* rnorm = reinterpret_cast<double*>(ws + off[12]);
  double* target = rnorm + pairs;
  // per-pair scales: every cycle starts from the true residual at unit norm
  // (r^T r stays inside the FP32 exponent range of the double-float pairs)
  double* cscale = rnorm + 2 * pairs;
  double* cinv = rnorm + 3 * pairs;
  double* clam = rnorm + 4 * pairs;
  int* want = reinterpret_cast<int*>(ws + off[13]);
  int* dstatus = want + pairs;
  int64_t* drows = reinterpret_cast<int64_t*>(ws + off[14]);
  int* dblk = reinterpret_cast<int*>(ws + off[15]);
  double2* Sblk = reinterpret_cast<double2*>(ws + off[16]);
  double2* r64b = reinterpret_cast<double2*>(ws + off[17]);
  const int k = P.k, G = P.nb;
  const bool bj = P.p > 0;
  std::vector<int> hblk = seg_blocks(hrows, P.S, k), cur_blk;
  std::vector<char> sys_active(P.S, 1);
  PG_CUDA_TRY(cudaMemcpyAsync(drows, hrows, sizeof(int64_t) * (P.S + 1), cudaMemcpyHostToDevice, s));
  PG_CUDA_TRY(cudaMemcpyAsync(dblk, hblk.data(), sizeof(int) * (P.S + 1), cudaMemcpyHostToDevice, s));
  PG_CUDA_TRY(cudaMemsetAsync(dstatus, 0, sizeof(int), s));
  const Seg g{drows, dblk, P.S};
  int hstatus = 0;
  k_sg_check<<<pg_blocks(P.n, 256), 256, 0, s>>>(rowptr, col, g, P.n, dstatus);
  PG_LAUNCH_CHECK();
  PG_CUDA_TRY(cudaMemcpyAsync(&hstatus, dstatus, sizeof(int), cudaMemcpyDeviceToHost, s));
  PG_CUDA_TRY(cudaStreamSynchronize(s));   // also keeps the host block map alive for the copies
  if (hstatus) {
    pg_set_error("pg_cocg_segments: a row references a column outside its own system");
    return PG_ERR_ARG;
  }
  if (bj) {
    k_fill_one<<<pg_blocks(P.n, 256), 256, 0, s>>>(Sd, P.n);
    for (int j = 0; j < P.S; ++j) {
      const BjInfo& B = P.bj[j];
      if (B.n == 0) continue;
      k_bj_check<<<pg_blocks(B.n, 256), 256, 0, s>>>(rowptr + hrows[j], col, B, dstatus);
    }
    PG_CUDA_TRY(cudaMemcpyAsync(&hstatus, dstatus, sizeof(int), cudaMemcpyDeviceToHost, s));
    PG_CUDA_TRY(cudaStreamSynchronize(s));
    if (hstatus) {
      pg_set_error("pg_cocg_segments: block-Jacobi needs the entity-block pattern (rows of one entity share their columns)");
      return PG_ERR_ARG;
    }
    for (int j = 0; j < P.S; ++j) {
      const BjInfo& B = P.bj[j];
      if (B.n == 0) continue;
      k_bj_factor<<<pg_blocks(B.n, 128), 128, 0, s>>>(rowptr + hrows[j], col, A, B, Sblk + P.soff[j], wd + hrows[j],
                                                       dstatus);
      k_bj_scale_matrix<<<pg_blocks(B.n, 128), 128, 0, s>>>(rowptr + hrows[j], col, A, B, Sblk + P.soff[j], At, ToDF());
    }
    k_wd_to_f32<<<pg_blocks(P.n, 256), 256, 0, s>>>(wd, P.n, wdf);
  } else {
    k_cg_scaling<<<pg_blocks(P.n, 256), 256, 0, s>>>(rowptr, col, A, P.n, Sd, wd, dstatus);
    k_df_scale_matrix<<<pg_blocks(P.n, 256), 256, 0, s>>>(rowptr, col, A, P.n, Sd, At, wdf, wd);
  }
  PG_LAUNCH_CHECK();
  std::vector<double> bnorm(pairs), rn(pairs), tgt(pairs), sc(pairs), sc_prev(pairs, 1.0), scal(4 * (size_t)pairs);
  std::vector<int> wnt(pairs);
  PG_KSWITCH(k, (k_sg_norm2<K><<<G, kThreads, 0, s>>>(b, g, part), k_sg_norm_final<K><<<1, kThreads, 0, s>>>(part, g, rnorm)));
  PG_LAUNCH_CHECK();
  PG_CUDA_TRY(cudaMemcpyAsync(bnorm.data(), rnorm, sizeof(double) * pairs, cudaMemcpyDeviceToHost, s));
  PG_CUDA_TRY(cudaMemcpyAsync(&hstatus, dstatus, sizeof(int), cudaMemcpyDeviceToHost, s));
  PG_CUDA_TRY(cudaStreamSynchronize(s));
  if (hstatus) {
    pg_set_error("pg_cocg_segments: zero diagonal entry (Jacobi scaling undefined)");
    return PG_ERR_BREAKDOWN;
  }
  Plan Pf{P.n, P.nnz, k, 1, 0, 1, sizeof(double2), BjInfo{}};
  const int64_t npr = P.nnz / (P.n > 0 ? P.n : 1);
  auto true_residual = [&]() { launch_spmv<double2>(Pf, rowptr, col, A, x, r64, b, nullptr, npr, s); };
  const char* mon_env = getenv("PG_KSP_MONITOR");
  const bool monitor = mon_env && mon_env[0] && mon_env[0] != '0';
  int64_t its = 0, checks = 0;
  int status = PG_OK;
  const int64_t max_it = o->max_it > 0 ? o->max_it : 100000;
  int chunk = o->check_every > 0 ? o->check_every : 50;
  bool first = true;
  const double delta = 1e-3;
  auto one_iteration = [&](cudaStream_t ss) {
    if (k == 1)
      k_sg_spmm<1, 4, 2><<<G, kThreads, 0, ss>>>(rowptr, col, At, g, pv, q, part, st, ctl);
    else
      PG_KSWITCH(k, (k_sg_spmm<K, 1, 2><<<G, kThreads, 0, ss>>>(rowptr, col, At, g, pv, q, part, st, ctl)));
    PG_KSWITCH(k, (k_sg_update<K><<<G, kThreads, 0, ss>>>(y, r, pv, q, wdf, g, st, part, part2, ctl, delta),
                   k_sg_pupdate<K><<<G, kThreads, 0, ss>>>(pv, r, g, st, ctl)));
  };
  const char* genv = getenv("PG_GRAPHS");
  const bool use_graphs = !(genv && genv[0] == '0');
  cudaStream_t cs = nullptr;
  cudaEvent_t ev_in = nullptr, ev_out = nullptr;
  cudaGraphExec_t gexec = nullptr;
  bool graph_failed = false;
  auto build_graph = [&]() {
    if (graph_failed) return;
    cudaGraph_t graph = nullptr;
    bool ok = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) == cudaSuccess &&
              cudaEventCreateWithFlags(&ev_in, cudaEventDisableTiming) == cudaSuccess &&
              cudaEventCreateWithFlags(&ev_out, cudaEventDisableTiming) == cudaSuccess;
    if (ok) ok = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
    if (ok) {
      for (int i = 0; i < kGraphIters; ++i) one_iteration(cs);
      ok = cudaStreamEndCapture(cs, &graph) == cudaSuccess && graph != nullptr;
    }
    if (ok) ok = cudaGraphInstantiate(&gexec, graph, 0) == cudaSuccess;
    if (graph) cudaGraphDestroy(graph);
    if (!ok) {
      cudaGetLastError();
      gexec = nullptr;
      graph_failed = true;
    }
  };
  struct GraphCleanup {
    cudaStream_t& cs;
    cudaEvent_t& a;
    cudaEvent_t& b;
    cudaGraphExec_t& gx;
    ~GraphCleanup() {
      if (gx) cudaGraphExecDestroy(gx);
      if (a) cudaEventDestroy(a);
      if (b) cudaEventDestroy(b);
      if (cs) cudaStreamDestroy(cs);
    }
  } graph_cleanup{cs, ev_in, ev_out, gexec};
  std::vector<CgState> hst(pairs);
  auto residual_norms = [&]() -> int {
    true_residual();
    PG_KSWITCH(k, (k_sg_norm2<K><<<G, kThreads, 0, s>>>(r64, g, part),
                   k_sg_norm_final<K><<<1, kThreads, 0, s>>>(part, g, rnorm)));
    PG_LAUNCH_CHECK();
    PG_CUDA_TRY(cudaMemcpyAsync(rn.data(), rnorm, sizeof(double) * pairs, cudaMemcpyDeviceToHost, s));
    return PG_OK;
  };
  for (;;) {
    const int e0 = residual_norms();
    if (e0) return e0;
    CgCtl hctl;
    PG_CUDA_TRY(cudaMemcpyAsync(&hctl, ctl, sizeof(CgCtl), cudaMemcpyDeviceToHost, s));
    PG_CUDA_TRY(cudaStreamSynchronize(s));
    if (!first && hctl.nonfinite) {
      pg_set_error("pg_cocg_segments: non-finite residual");
      status = PG_ERR_NONFINITE;
      break;
    }
    bool all = true;
    for (int t = 0; t < pairs; ++t) {
      if (monitor)
        fprintf(stderr, "pg_cocg_segments: check %lld its %lld system %d rhs %d true ||r||/||b|| = %.6e\n",
                (long long)checks, (long long)its, t / k, t % k, bnorm[t] > 0 ? rn[t] / bnorm[t] : 0.0);
      if (!isfinite(rn[t])) {
        pg_set_error("pg_cocg_segments: non-finite residual");
        status = PG_ERR_NONFINITE;
      }
      const double tb = o->rtol * bnorm[t];
      const bool ok = rn[t] <= tb || bnorm[t] == 0.0;
      wnt[t] = ok ? 0 : 1;
      sc[t] = rn[t] > 0.0 && isfinite(rn[t]) ? rn[t] : 1.0;
      tgt[t] = 0.5 * tb / sc[t];
      if (!ok) all = false;
    }
    if (status || all) break;
    if (its >= max_it) {
      status = PG_ERR_NOT_CONVERGED;
      break;
    }
    for (int t = 0; t < pairs; ++t) {
      scal[t] = rn[t] > 0.0 ? 1.0 : 0.0;
      scal[pairs + t] = sc[t];
      scal[2 * pairs + t] = 1.0 / sc[t];
      scal[3 * pairs + t] = sc_prev[t] / sc[t];
      sc_prev[t] = sc[t];
    }
    PG_CUDA_TRY(cudaMemcpyAsync(target, tgt.data(), sizeof(double) * pairs, cudaMemcpyHostToDevice, s));
    PG_CUDA_TRY(cudaMemcpyAsync(want, wnt.data(), sizeof(int) * pairs, cudaMemcpyHostToDevice, s));
    PG_CUDA_TRY(cudaMemcpyAsync(rnorm, scal.data(), sizeof(double) * pairs, cudaMemcpyHostToDevice, s));
    PG_CUDA_TRY(cudaMemcpyAsync(cscale, scal.data() + pairs, sizeof(double) * 3 * pairs, cudaMemcpyHostToDevice, s));
    PG_KSWITCH(k, (k_sg_scale_d2<K><<<pg_blocks(P.n * K, 256), 256, 0, s>>>(r64, g, P.n, cinv)));
    if (!first) PG_KSWITCH(k, (k_sg_scale_df<K><<<pg_blocks(P.n * K, 256), 256, 0, s>>>(pv, g, P.n, clam)));
    // systems already converged keep one idle block; the others take the rest
    for (int j = 0; j < P.S; ++j) {
      sys_active[j] = 0;
      for (int i = 0; i < k; ++i) sys_active[j] |= (char)wnt[j * k + i];
    }
    seg_rebalance(hrows, P.S, k, sys_active, G, cur_blk);
    if (cur_blk != hblk) {
      hblk = cur_blk;
      PG_CUDA_TRY(cudaMemcpyAsync(dblk, hblk.data(), sizeof(int) * (P.S + 1), cudaMemcpyHostToDevice, s));
    }
    if (bj)
      for (int j = 0; j < P.S; ++j) {
        const BjInfo& B = P.bj[j];
        if (B.n == 0) continue;
        PG_KSWITCH(k, (k_bj_apply<K><<<pg_blocks(B.n * K, 256), 256, 0, s>>>(Sblk + P.soff[j], B, r64 + hrows[j] * K,
                                                                             r64b + hrows[j] * K)));
      }
    PG_KSWITCH(k, (k_sg_start<K><<<G, kThreads, 0, s>>>(bj ? r64b : r64, Sd, g, r, y, pv, first ? 1 : 0, part),
                   k_sg_cycle_init<K><<<1, kThreads, 0, s>>>(part, g, st, rnorm, target, want, ctl, first ? 1 : 0)));
    first = false;
    const int steps = (int)((max_it - its) < chunk ? (max_it - its) : chunk);
    int done = 0;
    if (use_graphs && steps >= kGraphIters) {
      if (!gexec) build_graph();
      if (gexec) {
        cudaEventRecord(ev_in, s);
        cudaStreamWaitEvent(cs, ev_in, 0);
        for (; done + kGraphIters <= steps; done += kGraphIters) cudaGraphLaunch(gexec, cs);
        cudaEventRecord(ev_out, cs);
        cudaStreamWaitEvent(s, ev_out, 0);
      }
    }
    for (; done < steps; ++done) one_iteration(s);
    PG_LAUNCH_CHECK();
    PG_KSWITCH(k, (k_sg_scale_df<K><<<pg_blocks(P.n * K, 256), 256, 0, s>>>(y, g, P.n, cscale)));
    if (bj) {
      for (int j = 0; j < P.S; ++j) {
        const BjInfo& B = P.bj[j];
        if (B.n == 0) continue;
        PG_KSWITCH(k, (k_bj_apply_t_add<K><<<pg_blocks(B.n * K, 256), 256, 0, s>>>(
                           Sblk + P.soff[j], B, y + hrows[j] * K, x + hrows[j] * K, DfToD2())));
      }
    } else {
      PG_KSWITCH(k, (k_df_xupdate<K><<<pg_blocks(P.n * K, kThreads), kThreads, 0, s>>>(y, Sd, P.n, x)));
    }
    PG_CUDA_TRY(cudaMemcpyAsync(hst.data(), st, sizeof(CgState) * pairs, cudaMemcpyDeviceToHost, s));
    PG_CUDA_TRY(cudaStreamSynchronize(s));
    int used = 0;
    bool brk = false;
    for (int t = 0; t < pairs; ++t) {
      used = hst[t].its > used ? hst[t].its : used;
      brk = brk || hst[t].breakdown;
    }
    const int64_t cycle_its = used - its;
    its = used;
    ++checks;
    if (brk) {
      pg_set_error("pg_cocg_segments: breakdown (p^T A p = 0 or r^T r = 0)");
      status = PG_ERR_BREAKDOWN;
      const int e1 = residual_norms();
      if (e1) return e1;
      PG_CUDA_TRY(cudaStreamSynchronize(s));
      break;
    }
    int64_t c2 = cycle_its + cycle_its / 4 + 8;
    chunk = (int)(c2 < 16 ? 16 : (c2 > 4000 ? 4000 : c2));
  }
  if (its_out) {
    PG_CUDA_TRY(cudaMemcpyAsync(hst.data(), st, sizeof(CgState) * pairs, cudaMemcpyDeviceToHost, s));
    PG_CUDA_TRY(cudaStreamSynchronize(s));
    for (int t = 0; t < pairs; ++t) its_out[t] = first ? 0 : hst[t].its;
  }
  double worst = 0.0;
  for (int t = 0; t < pairs; ++t) {
    const double rr = bnorm[t] > 0 ? rn[t] / bnorm[t] : 0.0;
    if (relres_out) relres_out[t] = rr;
    worst = rr > worst ? rr : worst;
  }
  if (res) {
    res->iterations = its;
    res->restarts = checks;
    res->relres = worst;
    res->status = status;
  }
  if (status == PG_ERR_NOT_CONVERGED) pg_set_error("pg_cocg_segments: max_it reached before rtol");
  return status;
}

bool valid_k(int k) { return k == 1 || k == 2 || k == 4 || k == 8 || k == 16 || k == 32; }

}  // namespace

extern "C" void pg_gmres_default_opts(pg_gmres_opts* o) {
  if (!o) return;
  memset(o, 0, sizeof(*o));
  o->restart = 30;
  o->max_it = 10000;
  o->rtol = 1e-8;
  o->precision = 0;
  o->reorth = 0;
}

static Plan gmres_plan(int64_t n, int64_t nnz, int nrhs, const pg_gmres_opts* o) {
  Plan P{n, nnz, nrhs, o->restart, o->precision, pick_blocks(n, nrhs),
         o->precision ? sizeof(float2) : sizeof(double2)};
  if (o->block_p >= 1 && o->block_p <= 6) P.bj = BjInfo{o->block_edges, o->block_faces, o->block_volumes, o->block_p, n};
  return P;
}

extern "C" size_t pg_gmres_workspace_bytes(int64_t n, int64_t nnz, int nrhs, const pg_gmres_opts* opts) {
  if (!opts || n < 1 || !valid_k(nrhs)) return 0;
  Plan P = gmres_plan(n, nnz, nrhs, opts);
  size_t off[16];
  return ws_layout(P, off) + 256;
}

extern "C" int pg_gmres(const int64_t* rowptr, const int32_t* col, const double* vals, int64_t n, int64_t nnz,
                        const double* b, double* x, int nrhs, const pg_gmres_opts* opts, pg_gmres_result* result,
                        double* relres_per_rhs, void* workspace, size_t workspace_bytes, void* stream) {
  if (!opts || !rowptr || !col || !vals || !b || !x || n < 1 || nnz < n || !valid_k(nrhs)) {
    pg_set_error("pg_gmres: bad argument (nrhs must be 1, 2, 4, 8, 16 or 32)");
    return PG_ERR_ARG;
  }
  if (opts->restart < 1 || opts->restart > kMaxM || !(opts->rtol > 0.0) ||
      (opts->precision != 0 && opts->precision != 1)) {
    pg_set_error("pg_gmres: restart must be 1..64, rtol > 0, precision 0 or 1");
    return PG_ERR_ARG;
  }
  if (opts->block_p > 0) {
    const int64_t pp = opts->block_p;
    const int64_t nb_dofs = opts->block_edges * pp + opts->block_faces * pp * (pp - 1) +
                            opts->block_volumes * (pp * (pp - 1) * (pp - 2) / 2);
    if (opts->block_p > 6 || opts->block_edges < 0 || opts->block_faces < 0 || opts->block_volumes < 0 ||
        nb_dofs != n) {
      pg_set_error("pg_gmres: block-Jacobi entity counts do not match n");
      return PG_ERR_ARG;
    }
  }
  const size_t need = pg_gmres_workspace_bytes(n, nnz, nrhs, opts);
  if (!workspace || workspace_bytes < need) {
    pg_set_error("pg_gmres: workspace too small");
    return PG_ERR_WORKSPACE;
  }
  char* ws = reinterpret_cast<char*>(((uintptr_t)workspace + 255) & ~(uintptr_t)255);
  Plan P = gmres_plan(n, nnz, nrhs, opts);
  cudaStream_t s = pg_stream(stream);
  const double2* A = reinterpret_cast<const double2*>(vals);
  const double2* bb = reinterpret_cast<const double2*>(b);
  double2* xx = reinterpret_cast<double2*>(x);
  if (P.prec == 0) return run_gmres<double2>(P, rowptr, col, A, bb, xx, opts, result, relres_per_rhs, ws, s);
  return run_gmres<float2>(P, rowptr, col, A, bb, xx, opts, result, relres_per_rhs, ws, s);
}

extern "C" int pg_spmv_z(const int64_t* rowptr, const int32_t* col, const double* vals, int64_t n_rows, const double* x,
                         double* y, int nrhs, void* stream) {
  if (!rowptr || !col || !vals || !x || !y || n_rows < 1 || !valid_k(nrhs)) {
    pg_set_error("pg_spmv_z: bad argument");
    return PG_ERR_ARG;
  }
  Plan P{n_rows, 0, nrhs, 1, 0, 1, sizeof(double2)};
  launch_spmv<double2>(P, rowptr, col, reinterpret_cast<const double2*>(vals), reinterpret_cast<const double2*>(x),
                       reinterpret_cast<double2*>(y), nullptr, nullptr, 43, pg_stream(stream));
  PG_LAUNCH_CHECK();
  return PG_OK;
}

extern "C" int pg_spmv_c(const int64_t* rowptr, const int32_t* col, const float* vals, int64_t n_rows, const float* x,
                         float* y, int nrhs, void* stream) {
  if (!rowptr || !col || !vals || !x || !y || n_rows < 1 || !valid_k(nrhs)) {
    pg_set_error("pg_spmv_c: bad argument");
    return PG_ERR_ARG;
  }
  Plan P{n_rows, 0, nrhs, 1, 1, 1, sizeof(float2)};
  launch_spmv<float2>(P, rowptr, col, reinterpret_cast<const float2*>(vals), reinterpret_cast<const float2*>(x),
                      reinterpret_cast<float2*>(y), nullptr, nullptr, 43, pg_stream(stream));
  PG_LAUNCH_CHECK();
  return PG_OK;
}

extern "C" void pg_cocg_default_opts(pg_cocg_opts* o) {
  if (!o) return;
  memset(o, 0, sizeof(*o));
  o->max_it = 100000;
  o->rtol = 1e-8;
  o->precision = 0;
  o->check_every = 50;
}

static Plan cg_plan(int64_t n, int64_t nnz, int nrhs, const pg_cocg_opts* o) {
  int nb = pick_blocks(n, nrhs);
  if (nb < 152 * 16) nb = 152 * 16;  // partials also hold the SpMV's per-block sums
  Plan P{n, nnz, nrhs, 1, o->precision, nb, o->precision == 1 ? sizeof(float2) : sizeof(double2), BjInfo{}};
  P.bj = BjInfo{o->block_edges, o->block_faces, o->block_volumes, o->block_p, n};
  if (o->block_p < 1 || o->block_p > 6) P.bj.p = 0;
  return P;
}

extern "C" size_t pg_cocg_workspace_bytes(int64_t n, int64_t nnz, int nrhs, const pg_cocg_opts* opts) {
  if (!opts || n < 1 || !valid_k(nrhs)) return 0;
  Plan P = cg_plan(n, nnz, nrhs, opts);
  size_t off[20];
  return (opts->precision == 2 ? df_layout(P, off) : cg_layout(P, off)) + 256;
}

extern "C" int pg_cocg(const int64_t* rowptr, const int32_t* col, const double* vals, int64_t n, int64_t nnz,
                       const double* b, double* x, int nrhs, const pg_cocg_opts* opts, pg_gmres_result* result,
                       double* relres_per_rhs, void* workspace, size_t workspace_bytes, void* stream) {
  if (!opts || !rowptr || !col || !vals || !b || !x || n < 1 || nnz < n || !valid_k(nrhs) || !(opts->rtol > 0.0) ||
      opts->precision < 0 || opts->precision > 2) {
    pg_set_error("pg_cocg: bad argument (nrhs 1..32 power of two, rtol > 0, precision 0/1/2)");
    return PG_ERR_ARG;
  }
  if (opts->block_p > 0) {
    const int64_t pp = opts->block_p;
    const int64_t nb_dofs = opts->block_edges * pp + opts->block_faces * pp * (pp - 1) +
                            opts->block_volumes * (pp * (pp - 1) * (pp - 2) / 2);
    if (opts->block_p > 6 || opts->block_edges < 0 || opts->block_faces < 0 || opts->block_volumes < 0 ||
        nb_dofs != n) {
      pg_set_error("pg_cocg: block-Jacobi entity counts do not match n");
      return PG_ERR_ARG;
    }
  }
  const size_t need = pg_cocg_workspace_bytes(n, nnz, nrhs, opts);
  if (!workspace || workspace_bytes < need) {
    pg_set_error("pg_cocg: workspace too small");
    return PG_ERR_WORKSPACE;
  }
  char* ws = reinterpret_cast<char*>(((uintptr_t)workspace + 255) & ~(uintptr_t)255);
  Plan P = cg_plan(n, nnz, nrhs, opts);
  cudaStream_t s = pg_stream(stream);
  const double2* A = reinterpret_cast<const double2*>(vals);
  const double2* bb = reinterpret_cast<const double2*>(b);
  double2* xx = reinterpret_cast<double2*>(x);
  if (P.prec == 0) return run_cocg<double2>(P, rowptr, col, A, bb, xx, opts, result, relres_per_rhs, ws, s);
  if (P.prec == 2) return run_cocg_df(P, rowptr, col, A, bb, xx, opts, result, relres_per_rhs, ws, s);
  return run_cocg<float2>(P, rowptr, col, A, bb, xx, opts, result, relres_per_rhs, ws, s);
}

extern "C" size_t pg_cocg_multifreq_workspace_bytes(int64_t n, int64_t nnz, int nrhs) {
  if (n < 1 || !valid_k(nrhs)) return 0;
  pg_cocg_opts o;
  pg_cocg_default_opts(&o);
  o.precision = 2;
  Plan P = cg_plan(n, nnz, nrhs, &o);
  size_t off[20];
  return df_layout(P, off, true) + 256;
}

extern "C" int pg_cocg_multifreq(const int64_t* rowptr, const int32_t* col, const double* vals, int64_t n, int64_t nnz,
                                 const double* b, double* x, int nrhs, const double* col_scale,
                                 const pg_cocg_opts* opts, pg_gmres_result* result, double* relres_per_rhs,
                                 void* workspace, size_t workspace_bytes, void* stream) {
  if (!opts || !rowptr || !col || !vals || !b || !x || !col_scale || n < 1 || nnz < n || !valid_k(nrhs) ||
      !(opts->rtol > 0.0) || opts->precision != 2) {
    pg_set_error("pg_cocg_multifreq: bad argument (nrhs 1..32 power of two, rtol > 0, precision 2)");
    return PG_ERR_ARG;
  }
  for (int i = 0; i < nrhs; ++i)
    if (!(col_scale[i] > 0.0) || !isfinite(col_scale[i])) {
      pg_set_error("pg_cocg_multifreq: column frequency scales must be positive");
      return PG_ERR_ARG;
    }
  const size_t need = pg_cocg_multifreq_workspace_bytes(n, nnz, nrhs);
  if (!workspace || workspace_bytes < need) {
    pg_set_error("pg_cocg_multifreq: workspace too small");
    return PG_ERR_WORKSPACE;
  }
  char* ws = reinterpret_cast<char*>(((uintptr_t)workspace + 255) & ~(uintptr_t)255);
  Plan P = cg_plan(n, nnz, nrhs, opts);
  return run_cocg_df(P, rowptr, col, reinterpret_cast<const double2*>(vals), reinterpret_cast<const double2*>(b),
                     reinterpret_cast<double2*>(x), opts, result, relres_per_rhs, ws, pg_stream(stream), col_scale);
}

extern "C" size_t pg_cocg_segments_workspace_bytes(int64_t n, int64_t nnz, int nrhs, const int64_t* seg_rows,
                                                   int n_seg, const int64_t* seg_entities, const pg_cocg_opts* opts) {
  if (!opts || n < 1 || !valid_k(nrhs)) return 0;
  SegPlan P;
  if (seg_plan(n, nnz, nrhs, seg_rows, n_seg, seg_entities, opts->block_p, P) != PG_OK) return 0;
  size_t off[18];
  return sg_layout(P, off) + 256;
}

extern "C" int pg_cocg_segments(const int64_t* rowptr, const int32_t* col, const double* vals, int64_t n, int64_t nnz,
                                const int64_t* seg_rows, int n_seg, const int64_t* seg_entities, const double* b,
                                double* x, int nrhs, const pg_cocg_opts* opts, pg_gmres_result* result,
                                double* relres, int64_t* its, void* workspace, size_t workspace_bytes, void* stream) {
  if (!opts || !rowptr || !col || !vals || !b || !x || !seg_rows || n < 1 || nnz < n || n_seg < 1 ||
      !valid_k(nrhs) || !(opts->rtol > 0.0) || opts->precision != 2) {
    pg_set_error("pg_cocg_segments: bad argument (n_seg >= 1, nrhs 1..32 power of two, rtol > 0, precision 2)");
    return PG_ERR_ARG;
  }
  SegPlan P;
  if (seg_plan(n, nnz, nrhs, seg_rows, n_seg, seg_entities, opts->block_p, P) != PG_OK) {
    pg_set_error("pg_cocg_segments: seg_rows must rise from 0 to n; with block_p, seg_entities must give each "
                 "system's (edges, faces, elements) matching its rows");
    return PG_ERR_ARG;
  }
  const size_t need = pg_cocg_segments_workspace_bytes(n, nnz, nrhs, seg_rows, n_seg, seg_entities, opts);
  if (!workspace || workspace_bytes < need) {
    pg_set_error("pg_cocg_segments: workspace too small");
    return PG_ERR_WORKSPACE;
  }
  char* ws = reinterpret_cast<char*>(((uintptr_t)workspace + 255) & ~(uintptr_t)255);
  return run_cocg_seg(P, seg_rows, rowptr, col, reinterpret_cast<const double2*>(vals),
                      reinterpret_cast<const double2*>(b), reinterpret_cast<double2*>(x), opts, result, relres, its,
                      ws, pg_stream(stream));
}
