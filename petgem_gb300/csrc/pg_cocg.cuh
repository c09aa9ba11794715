// Shared pieces of the COCG solvers: per-RHS state and control block,
// last-block reductions, Jacobi and entity block-Jacobi setup, the
// double-float arithmetic and its reductions, and the solver entry points
// that cross translation units.
#pragma once
#include "pg_krylov.cuh"

namespace {

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

// ----------------------------------------------------------------------------
// Gradient correction (Hiptmair's hybrid smoother) on the Jacobi-scaled system
// At = S A S:  z = r + S^-1 G diag(G^T A G)^-1 G^T S^-1 r, which is
// B = D^-1 + G diag(G^T A G)^-1 G^T in the unscaled variables.  G is real;
// its rows (CSR) drive the prolongation, its transpose (rows ascending) the
// restriction, so both sums run in a fixed order.
// ----------------------------------------------------------------------------

__global__ void k_grad_sinv(const double2* S, int64_t n, double2* Sinv) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x)
    Sinv[r] = ddiv(make_double2(1.0, 0.0), S[r]);
}

// Gradient correction, later cycles: the recurrence continues (r, p, rho,
// the residual estimate are kept; y restarts at 0 after x += S y) instead
// of restarting from the true residual.  Replacing r by b - A x would inject
// the true residual's rounding in the directions the correction amplifies
// (gradient fields of nearly non-conducting regions, where invD is largest),
// which can make the iteration diverge; the FP64 recurrence needs no
// replacement.  RHS whose true residual converged stop (want = 0).
template <int K>
__global__ void k_cg_cycle_keep(CgState* st, const double* target, const int* want, CgCtl* ctl) {
  __shared__ int any;
  if (threadIdx.x == 0) any = 0;
  __syncthreads();
  if (threadIdx.x < K) {
    CgState& S = st[threadIdx.x];
    S.target = target[threadIdx.x];
    S.res0 = S.res;
    S.active = want[threadIdx.x] && S.active;
    if (S.active) atomicOr(&any, 1);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    ctl->any_active = any;
    ctl->nonfinite = 0;
    ctl->counter = 0;
  }
}

// FP32 restriction of the gradient correction, shared by the double-float and
// complex64 solvers: t = invD .* (G^T u), u = S^-1 r in FP32 (the correction
// only shapes the search direction).  Inside an iteration it runs only when
// this iteration's update ran (ctl->pending, cleared by the next product);
// start = 1 at a cycle start.
__global__ void k_to_f32(const double2* __restrict__ a, int64_t n, float2* __restrict__ out) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
    out[e] = make_float2((float)a[e].x, (float)a[e].y);
}

// acc += sum_j g_j v[c_j * K + rhs] over [j0, j1) of a map row (FP32 products
// of the FP64 map values), accumulated in entry order; four entries' index
// and value loads are issued before their four gathers, so a thread keeps
// four independent gathers in flight instead of one dependent chain.
template <int K>
__device__ __forceinline__ void grad_gather4(const int32_t* __restrict__ gc, const double* __restrict__ gv,
                                             const float2* __restrict__ v, int64_t j, int rhs, float2& acc) {
  int32_t c[4];
  float g[4];
  float2 w[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    c[i] = gc[j + i];
    g[i] = __double2float_rn(gv[j + i]);
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) w[i] = v[(int64_t)c[i] * K + rhs];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    acc.x = fmaf(g[i], w[i].x, acc.x);
    acc.y = fmaf(g[i], w[i].y, acc.y);
  }
}

template <int K>
__device__ __forceinline__ void grad_gather1(const int32_t* __restrict__ gc, const double* __restrict__ gv,
                                             const float2* __restrict__ v, int64_t j, int rhs, float2& acc) {
  const float g = __double2float_rn(gv[j]);
  const float2 w = v[(int64_t)gc[j] * K + rhs];
  acc.x = fmaf(g, w.x, acc.x);
  acc.y = fmaf(g, w.y, acc.y);
}

template <int K>
__device__ __forceinline__ void grad_row_acc(const int32_t* __restrict__ gc, const double* __restrict__ gv,
                                             const float2* __restrict__ v, int64_t j0, int64_t j1, int rhs,
                                             float2& acc) {
  int64_t j = j0;
  for (; j + 4 <= j1; j += 4) grad_gather4<K>(gc, gv, v, j, rhs, acc);
  for (; j < j1; ++j) grad_gather1<K>(gc, gv, v, j, rhs, acc);
}

template <int K>
__device__ __forceinline__ float2 grad_row_sum(const int32_t* __restrict__ gc, const double* __restrict__ gv,
                                               const float2* __restrict__ v, int64_t j0, int64_t j1, int rhs) {
  float2 acc = make_float2(0.f, 0.f);
  grad_row_acc<K>(gc, gv, v, j0, j1, rhs, acc);
  return acc;
}

// PC (several frequencies): A_j = Re A0 + i s_j Im A0 and G is real, so
// column j's diag(G^T A_j G) is Re d + i s_j Im d with d = diag(G^T A0 G)
// (invD holds d; cscale the s_j).  Re d vanishes on gradient columns
// (G^T K G = 0) but not on vector P1 columns.  K >= 4: a thread takes one
// column and 4 RHS (kGradQ), loading each gathered u row slice as two 16-byte
// vectors and the entry's index and value once for the 4; every RHS is
// still summed in entry order.  Launch ceil(gn * K / kGradQ(K)) threads.
__host__ __device__ constexpr int kGradQ(int k) { return k >= 4 ? 4 : 1; }

template <int K, bool PC = false>
__global__ void __launch_bounds__(kThreads) k_grad_restrict32(const int64_t* __restrict__ gtp,
                                                           const int32_t* __restrict__ gtr,
                                                           const double* __restrict__ gtv,
                                                           const float2* __restrict__ invD,
                                                           const float2* __restrict__ u, int64_t gn,
                                                           float2* __restrict__ t, const CgCtl* ctl, int start,
                                                           const float* __restrict__ cscale = nullptr) {
  if (!start && !ctl->pending) return;
  auto scaled = [&](int64_t c, int rhs, float2 acc) {
    if (PC) {
      // invD holds the diagonal d of G^T A0 G; column rhs divides by
      // Re d + i s_j Im d (scaled by the larger part against underflow)
      const float2 d = invD[c];
      float dx = d.x, dy = cscale[rhs] * d.y;
      const float m = fmaxf(fabsf(dx), fabsf(dy));
      if (m > 0.f) {
        dx /= m;
        dy /= m;
        const float den = m * fmaf(dx, dx, dy * dy);
        return make_float2(fmaf(acc.x, dx, acc.y * dy) / den, fmaf(acc.y, dx, -acc.x * dy) / den);
      }
      return make_float2(0.f, 0.f);
    }
    return cmul(invD[c], acc);
  };
  constexpr int Q = kGradQ(K), KQ = K / Q;
  const int64_t total = gn * KQ;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = e / KQ;
    if constexpr (Q == 1) {
      const int rhs = (int)(e % KQ);
      t[e] = scaled(c, rhs, grad_row_sum<K>(gtr, gtv, u, gtp[c], gtp[c + 1], rhs));
    } else {
      // RHS r0 .. r0 + 3: u rows and t are 8-byte complex values with K a
      // multiple of 4, so each slice starts on a 32-byte boundary
      const int r0 = (int)(e % KQ) * Q;
      float2 acc[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[q] = make_float2(0.f, 0.f);
      const int64_t j1 = gtp[c + 1];
#pragma unroll 2
      for (int64_t j = gtp[c]; j < j1; ++j) {
        const float g = __double2float_rn(gtv[j]);
        const float4* up = reinterpret_cast<const float4*>(u + (int64_t)gtr[j] * K + r0);
        const float4 a = up[0], b = up[1];
        acc[0].x = fmaf(g, a.x, acc[0].x);
        acc[0].y = fmaf(g, a.y, acc[0].y);
        acc[1].x = fmaf(g, a.z, acc[1].x);
        acc[1].y = fmaf(g, a.w, acc[1].y);
        acc[2].x = fmaf(g, b.x, acc[2].x);
        acc[2].y = fmaf(g, b.y, acc[2].y);
        acc[3].x = fmaf(g, b.z, acc[3].x);
        acc[3].y = fmaf(g, b.w, acc[3].y);
      }
      float2 w[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) w[q] = scaled(c, r0 + q, acc[q]);
      float4* tp = reinterpret_cast<float4*>(t + c * K + r0);
      tp[0] = make_float4(w[0].x, w[0].y, w[1].x, w[1].y);
      tp[1] = make_float4(w[2].x, w[2].y, w[3].x, w[3].y);
    }
  }
}

// true when some RHS ran this iteration's update (iter < 0: always)
template <int K>
__device__ __forceinline__ bool grad_due(const CgState* st, int iter) {
  if (iter < 0) return true;
  bool any = false;
  for (int i = 0; i < K; ++i) any |= st[i].beta_iter == iter;
  return any;
}

// t = invD .* (G^T u), u = S^-1 r (K RHS interleaved)
template <int K>
__global__ void __launch_bounds__(kThreads) k_grad_restrict(const int64_t* __restrict__ gtp,
                                                            const int32_t* __restrict__ gtr,
                                                            const double* __restrict__ gtv,
                                                            const double2* __restrict__ invD,
                                                            const double2* __restrict__ u, int64_t gn,
                                                            double2* __restrict__ t, const CgState* st, int iter) {
  if (!grad_due<K>(st, iter)) return;
  const int64_t total = gn * K;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = e / K;
    const double2 acc = grad_row_sum64<K>(gtr, gtv, u, gtp[c], gtp[c + 1], (int)(e % K));
    t[e] = cmul(invD[c], acc);
  }
}

// z = r + S^-1 (G t); partial rho = r^T z.  iter >= 0 (inside an iteration):
// the last block sets beta = rho / rho_old and rho for every RHS that ran
// this iteration's update.  iter < 0 (cycle start): partials only, and p = z
// when set_p.
template <int K>
__global__ void __launch_bounds__(kThreads) k_grad_prolong(const int64_t* __restrict__ gp,
                                                           const int32_t* __restrict__ gc,
                                                           const double* __restrict__ gv,
                                                           const double2* __restrict__ Sinv,
                                                           const double2* __restrict__ t,
                                                           const double2* __restrict__ r, int64_t n,
                                                           double2* __restrict__ z, double2* __restrict__ pv,
                                                           int set_p, double2* prho, CgState* st, CgCtl* ctl,
                                                           int iter) {
  if (!grad_due<K>(st, iter)) return;
  __shared__ double2 smem[2 * (kThreads / 32) * kMaxK];
  const int64_t total = n * K;
  const int64_t chunk = ((total + gridDim.x - 1) / gridDim.x + K - 1) / K * K;
  const int64_t lo = (int64_t)blockIdx.x * chunk, hi = min(total, lo + chunk);
  double2 rho = make_double2(0.0, 0.0);
  for (int64_t e = lo + threadIdx.x; e < hi; e += kThreads) {
    const int64_t row = e / K;
    const double2 acc = grad_row_sum64<K>(gc, gv, t, gp[row], gp[row + 1], (int)(e % K));
    const double2 re = r[e];
    const double2 ze = dadd(re, cmul(Sinv[row], acc));
    z[e] = ze;
    if (set_p) pv[e] = ze;
    rho = dadd(rho, cmul(re, ze));
  }
  block_reduce_rhs<K>(rho, smem, prho + (int64_t)blockIdx.x * K);
  if (iter >= 0 && arrive_last(&ctl->counter)) {
    const double2 rr = sum_partials<K>(prho, gridDim.x, threadIdx.x < K ? threadIdx.x : 0, smem);
    if (threadIdx.x < K) {
      CgState& S = st[threadIdx.x];
      if (S.beta_iter == iter) {
        if (S.rho.x == 0.0 && S.rho.y == 0.0) {
          S.breakdown = 1;
          S.active = 0;
          S.beta = make_double2(0.0, 0.0);
        } else {
          S.beta = ddiv(rr, S.rho);
        }
        S.rho = rr;
      } else {
        S.beta = make_double2(0.0, 0.0);
      }
    }
    if (threadIdx.x == 0) ctl->counter = 0;
  }
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

// The same when a thread holds 4 RHS, r0 .. r0 + 3 with r0 = 4 (lane % (K /
// 4)) (K >= 4): lanes with the same r0 are combined, then the warps in order.
template <int K>
__device__ void block_reduce_df_q4(const float4 (&rho)[4], float4* smf, double2* out) {
  constexpr int KQ = K / 4;
  float4 v[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    v[q] = rho[q];
#pragma unroll
    for (int off = 16; off >= KQ; off >>= 1) cdf_add(v[q], shfl_xor4(v[q], off));
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane < KQ) {
#pragma unroll
    for (int q = 0; q < 4; ++q) smf[warp * K + lane * 4 + q] = v[q];
  }
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

// spike: a cycle also ends when a column's residual estimate exceeds spike
// times its starting value (COCG's residual norm is not monotone; a
// recurrence carried far past such a spike has lost accuracy)
// GRAD (gradient correction): rho and beta are left to the prolongation,
// which forms z first.
template <int K, bool GRAD = false>
__device__ void cg_beta_final(const double2* prho, const double2* pw, int nblocks, CgState* st, CgCtl* ctl, int iter,
                              double delta, double2* smem, double spike = 1e3) {
  const int my = threadIdx.x < K ? threadIdx.x : 0;
  double2 rho = make_double2(0.0, 0.0);
  if constexpr (!GRAD) rho = sum_partials<K>(prho, nblocks, my, smem);
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
      if constexpr (!GRAD) {
        if (S.rho.x == 0.0 && S.rho.y == 0.0) {
          S.breakdown = 1;
          S.active = 0;
          S.beta = make_double2(0.0, 0.0);
        } else {
          S.beta = ddiv(rho, S.rho);
        }
        S.rho = rho;
      }
      if (S.res <= S.target || !isfinite(S.res)) S.active = 0;
      else if (S.res <= delta * S.res0 || S.res > spike * S.res0) atomicOr(&stop, 1);
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

__global__ void k_df_scale_matrix(const int64_t* rowptr, const int32_t* col, const double2* val, int64_t n,
                                  const double2* S, float4* out, float* wdf, const double* wd) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    const double2 sr = S[r];
    for (int64_t k = rowptr[r]; k < rowptr[r + 1]; ++k) out[k] = cdf_from(cmul(sr, cmul(val[k], S[col[k]])));
    wdf[r] = (float)wd[r];
  }
}

template <int K, bool PC = false>
__global__ void k_df_xupdate(const float4* __restrict__ y, const double2* __restrict__ S, int64_t n, double2* x) {
  const int64_t total = n * K;
  for (int64_t e = (int64_t)blockIdx.x * kThreads + threadIdx.x; e < total; e += (int64_t)gridDim.x * kThreads)
    x[e] = dadd(x[e], cmul(S[PC ? e : e / K], cdf_to(y[e])));
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

inline Plan cg_plan(int64_t n, int64_t nnz, int nrhs, const pg_cocg_opts* o) {
  int nb = pick_blocks(n, nrhs);
  if (nb < 152 * 16) nb = 152 * 16;  // partials also hold the SpMV's per-block sums
  Plan P{n, nnz, nrhs, 1, o->precision, nb, o->precision == 1 ? sizeof(float2) : sizeof(double2), BjInfo{}};
  P.bj = BjInfo{o->block_edges, o->block_faces, o->block_volumes, o->block_p, n};
  if (o->block_p < 1 || o->block_p > 6) P.bj.p = 0;
  P.gn = o->grad_rowptr && o->grad_cols > 0 ? o->grad_cols : 0;
  return P;
}

// ---- product variants shared by the double-float solvers ------------------
// The entity-group check and the on-line autotuner: at the first cycle of a
// solve each candidate product runs 3 times on the actual operands (the
// product is the first kernel of an iteration and recomputes alpha, so the
// extra runs change no solver state) and the fastest is kept.
// PG_AUTOTUNE=0 keeps the default variant.
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

bool autotune_enabled() {
  const char* e = getenv("PG_AUTOTUNE");
  return !(e && e[0] == '0');
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

}  // namespace

namespace pgk {

// workspace layout of the double-float COCG (mf: several frequencies)
size_t df_layout(const Plan& P, size_t* off /* 28 */, bool mf = false);
// double-float COCG; col_scale (host [k]) selects the several-frequencies form
int run_cocg_df(const Plan& P, const int64_t* rowptr, const int32_t* col, const double2* A, const double2* b, double2* x,
                const pg_cocg_opts* o, pg_gmres_result* res, double* relres_out, char* ws, cudaStream_t s,
                const double* col_scale = nullptr);

// workspace layout and driver of the complex64-inner / FP64-refinement COCG
size_t ir_layout(const Plan& P, size_t* off /* 16 */);
int run_cocg_ir(const Plan& P, const int64_t* rowptr, const int32_t* col, const double2* A, const double2* b,
                double2* x, const pg_cocg_opts* o, pg_gmres_result* res, double* relres_out, char* ws,
                cudaStream_t s);

}  // namespace pgk
