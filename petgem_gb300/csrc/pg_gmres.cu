// Restarted GMRES for petgem's complex system A x = b (petgem/solver.py:584-594,
// PETSc KSP with -ksp_type gmres and -pc_type jacobi or bjacobi), for one or
// several right-hand sides at once.
//
// Structure (same code for both precisions, templated on the Arnoldi scalar):
//   loop over restarts:
//     r = b - A x                    complex128 CSR SpMV/SpMM with the original A
//     stop when ||r|| <= rtol ||b|| for every RHS (true residual, FP64)
//     one Arnoldi cycle of m steps on  Ahat = A M^-1  (right preconditioning:
//     M = D, or the entity blocks A_aa), in the Arnoldi precision:
//     complex128 ("fp64") or complex64 ("mixed")
//     x += M^-1 V y                  FP64 update
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
#include "pg_krylov.cuh"

namespace {

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

// v~_0 = r / ||r|| (cast to C)
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

// Gradient correction, right preconditioning B = D^-1 T with
// T v = v + D G invD G^T v (invD = diag(G^T A G)^-1): the Arnoldi product is
// Ahat (T v), Ahat = A D^-1, and the update x += D^-1 T (V y).
// t = invD .* (G^T v)
template <typename C, int K>
__global__ void __launch_bounds__(kThreads) k_gm_restrict(const int64_t* __restrict__ gtp,
                                                          const int32_t* __restrict__ gtr,
                                                          const double* __restrict__ gtv,
                                                          const double2* __restrict__ invD,
                                                          const C* __restrict__ v, int64_t gn,
                                                          double2* __restrict__ t, const Ctl* ctl) {
  if (ctl && !ctl->any_active) return;
  const int64_t total = gn * K;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = e / K;
    const double2 acc = grad_row_sum64<K>(gtr, gtv, v, gtp[c], gtp[c + 1], (int)(e % K));
    t[e] = cmul(invD[c], acc);
  }
}

// u = v + d .* (G t)
template <typename C, int K>
__global__ void __launch_bounds__(kThreads) k_gm_prolong(const int64_t* __restrict__ gp,
                                                         const int32_t* __restrict__ gc,
                                                         const double* __restrict__ gv,
                                                         const double2* __restrict__ d,
                                                         const double2* __restrict__ t, const C* __restrict__ v,
                                                         int64_t n, C* __restrict__ u, const Ctl* ctl) {
  if (ctl && !ctl->any_active) return;
  const int64_t total = n * K;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t row = e / K;
    const double2 acc = grad_row_sum64<K>(gc, gv, t, gp[row], gp[row + 1], (int)(e % K));
    u[e] = cfrom<C>(dadd(to_d(v[e]), cmul(d[row], acc)));
  }
}

// x += dinv .* u
template <int K>
__global__ void k_gm_xadd(const double2* __restrict__ dinv, const double2* __restrict__ u, int64_t n,
                          double2* __restrict__ x) {
  const int64_t total = n * K;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x)
    x[e] = dadd(x[e], cmul(dinv[e / K], u[e]));
}

__global__ void k_recip(const double2* a, int64_t n, double2* out) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x)
    out[r] = ddiv(make_double2(1.0, 0.0), a[r]);
}

size_t ws_layout(const Plan& P, size_t* off /* 24 */) {
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
  // gradient correction: invD, t, u = T v (Arnoldi precision), d = diag A, ones
  put(16, P.gn ? sizeof(double2) * P.gn : 0);
  put(17, P.gn ? sizeof(double2) * P.gn * P.k : 0);
  put(18, P.gn ? sizeof(double2) * P.n * P.k : 0);   // Arnoldi precision in the steps, FP64 in the update
  put(19, P.gn ? sizeof(double2) * P.n : 0);
  put(20, P.gn ? sizeof(double2) * P.n : 0);
  return o;
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

template <typename C>
int run_gmres(const Plan& P, const int64_t* rowptr, const int32_t* col, const double2* A, const double2* b, double2* x,
              const pg_gmres_opts* o, pg_gmres_result* res, double* relres_out, char* ws, cudaStream_t s) {
  size_t off[24];
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
  const bool grad = P.gn > 0;   // diagonal Jacobi only (checked by pg_gmres)
  double2* invD = reinterpret_cast<double2*>(ws + off[16]);
  double2* gt = reinterpret_cast<double2*>(ws + off[17]);
  C* gu = reinterpret_cast<C*>(ws + off[18]);
  double2* dA = reinterpret_cast<double2*>(ws + off[19]);
  double2* ones = reinterpret_cast<double2*>(ws + off[20]);
  const unsigned gblocks = pg_blocks(P.gn * P.k, kThreads);
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
    if (grad) {
      k_recip<<<pg_blocks(P.n, 256), 256, 0, s>>>(dinv, P.n, dA);
      k_fill_one<<<pg_blocks(P.n, 256), 256, 0, s>>>(ones, P.n);
      k_grad_diag<<<pg_blocks(P.gn * 32, 256), 256, 0, s>>>(rowptr, col, A, o->gradt_rowptr, o->gradt_row, o->gradt_val,
                                                       P.gn, invD);
    }
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
  // One restart cycle's Arnoldi steps: the launches and their arguments are
  // the same every full cycle (j is fixed per step, converged RHS are
  // skipped through ctl on the device), so a full cycle is captured once in
  // a CUDA graph and replayed; small systems are bound by launch latency.
  auto arnoldi = [&](cudaStream_t ss, int steps) {
    for (int j = 0; j < steps; ++j) {
      C* vj = V + (int64_t)j * stride;
      C* w = V + (int64_t)(j + 1) * stride;
      if (grad) {
        PG_KSWITCH(k, (k_gm_restrict<C, K><<<gblocks, kThreads, 0, ss>>>(o->gradt_rowptr, o->gradt_row, o->gradt_val,
                                                                         invD, vj, P.gn, gt, ctl),
                       k_gm_prolong<C, K><<<pg_blocks(P.n * K, kThreads), kThreads, 0, ss>>>(
                           o->grad_rowptr, o->grad_col, o->grad_val, dA, gt, vj, P.n, gu, ctl)));
        launch_spmv<C>(P, rowptr, col, Ahat, gu, w, nullptr, ctl, npr, ss);
      } else {
        launch_spmv<C>(P, rowptr, col, Ahat, vj, w, nullptr, ctl, npr, ss);
      }
      const int passes = o->reorth ? 2 : 1;
      for (int pass = 0; pass < passes; ++pass) {
        PG_KSWITCH(k, (k_dots<C, K><<<nb, kThreads, 0, ss>>>(V, stride, w, P.n, j, dpart, ctl),
                       k_dots_final<C, K><<<1, 1024, 0, ss>>>(dpart, nb, j, m, st, coef, pass, ctl),
                       k_update<C, K><<<nb, kThreads, 0, ss>>>(V, stride, w, P.n, j, coef, st, pass, npart, ctl)));
      }
      PG_KSWITCH(k, (k_givens<K><<<1, 32 * K, 0, ss>>>(npart, nb, j, m, st, ctl, j == steps - 1)));
    }
  };
  const char* genv = getenv("PG_GRAPHS");
  const bool use_graphs = !(genv && genv[0] == '0');
  cudaStream_t cs = nullptr;
  cudaEvent_t ev_in = nullptr, ev_out = nullptr;
  cudaGraphExec_t gexec = nullptr;
  bool graph_failed = false;
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
  auto build_graph = [&]() {
    cudaGraph_t graph = nullptr;
    bool ok = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) == cudaSuccess &&
              cudaEventCreateWithFlags(&ev_in, cudaEventDisableTiming) == cudaSuccess &&
              cudaEventCreateWithFlags(&ev_out, cudaEventDisableTiming) == cudaSuccess;
    if (ok) ok = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
    if (ok) {
      arnoldi(cs, m);
      ok = cudaStreamEndCapture(cs, &graph) == cudaSuccess && graph != nullptr;
    }
    if (ok) ok = cudaGraphInstantiate(&gexec, graph, 0) == cudaSuccess;
    if (graph) cudaGraphDestroy(graph);
    if (!ok) {
      const cudaError_t e = cudaGetLastError();   // capture unavailable: keep launching directly
      if (monitor) fprintf(stderr, "pg_gmres: cycle graph not captured (%s); launching directly\n", cudaGetErrorString(e));
      gexec = nullptr;
      graph_failed = true;
    } else if (monitor) {
      fprintf(stderr, "pg_gmres: restart cycle of %d steps captured as a CUDA graph\n", m);
    }
  };
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
    bool replayed = false;
    if (use_graphs && steps == m && !graph_failed) {
      if (!gexec) build_graph();
      if (gexec) {
        cudaEventRecord(ev_in, s);
        cudaStreamWaitEvent(cs, ev_in, 0);
        cudaGraphLaunch(gexec, cs);
        cudaEventRecord(ev_out, cs);
        cudaStreamWaitEvent(s, ev_out, 0);
        replayed = true;
      }
    }
    if (!replayed) arnoldi(s, steps);
    PG_LAUNCH_CHECK();
    if (bj) {
      // x += M^-1 (V y): the combination into r (free until the next true residual), then the blocks
      PG_CUDA_TRY(cudaMemsetAsync(r, 0, sizeof(double2) * P.n * k, s));
      PG_KSWITCH(k, (k_backsolve<K><<<1, 32, 0, s>>>(st, m, ycoef),
                     k_update_x<C, K><<<pg_blocks(P.n * K, kThreads), kThreads, 0, s>>>(V, stride, steps, P.n,
                                                                                        ycoef, dinv, r),
                     k_bj_minv_apply_add<K><<<pg_blocks(P.n * K, 256), 256, 0, s>>>(Minv, P.bj, r, x)));
    } else if (grad) {
      // x += D^-1 T (V y): V y into r (free until the next true residual), T into gu, then scale and add
      PG_CUDA_TRY(cudaMemsetAsync(r, 0, sizeof(double2) * P.n * k, s));
      PG_KSWITCH(k, (k_backsolve<K><<<1, 32, 0, s>>>(st, m, ycoef),
                     k_update_x<C, K><<<pg_blocks(P.n * K, kThreads), kThreads, 0, s>>>(V, stride, steps, P.n,
                                                                                        ycoef, ones, r),
                     k_gm_restrict<double2, K><<<gblocks, kThreads, 0, s>>>(o->gradt_rowptr, o->gradt_row,
                                                                             o->gradt_val, invD, r, P.gn, gt, nullptr),
                     k_gm_prolong<double2, K><<<pg_blocks(P.n * K, kThreads), kThreads, 0, s>>>(
                         o->grad_rowptr, o->grad_col, o->grad_val, dA, gt, r, P.n, reinterpret_cast<double2*>(gu),
                         nullptr),
                     k_gm_xadd<K><<<pg_blocks(P.n * K, kThreads), kThreads, 0, s>>>(
                         dinv, reinterpret_cast<double2*>(gu), P.n, x)));
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
  P.gn = o->grad_rowptr && o->grad_cols > 0 ? o->grad_cols : 0;
  return P;
}

extern "C" size_t pg_gmres_workspace_bytes(int64_t n, int64_t nnz, int nrhs, const pg_gmres_opts* opts) {
  if (!opts || n < 1 || !valid_k(nrhs)) return 0;
  Plan P = gmres_plan(n, nnz, nrhs, opts);
  size_t off[24];
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
  if (opts->grad_rowptr) {
    if (!opts->grad_col || !opts->grad_val || !opts->gradt_rowptr || !opts->gradt_row || !opts->gradt_val ||
        opts->grad_cols < 1 || opts->grad_cols >= (int64_t(1) << 31) || opts->block_p > 0) {
      pg_set_error("pg_gmres: gradient correction needs all six G arrays, grad_cols >= 1 and diagonal Jacobi "
                   "(block_p 0)");
      return PG_ERR_ARG;
    }
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

