// COCG (conjugate orthogonal CG) for petgem's complex-symmetric system, in
// complex128 or with a complex64 matrix (FP64 recurrence), and the pg_cocg
// entry point, which also dispatches the double-float form (pg_cocg_df.cu).
// Replaces the KSPSolve of petgem/solver.py:584-594.
#include "pg_cocg.cuh"
#include "pg_sort.cuh"

namespace {

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

// The same product over the rows in the order perm (rows sorted by length):
// the warps of a launch see rows of one length, so no lane idles on a short
// row while its neighbours finish a long one.  Complex128 products are
// FP64-pipe bound and the pipe is charged per warp instruction, active lanes
// or not, so idle lanes and the shuffle-reduction adds are what separates the
// product from its 4 FMAs per stored entry.
template <typename CM, int G>
__global__ void __launch_bounds__(kThreads) k_cg_spmv_sorted(const int64_t* __restrict__ rowptr,
                                                             const int32_t* __restrict__ col,
                                                             const CM* __restrict__ val, int64_t n,
                                                             const int32_t* __restrict__ perm,
                                                             const CM* __restrict__ pm,
                                                             const double2* __restrict__ p64, CM* __restrict__ q,
                                                             double2* partial, CgState* st, CgCtl* ctl) {
  if (!ctl->any_active) return;
  __shared__ double2 smem[2 * (kThreads / 32) * kMaxK];
  const int lane = threadIdx.x % G;
  const int64_t groups = ((int64_t)gridDim.x * blockDim.x) / G;
  const int64_t gid = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / G;
  const int64_t warp_base = gid - (threadIdx.x & 31) / G;
  double2 mu = make_double2(0.0, 0.0);
  for (int64_t iw = warp_base; iw < n; iw += groups) {
    const int64_t i = iw + (gid - warp_base);
    const bool valid = i < n;
    const int64_t r = valid ? perm[i] : 0;
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

// sort keys: row lengths, values: row indices
__global__ void k_row_len_keys(const int64_t* rowptr, int64_t n, uint64_t* keys, int32_t* rows) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    keys[r] = (uint64_t)(rowptr[r + 1] - rowptr[r]);
    rows[r] = (int32_t)r;
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
// or grew above 1e3 * res0), or when all have converged.  GRAD (gradient
// correction): also u = S^-1 r; rho = r^T z and beta are left to
// k_grad_prolong.
template <typename CM, int K, bool GRAD = false>
__global__ void __launch_bounds__(kThreads) k_cg_update(double2* __restrict__ y, double2* __restrict__ r,
                                                        const double2* __restrict__ pv, const CM* __restrict__ q,
                                                        const double* __restrict__ wd, int64_t n, CgState* st,
                                                        double2* prho, double2* pw, CgCtl* ctl, int iter,
                                                        double delta, double2* __restrict__ u = nullptr,
                                                        const double2* __restrict__ Sinv = nullptr) {
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
    if constexpr (GRAD) {
      u[e] = cmul(Sinv[e / K], re);
    } else {
      rr += re.x * re.x - re.y * re.y;
      ri += 2 * re.x * re.y;
    }
    ww += (re.x * re.x + re.y * re.y) * wd[e / K];
  }
  if constexpr (!GRAD) block_reduce_rhs<K>(make_double2(rr, ri), smem, prho + (int64_t)blockIdx.x * K);
  block_reduce_rhs<K>(make_double2(ww, 0.0), smem, pw + (int64_t)blockIdx.x * K);
  if (arrive_last(&ctl->counter)) {
    const int my = threadIdx.x < K ? threadIdx.x : 0;
    double2 rho = make_double2(0.0, 0.0);
    if constexpr (!GRAD) rho = sum_partials<K>(prho, gridDim.x, my, smem);
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
        else if (S.res <= delta * S.res0 || S.res > 1e3 * S.res0) atomicOr(&stop, 1);
      } else if constexpr (!GRAD) {
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

// x += S y
template <int K>
__global__ void k_cg_xupdate(const double2* __restrict__ y, const double2* __restrict__ S, int64_t n, double2* x) {
  const int64_t total = n * K;
  for (int64_t e = (int64_t)blockIdx.x * kThreads + threadIdx.x; e < total; e += (int64_t)gridDim.x * kThreads)
    x[e] = dadd(x[e], cmul(S[e / K], y[e]));
}

size_t cg_layout(const Plan& P, size_t* off /* 28 */) {
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
  // complex128, one RHS: rows sorted by length for the product (perm, sort keys, sort workspace)
  const bool sorted = P.prec == 0 && P.k == 1 && P.n < (int64_t(1) << 31);
  put(14, sorted ? sizeof(int32_t) * P.n : 0);
  put(15, sorted ? sizeof(uint64_t) * P.n : 0);
  put(16, sorted ? pg::sort_workspace_bytes(P.n) : 0);
  // gradient correction: S^-1, diag(G^T A G)^-1, u = S^-1 r, t = invD G^T u, z
  put(17, P.gn ? sizeof(double2) * P.n : 0);
  put(20, P.gn ? sizeof(double2) * P.gn : 0);
  put(21, P.gn ? sizeof(double2) * P.n * P.k : 0);
  put(22, P.gn ? sizeof(double2) * P.gn * P.k : 0);
  put(23, P.gn ? sizeof(double2) * P.n * P.k : 0);
  return o;
}

// variant 0: rows in order, lanes per row from the row length; 2 / 4: rows
// in length order (perm) with 2 / 4 lanes per row
template <typename CM>
void launch_cg_spmv(const Plan& P, const int64_t* rowptr, const int32_t* col, const CM* val, const CM* pm,
                    const double2* p64, CM* q, double2* partial, CgState* st, CgCtl* ctl, int64_t npr, int grid,
                    cudaStream_t s, int variant = 0, const int32_t* perm = nullptr) {
  if (P.k == 1 && perm && variant == 2) {
    k_cg_spmv_sorted<CM, 2><<<grid, kThreads, 0, s>>>(rowptr, col, val, P.n, perm, pm, p64, q, partial, st, ctl);
    return;
  }
  if (P.k == 1 && perm && variant == 4) {
    k_cg_spmv_sorted<CM, 4><<<grid, kThreads, 0, s>>>(rowptr, col, val, P.n, perm, pm, p64, q, partial, st, ctl);
    return;
  }
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
  size_t off[28];
  cg_layout(P, off);
  const bool bj = P.bj.p > 0;
  double2* Sblk = reinterpret_cast<double2*>(ws + off[18]);
  double2* r64b = reinterpret_cast<double2*>(ws + off[19]);
  const bool sorted = P.prec == 0 && P.k == 1 && P.n < (int64_t(1) << 31);
  int32_t* perm = sorted ? reinterpret_cast<int32_t*>(ws + off[14]) : nullptr;
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
  // gradient correction (diagonal Jacobi, complex128 only; checked by pg_cocg)
  const bool grad = P.gn > 0;
  double2* Sinv = reinterpret_cast<double2*>(ws + off[17]);
  double2* invD = reinterpret_cast<double2*>(ws + off[20]);
  double2* gu = reinterpret_cast<double2*>(ws + off[21]);
  double2* gt = reinterpret_cast<double2*>(ws + off[22]);
  double2* gz = reinterpret_cast<double2*>(ws + off[23]);
  const unsigned gblocks = pg_blocks(P.gn * P.k, kThreads);
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
  if (sorted) {
    uint64_t* keys = reinterpret_cast<uint64_t*>(ws + off[15]);
    k_row_len_keys<<<pg_blocks(P.n, 256), 256, 0, s>>>(rowptr, P.n, keys, perm);
    PG_LAUNCH_CHECK();
    const int st0 = pg::sort_pairs(keys, perm, P.n, 32, ws + off[16], pg::sort_workspace_bytes(P.n), s);
    if (st0) return st0;
  }
  int variant = 0;
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
    if (grad) {
      k_grad_sinv<<<pg_blocks(P.n, 256), 256, 0, s>>>(S, P.n, Sinv);
      k_grad_diag<<<pg_blocks(P.gn * 32, 256), 256, 0, s>>>(rowptr, col, A, o->gradt_rowptr, o->gradt_row, o->gradt_val,
                                                       P.gn, invD);
    }
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
  std::vector<int> rec_done(k, 0);
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
    if (grad) {
      bool stalled = false, live = false;
      for (int i = 0; i < k; ++i) {
        if (!wnt[i]) continue;
        if (rec_done[i]) {
          stalled = true;
          wnt[i] = 0;
        } else {
          live = true;
        }
      }
      if (stalled && !live) {
        pg_set_error("pg_cocg: the recurrence reached rtol but the true residual did not (attainable accuracy of "
                     "the system in FP64)");
        status = PG_ERR_NOT_CONVERGED;
        break;
      }
    }
    PG_CUDA_TRY(cudaMemcpyAsync(target, tgt.data(), sizeof(double) * k, cudaMemcpyHostToDevice, s));
    PG_CUDA_TRY(cudaMemcpyAsync(want, wnt.data(), sizeof(int) * k, cudaMemcpyHostToDevice, s));
    if (bj) PG_KSWITCH(k, (k_bj_apply<K><<<pg_blocks(P.n * K, 256), 256, 0, s>>>(Sblk, P.bj, r64, r64b)));
    if (grad && !first) {
      PG_CUDA_TRY(cudaMemsetAsync(y, 0, sizeof(double2) * P.n * k, s));
      PG_KSWITCH(k, (k_cg_cycle_keep<K><<<1, 32, 0, s>>>(st, target, want, ctl)));
    } else if (grad) {
      // r = S r64, then z = r + S^-1 G invD G^T r64 (S^-1 r = r64), rho = r^T z
      PG_KSWITCH(k, (k_cg_start<CM, K><<<nb, kThreads, 0, s>>>(r64, S, P.n, r, y, pv, pm, 0, write_pm, part),
                     k_grad_restrict<K><<<gblocks, kThreads, 0, s>>>(o->gradt_rowptr, o->gradt_row, o->gradt_val,
                                                                     invD, r64, P.gn, gt, st, -1),
                     k_grad_prolong<K><<<nb, kThreads, 0, s>>>(o->grad_rowptr, o->grad_col, o->grad_val, Sinv, gt, r,
                                                               P.n, gz, pv, first ? 1 : 0, part, st, ctl, -1),
                     k_cg_cycle_init<K><<<1, 32 * K, 0, s>>>(part, nb, st, rnorm, target, want, ctl, first ? 1 : 0)));
    } else {
      PG_KSWITCH(k, (k_cg_start<CM, K><<<nb, kThreads, 0, s>>>(bj ? r64b : r64, S, P.n, r, y, pv, pm, first ? 1 : 0,
                                                               write_pm, part),
                     k_cg_cycle_init<K><<<1, 32 * K, 0, s>>>(part, nb, st, rnorm, target, want, ctl, first ? 1 : 0)));
    }
    if (first && sorted && autotune_enabled()) {
      // the product is the first kernel of an iteration and recomputes alpha,
      // so timing the candidates on the live operands changes no state
      variant = pick_fastest({0, 2, 4}, [&](int v) {
        launch_cg_spmv<CM>(P, rowptr, col, At, pm, pv, q, part, st, ctl, npr, spmv_grid, s, v, perm);
      }, s);
      PG_LAUNCH_CHECK();
      if (monitor) fprintf(stderr, "pg_cocg: product variant %d for n=%lld nnz=%lld\n", variant, (long long)P.n,
                           (long long)P.nnz);
    }
    first = false;
    const int steps = (int)((max_it - its) < chunk ? (max_it - its) : chunk);
    const double delta = P.prec ? 0.1 : 0.0;
    for (int it = 0; it < steps; ++it) {
      const int iter = (int)(launch_iter + it);
      launch_cg_spmv<CM>(P, rowptr, col, At, pm, pv, q, part, st, ctl, npr, spmv_grid, s, variant, perm);
      if (grad) {
        PG_KSWITCH(k, (k_cg_update<CM, K, true><<<nbu, kThreads, 0, s>>>(y, r, pv, q, wd, P.n, st, part, part2, ctl,
                                                                        iter, delta, gu, Sinv),
                       k_grad_restrict<K><<<gblocks, kThreads, 0, s>>>(o->gradt_rowptr, o->gradt_row, o->gradt_val,
                                                                       invD, gu, P.gn, gt, st, iter),
                       k_grad_prolong<K><<<nbu, kThreads, 0, s>>>(o->grad_rowptr, o->grad_col, o->grad_val, Sinv, gt,
                                                                  r, P.n, gz, pv, 0, part, st, ctl, iter),
                       k_cg_pupdate<CM, K><<<pg_blocks(P.n * K, kThreads), kThreads, 0, s>>>(pv, pm, gz, P.n, st,
                                                                                            iter, write_pm)));
      } else {
        PG_KSWITCH(k, (k_cg_update<CM, K><<<nbu, kThreads, 0, s>>>(y, r, pv, q, wd, P.n, st, part, part2, ctl, iter,
                                                                  delta),
                       k_cg_pupdate<CM, K><<<pg_blocks(P.n * K, kThreads), kThreads, 0, s>>>(pv, pm, r, P.n, st, iter,
                                                                                            write_pm)));
      }
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
    std::vector<int> hact(k);
    for (int i = 0; i < k; ++i) {
      PG_CUDA_TRY(cudaMemcpyAsync(&hits[i], &st[i].its, sizeof(int), cudaMemcpyDeviceToHost, s));
      PG_CUDA_TRY(cudaMemcpyAsync(&hbrk[i], &st[i].breakdown, sizeof(int), cudaMemcpyDeviceToHost, s));
      PG_CUDA_TRY(cudaMemcpyAsync(&hact[i], &st[i].active, sizeof(int), cudaMemcpyDeviceToHost, s));
    }
    PG_CUDA_TRY(cudaStreamSynchronize(s));
    if (grad) {
      // a recurrence that met its target ends; if its true residual then
      // misses rtol, the attainable accuracy is reached (checked below)
      for (int i = 0; i < k; ++i) rec_done[i] = rec_done[i] || (wnt[i] && !hact[i]);
    }
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
  if (status == PG_ERR_NOT_CONVERGED && its >= max_it) pg_set_error("pg_cocg: max_it reached before rtol");
  return status;
}

}  // namespace

using pgk::df_layout;
using pgk::ir_layout;
using pgk::run_cocg_df;
using pgk::run_cocg_ir;
extern "C" void pg_cocg_default_opts(pg_cocg_opts* o) {
  if (!o) return;
  memset(o, 0, sizeof(*o));
  o->max_it = 100000;
  o->rtol = 1e-8;
  o->precision = 0;
  o->check_every = 50;
  o->inner_rtol = 0.0;   // the solver's default: 1e-2, or 1e-4 with the gradient correction
}

extern "C" size_t pg_cocg_workspace_bytes(int64_t n, int64_t nnz, int nrhs, const pg_cocg_opts* opts) {
  if (!opts || n < 1 || !valid_k(nrhs)) return 0;
  Plan P = cg_plan(n, nnz, nrhs, opts);
  size_t off[28];
  if (opts->precision == 3) return ir_layout(P, off) + 256;
  return (opts->precision == 2 ? df_layout(P, off) : cg_layout(P, off)) + 256;
}

extern "C" int pg_cocg(const int64_t* rowptr, const int32_t* col, const double* vals, int64_t n, int64_t nnz,
                       const double* b, double* x, int nrhs, const pg_cocg_opts* opts, pg_gmres_result* result,
                       double* relres_per_rhs, void* workspace, size_t workspace_bytes, void* stream) {
  if (!opts || !rowptr || !col || !vals || !b || !x || n < 1 || nnz < n || !valid_k(nrhs) || !(opts->rtol > 0.0) ||
      opts->precision < 0 || opts->precision > 3) {
    pg_set_error("pg_cocg: bad argument (nrhs 1..32 power of two, rtol > 0, precision 0/1/2/3)");
    return PG_ERR_ARG;
  }
  if (opts->grad_rowptr) {
    if (!opts->grad_col || !opts->grad_val || !opts->gradt_rowptr || !opts->gradt_row || !opts->gradt_val ||
        opts->grad_cols < 1 || opts->grad_cols >= (int64_t(1) << 31) || opts->block_p > 0 ||
        opts->precision == 1) {
      pg_set_error("pg_cocg: gradient correction needs all six G arrays, grad_cols >= 1, precision 0, 2 or 3 and "
                   "diagonal Jacobi (block_p 0)");
      return PG_ERR_ARG;
    }
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
  if (P.prec == 3) return run_cocg_ir(P, rowptr, col, A, bb, xx, opts, result, relres_per_rhs, ws, s);
  return run_cocg<float2>(P, rowptr, col, A, bb, xx, opts, result, relres_per_rhs, ws, s);
}

